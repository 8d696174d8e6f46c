// Device-side layout of a batch of raw-physics scenes (shared by host and device code).
//
// A "scene" is what one pbd_simulate_with_constraints call advances: its bodies (entities), their
// colliders, its external constraints. A batch is any number of independent scenes laid out back to
// back; the plain single-scene form is a batch of one. All arrays live in HBM; per-scene ranges
// are prefix offsets. Poses are FP64 (the reference's r64 world_position / world_rotation); the
// remaining per-body quantities use the build's working type R (float for the FP32 build, double
// for the exact all-FP64 build).
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace rp {

// Status bits reported by the step kernel (rp_status values of the C ABI are built from them).
enum : uint32_t {
    ST_PAIR_OVERFLOW = 1u << 0,      // broad-phase pair list exceeded its capacity
    ST_CONTACT_OVERFLOW = 1u << 1,   // contact buffer exceeded its capacity
    ST_EPA_OVERFLOW = 1u << 2,       // EPA polytope outgrew its fixed per-warp storage
    ST_CLIP_OVERFLOW = 1u << 3,      // clipped polygon outgrew its per-warp storage
    ST_BARRIER_TIMEOUT = 1u << 4,    // a bounded grid barrier gave up; the frame was abandoned
    ST_DEGENERATE = 1u << 5,         // input the reference would reject with an assert
    ST_LEVEL_OVERFLOW = 1u << 6,     // dependency depth exceeded the level table
    ST_EPA_NOT_CONVERGED = 1u << 8,  // informational: the reference prints "EPA did not converge."
    // which degenerate condition set ST_DEGENERATE (each comes with it)
    ST_DEG_EPA_NORMAL = 1u << 9,     // an EPA face whose normal vanishes (epa.cpp:41 asserts)
    ST_DEG_EPA_COPLANAR = 1u << 10,  // an EPA face through the origin with every point in its plane (epa.cpp:72)
    ST_DEG_SKEW = 1u << 11,          // edge-edge contact of parallel edges (clipping.cpp:279)
    ST_DEG_MASK = ST_DEG_EPA_NORMAL | ST_DEG_EPA_COPLANAR | ST_DEG_SKEW,
};

// Collider kinds (Collider_Type, src/physics/collider.h:33-36)
enum : int32_t { COL_SPHERE = 0, COL_HULL = 1 };

// External constraint kinds (Constraint_Type, src/physics/pbd.h:14-20)
enum : int32_t { CON_POSITIONAL = 0, CON_COLLISION = 1, CON_MUTUAL_ORIENTATION = 2, CON_HINGE = 3, CON_SPHERICAL = 4 };

// One external constraint (the union of src/physics/pbd.h:22-77); lambdas live in the
// per-substep scratch copy, as copy_constraints resets them every substep (pbd.cpp:426-462).
struct ExtConstraint {
    int32_t type, e1, e2;    // e1/e2: global body indices
    int32_t a1, a2;          // hinge aligned axes | spherical swing axes
    int32_t l1, l2;          // hinge limit axes | spherical twist axes
    int32_t limited;
    double r1[3], r2[3];
    double compliance;
    double distance[3];
    double lo, hi;           // hinge limits | spherical swing limits
    double lo2, hi2;         // spherical twist limits
    float r1f[3], r2f[3];    // FP32 roundings of r1, r2 and compliance (the FP32 build's operands)
    float compliance_f;
};

struct Shape {               // one convex hull's topology (collider_convex_hull_create output)
    int32_t nv, nf;
    int32_t vert_off;        // into shape_verts (local, pre-scaled vertices, FP64)
    int32_t face_off;        // into face_normal (this hull's geometry)
    int32_t elem_off;        // into face_elem_start; the topology tables (elem_off, v2f/v2n/f2n_off) are
                             //     shared by every hull of one topology (scaled copies of one mesh)
    int32_t v2f_off, v2n_off;   // into csr_start for vertex -> faces, vertex -> neighbours
    int32_t f2n_off;            // into csr_start for face -> neighbour faces
    int32_t max_face_valence;
    int32_t max_face_neighbours;
};

// Per-pair state between the narrowphase kernels of the phase-major pipeline
enum : int32_t { WS_NONE = 0, WS_HIT = 1, WS_GENERAL = 2, WS_EPA_OK = 3, WS_EPA_FACE = 4, WS_FALLBACK = 5 };

// Phases of the step timed per frame (rp_phase_times). The persistent kernel times the whole
// narrowphase as PH_NARROW; the phase-major form splits it into the cull (PH_NARROW), GJK, EPA and
// contact-manifold kernels.
enum { PH_BROAD = 0, PH_ISLANDS, PH_SCHEDULE, PH_PREDICT, PH_TRANSFORM, PH_NARROW, PH_SOLVE, PH_VELOCITY, PH_VSOLVE,
       PH_GJK, PH_EPA, PH_MANIFOLD, PHASES };

struct StepParams {          // the arguments of pbd_simulate_with_constraints
    double dt;
    int32_t num_substeps;
    int32_t num_pos_iters;
    int32_t enable_collisions;
    int32_t pad;
};

struct Collider {
    int32_t type;           // COL_SPHERE / COL_HULL
    int32_t shape;           // hull: shape index
    float radius;            // sphere radius (the reference stores r32)
    int32_t tv_off;          // hull: offset of this collider's transformed vertices / normals
    int32_t tn_off;
};

template <typename R>
struct WorldView {
    // ---- batch layout --------------------------------------------------------------------
    int32_t num_scenes;
    const int32_t* scene_body;     // [S+1] body ranges
    const int32_t* scene_ext;      // [S+1] external constraint ranges
    const int32_t* scene_pair_cap; // [S+1] pair scratch ranges (capacity)
    const int32_t* scene_contact_cap; // [S+1] contact scratch ranges (capacity)
    const int32_t* scene_node_cap; // [S+1] solver node scratch ranges (ext + pairs)
    // ---- body state (mutable) ------------------------------------------------------------
    double4_32a* pos;        // world_position (w unused)
    double4_32a* rot;        // world_rotation (x, y, z, w)
    double4_32a* prev_pos;
    double4_32a* prev_rot;
    R* vel;              // [3N] linear_velocity
    R* omega;            // [3N] angular_velocity
    R* prev_vel;         // [3N]
    R* prev_omega;       // [3N]
    uint8_t* active;
    double* deact;       // deactivation_time
    // ---- body constants -------------------------------------------------------------------
    const R* inv_mass;
    const R* inertia;       // [6N] local inertia tensor, symmetric storage
    const R* inv_inertia;   // [6N]
    const R* material;      // [4N] static friction, dynamic friction, restitution, (unused)
    const double* radius;   // bounding_sphere_radius
    const float4* bound;    // [2N] geometric bound of the body's hulls in its local frame, rounded
                            // outwards: (box centre xyz, radius of the vertices about the body origin),
                            // (box half extents xyz, 1 when the body has a box, 0 when it has none)
    const uint8_t* fixed;
    const int32_t* col_start;   // [N+1] collider ranges
    const double* force;     // [3N] sum of external forces (calculate_external_force)
    const double* torque;    // [3N] sum of external torques (calculate_external_torque)
    // ---- geometry -------------------------------------------------------------------------
    const Collider* colliders;
    const Shape* shapes;
    const double* shape_verts;   // [3 * total verts] local vertices
    const double* face_normal;   // [3 * total faces] local face normals
    const float* shape_verts_f;  // FP32 copies of shape_verts / face_normal (the FP32 build's
    const float* face_normal_f;  // transform reads them without FP64 conversions)
    const int32_t* face_elem_start;  // [faces of the distinct topologies + 1] CSR starts (from Shape::elem_off)
    const int32_t* face_elem;        // vertex indices of faces
    const int32_t* csr_start;        // shared CSR start table for v2f / v2n / f2n
    const int32_t* csr_data;
    R* tverts;       // [3 * total transformed verts] transformed hull vertices (per collider)
    R* tnorms;       // [3 * total transformed normals]
    // ---- constraints ----------------------------------------------------------------------
    const ExtConstraint* ext;
    // ---- scratch ---------------------------------------------------------------------------
    int32_t* pair_count;     // [S] pairs found this step
    int2* pairs;             // broad-phase pairs (global body indices), in reference order
    int32_t* row_count;      // [N] broad-phase counts per row (scan workspace)
    uint32_t* sort_key;      // [2N] sort-based broad phase: radix-sort keys (ping-pong)
    int32_t* sort_val;       // [2N] body indices travelling with the keys
    int32_t* sort_hist;      // [256 * ceil(N / 256)] digit counts per tile of 256 keys
    float* sort_hi;          // [N] upper end of each body's x interval
    int32_t* uf_parent;      // [N] union-find parents (global body indices)
    uint8_t* island_awake;   // [N] per-root flag
    int32_t* node_body;      // [2 * nodes] the node's two bodies (-1 when fixed)
    int32_t* node_pred;      // [2 * nodes] predecessor node on each body (-1: none)
    int32_t* node_level;     // [nodes]
    int32_t* body_tl_count;  // [N] timeline lengths / fill counters
    int32_t* body_tl_start;  // [N+1] timeline CSR starts (per scene relative to node base)
    int32_t* body_tl;        // [2 * nodes] timeline entries
    // the substep's two sweep schedules (resched): position sweep (node_pred, node_level, level_*,
    // scene_levels) and velocity sweep (node_vpred, node_vlevel, vlevel_*, scene_vlevels)
    int32_t* level_count;    // [S * (max_levels+1)] nodes per level, then prefix
    int32_t* level_fill;     // [S * (max_levels+1)] fill counters; the last three words are flags
    int32_t* scan_tmp;       // [grid blocks] group-scan partial sums
    int32_t* level_nodes;    // [nodes] nodes sorted by level
    int32_t* scene_levels;   // [S] number of levels
    int32_t* node_vpred;     // [2 * nodes]
    int32_t* node_vlevel;    // [nodes]
    int32_t* vlevel_count;   // [S * (max_levels+1)]
    int32_t* vlevel_fill;    // [S * (max_levels+1)]
    int32_t* vlevel_nodes;   // [nodes]
    int32_t* scene_vlevels;  // [S]
    int32_t* act_list;       // [2 * nodes] active nodes of each schedule (position, then velocity)
    int32_t* act_count;      // [2 * S] their counts (zeroed by the substep's predict phase)
    int32_t sweep_order;     // SWEEP_REFERENCE (the reference's serial order) or SWEEP_COLOURED
    uint32_t* node_bits;     // [nodes / 32 + 1] phase-major form: bit (scene node base + k) set when pair node
                             //     k has contacts this substep (cleared before every substep's narrowphase)
    int32_t* scene_nodes;    // [S] number of live nodes (ext + pairs)
    int32_t* pair_cstart;    // [pairs] first contact of each pair
    int32_t* pair_ccount;    // [pairs]
    int32_t* contact_count;  // [S] contacts allocated this substep
    int32_t* work;           // [S] next broad-phase pair to narrowphase (dynamic work distribution)
    R* contacts;             // [12 * contacts] r1_lc, lambda_n, r2_lc, lambda_t, normal, (unused)
    double* ext_lambda;      // [4 * ext] per-substep lambdas of external constraints
    int32_t max_levels;
    // ---- phase-major pipeline (one kernel per phase over every scene of the batch) ----------
    const int32_t* body_scene;   // [N] scene of each body
    float4* pose_f;              // [2N] FP32 copy of the predicted pose (xyz, 0), (quaternion), written
                                 // by the predict phase (the orientation refreshed by the fold)
    float4* sdx;                 // [N] FP32 build: the position sweep's accumulated position correction
    float4* sdq;                 // [N]                 and orientation correction (delta form)
    float4* pred_d;              // [N] FP32 build: (float)(predicted position - previous position)
    float4* prev_qf;             // [N]             (float) previous orientation
    const int32_t* col_body;     // [colliders] body of each collider
    const uint8_t* single_hull;  // [bodies] 1: the body's only collider is a hull of at most 64 vertices
                                 //     (the narrowphase warp kernels' case)
    int32_t* work_list;          // [pair capacity] global pair slots narrowphased this frame
    int32_t* work_state;         // [pair capacity] per work item: WS_* below
    int32_t* gjk_list;           // [pair capacity] work items needing GJK this substep (queue[2] of them)
    int32_t* hit_list;           // [pair capacity] work items needing a manifold this substep (queue[3])
    R* work_simplex;             // [16 * pair capacity] GJK simplex of a hit (a, b, c, d)
    double* work_epa;            // [4 * pair capacity] EPA normal (FP64) and penetration of a hit
    float4* pair_base;           // [pair capacity] FP32 build: (float)(x_a - x_b) of a pair slot's predicted
                                 //     positions, rounded once per substep (the sweeps' solve frame)
    float4* ext_base;            // [external constraints] the same for each joint's two bodies
    float4* work_off;            // [pair capacity] FP32 build: body b's origin relative to body a's (xyz; the
                                 //     FP64 difference rounded once per pair and substep by k_cull)
    int32_t* fallback_list;      // [pair capacity] FP32 build: work items whose FP32 EPA or edge contact met a
                                 //     degenerate configuration, redone in FP64 (queue[5] of them)
    float* work_face;            // [12 * pair capacity] FP32 build: EPA's final face (three Minkowski points)
                                 //     and its FP32 normal, finished in FP64 by k_epa_finish
    int32_t* tstamp;             // [bodies] the substep (queue[4]) whose hull transform list took the body last
    int32_t* tlist;              // [bodies] bodies whose hulls this substep transforms (queue[7] of them)
    int32_t* queue;              // [16] [0] work items this frame, [1] next scene of a warp-per-scene sweep,
                                 //     [2] gjk_list length, [3] hit_list length, [4] substeps run since
                                 //     the world was built (phase-major form), [5] fallback_list length,
                                 //     [6] next of the CTA-swept scenes, [7] tlist length
    const int32_t* scene_order;  // [S] scenes by decreasing size (the order warps take them in)
    int32_t cta_scenes;          // the first cta_scenes of scene_order are swept by a whole CTA each
    int32_t max_colliders_per_body;
    int32_t solo_nodes;          // grid sweeps: levels of at most this many nodes run on CTA 0 alone
    // ---- control ----------------------------------------------------------------------------
    uint32_t* status;        // [S] status bits per scene
    unsigned int* barrier;   // [1] grid barrier arrival counter (zeroed before each launch sequence)
    unsigned long long wait_ns;   // bound of every device-side wait (grid barriers), nanoseconds
    unsigned long long* counters; // [32] diagnostics: gjk/epa iterations and cap hits, contacts, pair cycles
    unsigned long long* phase_ns; // [PHASES] time spent per phase of the step, seen by group rank 0
    int32_t* deg_first;      // [8] first degenerate condition met: ST_DEG_* bits (0: none yet), scene,
                             //     body slots a and b of the pair, substep (queue[4]) it was met in
};

}  // namespace rp
