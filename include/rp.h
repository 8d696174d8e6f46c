/*
 * raw-physics GB300 — C ABI of the rigid-body step.
 *
 * The hot path of raw-physics is one call per rendered frame,
 *   pbd_simulate_with_constraints(dt, entities, constraints, substeps, pos_iters, collisions)
 *   (src/physics/pbd.h:93-94, src/physics/pbd.cpp:468-747),
 * fed by the entity / collider / constraint API around it. This header exposes the same operations
 * over plain pointers and sizes, with every step computed by CUDA kernels on one GB300:
 *
 *   reference                                   this ABI
 *   collider_convex_hull_create (collider.h:48)   rp_hull_create
 *   collider_sphere_create      (collider.h:49)   rp_collider_desc{RP_COLLIDER_SPHERE, ...}
 *   entity_create / _fixed      (entity.h:52-55)  rp_entity_create
 *   entity_add_force            (entity.h:65)     rp_entity_add_force
 *   entity_clear_forces         (entity.h:66)     rp_entity_clear_forces
 *   pbd_*_constraint_*_init     (pbd.h:96-102)    rp_constraint_*
 *   pbd_simulate(_with_constraints) (pbd.h:93-94) rp_simulate
 *   Entity fields read/written in place          rp_state_get / rp_state_set (snapshot/restore)
 *   broad_get_collision_pairs   (broad.h:11)      rp_broad_pairs
 *   colliders_get_contacts      (collider.h:55)   rp_contacts
 *   obj_parse (src/render/obj.cpp:7) + examples_util_create_single_convex_hull_collider_array
 *                               (examples_util.cpp:5) rp_hull_from_obj
 *
 * Beyond the reference: the adjoint of the step (rp_adjoint_trajectory), a hull topology cache
 * (rp_hull_save / rp_hull_load), launch-mode control and an autotuner, a no-allocation contact
 * query, and diagnostics.
 *
 * Entities are numbered in creation order (the order entity_get_all returns, entity.cpp:88).
 * A world holds one or more independent scenes; rp_simulate advances all of them in one launch
 * (the batched form). Every function returns RP_OK or a negative rp_status; nothing aborts.
 *
 * The C++-mangled pbd_simulate / pbd_simulate_with_constraints drop-in built on this ABI is declared
 * in include/rp_compat.h.
 */
#ifndef RP_GB300_H
#define RP_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rp_world rp_world;
typedef int32_t rp_status;

enum {
    RP_OK = 0,
    RP_ERR_INVALID = -1,        /* bad argument (unknown entity, bad size, NaN pose, ...) */
    RP_ERR_CUDA = -2,           /* a CUDA call failed (message in rp_last_error) */
    RP_ERR_NO_DEVICE = -3,      /* no CUDA device / the CUDA extension cannot run here */
    RP_ERR_CAPACITY = -4,       /* a scratch buffer could not be grown enough */
    RP_ERR_DEGENERATE = -5,     /* geometry the reference rejects with an assert */
    RP_ERR_TIMEOUT = -6,        /* a bounded device-side wait gave up */
    RP_ERR_STATE = -7           /* call not allowed in the current state */
};

enum { RP_PRECISION_FP32 = 0, RP_PRECISION_FP64 = 1 };
/* RP_PRECISION_FP32: FP32 arithmetic, FP64 positions / orientations and EPA face test.
 * RP_PRECISION_FP64: every quantity in FP64, evaluated in the reference's operation order without
 *                    FMA contraction (reproduces the reference's FP64 results). */

/* How a frame is launched (rp_world_set_mode). Both give identical results.
 * RP_MODE_PHASED:     one small kernel per phase (setup, predict, hull transform, GJK, EPA, contact
 *                     manifold, position and velocity sweeps) over every scene, the frame replayed
 *                     from a captured CUDA graph. The default.
 * RP_MODE_PERSISTENT: one persistent kernel per frame (a CTA per scene, or a cooperative grid on a
 *                     single large scene).
 * RP_MODE_AUTO:       RP_MODE_PHASED unless the environment variable RP_MODE is "persistent". */
enum { RP_MODE_AUTO = 0, RP_MODE_PERSISTENT = 1, RP_MODE_PHASED = 2 };

enum { RP_COLLIDER_SPHERE = 0, RP_COLLIDER_HULL = 1 };        /* Collider_Type, collider.h:33-36 */
enum { RP_AXIS_POS_X = 0, RP_AXIS_NEG_X, RP_AXIS_POS_Y, RP_AXIS_NEG_Y, RP_AXIS_POS_Z, RP_AXIS_NEG_Z }; /* PBD_Axis_Type */

#define RP_STATE_DOUBLES 28
/* Per-entity state record of rp_state_get / rp_state_set (all FP64):
 *  0..2 world_position  3..6 world_rotation (x,y,z,w)  7..9 linear_velocity  10..12 angular_velocity
 * 13..15 previous_world_position  16..19 previous_world_rotation  20..22 previous_linear_velocity
 * 23..25 previous_angular_velocity  26 active (0/1)  27 deactivation_time */

#define RP_CONTACT_DOUBLES 9   /* rp_contacts record: collision_point1[3], collision_point2[3], normal[3] */

typedef struct {
    int32_t type;      /* RP_COLLIDER_SPHERE or RP_COLLIDER_HULL */
    int32_t hull;      /* hull id from rp_hull_create (hulls) */
    float radius;      /* sphere radius (spheres) */
} rp_collider_desc;

/* -- world ------------------------------------------------------------------------------------ */
/* device >= 0: a world on that CUDA device (a GPU of compute capability 10.x or newer is required).
 * device == -1: a host-only world for set-up queries (hulls, mass properties, state snapshots);
 * any call that needs the GPU then returns RP_ERR_NO_DEVICE. */
rp_status rp_world_create(rp_world** out, int32_t device, int32_t precision);
void      rp_world_destroy(rp_world* w);
/* Use an existing cudaStream_t (passed as void*) for every launch and copy of this world. */
rp_status rp_world_set_stream(rp_world* w, void* cuda_stream);
/* Adjoint of the step (no counterpart in the reference): for every scene, the loss
 * |x_e(T) - target|^2 of one entity e = loss_entity[scene] after `frames` frames (dt, substeps,
 * iterations and enable_collisions as rp_simulate, gravity as set, no other forces) and its gradient
 * with respect to every entity's initial linear and angular velocity (grad_v, grad_w: 3 doubles per
 * entity), mass (grad_mass) and static / dynamic friction (grad_friction, 2 per entity, may be NULL).
 * Everything the step does is differentiated: free motion, the external joints (positional, mutual
 * orientation, hinge, spherical, limits included) and, with collisions, hull-hull contacts (the EPA
 * normal and clipped contact points as functions of the poses, the normal and static-friction
 * solves, the velocity solver with dynamic friction and restitution). Discrete events are held
 * fixed: the broad-phase pairs and awake bodies of every frame, every branch (a limit or a contact
 * acting, static friction holding), the support features GJK, EPA and the clipping select; the
 * clipping's float roundings are differentiated as identity. Static friction only enters through a
 * comparison, so its gradient is zero. Scenes whose contact pairs involve sphere colliders report
 * RP_ERR_INVALID with collisions on. The forward pass is the all-FP64 step: its loss equals the FP64
 * build's. Reverse mode over a tape, one scene per GPU thread, with the trajectory checkpointed
 * every `checkpoint_every` frames and recomputed segment by segment. Starts from the world's current
 * state, which it does not change. target: 3 doubles per scene. */
rp_status rp_adjoint_trajectory(rp_world* w, double dt, uint32_t num_substeps, uint32_t num_pos_iters,
                                int32_t enable_collisions, uint32_t frames, uint32_t checkpoint_every,
                                const int32_t* loss_entity, const double* target, double* loss_out, double* grad_v,
                                double* grad_w, double* grad_mass, double* grad_friction);
rp_status rp_world_set_mode(rp_world* w, int32_t mode);
/* Gauss–Seidel order of the constraint sweeps. RP_SWEEP_REFERENCE (default): the reference's serial
 * order (pbd.cpp:615-620 and the velocity pass's loop), swept level by level over the substep's active
 * constraints; results are the reference's (bit for bit in RP_PRECISION_FP64). RP_SWEEP_COLOURED:
 * graph-coloured sweeps, constraints that share a dynamic body get different colours and the sweep
 * runs colour by colour; a different Gauss–Seidel order with fewer dependent steps (a joint chain takes
 * two or three colours instead of one step per link). Its results differ from the reference's by the
 * reordering (measured per-step error against the FP64 oracle: bench.py's step_err); the autotuner
 * then also picks the colouring's priority scheme. No counterpart in the reference. */
enum { RP_SWEEP_REFERENCE = 0, RP_SWEEP_COLOURED = 1 };
rp_status rp_world_set_sweep_order(rp_world* w, int32_t order);
/* How a batch's sweeps spread scenes over the GPU (a launch shape: the same schedule under every
 * choice, so FP64 results are identical and FP32 results agree to rounding):
 * 0 one warp per scene (the default), 1 one CTA per scene, n >= 2 a whole CTA for every scene whose
 * sweep cost (dynamic bodies + 8 per joint) is n or more and one warp for each other scene.
 * rp_autotune chooses among these (its choice[2]). No counterpart in the reference. */
rp_status rp_world_set_sweep_assignment(rp_world* w, int32_t cta);
/* Bound of every device-side wait of this world (the grid barriers of a single large scene's
 * cooperative kernels), in microseconds; 1 s by default, at most 60 s; 0 gives up at the first wait
 * that finds its barrier incomplete. A wait that runs out abandons the frame: every CTA leaves the
 * launch, the frame's remaining kernels return at once, rp_simulate restores the state it started
 * from and returns RP_ERR_TIMEOUT (forces stay pending). The world stays usable. No counterpart in
 * the reference, which has no device waits. */
rp_status rp_world_set_wait_limit(rp_world* w, uint64_t microseconds);
/* Autotuner (no counterpart in the reference): times `frames` frames of the world's current scenes
 * from their current state under each candidate launch configuration — launch mode, threads per
 * collider in the hull transform (4/8/16/32), and the sweep layout (levels swept by one CTA below
 * 128..2048 nodes for one large scene; for a batch, which scenes a warp and which a whole CTA sweeps) —
 * keeps the fastest, and restores the state. Every configuration runs the same schedule: results are
 * identical in RP_PRECISION_FP64 and agree to rounding in RP_PRECISION_FP32 (each kernel instantiation
 * may contract multiply-adds differently). Each candidate is timed twice; one replaces the default only
 * when at least 1 % faster. Call it with
 * no forces pending. choice receives {mode, transform threads, batch sweep assignment (0: a warp per
 * scene, 1: a CTA per scene, n >= 2: a CTA for scenes of n or more bodies plus 8 per joint, a warp for
 * the rest), solo level size}. */
rp_status rp_autotune(rp_world* w, double dt, uint32_t num_substeps, uint32_t num_pos_iters, int32_t enable_collisions,
                      uint32_t frames, int32_t choice[4]);
const char* rp_last_error(void);
/* Adds a new empty scene; scene 0 exists from creation. */
rp_status rp_scene_create(rp_world* w, int32_t* out_scene);

/* -- geometry ---------------------------------------------------------------------------------- */
/* collider_convex_hull_create (src/physics/collider.cpp:194-364) from a triangle list: num_vertices
 * FP64 positions (already scaled, as examples_util.cpp:5-24 does) and num_indices indices
 * (3 per triangle, counter-clockwise seen from outside). Identical hulls are shared. */
rp_status rp_hull_create(rp_world* w, const double* vertices, uint32_t num_vertices, const uint32_t* indices,
                         uint32_t num_indices, int32_t* out_hull);
/* A hull whose topology the caller already holds, in the reference's Collider_Convex_Hull form
 * (collider.h:15-24) flattened to CSR: unique vertices, face normals, face boundary loops, and the
 * vertex->faces, vertex->neighbours, face->neighbours lists, each *_start array having one more entry
 * than rows. Used by the pbd_simulate drop-in, which forwards the caller's own colliders. */
rp_status rp_hull_create_from_topology(rp_world* w, const double* vertices, int32_t num_vertices, const double* face_normals,
                                       int32_t num_faces, const int32_t* face_start, const int32_t* face_elements,
                                       const int32_t* v2f_start, const int32_t* v2f, const int32_t* v2n_start,
                                       const int32_t* v2n, const int32_t* f2n_start, const int32_t* f2n,
                                       int32_t* out_hull);
/* Hull preprocessing (no counterpart in the reference, which rebuilds every hull from its OBJ file at
 * start-up). rp_hull_from_obj: a hull from an OBJ file's `v` and `f` lines (indices 1-based or
 * negative; texture / normal indices ignored), one vertex per face corner in face order and positions
 * stored as FP32 then scaled per axis in FP64, as obj_parse (src/render/obj.cpp:7-80) and
 * examples_util.cpp:5-24 do, polygons triangulated by the ear clipping of the reference's OBJ
 * loader (tinyobj, include/tiny_obj_loader.h) so that the corner order is the reference's.
 * rp_hull_save writes a built hull's
 * topology to a binary file (little-endian, checksummed); rp_hull_load restores it without
 * rebuilding (RP_ERR_INVALID on a bad or corrupt file). */
rp_status rp_hull_from_obj(rp_world* w, const char* path, const double scale[3], int32_t* out_hull);
rp_status rp_hull_save(rp_world* w, int32_t hull, const char* path);
rp_status rp_hull_load(rp_world* w, const char* path, int32_t* out_hull);
/* Topology queries of a built hull (for tests): counts, then the arrays. */
rp_status rp_hull_info(rp_world* w, int32_t hull, int32_t* num_vertices, int32_t* num_faces);
/* One topology table of a hull in CSR form: which = 0 face boundary loops, 1 vertex->faces,
 * 2 vertex->neighbours, 3 face->neighbours. start_out gets rows+1 entries, data_out the entries;
 * either may be NULL to query *num_rows / *num_data first. */
rp_status rp_hull_topology(rp_world* w, int32_t hull, int32_t which, int32_t* start_out, int32_t* data_out, int32_t cap,
                           int32_t* num_rows, int32_t* num_data);
/* Unique vertices (3 per vertex) and face normals (3 per face) of a hull, FP64. */
rp_status rp_hull_geometry(rp_world* w, int32_t hull, double* vertices_out, double* normals_out);
rp_status rp_hull_face(rp_world* w, int32_t hull, int32_t face, double normal[3], int32_t* elements, int32_t cap,
                       int32_t* num_elements);

/* -- entities ------------------------------------------------------------------------------------ */
/* entity_create / entity_create_fixed (src/entity.cpp:24-65): bounding radius, inverse mass and the
 * point-mass inertia tensor are derived as the reference derives them. Returns the entity index. */
rp_status rp_entity_create(rp_world* w, int32_t scene, const double position[3], const double rotation[4], double mass,
                           int32_t fixed, const rp_collider_desc* colliders, uint32_t num_colliders,
                           double static_friction, double dynamic_friction, double restitution, int32_t* out_entity);
rp_status rp_entity_set_velocity(rp_world* w, int32_t entity, const double linear[3], const double angular[3]);
/* n calls of rp_entity_create with one collider each (cols[i]), plus optional initial velocities
 * (vel / omega: 3 doubles per entity, or NULL for zero); arrays hold one entry per entity (pos: 3,
 * rot: 4). All or nothing: on error no entity is added. *out_first receives the first new entity.
 * Bulk form for batches of many scenes; no counterpart in the reference. */
rp_status rp_entities_create(rp_world* w, uint32_t n, const int32_t* scene, const double* pos, const double* rot,
                             const double* mass, const int32_t* fixed, const rp_collider_desc* cols, const double* mus,
                             const double* mud, const double* rest, const double* vel, const double* omega,
                             int32_t* out_first);
/* entity_add_force: applies to every frame of the next rp_simulate call and is then cleared, as the
 * reference's callers clear forces after every frame (src/examples/stack.cpp:100-102). */
rp_status rp_entity_add_force(rp_world* w, int32_t entity, const double position[3], const double force[3],
                              int32_t local_coords);
rp_status rp_entity_clear_forces(rp_world* w, int32_t entity);
/* Persistent gravity: before every step each entity gets the force (0, -g / inverse_mass, 0), added
 * after its other forces, as the example scenes do (src/examples/stack.cpp:93-96). 0 disables it. */
rp_status rp_world_set_gravity(rp_world* w, double g);
rp_status rp_entity_get_mass_properties(rp_world* w, int32_t entity, double* inverse_mass, double inertia[9],
                                        double inverse_inertia[9], double* bounding_radius);
/* Overrides what rp_entity_create derived (a caller that edited Entity::inverse_mass or the
 * inertia tensors, as the drop-in forwards them). Row-major 3x3 tensors; must be symmetric. */
rp_status rp_entity_set_mass_properties(rp_world* w, int32_t entity, double inverse_mass, const double inertia[9],
                                        const double inverse_inertia[9], double bounding_radius);
int32_t   rp_num_entities(const rp_world* w);

/* -- external constraints (src/physics/pbd.h:96-102); entities must share a scene --------------- */
rp_status rp_constraint_positional(rp_world* w, int32_t e1, int32_t e2, const double r1[3], const double r2[3],
                                   double compliance, const double distance[3], int32_t* out);
rp_status rp_constraint_mutual_orientation(rp_world* w, int32_t e1, int32_t e2, double compliance, int32_t* out);
rp_status rp_constraint_hinge(rp_world* w, int32_t e1, int32_t e2, const double r1[3], const double r2[3], double compliance,
                              int32_t e1_aligned_axis, int32_t e2_aligned_axis, int32_t limited, int32_t e1_limit_axis,
                              int32_t e2_limit_axis, double lower_limit, double upper_limit, int32_t* out);
rp_status rp_constraint_spherical(rp_world* w, int32_t e1, int32_t e2, const double r1[3], const double r2[3],
                                  int32_t e1_swing_axis, int32_t e2_swing_axis, int32_t e1_twist_axis,
                                  int32_t e2_twist_axis, double swing_lower, double swing_upper, double twist_lower,
                                  double twist_upper, int32_t* out);

/* -- stepping ------------------------------------------------------------------------------------ */
/* pbd_simulate_with_constraints for every scene of the world: num_steps frames of dt each, all on
 * the device (one persistent launch per frame), then forces added with rp_entity_add_force are
 * cleared. dt <= 0 is a no-op, as in the reference (pbd.cpp:471). Asynchronous with respect to the
 * host unless a state read follows; device status is checked by rp_sync. */
rp_status rp_simulate(rp_world* w, double dt, uint32_t num_substeps, uint32_t num_pos_iters, int32_t enable_collisions,
                      uint32_t num_steps);
/* Waits for the world's stream and folds device status into the return value. */
rp_status rp_sync(rp_world* w);
/* Device status bits accumulated since the last call (RP_STATUS_* below). */
rp_status rp_last_status(rp_world* w, uint32_t* bits);
enum {
    RP_STATUS_PAIR_OVERFLOW = 1 << 0,     /* broad-phase pairs exceeded the scratch (the step is redone larger) */
    RP_STATUS_CONTACT_OVERFLOW = 1 << 1,  /* contacts exceeded the scratch (the step is redone larger) */
    RP_STATUS_EPA_OVERFLOW = 1 << 2,      /* an EPA polytope outgrew its fixed storage; that pair was dropped */
    RP_STATUS_CLIP_OVERFLOW = 1 << 3,     /* a clipped polygon outgrew its fixed storage */
    RP_STATUS_BARRIER_TIMEOUT = 1 << 4,   /* a bounded device barrier gave up (rp_simulate undoes the call) */
    RP_STATUS_DEGENERATE = 1 << 5,        /* geometry the reference would reject with an assert */
    RP_STATUS_LEVEL_OVERFLOW = 1 << 6,    /* solver dependency depth exceeded its table */
    RP_STATUS_EPA_NOT_CONVERGED = 1 << 8, /* informational: EPA hit its iteration cap (reference prints a warning) */
    /* which condition raised RP_STATUS_DEGENERATE (each comes with it) */
    RP_STATUS_DEG_EPA_NORMAL = 1 << 9,    /* an EPA face whose normal vanishes (epa.cpp:41 asserts) */
    RP_STATUS_DEG_EPA_COPLANAR = 1 << 10, /* an EPA face through the origin, every point in its plane (epa.cpp:72) */
    RP_STATUS_DEG_SKEW = 1 << 11          /* edge-edge contact of parallel edges (clipping.cpp:279) */
};
/* The first degenerate condition the world met since the last call (the call clears it): out[0] its
 * RP_STATUS_DEG_* bits (0: none), out[1] scene, out[2] / out[3] the pair's entities, out[4] the
 * substep it was met in, counted from the world's last device build (phase-major and persistent
 * forms). No counterpart in the reference, which aborts on these conditions. */
rp_status rp_degenerate_info(rp_world* w, int64_t out[5]);

/* -- state --------------------------------------------------------------------------------------- */
rp_status rp_state_get(rp_world* w, double* out /* num_entities * RP_STATE_DOUBLES */);
rp_status rp_state_set(rp_world* w, const double* in);

/* colliders_update (src/physics/collider.h:51, collider.cpp:409-446) of every entity's hull colliders
 * at its current pose, computed on the device in FP64 with the reference's arithmetic (for worlds of
 * either precision): vertices_out receives 3 doubles per hull vertex, normals_out 3 per hull face
 * (unit), entity by entity in creation order, collider by collider (sphere colliders take no room).
 * rp_transformed_hulls_size gives the two counts. This is the caller prelude the reference's examples
 * run on the host before every step (src/examples/stack.cpp:88-91); the pbd_simulate drop-in uses it
 * to refresh its callers' transformed geometry. */
rp_status rp_transformed_hulls_size(rp_world* w, uint64_t* num_vertices, uint64_t* num_normals);
rp_status rp_transformed_hulls(rp_world* w, double* vertices_out, double* normals_out);

/* -- diagnostics and known-answer entry points --------------------------------------------------- */
/* broad_get_collision_pairs of one scene on the current state: entity-index pairs in the reference's
 * order. *count receives the total even when it exceeds cap. */
rp_status rp_broad_pairs(rp_world* w, int32_t scene, uint32_t* out_pairs, uint32_t cap, uint32_t* count);
/* colliders_update + colliders_get_contacts for one entity pair on the current state, computed by
 * the device narrowphase. out: RP_CONTACT_DOUBLES per contact. */
rp_status rp_contacts(rp_world* w, int32_t e1, int32_t e2, double* out, uint32_t cap, uint32_t* count);
/* rp_contacts without any allocation: no cudaMalloc / cudaFree and no host heap allocation in the
 * call. For callers that must not allocate mid-frame: a frame loop that draws or logs contact points
 * between steps (a device allocation synchronises the whole device and stalls the other streams on
 * it), or a caller with a fixed memory budget. The contacts are computed into a static device scratch
 * of at most 64 contacts and copied into out; cap > 64 is rejected with RP_ERR_CAPACITY, a pair with
 * more contacts reports its full count with the first cap written (cap 0 only counts).
 *
 * Like every call on a world, it must be serialised with the other calls on the same world (it reads
 * the world's buffers and its kernel rewrites the pair's transformed hull vertices); a caller that
 * queries from a second thread takes its own lock around both threads' calls.
 * The world must already be built on the device (it has been stepped), else RP_ERR_STATE. Host-side
 * state edits since the last step (rp_entity_set_velocity) are uploaded first through the world's
 * existing staging buffer, without allocating; an edit that changes the layout (a new entity,
 * constraint or hull) needs a step first (RP_ERR_STATE says so).
 * The first call on a device looks up the scratch's address (set-up) and should come before any
 * stream capture; every call synchronises the world's stream, so none may be made while that stream is
 * being captured. The address stays valid for the process's lifetime: a cudaDeviceReset while the
 * library is loaded is not supported. Calls on the same device must not overlap: they share the
 * scratch. No counterpart in the reference. */
#define RP_NOALLOC_MAX_CONTACTS 64
rp_status rp_contacts_noalloc(rp_world* w, int32_t e1, int32_t e2, double* out, uint32_t cap, uint32_t* count);
/* The collision constraints of the last substep of the last rp_simulate call, in the reference's
 * constraint order (pairs in broad-phase order, contacts in manifold order): entity pairs (2 per
 * contact) and 11 doubles per contact: r1_lc[3], r2_lc[3], normal[3], lambda_n, lambda_t
 * (clipping_contact_to_collision_constraint, pbd.cpp:408-424). *count receives the total. */
rp_status rp_last_contacts(rp_world* w, int32_t scene, int32_t* pairs_out, double* out, uint32_t cap, uint32_t* count);
/* Counters accumulated since creation: [0] GJK iterations, [1] EPA iterations, [2] EPA calls,
 * [3] steps, [4] substeps, [5] contacts generated, [6] broad-phase pairs (summed over steps),
 * [7] solver levels (summed over steps), [8] GJK calls that hit the 100-iteration cap,
 * [9] EPA calls that hit the 100-iteration cap, [10] largest narrowphase cost of one pair
 * (SM clock cycles), [11] narrowphase cycles summed over pairs, [12] pairs narrowphased,
 * [13] pairs skipped because their bounding box and sphere are certainly apart, [14] GJK cycles,
 * [15] EPA cycles, [16] contact-manifold cycles (summed over calls), [17] GJK cycles spent in
 * support mapping, [18] GJK runs ended early on a repeated state (they would have reached the
 * iteration cap and returned no collision), [19] EPA set-up cycles (hull staging, simplex load),
 * [20] EPA support-mapping cycles, [21] manifold set-up cycles, [22] contact write-out cycles,
 * [23] pairs the FP32 build redid in FP64 because FP32 rounding made their EPA polytope or edge
 * contact degenerate (phase-major form). Cycle counters of the phase-major kernels are summed per
 * warp. */
/* The sweep schedules of the last substep of the last rp_simulate call for one scene: per solver
 * node (the scene's external constraints, then its broad-phase pairs, in constraint order) its level
 * (RP_SWEEP_REFERENCE) or colour (RP_SWEEP_COLOURED) in the position sweep (which = 0) or the
 * velocity sweep (which = 1), -1 when the node does nothing there, and its two dynamic entities
 * (-1 for a fixed body). *count receives the node count; level_out / bodies_out may be NULL. */
rp_status rp_last_schedule(rp_world* w, int32_t scene, int32_t which, int32_t* level_out, int32_t* bodies_out,
                           uint32_t cap, uint32_t* count);
#define RP_NUM_COUNTERS 24
rp_status rp_counters(rp_world* w, uint64_t out[RP_NUM_COUNTERS]);
/* Kernel launches issued by this world since creation (every launch of the CUDA extension). */
uint64_t  rp_kernel_launches(const rp_world* w);
/* Device time per phase of the step since creation, in ms (summed over frames): [0] broad phase,
 * [1] islands and sleeping, [2] solver schedule, [3] predict, [4] hull transform, [5] narrowphase
 * (persistent kernel: all of it; phase-major form: the cull kernel), [6] position solve, [7] velocity
 * update, [8] velocity solve, [9] GJK, [10] EPA, [11] contact manifold (the phase-major form's
 * narrowphase kernels). The phase-major form is timed with CUDA events after each kernel while
 * timing is on (rp_set_timing; those frames run outside the CUDA graph); the persistent kernel with
 * the global timer as seen by each scene's first thread. */
#define RP_NUM_PHASES 12
rp_status rp_phase_times(rp_world* w, double out_ms[RP_NUM_PHASES]);
/* Bytes copied host->device (out[0]) and device->host (out[1]) by state and force transfers. */
rp_status rp_transfer_bytes(rp_world* w, uint64_t out[2]);
/* Average duration of the step kernel over the last rp_simulate, measured with CUDA events on the
 * world's stream (milliseconds per launch; 0 if timing is off). */
rp_status rp_set_timing(rp_world* w, int32_t enabled);
rp_status rp_last_step_ms(rp_world* w, double* ms_per_launch);

#ifdef __cplusplus
}
#endif
#endif
