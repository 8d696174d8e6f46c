// Host-side entry points of the two precision builds of the step kernels (rp_kernels_f32.cu,
// rp_kernels_f64.cu). Plain C++: the runtime in rp_host.cpp calls these without device code.
#pragma once
#include <cuda_runtime.h>
#include "rp_world.h"

namespace rp {

// Launch shapes of the phase-major pipeline, chosen once per device (occupancy) and per world.
struct PipeConfig {
    int sms = 0;
    int cull_blocks = 0, gjk_blocks = 0, epa_blocks = 0, manifold_blocks = 0, general_blocks = 0;
    int setup_grid_blocks = 0, sweep_grid_blocks = 0, vsweep_grid_blocks = 0, sweep_warp_blocks = 0;
    // tunable (rp_autotune): the schedule does not depend on them (FP64 results identical, FP32 to rounding)
    int transform_group = 4;     // threads per collider in the hull transform
    int sweep_cta = 0;           // batched sweeps: one CTA per scene instead of one warp per scene
};
struct PipeDims {
    int nbodies = 0, ncolliders = 0, next = 0, num_scenes = 0;
    int node_words = 0;  // words of the node bitmap (node capacity / 32 + 1)
    int grid_mode = 0;   // one large scene: cooperative setup and sweeps
};
// Optional events recorded after each phase (timing runs; never inside a captured graph).
struct PipeMarks {
    cudaEvent_t* ev = nullptr;
    int* phase = nullptr;
    int n = 0, cap = 0;
};

#define RP_DECLARE_LAUNCHERS(SUF, R)                                                                          \
    size_t smem_bytes_##SUF();                                                                                \
    cudaError_t configure_##SUF();                                                                            \
    int grid_blocks_per_sm_##SUF();                                                                           \
    cudaError_t step_##SUF(const WorldView<R>& W, const StepParams& P, bool grid, int blocks, cudaStream_t st); \
    cudaError_t broad_##SUF(const WorldView<R>& W, int scene, int grid_blocks, cudaStream_t st);              \
    cudaError_t contacts_##SUF(const WorldView<R>& W, int a, int b, double* out, int cap, int* count, cudaStream_t st); \
    cudaError_t state_io_##SUF(const WorldView<R>& W, double* rec, const int32_t* slot_entity, int n, bool pack, cudaStream_t st); \
    cudaError_t pipe_configure_##SUF(PipeConfig& c, int sms);                                                 \
    cudaError_t pipe_frame_##SUF(const WorldView<R>& W, const StepParams& P, const PipeConfig& c, const PipeDims& d, \
                                 cudaStream_t st, PipeMarks* marks);                                          \
    int pipe_launches_##SUF(const StepParams& P);

// Adjoint of the substep (rp_adjoint.cu): one scene per thread.
struct AdjGeom {                           // the world's collider geometry (FP64), shared by all scenes
    const Collider* colliders;
    const Shape* shapes;
    const double* shape_verts;
    const double* face_normal;
    const int32_t* face_elem_start;
    const int32_t* face_elem;
    const int32_t* csr_start;
    const int32_t* csr_data;
    const int32_t* col_start;              // [N+1] collider ranges by body slot
    const double* radius;                  // [N] bounding_sphere_radius by body slot
};
struct AdjointParams {
    double dt, gravity;
    int substeps, pos_iters, frames, checkpoint_every;
    int collisions;                        // enable_collisions of the differentiated step
    AdjGeom geom;
};
// Status bits of one scene's adjoint
enum : int { ADJ_ST_TAPE = 1, ADJ_ST_BAD_TAPE = 2, ADJ_ST_UNSUPPORTED = 4, ADJ_ST_PAIRS = 8, ADJ_ST_CONTACTS = 16,
             ADJ_ST_NARROW = 32 };
struct AdjointScene {
    int nb, ne, body0;                     // the scene's bodies are world slots body0 .. body0 + nb
    const ExtConstraint* ext;              // its external constraints (global slots)
    const double* start;                   // [13 nb] x, q, v, w at the trajectory start
    const double* invm;                    // [nb]
    const double* inertia;                 // [6 nb] local inertia (symmetric storage: xx yy zz xy xz yz)
    const double* inv_inertia;             // [6 nb] local inverse inertia
    const double* material;                // [3 nb] static friction, dynamic friction, restitution
    const double* prev_vel;                // [6 nb] previous linear and angular velocity (fixed bodies keep theirs)
    const double* deact0;                  // [nb] deactivation time at the start
    const uint8_t* active0;                // [nb] awake flag at the start
    const uint8_t* fixed;                  // [nb]
    int loss_body;                         // scene-local body of the loss |x - target|^2
    double target[3];
    int tv0, tn0, ntv, ntn;                // the scene's transformed vertices / normals (global offset, count)
    int pair_cap, contact_cap;
    double* checkpoints;                   // [(frames / K + 1) * 15 nb]: state, deactivation time, awake flag
    double* segment;                       // [(K * substeps + 1) * 13 nb]
    double* work;                          // [13 nb]
    double* deact;                         // [nb]
    uint8_t* active;                       // [nb]
    uint8_t* active_seg;                   // [K nb] awake flags of each frame of the segment
    int2* pairs;                           // [K pair_cap] broad-phase pairs of each frame of the segment
    int* npairs;                           // [K]
    int* uf;                               // [nb] union-find parents
    uint8_t* awake;                        // [nb]
    int* stamp;                            // [nb] substep of the body's last hull transform
    void* tv_d; void* tn_d;                // transformed vertices / normals, scalar pass
    void* tv_a; void* tn_a;                // taped pass
    double* tv_val; double* tn_val;        // their values (every decision is taken on these)
    void* con_d; void* con_a;              // [contact_cap] contact constraints of the substep
    void* clip_d; void* clip_a;            // clipping buffers
    void* epa;                             // EPA polytope
    double* grad_state;                    // [13 nb] adjoint of the state (ends as d loss / d start)
    double* grad_invm;                     // [nb]
    double* grad_mu;                       // [2 nb] static, dynamic friction
    double* loss;                          // [1]
    int* status;                           // [1] ADJ_ST_* bits
    long long* prof;                       // [6] SM cycles: forward, segment recompute, taped substeps, reverse
                                           //     sweeps; largest and total tape entries of a substep
    void* bodies_d;                        // nb bodies of the scalar pass
    void* bodies_a;                        // nb bodies of the taped pass
    double* lam_d;                         // [4 ne]
    void* lam_a;                           // [4 ne] taped lambdas
    int2* tape_ab;
    double2* tape_d;
    double* tape_adj;
    int tape_cap;
};
cudaError_t adjoint_launch(AdjointScene* d_scenes, int nscenes, const AdjointParams& P, cudaStream_t st);
size_t adjoint_body_bytes(bool tape);
size_t adjoint_var_bytes();
// scratch sizes of the contact pipeline: contact record, clipping buffers (per pass), EPA polytope
size_t adjoint_contact_bytes(bool tape);
size_t adjoint_clip_bytes(bool tape);
size_t adjoint_epa_bytes();

// colliders_update (collider.cpp:409-446) of every hull collider at its body's current pose, in FP64
// with the reference's arithmetic (built with -fmad=false in rp_kernels_f64.cu): world-space vertices
// and unit face normals at each collider's transformed-geometry offsets (tv_off / tn_off, 3 doubles
// each). Works for worlds of either precision: it reads only FP64 poses and shapes.
struct WorldHullsArgs {
    const Collider* colliders;
    const int32_t* col_body;
    const Shape* shapes;
    const double* shape_verts;
    const double* face_normal;
    const double4_32a* pos;
    const double4_32a* rot;
    int ncolliders;
    double* vertices_out;
    double* normals_out;
};
cudaError_t world_hulls(const WorldHullsArgs& a, cudaStream_t st);

// No-allocation contact query: contacts per call held by its static device scratch (rp_noalloc.cu).
constexpr int NOALLOC_MAX_CONTACTS = 64;
cudaError_t noalloc_scratch(int device, double** contacts, int** count);

RP_DECLARE_LAUNCHERS(f32, float)
RP_DECLARE_LAUNCHERS(f64, double)
#undef RP_DECLARE_LAUNCHERS

}  // namespace rp
