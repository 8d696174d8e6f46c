// Host-side entry points of the two precision builds of the step kernels (rp_kernels_f32.cu,
// rp_kernels_f64.cu). Plain C++: the runtime in rp_host.cpp calls these without device code.
#pragma once
#include <cuda_runtime.h>
#include "rp_world.h"

namespace rp {

// Launch shapes of the phase-major pipeline, chosen once per device (occupancy) and per world.
struct PipeConfig {
    int sms = 0;
    int cull_blocks = 0, gjk_blocks = 0, epa_blocks = 0, manifold_blocks = 0;
    int setup_grid_blocks = 0, sweep_grid_blocks = 0, vsweep_grid_blocks = 0, sweep_warp_blocks = 0;
    // tunable (rp_autotune): results do not depend on them
    int transform_group = 8;     // threads per collider in the hull transform
    int sweep_cta = 0;           // batched sweeps: one CTA per scene instead of one warp per scene
};
struct PipeDims {
    int nbodies = 0, ncolliders = 0, next = 0, num_scenes = 0;
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
    cudaError_t broad_##SUF(const WorldView<R>& W, int scene, cudaStream_t st);                               \
    cudaError_t contacts_##SUF(const WorldView<R>& W, int a, int b, double* out, int cap, int* count, cudaStream_t st); \
    cudaError_t pipe_configure_##SUF(PipeConfig& c, int sms);                                                 \
    cudaError_t pipe_frame_##SUF(const WorldView<R>& W, const StepParams& P, const PipeConfig& c, const PipeDims& d, \
                                 cudaStream_t st, PipeMarks* marks);                                          \
    int pipe_launches_##SUF(const StepParams& P);

// No-allocation contact query: contacts per call held by its static device scratch (rp_noalloc.cu).
constexpr int NOALLOC_MAX_CONTACTS = 64;
cudaError_t noalloc_scratch(int device, double** contacts, int** count);

RP_DECLARE_LAUNCHERS(f32, float)
RP_DECLARE_LAUNCHERS(f64, double)
#undef RP_DECLARE_LAUNCHERS

}  // namespace rp
