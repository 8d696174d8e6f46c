// Host-side entry points of the two precision builds of the step kernels (rp_kernels_f32.cu,
// rp_kernels_f64.cu). Plain C++: the runtime in rp_host.cpp calls these without device code.
#pragma once
#include <cuda_runtime.h>
#include "rp_world.h"

namespace rp {

#define RP_DECLARE_LAUNCHERS(SUF, R)                                                                          \
    size_t smem_bytes_##SUF();                                                                                \
    cudaError_t configure_##SUF();                                                                            \
    int grid_blocks_per_sm_##SUF();                                                                           \
    cudaError_t step_##SUF(const WorldView<R>& W, const StepParams& P, bool grid, int blocks, cudaStream_t st); \
    cudaError_t broad_##SUF(const WorldView<R>& W, int scene, cudaStream_t st);                               \
    cudaError_t contacts_##SUF(const WorldView<R>& W, int a, int b, double* out, int cap, int* count, cudaStream_t st);

RP_DECLARE_LAUNCHERS(f32, float)
RP_DECLARE_LAUNCHERS(f64, double)
#undef RP_DECLARE_LAUNCHERS

}  // namespace rp
