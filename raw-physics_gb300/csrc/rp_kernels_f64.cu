// All-FP64 build of the step kernels, compiled with -fmad=false: the reference's FP64 arithmetic.
#include "rp_kernels.cuh"

namespace rp {
size_t smem_bytes_f64() { return Launcher<double, true>::smem_bytes(); }
cudaError_t configure_f64() { return Launcher<double, true>::configure(); }
int grid_blocks_per_sm_f64() { return Launcher<double, true>::grid_blocks_per_sm(); }
cudaError_t step_f64(const WorldView<double>& W, const StepParams& P, bool grid, int blocks, cudaStream_t st) {
    return Launcher<double, true>::step(W, P, grid, blocks, st);
}
cudaError_t broad_f64(const WorldView<double>& W, int scene, int grid_blocks, cudaStream_t st) {
    return Launcher<double, true>::broad(W, scene, grid_blocks, st);
}
cudaError_t contacts_f64(const WorldView<double>& W, int a, int b, double* out, int cap, int* count, cudaStream_t st) {
    return Launcher<double, true>::contacts(W, a, b, out, cap, count, st);
}
}  // namespace rp
