// FP32 build of the step kernels: FP32 arithmetic with FP64 poses and EPA face test.
#include "rp_kernels.cuh"

namespace rp {
size_t smem_bytes_f32() { return Launcher<float, false>::smem_bytes(); }
cudaError_t configure_f32() { return Launcher<float, false>::configure(); }
int grid_blocks_per_sm_f32() { return Launcher<float, false>::grid_blocks_per_sm(); }
cudaError_t step_f32(const WorldView<float>& W, const StepParams& P, bool grid, int blocks, cudaStream_t st) {
    return Launcher<float, false>::step(W, P, grid, blocks, st);
}
cudaError_t broad_f32(const WorldView<float>& W, int scene, int grid_blocks, cudaStream_t st) {
    return Launcher<float, false>::broad(W, scene, grid_blocks, st);
}
cudaError_t state_io_f32(const WorldView<float>& W, double* rec, const int32_t* slot_entity, int n, bool pack, cudaStream_t st) {
    return Launcher<float, false>::state_io(W, rec, slot_entity, n, pack, st);
}
cudaError_t contacts_f32(const WorldView<float>& W, int a, int b, double* out, int cap, int* count, cudaStream_t st) {
    return Launcher<float, false>::contacts(W, a, b, out, cap, count, st);
}
}  // namespace rp
