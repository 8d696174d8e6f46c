// FP32 build of the phase-major pipeline kernels.
#include "rp_pipeline.cuh"
#include "rp_launch.h"

namespace rp {
cudaError_t pipe_configure_f32(PipeConfig& c, int sms) { return PipeLauncher<float, false>::configure(c, sms); }
cudaError_t pipe_frame_f32(const WorldView<float>& W, const StepParams& P, const PipeConfig& c, const PipeDims& d,
                           cudaStream_t st, PipeMarks* marks) {
    return PipeLauncher<float, false>::frame(W, P, c, d, st, marks);
}
int pipe_launches_f32(const StepParams& P) { return PipeLauncher<float, false>::launches_per_frame(P); }
}  // namespace rp
