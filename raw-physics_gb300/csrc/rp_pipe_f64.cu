// All-FP64 build of the phase-major pipeline kernels (compiled without FMA contraction).
#include "rp_pipeline.cuh"
#include "rp_launch.h"

namespace rp {
cudaError_t pipe_configure_f64(PipeConfig& c, int sms) { return PipeLauncher<double, true>::configure(c, sms); }
cudaError_t pipe_frame_f64(const WorldView<double>& W, const StepParams& P, const PipeConfig& c, const PipeDims& d,
                           cudaStream_t st, PipeMarks* marks) {
    return PipeLauncher<double, true>::frame(W, P, c, d, st, marks);
}
int pipe_launches_f64(const StepParams& P) { return PipeLauncher<double, true>::launches_per_frame(P); }
}  // namespace rp
