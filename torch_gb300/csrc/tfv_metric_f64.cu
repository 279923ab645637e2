// Metric / face-boundary kernels, double precision (built with -fmad=false:
// the reference's rounding).
#define TFV_METRIC_R double
#define TFV_METRIC_LAUNCH metric_launch_f64
#define TFV_RUSANOV_LAUNCH rusanov_launch_f64
#include "tfv_metric_inst.inc"

namespace tfv {
cudaError_t metric_reduce(const double* part, int nblocks, int nv, double* out, cudaStream_t s) {
  metric_reduce_kernel<<<1, 256, 0, s>>>(part, nblocks, nv, out);
  return cudaGetLastError();
}
}  // namespace tfv
