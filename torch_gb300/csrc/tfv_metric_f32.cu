// Metric / face-boundary kernels, single precision (FMA contraction,
// approximate division and square root); sums in double precision.
#define TFV_METRIC_R float
#define TFV_METRIC_LAUNCH metric_launch_f32
#define TFV_RUSANOV_LAUNCH rusanov_launch_f32
#include "tfv_metric_inst.inc"
