// Metric / face-boundary kernels, single precision (FMA contraction,
// approximate division and square root); sums in double precision.
#define TFV_METRIC_R float
// column-marching kernels: three 256-thread CTAs per SM (80 registers)
#define TFV_MARCH_MIN_BLOCKS 3
// one thread per x face: four CTAs per SM (64 registers)
#define TFV_FACE_MIN_BLOCKS 4
#define TFV_METRIC_LAUNCH metric_launch_f32
#define TFV_RUSANOV_LAUNCH rusanov_launch_f32
#include "tfv_metric_inst.inc"
