// Single-precision 3D step kernels: the bulk FP32 path (contraction and fast
// division/square root allowed by the build flags; conservation sums and time
// stay in double).
#define REAL float
// 80 registers: three 256-thread CTAs per SM (24 warps) without spills
#define TFV_HYDRO_MIN_BLOCKS 3
#define TFV_FIXED_SHAPES 1
#define TFV_WITH_2D 0
#define TFV_WITH_3D 1
#define TFV_LAUNCH3_NAME launch_step3_f32
#define TFV_HLLC_NAME launch_hllc_f32
#define TFV_WITH_1D 0
#define TFV_CHECK_READ_NAME check_read_f32_3d
#define TFV_OCC3_NAME occupancy3_f32
#include "tfv_inst.inc"
