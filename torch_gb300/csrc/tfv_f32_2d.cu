// Single-precision 2D step kernels (see tfv_f32_3d.cu).
#define REAL float
#define TFV_HYDRO_MIN_BLOCKS 3
#define TFV_FIXED_SHAPES 1
#define TFV_WITH_2D 1
#define TFV_WITH_3D 0
#define TFV_LAUNCH2_NAME launch_step2_f32
#define TFV_WITH_1D 1
#define TFV_LAUNCH1_NAME launch_step1_f32
#define TFV_CHECK_READ_NAME check_read_f32_2d
#define TFV_OCC2_NAME occupancy2_f32
#include "tfv_inst.inc"
