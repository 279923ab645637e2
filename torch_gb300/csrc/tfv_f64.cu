// Double-precision step kernels: the reference-faithful path.  Built with
// -fmad=false so every product and sum rounds separately, as in NumPy.
#define REAL double
#define TFV_DEFINE_SHARED_KERNELS
// double precision needs ~250 registers; one CTA bound, 128-thread tiles
#define TFV_HYDRO_MIN_BLOCKS 1
#define TFV_FIXED_SHAPES 0
#define TFV_WITH_2D 1
#define TFV_WITH_3D 1
#define TFV_LAUNCH2_NAME launch_step2_f64
#define TFV_LAUNCH3_NAME launch_step3_f64
#define TFV_HLLC_NAME launch_hllc_f64
#define TFV_WITH_1D 1
#define TFV_LAUNCH1_NAME launch_step1_f64
#define TFV_CHECK_READ_NAME check_read_f64
#define TFV_OCC2_NAME occupancy2_f64
#define TFV_OCC3_NAME occupancy3_f64
#include "tfv_inst.inc"

namespace tfv {
cudaError_t launch_finalize(const StepArgs& A, int mode, int fp32, double* integrals_out,
                            cudaStream_t s) {
  const dim3 grid(A.fin_slices > 0 ? A.fin_slices : 1, A.ninst);
  finalize_kernel<<<grid, kFinalizeThreads, 0, s>>>(A, mode, fp32, integrals_out);
  return cudaGetLastError();
}
}  // namespace tfv
