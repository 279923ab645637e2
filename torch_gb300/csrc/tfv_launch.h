// Launchers exported by the per-precision translation units.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "tfv_types.h"

namespace tfv {

// kOpWavesStep: the 1D chain's wave-speed pass inside a step (keeps the step's
// source sums and ORs its flags into those of the earlier kernels);
// kOpStep1d: the fused inert 1D step; kOpWavesFallback: the wave-speed pass
// for the instances whose step was redone at first order; kOpWavesPlan: wave
// maxima and flags of the current state without its integrals (re-planning)
enum : int { kOpHydro = 0, kOpFallback = 1, kOpWaves = 2, kOpReact1 = 3, kOpReact2 = 4,
             kOpSpecies = 5, kOpGamma = 6, kOpWavesStep = 7,
             kOpStep1d = 8, kOpWavesFallback = 9, kOpWavesPlan = 10 };

// lim selects the limiter instantiation of the step kernel (ignored otherwise).
cudaError_t launch_step1_f64(int op, bool varg, int lim, const StepArgs& A, int grid, int block,
                             cudaStream_t s);
cudaError_t launch_step1_f32(int op, bool varg, int lim, const StepArgs& A, int grid, int block,
                             cudaStream_t s);
cudaError_t launch_step2_f64(int op, bool varg, int lim, const StepArgs& A, int grid, int block,
                             cudaStream_t s);
cudaError_t launch_step3_f64(int op, bool varg, int lim, const StepArgs& A, int grid, int block,
                             cudaStream_t s);
cudaError_t launch_step2_f32(int op, bool varg, int lim, const StepArgs& A, int grid, int block,
                             cudaStream_t s);
cudaError_t launch_step3_f32(int op, bool varg, int lim, const StepArgs& A, int grid, int block,
                             cudaStream_t s);
cudaError_t launch_hllc_f64(int nv, int64_t n, const void* ul, const void* ur, const void* gl,
                            const void* gr, void* out, cudaStream_t s);
cudaError_t launch_hllc_f32(int nv, int64_t n, const void* ul, const void* ur, const void* gl,
                            const void* gr, void* out, cudaStream_t s);
#if TFV_CHECKED
cudaError_t check_read_f64(unsigned long long* out);
cudaError_t check_read_f32_3d(unsigned long long* out);
cudaError_t check_read_f32_2d(unsigned long long* out);
#endif
// Resident step-kernel CTAs per SM for a tile shape (0 when unknown).
int occupancy2_f64(bool varg, int tx);
int occupancy3_f64(bool varg, int tx, int ty);
int occupancy2_f32(bool varg, int tx);
int occupancy3_f32(bool varg, int tx, int ty);
cudaError_t launch_finalize(const StepArgs& A, int mode, int fp32, double* integrals_out,
                            cudaStream_t s);

// Error text of the C ABI (tfv_last_error), shared by the host units.
int host_fail(int code, const char* msg);
int host_cuda_fail(cudaError_t e, const char* where);

}  // namespace tfv
