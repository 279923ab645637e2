// Launchers of the metric / face-boundary kernels (one per precision) and
// the block-partial reduction.
#pragma once

#include <cuda_runtime.h>

#include "tfv_metric.h"

namespace tfv {

enum : int {
  kMOpPrim = 0,      // primitives, gamma, geometric source (+ partials of source * volume)
  kMOpFace = 1,      // arg = direction: area-weighted Rusanov fluxes and fraction transport
  kMOpUpdate = 2,    // arg = SSPRK2 stage (1 or 2)
  kMOpOutward = 3,   // partials of the boundary-plane flux differences
  kMOpRate = 4,      // CFL rate maximum
  kMOpReact = 5,     // arg = 0: reaction half into Uout; 1: closing half in place + source partials
  kMOpIntegral = 6,  // partials of the state integral
  kMOpMarchUpdate = 7,  // arg = SSPRK2 stage: last-direction faces + update (2D / 3D)
};

cudaError_t metric_launch_f64(int op, int dim, const MArgs<double>& A, int arg, int grid,
                              cudaStream_t s);
cudaError_t metric_launch_f32(int op, int dim, const MArgs<float>& A, int arg, int grid,
                              cudaStream_t s);
// Rusanov fluxes of n faces (rows [nv][n], primitive face states)
cudaError_t rusanov_launch_f64(int nv, int64_t n, int dir, const void* l, const void* r,
                               const void* gl, const void* gr, void* out, int grid,
                               cudaStream_t s);
cudaError_t rusanov_launch_f32(int nv, int64_t n, int dir, const void* l, const void* r,
                               const void* gl, const void* gr, void* out, int grid,
                               cudaStream_t s);
// out[v] = sum over blocks b < nblocks of part[b * 8 + v], v < nv, in block order
cudaError_t metric_reduce(const double* part, int nblocks, int nv, double* out, cudaStream_t s);

}  // namespace tfv
