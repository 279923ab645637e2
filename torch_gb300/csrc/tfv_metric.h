// Metric / face-boundary finite volumes: descriptors shared by the host
// driver and the kernels (python/cfdSolver/torchFiniteVolume.py,
// torchGeometry.py, torchBoundaries.py).
#pragma once

#include <stdint.h>

#include "tfv_types.h"

namespace tfv {

enum MFaceType : int32_t {
  kFaceOutflow = 0,
  kFaceWall = 1,
  kFacePeriodic = 2,
  kFaceInflow = 3,
  kFacePressureOutlet = 4,
  kFaceStagnation = 5,
};

enum MGeometry : int32_t {
  kGeoCartesian = 0,
  kGeoCylindrical = 1,
  kGeoAnnular = 2,
  kGeoSpherical = 3,
};

// error bits raised by the kernels, read by the host after each stage
enum : int32_t {
  kMErrReservoirSolution = 1,  // stagnation inlet: negative discriminant
  kMErrReservoirSupply = 2,    // stagnation inlet: inflow against the interior
  kMErrBackflow = 4,           // pressure outlet backflow without a backflow state
  kMErrNonphysical = 8,        // stage / result state not physical
  kMErrFraction = 16,          // stage / result fraction outside [-1e-12, 1 + 1e-12]
  kMErrChemistry = 32,         // reaction input rejected
  kMErrRate = 64,              // wave-speed rate not finite
  kMErrFinal = 128,            // state after the closing reaction half not physical
};

// One face boundary in the kernels' arithmetic type (converted once on the
// host, so single-precision kernels do no double-precision conversions).
template <typename R>
struct MFace {
  int32_t type;
  int32_t has_backflow;
  R prim[5];   // inflow primitive state, or the pressure outlet's backflow state
  R lam, beta; // fractions carried in by inflow / backflow / reservoir
  R gam;       // gamma(lam) of the carried-in gas (reactive sessions)
  R pressure;  // pressure outlet
  R p0, t0, rgas;  // stagnation inlet: total pressure, temperature, gas constant
};

// Unsigned 32-bit division by an invariant divisor d as a multiply-high, an
// add and a shift (Granlund and Montgomery, "Division by invariant integers
// using multiplication", PLDI 1994, unsigned case with N = 32): with
// l = ceil(log2 d) and m = floor(2^32 (2^l - d) / d) + 1, the quotient of
// every n < 2^32 is (mulhi(m, n) + n) >> l, the sum formed in 64 bits.
struct UDiv {
  uint32_t d, m, l;
};
inline UDiv make_udiv(uint32_t d) {
  UDiv v;
  v.d = d;
  v.l = 0;
  while (v.l < 32 && (uint64_t(1) << v.l) < d) ++v.l;
  v.m = (uint32_t)(((uint64_t(1) << 32) * ((uint64_t(1) << v.l) - d)) / d + 1);
  return v;
}

constexpr int kMReduceBlocks = 512;  // fixed block count of every reduction (deterministic)
constexpr int kMChunk = 32;          // longest run of y / z faces marched by one thread
constexpr int kMXRun = 4;            // x faces per thread in the single-precision x march

template <typename R>
struct MArgs {
  int32_t n[3];       // cells along x, y, z (1 beyond the active axes)
  int64_t nc;         // cells
  int64_t nf[3];      // faces per direction
  // cell and face indexes below 2^31: decoded with the invariant divisors
  // n[0], n[1], n[0] + 1 and n[1] + 1 instead of 64-bit division
  int32_t idx32;
  UDiv dn0, dn1, dn0f, dn1f;
  // x faces marched in short runs by threads adjacent along x (run index
  // fastest, dnch its count per row); 0: threads adjacent along y
  int32_t xlanes;
  UDiv dnch;
  int32_t nfrac;      // transported fractions (0, 1 or 2)
  int32_t reactive;   // gamma from lambda (SI closure)
  int32_t limiter;    // 0 VanLeer, 1 Albada, 2 MINBEE, 3 Superbee, 4 Unos
  int32_t geometry;
  int32_t first_order;
  int32_t chunk;      // y / z faces per thread of the marching face kernel
  int32_t znd;
  double gamma;
  R gam;              // gamma in the arithmetic type
  double dt;          // stage time step
  int32_t periodic[3];  // face pair of each direction is periodic
  const MFace<R>* face;  // [6] in device memory (x_min, x_max, y_min, ...)
  InstDesc chem;      // chemistry constants (q, ea, a, closure) for react_cell
  const R* vf[3];     // volume factors per axis
  const R* ff[3][3];  // face-area factors [direction][axis]
  // inputs of the kernel at hand
  const R* U;         // state
  const R* Q[2];      // fractions (lambda, beta) of that state
  const R* U0;        // stage base state (SSPRK2) / start state (reaction)
  const R* Q0[2];
  const R* Us;        // stage state (second SSPRK2 stage) / hydro state (reaction)
  const R* Qs[2];
  // outputs and scratch
  R* P;               // primitives [nv][nc]
  R* G;               // gamma [nc] (reactive)
  R* S;               // sound speed sqrt(gamma p / rho) [nc] of the primitives in P
  R* K;               // d state / dt [nv][nc]
  R* W[3];            // area-weighted fluxes per direction [nv][nf]
  R* T[3];            // area-weighted fraction transport per direction [nfrac][nf]
  R* Uout;
  R* Qout[2];
  double* part;       // [kMReduceBlocks][8] partial sums
  unsigned long long* rate_max;  // bit pattern of the largest positive rate
  int32_t* err;
};

}  // namespace tfv
