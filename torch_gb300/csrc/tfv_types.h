// Host/device shared descriptors of the batched finite-volume engine.
#pragma once

#include <stdint.h>

namespace tfv {

constexpr int kMaxRing = 3;
constexpr int kFinalizeSlice = 128;  // tiles reduced by one finalize CTA

// Read-only per-instance description (uploaded once per bind).
struct InstDesc {
  int32_t dim;
  int32_t nring;
  int32_t n[3];          // cells along x, y, z
  int32_t bc[3];         // TFV_BC_* along x, y, z
  int32_t limiter;
  int32_t reactive;
  int32_t model;         // TFV_ARRHENIUS / TFV_ZND
  int32_t closure;       // TFV_CLOSURE_*
  int32_t var_gamma;     // gamma per cell from the gamma buffer
  int32_t controller, variant, wavespeed;  // 1D options
  int32_t tile0, ntiles; // range of this instance in the tile table
  int32_t has_flux_out;
  int32_t flux_nv;       // components written to flux_out (all for return_fluxes, 1 = mass)
  int32_t tma;           // tensor maps of this instance's buffers are valid
  int64_t ncell;
  int64_t max_steps;
  double h[3];
  double vol;            // hx*hy*hz over the active axes
  double cfl, gamma, t_end;
  float gamma_f;         // gamma in single precision (no per-cell conversion)
  int32_t pad_gamma;
  double q, ea, a;       // chemistry constants
  double inlet[4];       // conservative 2D inlet state (gamma 1.4)
  void* U[kMaxRing];
  void* lam[kMaxRing];
  void* beta[kMaxRing];
  void* gam;             // per-cell gamma (batch precision), var_gamma only
  void* flux_out[3];
  void* scratch;         // 1D scratch (recon l/r and fluxes)
};

// Mutable per-instance scalars (device resident).
struct InstState {
  double time;
  double dt;             // dt of the step about to run
  double initial[5];
  double boundary[5];
  double source[5];
  int64_t steps;
  int32_t cur;           // ring index of the current state
  int32_t status;        // TFV_READY ...
  int32_t fb_word;       // set by the step kernels when the fallback is needed
  int32_t fallback_steps;
  int32_t last_fallback;
  int32_t retry;         // reactive dt halvings taken in this step
  double dt_allowed;     // reactive: CFL dt of the half-reacted state
  double coef_half[3];   // (0.5*dt)/h_d, predictor coefficients
  double coef_full[3];   // dt/h_d, update coefficients
};

// One tile of work: an in-plane block of one instance over a chunk of
// planes along the marching axis (z in 3D, y in 2D, x-chunks in 1D).
struct Tile {
  int32_t inst;
  int32_t x0, y0;
  int32_t p0, p1;
  int32_t pad_;
};

struct StepArgs {
  const InstDesc* desc;
  InstState* st;
  const Tile* tiles;
  int32_t ntiles;
  int32_t tx, ty;
  int32_t ninst;
  int32_t src_off;  // ring offset (from cur) of the state a kernel reads
  int32_t dst_off;  // ring offset of the state it writes
  int32_t t_begin;  // tile range of this launch
  int32_t t_end;
  const void* tmaps;  // [ninst][4] CUtensorMap (128 B each): ring buffers 0..2, gamma
  double* t_bsum;  // [ntiles][3][5] boundary face sums per direction
  double* t_wmax;  // [ntiles][3] max(|u_d| + a) of the new state
  double* t_sum;   // [ntiles][5] integrals / source partial sums
  int32_t* t_flags;// [ntiles] bit0: nonphysical result, bit1: gate, bit2: species
  double* fin_part;  // [ninst][fin_slices][24] finalize slice records
  int32_t* fin_cnt;  // [ninst] finalize slices arrived (reset by the last)
  int32_t fin_slices;
  const unsigned char* ws_lo;  // workspace range (address checks of the checked build)
  const unsigned char* ws_hi;
};

enum : int32_t {
  kFlagNonphysical = 1,
  kFlagGate = 2,
  kFlagSpecies = 4,
  kFlagChemistry = 8,
};

// Threads per CTA of the step kernel for a tx x ty tile.  A single-precision
// tile whose cell count is not a whole number of warps gets the ring cells
// (2 tx + 2 ty + 4 in 3D, 2 in 2D) on the lanes after its owners, rounded up
// to whole warps, when that fits 256 threads: each lane then does one cell
// stage per plane, and no warp a second one before the plane's barrier.
// Every other tile takes one thread per owned cell.
#if defined(__CUDACC__)
#define TFV_HOST_DEVICE __host__ __device__
#else
#define TFV_HOST_DEVICE
#endif
inline TFV_HOST_DEVICE int step_threads(int dim, bool exact, int tx, int ty) {
  const int nt = tx * (dim == 3 ? ty : 1);
  if (!exact && dim >= 2 && nt % 32 != 0) {
    const int ring = dim == 3 ? 2 * tx + 2 * ty + 4 : 2;
    const int t = (nt + ring + 31) / 32 * 32;
    if (t <= 256) return t;
  }
  return nt;
}

}  // namespace tfv
