// Kernels of the batched finite-volume engine (2D / 3D).
//
// hydro_kernel — the fused step.  A CTA owns a tile of TX x TY cells in the
// (x, y) plane of a 3D grid (TX cells along x of a 2D grid) and marches
// along the last axis (z in 3D, y in 2D) through a chunk of planes.  Per
// plane it
//   1. stages the conserved state of plane p+1 with a 2-cell in-plane halo
//      in shared memory (ghost cells by the boundary rules), keeping planes
//      p-1, p, p+1 in a 3-slot ring;
//   2. computes limited slopes and the Hancock predictor on the tile plus a
//      1-cell in-plane ring (the "cross" region), and stores predictor and
//      in-plane slopes in shared memory;
//   3. evaluates HLLC on every in-plane face of the tile once;
//   4. evaluates HLLC on the marching-axis face below each owned cell from
//      registers (the face state above the previous plane is carried), and
//      finishes the conservative update of plane p-1 in registers, in the
//      reference's order U - cx dFx - cy dFy - cz dFz.
// Each cell's state is read from HBM once per step (plus the in-plane halo,
// served by L2) and written once.  The epilogue reduces, per tile, the wave
// speeds of the new state for the next CFL dt, the boundary-face flux sums
// for the conservation audit and the positivity flags.
//
// Reference: python/cfdSolver/torchSolver3D.py:122-203 (_hydro),
// python/cfdSolver/torchSolver2D.py:274-466 (muscl_hancock_step_2d),
// python/cfdSolver/torchFlux.py:6-248, python/cfdSolver/torchSession.py:
// 333-360 (dt), 498-508 (boundary integral).
#pragma once

#include "tfv_physics.cuh"
#include "tfv_types.h"

namespace tfv {

enum : int { kBcOpen = 0, kBcReflective = 1, kBcPeriodic = 2, kBcInflow = 3 };
constexpr int kFinalizeThreads = 256;  // threads of a finalize CTA
constexpr int kPartVals = 23;          // partials per tile: 3 maxima, 15 boundary sums, 5 integrals

// an int carried in a double slot of the finalize records (bit copy)
__device__ __forceinline__ double __int_as_double_bits(int v) {
  return __longlong_as_double((long long)(unsigned)v);
}
__device__ __forceinline__ int __double_bits_as_int(double v) {
  return (int)(unsigned)__double_as_longlong(v);
}

enum : int { kReady = 0, kDone = 1, kErrMaxSteps = 2, kErrStall = 3, kErrNonphysical = 4,
             kErrReactive = 5, kErrSpecies = 6, kErrChemistry = 7, kRetry = 8,
             kErrDeviceWait = 9 };

// Source index of padded coordinate i on an axis of n >= 2 cells (at most two
// cells outside), following np.pad 'edge' / 'symmetric' / 'wrap'
// (python/cfdSolver/torchSolver3D.py:47-70).
__device__ __forceinline__ int map_axis(int i, int n, int bc, bool& ghost) {
  ghost = (i < 0) || (i >= n);
  if (!ghost) return i;
  if (bc == kBcReflective) return i < 0 ? -1 - i : 2 * n - 1 - i;
  if (bc == kBcPeriodic) return i < 0 ? i + n : i - n;
  return i < 0 ? 0 : n - 1;
}

// --------------------------------------------------------------------------
// Checked build (TFV_CHECKED=1): every global and shared index of the step
// kernels is tested against the extent of its buffer; the first violation is
// recorded (site, block, index, extent) and the access is skipped.  The
// record is per translation unit; the host reads it after each launch.
// --------------------------------------------------------------------------
#if TFV_CHECKED
static __device__ unsigned long long g_check[4];
static __device__ __noinline__ void check_fail(int site, long long idx, long long lim) {
  if (atomicCAS(&g_check[0], 0ull, (unsigned long long)site) == 0ull) {
    g_check[1] = blockIdx.x;
    g_check[2] = (unsigned long long)idx;
    g_check[3] = (unsigned long long)lim;
  }
}
static __device__ __forceinline__ bool in_range(int site, long long idx, long long lim) {
  if (idx >= 0 && idx < lim) return true;
  check_fail(site, idx, lim);
  return false;
}
#define TFV_IN(site, idx, lim) ::tfv::in_range((site), (long long)(idx), (long long)(lim))
// address checks: a state store must lie outside the workspace, a scratch
// store inside [lo, hi)
static __device__ __forceinline__ bool outside(int site, const void* p, const void* lo,
                                               const void* hi) {
  const char* c = (const char*)p;
  if (c < (const char*)lo || c >= (const char*)hi) return true;
  check_fail(site, (long long)(c - (const char*)lo), (long long)((const char*)hi - (const char*)lo));
  return false;
}
static __device__ __forceinline__ bool inside(int site, const void* p, const void* lo,
                                              const void* hi) {
  const char* c = (const char*)p;
  if (c >= (const char*)lo && c < (const char*)hi) return true;
  check_fail(site, (long long)(c - (const char*)lo), (long long)((const char*)hi - (const char*)lo));
  return false;
}
#define TFV_OUTSIDE(site, p, lo, hi) ::tfv::outside((site), (p), (lo), (hi))
#define TFV_INSIDE(site, p, lo, hi) ::tfv::inside((site), (p), (lo), (hi))
#else
#define TFV_IN(site, idx, lim) true
#define TFV_OUTSIDE(site, p, lo, hi) true
#define TFV_INSIDE(site, p, lo, hi) true
#endif

// --------------------------------------------------------------------------
// Deterministic block reductions (fixed shuffle tree, warps summed in order).
// --------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ int warp_or(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v |= __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Sum of `v` over the block; result valid in thread 0.  scratch >= 32 doubles.
__device__ __forceinline__ double block_sum(double v, double* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < nw; ++w) t += scratch[w];
  }
  return t;
}
__device__ __forceinline__ double block_max(double v, double* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < nw; ++w) t = fmax(t, scratch[w]);
  }
  return t;
}
// Single-precision maximum (exact: the result equals the double maximum of
// the same values) without double-precision arithmetic.
__device__ __forceinline__ float block_max(float v, double* scratch_d) {
  float* scratch = reinterpret_cast<float*>(scratch_d);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  float t = 0.0f;
  if (threadIdx.x == 0) {
    for (int w = 0; w < nw; ++w) t = fmaxf(t, scratch[w]);
  }
  return t;
}
__device__ __forceinline__ int block_or(int v, int* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_or(v);
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  int t = 0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < nw; ++w) t |= scratch[w];
  }
  return t;
}


// --------------------------------------------------------------------------
// Tensor-memory-accelerator staging (cp.async.bulk.tensor + mbarrier).
// Every wait is bounded: after kWaitLimit polls the caller reports an error
// instead of spinning forever.
// --------------------------------------------------------------------------
constexpr uint32_t kWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// The tensor maps live in the workspace and are written by host copies
// between launches; a workspace can reuse the address of an earlier batch's
// maps.  Acquire each map through the tensormap proxy before its first use
// so that no stale cached descriptor is used.
__device__ __forceinline__ void fence_tensormap_acquire(const void* map) {
  asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;" ::"l"(map) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Bounded wait for the phase with the given parity; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const void* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const void* map, int x, int y, int z,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_4d(void* dst, const void* map, int x, int y, int z,
                                            int w, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
      : "memory");
}

// --------------------------------------------------------------------------
// Geometry helper: the grid seen as planes along the marching axis.
// 3D: (a, b, p) = (x, y, z); 2D: (a, b, p) = (x, -, y).
// --------------------------------------------------------------------------
template <int DIM>
struct Geo {
  int na, nb, np;   // extents
  int bca, bcb, bcp;
  int64_t ps, cs;   // plane stride, component stride
  __device__ __forceinline__ void init(const InstDesc& d) {
    na = d.n[0];
    nb = DIM == 3 ? d.n[1] : 1;
    np = DIM == 1 ? 1 : d.n[DIM - 1];  // a 1D grid is a single row
    bca = d.bc[0];
    bcb = DIM == 3 ? d.bc[1] : kBcOpen;
    bcp = DIM == 1 ? kBcOpen : d.bc[DIM - 1];
    ps = (int64_t)na * nb;
    cs = ps * np;
  }
};

// Value of component c (c == NV: gamma) at padded coordinates (a, b, p).
template <typename R, int DIM>
__device__ __forceinline__ R fetch_padded(const InstDesc& d, const Geo<DIM>& g, const R* U,
                                          const R* gam, int c, int a, int b, int p) {
  constexpr int NV = DIM + 2;
  bool ga, gb = false, gp;
  const int sa = map_axis(a, g.na, g.bca, ga);
  const int sb = DIM == 3 ? map_axis(b, g.nb, g.bcb, gb) : 0;
  const int sp = map_axis(p, g.np, g.bcp, gp);
  if (DIM == 2 && g.bcp == kBcInflow && p < 0) {
    return c < NV ? R(d.inlet[c]) : R(1.4);
  }
  const int64_t off = (int64_t)sp * g.ps + (int64_t)sb * g.na + sa;
  if (!TFV_IN(1, off, g.cs) || !TFV_IN(2, c, NV + 1)) return R(0);
  if (c == NV) return gam ? gam[off] : desc_gamma(d, R(0));
  R v = U[c * g.cs + off];
  if ((c == 1 && ga && g.bca == kBcReflective) ||
      (DIM == 3 && c == 2 && gb && g.bcb == kBcReflective) ||
      (c == DIM && gp && g.bcp == kBcReflective))
    v = -v;
  return v;
}

// --------------------------------------------------------------------------
// Shared-memory layout of one hydro tile.
// --------------------------------------------------------------------------
template <typename R, int DIM, bool VARG>
struct HydroSmem {
  static constexpr int NV = DIM + 2;
  static constexpr int NL = NV + (VARG ? 1 : 0);
  static constexpr int kMaxRingItems = 3;  // ring + corner cells per thread
  static constexpr int kMaxFaceItems = 4;  // in-plane faces per thread
  // x offset of cell a = 0 in a staged row: a tensor-copy box must start on a
  // 16-byte boundary, so the row holds 16 bytes of halo on each side.
  static constexpr int kXo = 16 / (int)sizeof(R);
  int tx, ty, pw, ph, bw, bh, xo, nthreads;
  size_t slot_elems;  // elements per ring slot (128-byte multiple)
  size_t ring_off, bar_off, box_off, fa_off, fb_off, bs_off, red_off, items_off, bytes;
  __host__ __device__ void init(int tx_, int ty_) {
    tx = tx_;
    ty = DIM == 3 ? ty_ : 1;
    nthreads = step_threads(DIM, Exact<R>::value, tx, ty);
    xo = kXo;
    pw = tx + 2 * kXo;
    ph = DIM == 3 ? ty + 4 : 1;
    bw = tx + 2;
    bh = DIM == 3 ? ty + 2 : 1;
    slot_elems = ((size_t)NL * ph * pw * sizeof(R) + 127) / 128 * 128 / sizeof(R);
    size_t o = 0;
    ring_off = o;  // dynamic shared memory starts 128-byte aligned
    o += sizeof(R) * 3 * slot_elems;
    bar_off = o;   // one mbarrier per ring slot
    o += 8 * 4;
    o = (o + 15) & ~size_t(15);
    box_off = o;
    o += sizeof(R) * (DIM == 3 ? 3 : 2) * NV * bh * bw;
    o = (o + 15) & ~size_t(15);
    fa_off = o;
    o += sizeof(R) * NV * ty * (tx + 1);
    o = (o + 15) & ~size_t(15);
    fb_off = o;
    if (DIM == 3) o += sizeof(R) * NV * (ty + 1) * tx;
    o = (o + 15) & ~size_t(15);
    bs_off = o;  // boundary-face accumulators (double)
    o += sizeof(double) * (2 * ty * NV + (DIM == 3 ? 2 * tx * NV : 0) + 2 * NV);
    red_off = o;  // reduction scratch
    o += sizeof(double) * 40;
    items_off = o;  // per-thread ring and face work items, packed
    o += sizeof(int) * (kMaxRingItems + kMaxFaceItems) * nthreads;
    bytes = ((o + 15) & ~size_t(15)) + 128;  // + room to align the base to 128 bytes
  }
};

template <typename R, int DIM, bool VARG>
struct HydroTile {
  static constexpr int NV = DIM + 2;
  static constexpr int NL = NV + (VARG ? 1 : 0);
  static constexpr int MD = DIM - 1;  // marching direction

  // Stage plane p of the padded state (2-cell in-plane halo) into `dst`.
  static __device__ __forceinline__ void load_plane(const InstDesc& d, const Geo<DIM>& g,
                                                    const R* U, const R* gam, R* dst,
                                                    const HydroSmem<R, DIM, VARG>& S, int x0,
                                                    int y0, int ax, int by, int p) {
    const int w = ax + 4;
    const int h = DIM == 3 ? by + 4 : 1;
    const int plane = S.ph * S.pw;
    const bool inside_p = (p >= 0 && p < g.np);
    const bool inside_a = (x0 >= 2 && x0 + ax + 2 <= g.na);
    const bool inside_b = DIM == 2 || (y0 >= 2 && y0 + by + 2 <= g.nb);
    // one warp per staged row (component c, in-plane row lb); lanes along x
    const int nrows = NL * h;
    const int lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    if (inside_p && inside_a && inside_b) {
      const int64_t base = (int64_t)p * g.ps + (int64_t)(DIM == 3 ? y0 - 2 : 0) * g.na + (x0 - 2);
      for (int row = threadIdx.x >> 5; row < nrows; row += nwarps) {
        const int c = row / h;
        const int lb = row - c * h;
        const R* srow = (VARG && c == NV) ? gam + base + (int64_t)lb * g.na
                                          : U + c * g.cs + base + (int64_t)lb * g.na;
        R* drow = dst + c * plane + lb * S.pw + (S.xo - 2);
        for (int la = lane; la < w; la += 32) {
          if (!TFV_IN(3, base + (int64_t)lb * g.na + la, g.cs) ||
              !TFV_IN(4, c * plane + lb * S.pw + (S.xo - 2) + la, (int64_t)S.slot_elems))
            continue;
          drow[la] = srow[la];
        }
      }
    } else {
      for (int row = threadIdx.x >> 5; row < nrows; row += nwarps) {
        const int c = row / h;
        const int lb = row - c * h;
        R* drow = dst + c * plane + lb * S.pw + (S.xo - 2);
        for (int la = lane; la < w; la += 32) {
          if (!TFV_IN(5, c * plane + lb * S.pw + (S.xo - 2) + la, (int64_t)S.slot_elems)) continue;
          drow[la] = fetch_padded<R, DIM>(d, g, U, VARG ? gam : (const R*)nullptr, c, x0 - 2 + la,
                                          DIM == 3 ? y0 - 2 + lb : 0, p);
        }
      }
    }
  }

  // After a tensor copy of an in-range plane: rewrite the in-plane ghost
  // cells (outside the domain, zero-filled by the copy) by the boundary
  // rules.  Only tiles touching an in-plane domain edge have any.
  static __device__ __forceinline__ void fix_ghosts(const InstDesc& d, const Geo<DIM>& g,
                                                    const R* U, const R* gam, R* dst,
                                                    const HydroSmem<R, DIM, VARG>& S, int x0,
                                                    int y0, int ax, int by, int p) {
    const int H = DIM == 3 ? by + 4 : 1;
    const int aL = x0 == 0 ? 2 : 0;
    const int aR = max(0, x0 + ax + 2 - g.na);
    const int bL = (DIM == 3 && y0 == 0) ? 2 : 0;
    const int bR = DIM == 3 ? max(0, y0 + by + 2 - g.nb) : 0;
    const int wm = ax + 4 - aL - aR;
    const int n1 = (aL + aR) * H;  // ghost columns, every row
    const int n2 = (bL + bR) * wm; // ghost rows, the other columns
    const int n = n1 + n2;
    if (n == 0) return;
    const int cplane = S.ph * S.pw;
    for (int e = threadIdx.x; e < NL * n; e += blockDim.x) {
      const int c = e / n;
      const int r = e - c * n;
      int la, lb;  // needed-region coordinates: a = la - 2, b = lb - 2
      if (r < n1) {
        const int col = r / H;
        lb = r - col * H;
        la = col < aL ? col : (ax + 4 - aR) + (col - aL);
      } else {
        const int q = r - n1;
        const int row = q / wm;
        la = aL + (q - row * wm);
        lb = row < bL ? row : (by + 4 - bR) + (row - bL);
      }
      if (!TFV_IN(6, c * cplane + lb * S.pw + la + (S.xo - 2), (int64_t)S.slot_elems)) continue;
      dst[c * cplane + lb * S.pw + la + (S.xo - 2)] = fetch_padded<R, DIM>(
          d, g, U, VARG ? gam : (const R*)nullptr, c, x0 - 2 + la, DIM == 3 ? y0 - 2 + lb : 0, p);
    }
  }
};

// Cell stage at local position (a, b) of the current plane: limited slopes in
// every direction and the Hancock predictor (python/cfdSolver/torchSolver3D.py:
// 135-151, python/cfdSolver/torchSolver2D.py:305-377).  Writes predictor and
// in-plane slopes to the box; returns the marching-axis slope; sets *gate when
// a predicted face state is nonphysical (3D gate, torchSolver3D.py:152-159).
// check_gate false skips the gate: the single-precision step gates the face
// states of in-domain cells inside HLLC (hllc_gated), where each of them is
// consumed, and calls this with the gate only for ghost cells, whose outer
// face states no face consumes.
template <typename R, int DIM, bool VARG, int LIM>
__device__ __forceinline__ void cell_stage(const R* ringm, const R* ringc, const R* ringp,
                                           R* box, const HydroSmem<R, DIM, VARG>& S, int a,
                                           int b, R gconst, const R* coefh, R* ubar, R* smarch,
                                           bool& gate, bool check_gate = true) {
  constexpr int NV = DIM + 2;
  const int plane = S.ph * S.pw;
  const int li = (DIM == 3 ? (b + 2) * S.pw : 0) + (a + S.xo);
  const int bi = (DIM == 3 ? (b + 1) * S.bw : 0) + (a + 1);
  const int bplane = S.bh * S.bw;
  R* bub = box;                   // predictor
  R* bsa = box + NV * bplane;     // slope along a (x)
  R* bsb = box + 2 * NV * bplane; // slope along b (y), 3D only
#if TFV_CHECKED
  if (!TFV_IN(7, li - (DIM == 3 ? S.pw : 0) - 1, plane) ||
      !TFV_IN(8, li + (DIM == 3 ? S.pw : 0) + 1, plane) || !TFV_IN(9, bi, bplane)) {
    for (int c = 0; c < NV; ++c) ubar[c] = smarch[c] = R(0);
    return;
  }
#endif
  const R g = VARG ? ringc[NV * plane + li] : gconst;

  R u[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) {
    u[c] = ringc[c * plane + li];
    ubar[c] = u[c];
  }
#pragma unroll
  for (int dd = 0; dd < DIM; ++dd) {
    R s[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) {
      R um, up;
      if (dd == 0) {
        um = ringc[c * plane + li - 1];
        up = ringc[c * plane + li + 1];
      } else if (dd == (DIM - 1)) {
        um = ringm[c * plane + li];
        up = ringp[c * plane + li];
      } else {
        um = ringc[c * plane + li - S.pw];
        up = ringc[c * plane + li + S.pw];
      }
      s[c] = limited_slope<R, DIM, LIM>(um, u[c], up);
    }
    R vp[NV], vm[NV], fp[NV], fm[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) {
      vp[c] = u[c] + R(0.5) * s[c];
      vm[c] = u[c] - R(0.5) * s[c];
    }
    if (DIM == 3) {
      flux3<R>(vp, g, dd + 1, fp);
      flux3<R>(vm, g, dd + 1, fm);
    } else {
      flux2<R>(vp, g, dd, fp);
      flux2<R>(vm, g, dd, fm);
    }
    if constexpr (!Exact<R>::value && DIM == 3) {
      // single precision 3D: the mass fluxes are the normal momenta
      // (flux3), so their difference is the normal momentum's slope
      ubar[0] = ubar[0] - coefh[dd] * s[dd + 1];
#pragma unroll
      for (int c = 1; c < NV; ++c) ubar[c] = ubar[c] - coefh[dd] * (fp[c] - fm[c]);
    } else {
#pragma unroll
      for (int c = 0; c < NV; ++c) ubar[c] = ubar[c] - coefh[dd] * (fp[c] - fm[c]);
    }
    if (dd == 0) {
#pragma unroll
      for (int c = 0; c < NV; ++c) bsa[c * bplane + bi] = s[c];
    } else if (dd == (DIM - 1)) {
#pragma unroll
      for (int c = 0; c < NV; ++c) smarch[c] = s[c];
    } else {
#pragma unroll
      for (int c = 0; c < NV; ++c) bsb[c * bplane + bi] = s[c];
    }
  }
  if (DIM == 2) {
    // predictor floors (python/cfdSolver/torchSolver2D.py:367-377)
    ubar[0] = np_max(ubar[0], R(kFloor));
    const R ke = (R(0.5) * (ubar[1] * ubar[1] + ubar[2] * ubar[2])) / ubar[0];
    const R pb = (g - R(1)) * (ubar[3] - ke);
    if (pb < R(kFloor)) ubar[3] = R(kFloor) / (g - R(1)) + ke;
  }
#pragma unroll
  for (int c = 0; c < NV; ++c) bub[c * bplane + bi] = ubar[c];
  if (DIM == 3 && check_gate) {
    // predictor gate on every predicted face state
    bool ok = true;
#pragma unroll
    for (int dd = 0; dd < DIM; ++dd) {
      R lo[NV], hi[NV];
#pragma unroll
      for (int c = 0; c < NV; ++c) {
        const R s = dd == 0 ? bsa[c * bplane + bi]
                            : (dd == 1 ? bsb[c * bplane + bi] : smarch[c]);
        lo[c] = ubar[c] + R(-0.5) * s;
        hi[c] = ubar[c] + R(0.5) * s;
      }
      ok = ok && physical_cell<R, NV>(lo) && physical_cell<R, NV>(hi);
    }
    if (!ok) gate = true;
  }
}

// Wave speeds max(|u_d| + a) of one updated cell for the next CFL dt.
// 3D: session _dt (python/cfdSolver/torchSession.py:356-360, no floors).
// 2D: compute_cfl_dt_2d on floored primitives (torchSolver2D.py:512-530).
template <typename R, int DIM>
__device__ __forceinline__ void wave_speeds(const R* u, R g, R* w) {
  if (DIM == 3) {
    const R rho = u[0];
    const R s = (u[1] * u[1] + u[2] * u[2]) + u[3] * u[3];
    if constexpr (Exact<R>::value) {
      const R p = (g - R(1)) * (u[4] - (R(0.5) * s) / rho);
      const R a = sqrt((g * p) / rho);
#pragma unroll
      for (int k = 0; k < 3; ++k) w[k] = fabs(u[k + 1] / rho) + a;
    } else {
      const R irho = rcp(rho);
      const R p = (g - R(1)) * (u[4] - R(0.5) * s * irho);
      const R a = sqrt(g * p * irho);
#pragma unroll
      for (int k = 0; k < 3; ++k) w[k] = fabs(u[k + 1] * irho) + a;
    }
  } else if (DIM == 1) {
    // hydro_dt_1d: uconsv_to_uprim + sound_speed_calc (pressure floored at 0)
    const R rho = np_max(u[0], R(kFloor));
    const R v = u[1] / rho;
    const R p = np_max((u[2] - (R(0.5) * rho) * (v * v)) * (g - R(1)), R(kFloor));
    w[0] = fabs(v) + sqrt((g * np_max(p, R(0))) / np_max(rho, R(kFloor)));
  } else {
    const R rho = np_max(u[0], R(kFloor));
    const R vx = u[1] / rho;
    const R vy = u[2] / rho;
    const R p = np_max((g - R(1)) * (u[3] - (R(0.5) * rho) * (vx * vx + vy * vy)), R(kFloor));
    const R a = sqrt((g * np_max(p, R(kFloor))) / np_max(rho, R(kFloor)));
    w[0] = fabs(vx) + a;
    w[1] = fabs(vy) + a;
  }
}

// FP64 sum over the CTA of the marching-axis boundary fluxes (first and last
// plane of the domain only).  Kept out of line so that the conversions to
// double stay on this rare path instead of being hoisted into every plane.
template <typename R, int NV>
struct FaceFlux {
  R v[NV];
};
template <typename R, int NV>
__device__ __noinline__ void march_boundary_sum(FaceFlux<R, NV> ff, double* red, double* out) {
#pragma unroll
  for (int c = 0; c < NV; ++c) {
    const double s = block_sum((double)ff.v[c], red);
    if (threadIdx.x == 0) out[c] += s;
  }
}

template <typename T>
__device__ __forceinline__ T* smem_at(unsigned char* base, size_t off) {
  return reinterpret_cast<T*>(base + off);
}

// One tile of the fused second-order step.
// Returns false when a bounded wait on a tensor copy gave up (the instance's
// status is set to kErrDeviceWait and the kernel stops).
template <typename R, int DIM, bool VARG, int LIM>
__device__ bool hydro_tile(const StepArgs& A, int t, unsigned char* smem,
                           const HydroSmem<R, DIM, VARG>& S, uint32_t& bar_phase) {
  constexpr int NV = DIM + 2;
  constexpr int NL = NV + (VARG ? 1 : 0);
  constexpr int MD = DIM - 1;
  if (!TFV_IN(10, t, A.ntiles)) return true;
  const Tile T = A.tiles[t];
  if (!TFV_IN(11, T.inst, A.ninst)) return true;
  const InstDesc& d = A.desc[T.inst];
  InstState& st = A.st[T.inst];
  if (st.status != kReady) return true;  // uniform over the CTA
  Geo<DIM> g;
  g.init(d);
  const int src = (st.cur + A.src_off) % d.nring;
  const int dst = (st.cur + A.dst_off) % d.nring;
  const R* U = (const R*)d.U[src];
  R* Un = (R*)d.U[dst];
  const R* gam = VARG ? (const R*)d.gam : nullptr;
  const double dt = st.dt;
  const R gconst = desc_gamma(d, R(0));
  (void)dt;
  R coefh[DIM], cu[DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    coefh[k] = R(st.coef_half[k]);  // (0.5*dt)/h_d, computed when dt was planned
    cu[k] = R(st.coef_full[k]);     // dt/h_d
  }
  const int x0 = T.x0, y0 = T.y0, p0 = T.p0, p1 = T.p1;
  const int ax = min(S.tx, g.na - x0);
  const int by = DIM == 3 ? min(S.ty, g.nb - y0) : 1;
  if (!TFV_IN(12, ax - 1, S.tx) || !TFV_IN(13, by - 1, S.ty) || !TFV_IN(14, p0, p1) ||
      !TFV_IN(15, p1 - 1, g.np) || !TFV_IN(16, blockDim.x - 1, S.nthreads) ||
      !TFV_IN(17, (int)src, d.nring) || !TFV_IN(18, (int)dst, d.nring))
    return true;
  const int nint = ax * by;
  const int tid = threadIdx.x;
  const bool owner = tid < nint;
  const int oa = owner ? tid % ax : 0;
  const int ob = owner ? tid / ax : 0;
  const bool at_x0 = (x0 == 0), at_x1 = (x0 + ax == g.na);
  const bool at_y0 = DIM == 3 && y0 == 0, at_y1 = DIM == 3 && (y0 + by == g.nb);

  const int plane = (int)S.slot_elems;
  const int cplane = S.ph * S.pw;
  const int bplane = S.bh * S.bw;
  R* ring = smem_at<R>(smem, S.ring_off);
  R* box = smem_at<R>(smem, S.box_off);
  R* fa = smem_at<R>(smem, S.fa_off);
  R* fb = smem_at<R>(smem, S.fb_off);
  double* bs = smem_at<double>(smem, S.bs_off);
  double* red = smem_at<double>(smem, S.red_off);
  const int nbs = 2 * S.ty * NV + (DIM == 3 ? 2 * S.tx * NV : 0) + 2 * NV;
  for (int e = tid; e < nbs; e += blockDim.x) bs[e] = 0.0;
  double* bs_a = bs;                                   // [2][ty][NV]
  double* bs_b = bs + 2 * S.ty * NV;                   // [2][tx][NV] (3D)
  double* bs_m = bs_b + (DIM == 3 ? 2 * S.tx * NV : 0);// [2][NV]
  const int fa_plane = S.ty * (S.tx + 1);
  const int fb_plane = (S.ty + 1) * S.tx;

  auto slot_of = [&](int p) { return (p - p0 + 2) % 3; };
  auto slot = [&](int p) { return ring + slot_of(p) * plane; };
  // Staging: an in-range plane of a tensor-copy-enabled instance arrives by
  // one cp.async.bulk.tensor per plane (plus one for gamma); ghost planes
  // and other instances use plain loads.
  const bool use_tma = d.tma != 0;
  const bool edge_tile = x0 == 0 || x0 + ax + 2 > g.na ||
                         (DIM == 3 && (y0 == 0 || y0 + by + 2 > g.nb));
  const char* maps = reinterpret_cast<const char*>(A.tmaps) + (size_t)T.inst * 4 * 128;
  const void* map_u = maps + src * 128;
  const void* map_g = maps + 3 * 128;
  const uint32_t box_bytes = (uint32_t)(sizeof(R) * NV * S.ph * S.pw);
  const uint32_t gbox_bytes = VARG ? (uint32_t)(sizeof(R) * S.ph * S.pw) : 0u;
  uint64_t* bars = smem_at<uint64_t>(smem, S.bar_off);
  bool waited_ok = true;
  if (use_tma && tid == 0) {
    fence_tensormap_acquire(map_u);
    if (VARG) fence_tensormap_acquire(map_g);
  }
  auto stage_begin = [&](int p) {
    R* dst = slot(p);
    if (use_tma && p >= 0 && p < g.np) {
      if (tid == 0) {
        uint64_t* bar = bars + slot_of(p);
        fence_proxy_async();  // earlier generic accesses to the slot come first
        mbar_expect_tx(bar, box_bytes + gbox_bytes);
        if (DIM == 3) {
          tma_load_4d(dst, map_u, x0 - S.xo, y0 - 2, p, 0, bar);
          if (VARG) tma_load_3d(dst + NV * cplane, map_g, x0 - S.xo, y0 - 2, p, bar);
        } else {
          tma_load_3d(dst, map_u, x0 - S.xo, p, 0, bar);
          if (VARG) tma_load_2d(dst + NV * cplane, map_g, x0 - S.xo, p, bar);
        }
      }
    } else {
      HydroTile<R, DIM, VARG>::load_plane(d, g, U, gam, dst, S, x0, y0, ax, by, p);
    }
  };
  auto stage_end = [&](int p) {
    if (use_tma && p >= 0 && p < g.np) {
      const int sidx = slot_of(p);
      const uint32_t parity = (bar_phase >> sidx) & 1u;
      bar_phase ^= 1u << sidx;
      if (!mbar_wait(bars + sidx, parity)) {
        waited_ok = false;
        mbar_wait(bars + sidx, parity);  // give the copy in flight a second bound
      }
      if (edge_tile)
        HydroTile<R, DIM, VARG>::fix_ghosts(d, g, U, gam, slot(p), S, x0, y0, ax, by, p);
    }
  };
  stage_begin(p0 - 2);
  stage_begin(p0 - 1);
  stage_begin(p0);
  stage_end(p0 - 2);
  stage_end(p0 - 1);
  stage_end(p0);
  if (__syncthreads_or(!waited_ok)) {
    if (tid == 0) st.status = kErrDeviceWait;
    return false;
  }

  R Tprev[NV], Fprev[NV], Pprev[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) Tprev[c] = Fprev[c] = Pprev[c] = R(0);
  R gprev = gconst;
  R wmax[DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k) wmax[k] = R(0);
  bool bad = false, gate = false;
  R* fout[3] = {(R*)d.flux_out[0], (R*)d.flux_out[1], (R*)d.flux_out[2]};
  const bool want_flux = d.has_flux_out != 0;
  const int nvo = d.flux_nv;

  // domain corners of the active box that this tile must gate (3D)
  int ncorner = 0;
  int corner_a[4], corner_b[4];
  if (DIM == 3) {
    if (at_x0 && at_y0) { corner_a[ncorner] = -1; corner_b[ncorner++] = -1; }
    if (at_x1 && at_y0) { corner_a[ncorner] = ax; corner_b[ncorner++] = -1; }
    if (at_x0 && at_y1) { corner_a[ncorner] = -1; corner_b[ncorner++] = by; }
    if (at_x1 && at_y1) { corner_a[ncorner] = ax; corner_b[ncorner++] = by; }
  }

  // Per-thread work items, computed once per tile and kept in shared memory:
  // ring/corner cells of the cross region and in-plane faces, packed as
  // (kind << 30) | ((i + 1) << 15) | (j + 1).
  int* items = smem_at<int>(smem, S.items_off);
  const int NT = blockDim.x;
  constexpr int MR = HydroSmem<R, DIM, VARG>::kMaxRingItems;
  const int nring_cells = DIM == 3 ? 2 * ax + 2 * by : 2;
  // ring items start at the first lane after the owners when the CTA has
  // lanes for them (step_threads), else at thread 0
  const int r0 = NT > S.tx * S.ty ? S.tx * S.ty : 0;
  int n_ritems = 0;
  for (int q = tid - r0; q >= 0 && q < nring_cells + ncorner; q += NT - r0) {
    int a, b;
    if (q < nring_cells) {
      if (DIM == 3) {
        if (q < by) { a = -1; b = q; }
        else if (q < 2 * by) { a = ax; b = q - by; }
        else if (q < 2 * by + ax) { a = q - 2 * by; b = -1; }
        else { a = q - 2 * by - ax; b = by; }
      } else {
        a = q == 0 ? -1 : ax;
        b = 0;
      }
    } else {
      a = corner_a[q - nring_cells];
      b = corner_b[q - nring_cells];
    }
    if (!TFV_IN(19, n_ritems, MR)) break;
    items[n_ritems * NT + tid] = ((a + 1) << 15) | (b + 1);
    ++n_ritems;
  }
  const int nfa = (ax + 1) * by;
  const int nfb = DIM == 3 ? ax * (by + 1) : 0;
  int n_fitems = 0;
  // the faces do not divide evenly over the threads: the ones that take one
  // more face than the rest start at warp 2, so that they share no warp (and
  // no scheduler) with the ring cells of warps 0 and 1; with ring lanes after
  // the owners they start at thread 0
  const int tface = r0 ? tid : (tid + NT - 64 % NT) % NT;
  for (int w = tface; w < nfa + nfb; w += NT) {
    int packed;
    if (w < nfa) {
      const int af = w % (ax + 1), b = w / (ax + 1);
      packed = ((af + 1) << 15) | (b + 1);
    } else {
      const int q = w - nfa;
      const int a = q % ax, bf = q / ax;
      packed = (1 << 30) | ((a + 1) << 15) | (bf + 1);
    }
    if (!TFV_IN(20, n_fitems, (HydroSmem<R, DIM, VARG>::kMaxFaceItems))) break;
    items[(MR + n_fitems) * NT + tid] = packed;
    ++n_fitems;
  }

  for (int it = p0 - 1; it <= p1; ++it) {
    const R* rm = slot(it - 1);
    const R* rc = slot(it);
    const R* rp = slot(it + 1);
    const bool full = (it >= p0 && it < p1);
    const bool edge_plane = DIM == 3 && (it == -1 || it == g.np);
    const int nr_now = (full || edge_plane) ? n_ritems : 0;
    R Bn[NV], Tn[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) Bn[c] = Tn[c] = R(0);
    // k = -1: the owned interior cell; k >= 0: ring / corner cells
    for (int k = owner ? -1 : 0; k < nr_now; ++k) {
      int a = oa, b = ob;
      if (k >= 0) {
        const int pk = items[k * NT + tid];
        a = ((pk >> 15) & 0x7fff) - 1;
        b = (pk & 0x7fff) - 1;
      }
      R ub[NV], sm[NV];
      // ghost cells (outside the domain) keep the explicit gate; the face
      // states of in-domain cells are gated where HLLC consumes them (FP32)
      const bool ghost = it < 0 || it >= g.np || x0 + a < 0 || x0 + a >= g.na ||
                         (DIM == 3 && (y0 + b < 0 || y0 + b >= g.nb));
      cell_stage<R, DIM, VARG, LIM>(rm, rc, rp, box, S, a, b, gconst, coefh, ub, sm, gate,
                                    Exact<R>::value || ghost);
      if (k < 0) {
#pragma unroll
        for (int c = 0; c < NV; ++c) {
          Bn[c] = ub[c] - R(0.5) * sm[c];
          Tn[c] = ub[c] + R(0.5) * sm[c];
        }
      }
    }
    __syncthreads();  // box complete; ring slot of plane it-1 free
    const bool stage_next = it + 2 <= p1 + 1;
    if (stage_next) stage_begin(it + 2);
    if (full) {
      const R* bub = box;
      for (int k = 0; k < n_fitems; ++k) {
        const int pk = items[(MR + k) * NT + tid];
        const int kind = pk >> 30;  // 0: face normal to x, 1: normal to y (3D)
        const int i = ((pk >> 15) & 0x7fff) - 1;
        const int j = (pk & 0x7fff) - 1;
        // left cell's box index, step to the right cell, slope array
        const int bl = kind == 0 ? (DIM == 3 ? (j + 1) * S.bw : 0) + i : j * S.bw + i + 1;
        const int br = bl + (kind == 0 ? 1 : S.bw);
        if (!TFV_IN(21, bl, bplane) || !TFV_IN(22, br, bplane)) continue;
        const R* bsl = box + (kind == 0 ? 1 : 2) * NV * bplane;
        // rotation into the normal basis: swap rows 1 and 2 for y faces
        R ul[NV], ur[NV], f[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) {
          const int cc = (kind == 1 && c == 1) ? 2 : ((kind == 1 && c == 2) ? 1 : c);
          ul[c] = bub[cc * bplane + bl] + R(0.5) * bsl[cc * bplane + bl];
          ur[c] = bub[cc * bplane + br] - R(0.5) * bsl[cc * bplane + br];
        }
        R gl = gconst, gr = gconst;
        if (VARG) {
          const int li = kind == 0 ? (DIM == 3 ? (j + 2) * S.pw : 0) + i - 1 + S.xo
                                   : (j + 1) * S.pw + i + S.xo;
          gl = rc[NV * cplane + li];
          gr = rc[NV * cplane + li + (kind == 0 ? 1 : S.pw)];
        }
        if constexpr (Exact<R>::value || DIM != 3)
          hllc<R, NV - 3>(ul, ur, gl, gr, f);
        else
          hllc_gated<NV - 3>(ul, ur, gl, gr, f, gate);
        R F[NV];  // back to Cartesian order
#pragma unroll
        for (int c = 0; c < NV; ++c) F[c] = kind == 1 ? (c == 1 ? f[2] : (c == 2 ? f[1] : f[c])) : f[c];
        if (kind == 0) {
          const int af = i, b = j;
#pragma unroll
          for (int c = 0; c < NV; ++c)
            if (TFV_IN(23, b * (S.tx + 1) + af, fa_plane)) fa[c * fa_plane + b * (S.tx + 1) + af] = F[c];
          if (want_flux && fout[0]) {
            const int64_t nf = (int64_t)g.na + 1;
#pragma unroll
            for (int c = 0; c < NV; ++c)
              if (c < nvo) fout[0][((int64_t)(c * g.np + it) * g.nb + (y0 + b)) * nf + x0 + af] = F[c];
          }
        } else {
          const int a = i, bf = j;
#pragma unroll
          for (int c = 0; c < NV; ++c)
            if (TFV_IN(24, bf * S.tx + a, fb_plane)) fb[c * fb_plane + bf * S.tx + a] = F[c];
          if (want_flux && fout[1]) {
#pragma unroll
            for (int c = 0; c < NV; ++c)
              if (c < nvo) fout[1][((int64_t)(c * g.np + it) * (g.nb + 1) + (y0 + bf)) * g.na + x0 + a] = F[c];
          }
        }
      }
    }
    if (stage_next) stage_end(it + 2);
    if (__syncthreads_or(!waited_ok)) {  // in-plane fluxes complete; plane it+2 staged
      if (tid == 0) st.status = kErrDeviceWait;
      return false;
    }
    if (full && (at_x0 || at_x1 || at_y0 || at_y1)) {
      // FP64 sums of the domain-boundary in-plane faces, read back from shared
      // memory by tiles that touch an edge (interior tiles carry no FP64 work);
      // each entry belongs to one thread and accumulates plane by plane
      const int nxb = 2 * S.ty * NV;
      const int nyb = DIM == 3 ? 2 * S.tx * NV : 0;
      for (int e = tid; e < nxb + nyb; e += NT) {
        if (e < nxb) {
          const int side = e / (S.ty * NV), b = (e / NV) % S.ty, c = e % NV;
          if (b < by && (side ? at_x1 : at_x0))
            bs_a[e] += (double)fa[c * fa_plane + b * (S.tx + 1) + (side ? ax : 0)];
        } else {
          const int q = e - nxb;
          const int side = q / (S.tx * NV), a = (q / NV) % S.tx, c = q % NV;
          if (a < ax && (side ? at_y1 : at_y0))
            bs_b[q] += (double)fb[c * fb_plane + (side ? by : 0) * S.tx + a];
        }
      }
    }
    R Fm[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) Fm[c] = R(0);
    if (owner) {
      const int li = (DIM == 3 ? (ob + 2) * S.pw : 0) + oa + S.xo;
      const R gcur = VARG ? rc[NV * cplane + li] : gconst;
      if (it >= p0) {
        if constexpr (Exact<R>::value || DIM != 3)
          hllc_cartesian<R, NV>(Tprev, Bn, gprev, gcur, MD, Fm);
        else
          hllc_cartesian_gated<NV>(Tprev, Bn, gprev, gcur, MD, Fm, gate);
        if (want_flux && fout[MD]) {
#pragma unroll
          for (int c = 0; c < NV; ++c)
            if (c < nvo) fout[MD][((int64_t)(c * (g.np + 1) + it) * g.nb + (y0 + ob)) * g.na + x0 + oa] = Fm[c];
        }
        if (it > p0) {
          R un[NV];
#pragma unroll
          for (int c = 0; c < NV; ++c) un[c] = Pprev[c] - cu[MD] * (Fm[c] - Fprev[c]);
          const int64_t off = (int64_t)(it - 1) * g.ps + (int64_t)(y0 + ob) * g.na + (x0 + oa);
#pragma unroll
          for (int c = 0; c < NV; ++c)
            if (TFV_IN(25, off, g.cs) && TFV_OUTSIDE(60, Un + c * g.cs + off, A.ws_lo, A.ws_hi))
              Un[c * g.cs + off] = un[c];
          if (!physical_cell<R, NV>(un)) bad = true;
          R w[DIM];
          wave_speeds<R, DIM>(un, gprev, w);
#pragma unroll
          for (int k = 0; k < DIM; ++k) wmax[k] = fmax(wmax[k], w[k]);
        }
#pragma unroll
        for (int c = 0; c < NV; ++c) Fprev[c] = Fm[c];
      }
      if (full) {
        const int fi = ob * (S.tx + 1) + oa;
#pragma unroll
        for (int c = 0; c < NV; ++c)
          Pprev[c] = rc[c * cplane + li] - cu[0] * (fa[c * fa_plane + fi + 1] - fa[c * fa_plane + fi]);
        if (DIM == 3) {
          const int gi = ob * S.tx + oa;
#pragma unroll
          for (int c = 0; c < NV; ++c)
            Pprev[c] = Pprev[c] - cu[1] * (fb[c * fb_plane + gi + S.tx] - fb[c * fb_plane + gi]);
        }
      }
#pragma unroll
      for (int c = 0; c < NV; ++c) Tprev[c] = Tn[c];
      gprev = gcur;
    }
    if (it >= p0 && (it == 0 || it == g.np)) {  // march-axis boundary faces
      FaceFlux<R, NV> ff;
#pragma unroll
      for (int c = 0; c < NV; ++c) ff.v[c] = owner ? Fm[c] : R(0);
      march_boundary_sum<R, NV>(ff, red, bs_m + (it == 0 ? 0 : NV));
    }
  }

  // tile epilogue: flags, wave maxima, boundary sums
  int fl = (bad ? kFlagNonphysical : 0) | (gate ? kFlagGate : 0);
  fl = block_or(fl, reinterpret_cast<int*>(red));
  double wm[DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k) wm[k] = (double)block_max(owner ? wmax[k] : R(0), red);
  __syncthreads();
  if (tid == 0) {
    double* out = A.t_bsum + (size_t)t * 15;
    for (int c = 0; c < NV; ++c) {
      double sa = 0.0;
      for (int b = 0; b < S.ty; ++b) sa += bs_a[(1 * S.ty + b) * NV + c] - bs_a[(0 * S.ty + b) * NV + c];
      out[0 * 5 + c] = sa;
      if (DIM == 3) {
        double sb = 0.0;
        for (int a = 0; a < S.tx; ++a) sb += bs_b[(1 * S.tx + a) * NV + c] - bs_b[(0 * S.tx + a) * NV + c];
        out[1 * 5 + c] = sb;
      }
      out[MD * 5 + c] = bs_m[NV + c] - bs_m[c];
    }
    for (int k = 0; k < DIM; ++k) A.t_wmax[(size_t)t * 3 + k] = wm[k];
    A.t_flags[t] = fl;
    if (fl & (kFlagNonphysical | kFlagGate)) atomicOr(&st.fb_word, fl);
  }
  __syncthreads();
  return true;
}

// TX, TY > 0: tile shape fixed at compile time (shared-memory offsets become
// immediates); 0: taken from the launch arguments.
template <typename R, int DIM, bool VARG, int LIM, int TX, int TY>
__global__ void __launch_bounds__(256, TFV_HYDRO_MIN_BLOCKS) hydro_kernel(StepArgs A) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // align by pointer arithmetic on the shared array (an integer round trip
  // would hide the address space and turn every shared access generic)
  unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  HydroSmem<R, DIM, VARG> S;
  S.init(TX > 0 ? TX : A.tx, TY > 0 ? TY : A.ty);
  if (threadIdx.x == 0) {
    uint64_t* bars = smem_at<uint64_t>(smem, S.bar_off);
    for (int k = 0; k < 3; ++k) mbar_init(bars + k, 1);
    fence_mbar_init();
  }
  __syncthreads();
  uint32_t bar_phase = 0;  // parity of the next completion of each slot's barrier
  for (int t = A.t_begin + blockIdx.x; t < A.t_end; t += gridDim.x)
    if (!hydro_tile<R, DIM, VARG, LIM>(A, t, smem, S, bar_phase)) break;
}

// --------------------------------------------------------------------------
// First-order fallback (whole step), run only when a tile flagged the
// instance.  3D: Rusanov on padded cells (python/cfdSolver/torchSolver3D.py:
// 162-176); 2D: LLF with floored primitives (torchSolver2D.py:419-462).
// --------------------------------------------------------------------------
template <typename R, int DIM>
__device__ __forceinline__ void first_order_face(const R* L, const R* Rr, R gl, R gr, int dd,
                                                 R* F) {
  constexpr int NV = DIM + 2;
  if (DIM == 3) {
    const int m = dd + 1;
    R fl[NV], fr[NV];
    flux3<R>(L, gl, m, fl);
    flux3<R>(Rr, gr, m, fr);
    const R sl_ = (L[1] * L[1] + L[2] * L[2]) + L[3] * L[3];
    const R sr_ = (Rr[1] * Rr[1] + Rr[2] * Rr[2]) + Rr[3] * Rr[3];
    const R pl = (gl - R(1)) * (L[4] - (R(0.5) * sl_) / L[0]);
    const R pr = (gr - R(1)) * (Rr[4] - (R(0.5) * sr_) / Rr[0]);
    const R speed = np_max(fabs(L[m] / L[0]) + sqrt((gl * pl) / L[0]),
                           fabs(Rr[m] / Rr[0]) + sqrt((gr * pr) / Rr[0]));
#pragma unroll
    for (int c = 0; c < NV; ++c) F[c] = R(0.5) * ((fl[c] + fr[c]) - speed * (Rr[c] - L[c]));
  } else {
    R f[2][NV], cs[2];
    const R* uu[2] = {L, Rr};
    const R gg[2] = {gl, gr};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const R* u = uu[k];
      const R rho = np_max(u[0], R(kFloor));
      const R ux = u[1] / rho;
      const R vy = u[2] / rho;
      const R p = np_max((gg[k] - R(1)) * (u[3] - (R(0.5) * rho) * (ux * ux + vy * vy)), R(kFloor));
      const R snd = sqrt((gg[k] * np_max(p, R(kFloor))) / np_max(rho, R(kFloor)));
      const R vn = dd == 0 ? ux : vy;
      if (dd == 0) {
        f[k][0] = u[1];
        f[k][1] = u[1] * ux + p;
        f[k][2] = u[2] * ux;
        f[k][3] = ux * (u[3] + p);
      } else {
        f[k][0] = u[2];
        f[k][1] = u[1] * vy;
        f[k][2] = u[2] * vy + p;
        f[k][3] = vy * (u[3] + p);
      }
      cs[k] = fabs(vn) + snd;
    }
    const R speed = np_max(cs[0], cs[1]);
#pragma unroll
    for (int c = 0; c < NV; ++c) F[c] = R(0.5) * ((f[0][c] + f[1][c]) - speed * (Rr[c] - L[c]));
  }
}

template <typename R, int DIM, bool VARG>
__global__ void __launch_bounds__(256) fallback_kernel(StepArgs A) {
  constexpr int NV = DIM + 2;
  __shared__ double red[40];
  {
    // usually no instance is flagged: one look at the instance states instead
    // of walking the tile table
    int any = 0;
    for (int k = threadIdx.x; k < A.ninst; k += blockDim.x)
      any |= (A.st[k].status == kReady && A.st[k].fb_word != 0);
    if (!__syncthreads_or(any)) return;
  }
  for (int t = A.t_begin + blockIdx.x; t < A.t_end; t += gridDim.x) {
    if (!TFV_IN(28, t, A.ntiles)) continue;
    const Tile T = A.tiles[t];
    if (!TFV_IN(29, T.inst, A.ninst)) continue;
    const InstDesc& d = A.desc[T.inst];
    InstState& st = A.st[T.inst];
    if (st.status != kReady || st.fb_word == 0) continue;  // uniform
    Geo<DIM> g;
    g.init(d);
    const int src = (st.cur + A.src_off) % d.nring;
    const int dst = (st.cur + A.dst_off) % d.nring;
    const R* U = (const R*)d.U[src];
    R* Un = (R*)d.U[dst];
    const R* gam = VARG ? (const R*)d.gam : nullptr;
    const double dt = st.dt;
    (void)dt;
    R cu[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) cu[k] = R(st.coef_full[k]);
    const int ax = min(A.tx, g.na - T.x0);
    const int by = DIM == 3 ? min(A.ty, g.nb - T.y0) : 1;
    const bool owner = (int)threadIdx.x < ax * by;
    const int a = T.x0 + (owner ? (int)threadIdx.x % ax : 0);
    const int b = DIM == 3 ? T.y0 + (owner ? (int)threadIdx.x / ax : 0) : 0;
    double acc[DIM][NV];
#pragma unroll
    for (int k = 0; k < DIM; ++k)
#pragma unroll
      for (int c = 0; c < NV; ++c) acc[k][c] = 0.0;
    R wmax[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) wmax[k] = R(0);
    bool bad = false;
    R* fout[3] = {(R*)d.flux_out[0], (R*)d.flux_out[1], (R*)d.flux_out[2]};
    if (owner) {
      for (int p = T.p0; p < T.p1; ++p) {
        R u[NV], un[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) {
          u[c] = fetch_padded<R, DIM>(d, g, U, gam, c, a, b, p);
          un[c] = u[c];
        }
        const R gc = VARG ? fetch_padded<R, DIM>(d, g, U, gam, NV, a, b, p) : desc_gamma(d, R(0));
#pragma unroll
        for (int dd = 0; dd < DIM; ++dd) {
          const int ia = dd == 0 ? 1 : 0;
          const int ib = (DIM == 3 && dd == 1) ? 1 : 0;
          const int ip = dd == DIM - 1 ? 1 : 0;
          R lo[NV], hi[NV], Fm[NV], Fp[NV];
#pragma unroll
          for (int c = 0; c < NV; ++c) {
            lo[c] = fetch_padded<R, DIM>(d, g, U, gam, c, a - ia, b - ib, p - ip);
            hi[c] = fetch_padded<R, DIM>(d, g, U, gam, c, a + ia, b + ib, p + ip);
          }
          const R glo = VARG ? fetch_padded<R, DIM>(d, g, U, gam, NV, a - ia, b - ib, p - ip) : gc;
          const R ghi = VARG ? fetch_padded<R, DIM>(d, g, U, gam, NV, a + ia, b + ib, p + ip) : gc;
          first_order_face<R, DIM>(lo, u, glo, gc, dd, Fm);
          first_order_face<R, DIM>(u, hi, gc, ghi, dd, Fp);
#pragma unroll
          for (int c = 0; c < NV; ++c) un[c] = un[c] - cu[dd] * (Fp[c] - Fm[c]);
          const int idx = dd == 0 ? a : (dd == DIM - 1 ? p : b);
          const int n = dd == 0 ? g.na : (dd == DIM - 1 ? g.np : g.nb);
          if (idx == 0) {
#pragma unroll
            for (int c = 0; c < NV; ++c) acc[dd][c] -= (double)Fm[c];
          }
          if (idx == n - 1) {
#pragma unroll
            for (int c = 0; c < NV; ++c) acc[dd][c] += (double)Fp[c];
          }
          if (d.has_flux_out && fout[dd]) {
            // face arrays: the axis dd has n+1 faces
            const int fa_n = dd == 0 ? g.na + 1 : g.na;
            const int fb_n = (DIM == 3 && dd == 1) ? g.nb + 1 : g.nb;
            const int fp_n = dd == DIM - 1 ? g.np + 1 : g.np;
            (void)fp_n;
#pragma unroll
            for (int c = 0; c < NV; ++c) {
              if (c >= d.flux_nv) continue;
              const int64_t base = (int64_t)c * (dd == DIM - 1 ? g.np + 1 : g.np);
              fout[dd][((base + p) * fb_n + b) * fa_n + a] = Fm[c];
              if (idx == n - 1)
                fout[dd][((base + p + ip) * fb_n + b + ib) * fa_n + a + ia] = Fp[c];
            }
          }
        }
        const int64_t off = (int64_t)p * g.ps + (int64_t)b * g.na + a;
#pragma unroll
        for (int c = 0; c < NV; ++c)
          if (TFV_IN(26, off, g.cs) && TFV_OUTSIDE(61, Un + c * g.cs + off, A.ws_lo, A.ws_hi))
            Un[c * g.cs + off] = un[c];
        if (!physical_cell<R, NV>(un)) bad = true;
        R w[DIM];
        wave_speeds<R, DIM>(un, gc, w);
#pragma unroll
        for (int k = 0; k < DIM; ++k) wmax[k] = fmax(wmax[k], w[k]);
      }
    }
    int fl = block_or(bad ? kFlagNonphysical : 0, reinterpret_cast<int*>(red));
    double sums[DIM][NV];
#pragma unroll
    for (int k = 0; k < DIM; ++k)
#pragma unroll
      for (int c = 0; c < NV; ++c) sums[k][c] = block_sum(acc[k][c], red);
    double wm[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) wm[k] = (double)block_max(owner ? wmax[k] : R(0), red);
    if (threadIdx.x == 0) {
      double* out = A.t_bsum + (size_t)t * 15;
      for (int k = 0; k < DIM; ++k)
        for (int c = 0; c < NV; ++c) out[k * 5 + c] = sums[k][c];
      for (int k = 0; k < DIM; ++k) A.t_wmax[(size_t)t * 3 + k] = wm[k];
      A.t_flags[t] = fl;
    }
    __syncthreads();
  }
}

// --------------------------------------------------------------------------
// Wave-speed maxima of the current state (initial / re-planned dt).
// --------------------------------------------------------------------------
template <typename R, int DIM, bool VARG>
// sums: also the integrals of the state (bind, integrals); re-planning needs
// only the wave maxima and flags.
__global__ void __launch_bounds__(256) waves_kernel(StepArgs A, int sums) {
  constexpr int NV = DIM + 2;
  __shared__ double red[40];
  for (int t = A.t_begin + blockIdx.x; t < A.t_end; t += gridDim.x) {
    if (!TFV_IN(30, t, A.ntiles)) continue;
    const Tile T = A.tiles[t];
    if (!TFV_IN(31, T.inst, A.ninst)) continue;
    const InstDesc& d = A.desc[T.inst];
    const InstState& st = A.st[T.inst];
    Geo<DIM> g;
    g.init(d);
    const R* U = (const R*)d.U[(st.cur + A.src_off) % d.nring];
    const R* gam = VARG ? (const R*)d.gam : nullptr;
    const int ax = min(A.tx, g.na - T.x0);
    const int by = DIM == 3 ? min(A.ty, g.nb - T.y0) : 1;
    const bool owner = (int)threadIdx.x < ax * by;
    const int a = T.x0 + (owner ? (int)threadIdx.x % ax : 0);
    const int b = DIM == 3 ? T.y0 + (owner ? (int)threadIdx.x / ax : 0) : 0;
    R wmax[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) wmax[k] = R(0);
    bool bad = false;
    double sum[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) sum[c] = 0.0;
    if (owner) {
      // planes in groups of four: every load of a group is issued before the
      // first is used (one column per thread leaves little other parallelism);
      // the sums still run plane by plane in order
      constexpr int G4 = 4;
      for (int p = T.p0; p < T.p1; p += G4) {
        R u[G4][NV];
        R gc[G4];
#pragma unroll
        for (int q = 0; q < G4; ++q) {
          const int64_t off = (int64_t)(p + q) * g.ps + (int64_t)b * g.na + a;
          const bool in = p + q < T.p1 && TFV_IN(27, off, g.cs);
#pragma unroll
          for (int c = 0; c < NV; ++c) u[q][c] = in ? U[c * g.cs + off] : R(1);
          gc[q] = VARG ? (in ? gam[off] : R(1.4)) : desc_gamma(d, R(0));
        }
#pragma unroll
        for (int q = 0; q < G4; ++q) {
          if (p + q >= T.p1) break;
          if (sums) {
#pragma unroll
            for (int c = 0; c < NV; ++c) sum[c] += (double)u[q][c];
          }
          if (!physical_cell<R, NV>(u[q])) bad = true;
          R w[DIM];
          wave_speeds<R, DIM>(u[q], gc[q], w);
#pragma unroll
          for (int k = 0; k < DIM; ++k) wmax[k] = fmax(wmax[k], w[k]);
        }
      }
    }
    int fl = block_or(bad ? kFlagNonphysical : 0, reinterpret_cast<int*>(red));
    double wm[DIM], sm[NV];
#pragma unroll
    for (int k = 0; k < DIM; ++k) wm[k] = (double)block_max(owner ? wmax[k] : R(0), red);
#pragma unroll
    for (int c = 0; c < NV; ++c) sm[c] = sums ? block_sum(sum[c], red) : 0.0;  // uniform
    if (threadIdx.x == 0) {
      for (int k = 0; k < DIM; ++k) A.t_wmax[(size_t)t * 3 + k] = wm[k];
      if (sums)
        for (int c = 0; c < NV; ++c) A.t_sum[(size_t)t * 5 + c] = sm[c];
      A.t_flags[t] = fl;
    }
    __syncthreads();
  }
}

// --------------------------------------------------------------------------
// Per-instance finalize: commit the step (ring swap, boundary integral,
// time, steps), then plan the next dt (python/cfdSolver/torchSession.py:
// 379-396, 498-522).  mode 0: commit + plan; 1: plan only; 2: integrals only;
// 3: record the initial integrals, then plan (bind); 4: reactive dt check
// after the first half reaction (accept, or halve dt and retry, at most 60
// attempts; torchSession.py:401-411).  One CTA per instance.
// --------------------------------------------------------------------------
// CFL dt from the wave-speed maxima w (python/cfdSolver/torchSession.py:333-360):
// 3D cfl / sum_d max(|u_d|+a)/h_d; 2D on floored primitives including the
// inlet ghost rows, 1e-3 when the speeds vanish; 1D min of the wave-speed and
// hydro estimates (w[0] = max |S|, w[1] = max(|u| + a)).
__device__ __forceinline__ double cfl_dt(const InstDesc& d, const double* w) {
  if (d.dim == 3) {
    const double total = (w[0] / d.h[0] + w[1] / d.h[1]) + w[2] / d.h[2];
    return d.cfl / total;
  }
  if (d.dim == 2) {
    double w0 = w[0], w1 = w[1];
    if (d.bc[1] == kBcInflow) {  // the inlet ghost rows take part in the 2D dt
      const double rho = fmax(d.inlet[0], 1e-12);
      const double ux = d.inlet[1] / rho, vy = d.inlet[2] / rho;
      const double p = fmax((1.4 - 1.0) * (d.inlet[3] - (0.5 * rho) * (ux * ux + vy * vy)), 1e-12);
      const double a = sqrt((1.4 * fmax(p, 1e-12)) / fmax(rho, 1e-12));
      w0 = fmax(w0, fabs(ux) + a);
      w1 = fmax(w1, fabs(vy) + a);
    }
    const double total = w0 / d.h[0] + w1 / d.h[1];
    return total <= 1e-12 ? 1e-3 : d.cfl / total;
  }
  const double dw = w[0] > 0 ? (d.cfl * d.h[0]) / w[0] : 1e-6;
  const double dh = d.cfl * d.h[0] / w[1];
  return dh < dw ? dh : dw;
}

__device__ __forceinline__ void set_dt(const InstDesc& d, InstState& st, double dt) {
  st.dt = dt;
  for (int k = 0; k < 3; ++k) {
    st.coef_half[k] = (0.5 * dt) / d.h[k];
    st.coef_full[k] = dt / d.h[k];
  }
}

__device__ __forceinline__ void plan_next(const InstDesc& d, InstState& st, const double* w,
                                          int fp32) {
  if (st.time == d.t_end) {
    st.status = kDone;
    return;
  }
  if (st.steps >= d.max_steps) {
    st.status = kErrMaxSteps;
    return;
  }
  double dt = cfl_dt(d, w);
  if (fp32) dt = (double)(float)dt;
  const double rem = d.t_end - st.time;
  if (rem < dt) dt = rem;
  set_dt(d, st, dt);
  if (!isfinite(dt) || dt <= 0.0 || st.time + dt == st.time) {
    st.status = kErrStall;
    return;
  }
  st.status = kReady;
}

// plan_next run by one warp: the independent FP64 divisions (w_d / h_d of the
// CFL reduction, the dt / h_d coefficients) go to separate lanes.  Every
// value keeps the expression and operation order of the serial form, so the
// results are identical; GB300's double-precision pipe is narrow, and a
// single thread's chain of divisions was the finalize kernel's critical path.
__device__ __forceinline__ void plan_next_warp(const InstDesc& d, InstState& st, const double* w,
                                               int fp32, int lane) {
  if (st.time == d.t_end) {
    if (lane == 0) st.status = kDone;
    return;
  }
  if (st.steps >= d.max_steps) {
    if (lane == 0) st.status = kErrMaxSteps;
    return;
  }
  double dt;
  if (d.dim == 3) {
    const double q = lane < 3 ? w[lane] / d.h[lane] : 0.0;
    const double q0 = __shfl_sync(0xffffffffu, q, 0);
    const double q1 = __shfl_sync(0xffffffffu, q, 1);
    const double q2 = __shfl_sync(0xffffffffu, q, 2);
    const double total = (q0 + q1) + q2;
    dt = d.cfl / total;
  } else {
    dt = cfl_dt(d, w);
  }
  if (fp32) dt = (double)(float)dt;
  const double rem = d.t_end - st.time;
  if (rem < dt) dt = rem;
  if (lane < 3) {
    st.coef_half[lane] = (0.5 * dt) / d.h[lane];
  } else if (lane < 6) {
    st.coef_full[lane - 3] = dt / d.h[lane - 3];
  } else if (lane == 6) {
    st.dt = dt;
    st.status = (!isfinite(dt) || dt <= 0.0 || st.time + dt == st.time) ? kErrStall : kReady;
  }
}

// --------------------------------------------------------------------------
// Chemistry: exponential-midpoint Arrhenius / two-stage ZND source on the
// 1D projection of a cell (python/cfdSolver/torchSolver.py:708-789 via
// reaction_step_2d / reaction_step_3d, torchSolver2D.py:474-509,
// torchSolver3D.py:225-243).  Closure SI: gamma(lambda), T = p M / (rho R_u),
// rate = A exp(-Ea / (8.314 T)); closure nondimensional: constant gamma,
// T = p / rho, rate = A exp(-Ea_over_R / T).
// --------------------------------------------------------------------------
__device__ __forceinline__ double texp(double x) { return exp(x); }
__device__ __forceinline__ float texp(float x) { return expf(x); }

template <typename R>
__device__ __forceinline__ R gamma_of_lambda(R lam) {
  return (R(4.5) - lam) / (R(3.5) - lam);
}

// Chemistry constants of an instance in the arithmetic type, converted once
// per tile rather than per cell (a double-to-float conversion runs on the
// narrow FP64 pipe).
template <typename R>
struct Chem {
  int closure;
  R q, ea, a, gamma;
  __device__ __forceinline__ explicit Chem(const InstDesc& d)
      : closure(d.closure), q(R(d.q)), ea(R(d.ea)), a(R(d.a)), gamma(desc_gamma(d, R(0))) {}
};

template <typename R>
__device__ __forceinline__ R reaction_rate(const Chem<R>& d, R lam, R s0, R s1, R s2) {
  const bool si = d.closure == 0;
  const R g = si ? gamma_of_lambda(lam) : d.gamma;
  // uconsv_to_uprim (torchSolver.py:117-127)
  const R rho = np_max(s0, R(kFloor));
  const R u = s1 / rho;
  const R p = np_max((s2 - (R(0.5) * rho) * (u * u)) * (g - R(1)), R(kFloor));
  R t;
  if (si) {
    // temp_calc (torchSolver.py:90-114)
    const R rho2 = np_max(rho, R(kFloor));
    const R molar = (lam * R(2.0 / 3.0)) * R(2.016) + (lam * R(1.0 / 3.0)) * R(32.0) +
                    (R(1) - lam) * R(18.016);
    t = np_max((p * molar) / (rho2 * R(8314.46)), R(kFloor));
    return d.a * texp(-d.ea / (R(8.314) * t));
  }
  t = np_max(p / rho, R(kFloor));
  return d.a * texp(-d.ea / t);
}

// One cell: returns false when the reference would reject the input
// (reactant fraction outside [0,1] or not finite, nonphysical 1D state,
// induction fraction outside [0,1]).
template <typename R, int DIM>
__device__ __forceinline__ bool react_cell(const Chem<R>& d, R* u, R& lam, R& beta, bool znd,
                                           double dt_r) {
  constexpr int NV = DIM + 2;
  const R s0 = u[0], s1 = u[1];
  R s2 = u[NV - 1];  // 1D: the state itself (torchSession.py:365-369)
  if (DIM > 1) {     // 2D/3D: move the transverse kinetic energy out of E
    R st = u[2] * u[2];
    if (DIM == 3) st = st + u[3] * u[3];
    s2 = u[NV - 1] - (R(0.5) * st) / u[0];
  }
  bool ok = finite_(lam) && lam >= R(0) && lam <= R(1);
  const R e1 = s2 - (R(0.5) * (s1 * s1)) / s0;
  ok = ok && finite_(s0) && finite_(s1) && finite_(s2) && s0 > R(kFloor) && e1 > R(kFloor);
  const R beta_n = znd ? beta : R(1);
  if (znd) ok = ok && finite_(beta) && beta >= R(0) && beta <= R(1);
  const R q = d.q;
  const R lam_n = lam;
  auto advance = [&](R rate, R duration, R& lam_out, R& beta_out) {
    if (znd) {
      const R floor_rate = Exact<R>::value ? R(1e-300) : R(1e-30);
      const R active = np_max(R(0), duration - beta_n / np_max(rate, floor_rate));
      lam_out = lam_n * texp((R(-5.0) * rate) * active);
      beta_out = np_min(np_max(beta_n - rate * duration, R(0)), R(1));
    } else {
      lam_out = lam_n * texp((-rate) * duration);
      beta_out = R(0);
    }
  };
  R lam_mid, beta_mid;
  advance(reaction_rate<R>(d, lam_n, s0, s1, s2), R(0.5 * dt_r), lam_mid, beta_mid);
  const R s2_mid = s2 + (q * s0) * (lam_n - lam_mid);
  R lam_new, beta_new;
  advance(reaction_rate<R>(d, lam_mid, s0, s1, s2_mid), R(dt_r), lam_new, beta_new);
  const R s2_new = s2 + (q * s0) * (lam_n - lam_new);
  u[NV - 1] = DIM == 1 ? s2_new : u[NV - 1] + (s2_new - s2);
  lam = lam_new;
  if (znd) beta = beta_new;
  return ok;
}

// Reaction half step over every tile.  stage 1: start (ring cur) -> heated
// (cur+1) and gamma(lambda) for the hydro step; wave maxima for the reactive
// dt check.  stage 2: hydro (cur+2) -> new (cur+1, where the heated state
// was), source partial sums (old - start + new - hydro) and the wave maxima of
// the new state for the next dt (python/cfdSolver/torchSession.py:401-411,
// 510-517).
template <typename R, int DIM, bool VARG>
__global__ void __launch_bounds__(256) react_kernel(StepArgs A, int stage) {
  constexpr int NV = DIM + 2;
  __shared__ double red[40];
  for (int t = A.t_begin + blockIdx.x; t < A.t_end; t += gridDim.x) {
    const Tile T = A.tiles[t];
    const InstDesc& d = A.desc[T.inst];
    InstState& st = A.st[T.inst];
    const int status = st.status;
    if (!(status == kReady || (stage == 1 && status == kRetry))) continue;  // uniform
    Geo<DIM> g;
    g.init(d);
    const int cur = st.cur;
    const int i0 = cur % d.nring, i1 = (cur + 1) % d.nring, i2 = (cur + 2) % d.nring;
    const R* Usrc = (const R*)d.U[stage == 1 ? i0 : i2];
    R* Udst = (R*)d.U[i1];
    const R* Ustart = (const R*)d.U[i0];
    const R* Lsrc = (const R*)d.lam[stage == 1 ? i0 : i2];
    R* Ldst = (R*)d.lam[i1];
    const bool znd = d.model == 1;
    const R* Bsrc = znd ? (const R*)d.beta[stage == 1 ? i0 : i2] : nullptr;
    R* Bdst = znd ? (R*)d.beta[i1] : nullptr;
    R* gam = VARG ? (R*)d.gam : nullptr;
    const double half = 0.5 * st.dt;
    const Chem<R> chem(d);
    const int ax = min(A.tx, g.na - T.x0);
    const int by = DIM == 3 ? min(A.ty, g.nb - T.y0) : 1;
    const bool owner = (int)threadIdx.x < ax * by;
    const int a = T.x0 + (owner ? (int)threadIdx.x % ax : 0);
    const int b = DIM == 3 ? T.y0 + (owner ? (int)threadIdx.x / ax : 0) : 0;
    R wmax[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) wmax[k] = R(0);
    double src[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) src[c] = 0.0;
    // single precision: this thread's column of source terms summed with
    // compensation (Kahan), converted once; the tile and global sums are FP64
    R ksum[NV], kcomp[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) ksum[c] = kcomp[c] = R(0);
    int fl = 0;
    if (owner) {
      for (int p = T.p0; p < T.p1; ++p) {
        const int64_t off = (int64_t)p * g.ps + (int64_t)b * g.na + a;
        R u[NV], hyd[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) {
          u[c] = Usrc[c * g.cs + off];
          hyd[c] = u[c];
        }
        R lam = Lsrc[off];
        R beta = znd ? Bsrc[off] : R(1);
        if (!react_cell<R, DIM>(chem, u, lam, beta, znd, half)) fl |= kFlagChemistry;
        if (stage == 2) {
#pragma unroll
          for (int c = 0; c < NV; ++c) {
            if constexpr (Exact<R>::value) {
              const double old = Udst[c * g.cs + off];  // heated state of this step
              const double start = Ustart[c * g.cs + off];
              src[c] += ((old - start) + u[c]) - hyd[c];
            } else {
              const R old = Udst[c * g.cs + off];
              const R start = Ustart[c * g.cs + off];
              const R y = (((old - start) + u[c]) - hyd[c]) - kcomp[c];
              const R t = ksum[c] + y;
              kcomp[c] = (t - ksum[c]) - y;
              ksum[c] = t;
            }
          }
          if (!physical_cell<R, NV>(u)) fl |= kFlagNonphysical;
        }
#pragma unroll
        for (int c = 0; c < NV; ++c) Udst[c * g.cs + off] = u[c];
        Ldst[off] = lam;
        if (znd) Bdst[off] = beta;
        const R gc = (chem.closure == 0) ? gamma_of_lambda(lam) : chem.gamma;
        if (VARG && stage == 1) gam[off] = gc;
        R w[DIM];
        wave_speeds<R, DIM>(u, gc, w);
#pragma unroll
        for (int k = 0; k < DIM; ++k) wmax[k] = fmax(wmax[k], w[k]);
      }
    }
    fl = block_or(fl, reinterpret_cast<int*>(red));
    double wm[DIM], sm[NV];
#pragma unroll
    for (int k = 0; k < DIM; ++k) wm[k] = (double)block_max(owner ? wmax[k] : R(0), red);
#pragma unroll
    for (int c = 0; c < NV; ++c) {
      if constexpr (!Exact<R>::value) src[c] = (double)ksum[c] - (double)kcomp[c];
      sm[c] = stage == 2 ? block_sum(src[c], red) : 0.0;
    }
    if (threadIdx.x == 0) {
      for (int k = 0; k < DIM; ++k) A.t_wmax[(size_t)t * 3 + k] = wm[k];
      if (stage == 2) {
        for (int c = 0; c < NV; ++c) A.t_sum[(size_t)t * 5 + c] = sm[c];
        A.t_flags[t] |= fl;
      } else {
        A.t_flags[t] = fl;
      }
    }
    __syncthreads();
  }
}

// Species transport with the hydro mass fluxes: first-order upwind in every
// direction (python/cfdSolver/torchSolver3D.py:246-256,
// torchSolver2D.py:659-667).  q = lambda (and beta) of the heated state
// (ring cur+1) -> ring cur+2.  Scalar ghost cells: no sign change; the 2D
// inlet rows hold fresh mixture (1).
template <typename R, int DIM>
__device__ __forceinline__ R fetch_scalar(const InstDesc& d, const Geo<DIM>& g, const R* q, int a,
                                          int b, int p) {
  bool ga, gb = false, gp;
  const int sa = map_axis(a, g.na, g.bca, ga);
  const int sb = DIM == 3 ? map_axis(b, g.nb, g.bcb, gb) : 0;
  const int sp = map_axis(p, g.np, g.bcp, gp);
  if (DIM == 2 && g.bcp == kBcInflow && p < 0) return R(1);
  return q[(int64_t)sp * g.ps + (int64_t)sb * g.na + sa];
}

template <typename R, int DIM>
__global__ void __launch_bounds__(256) species_kernel(StepArgs A) {
  __shared__ int red[40];
  for (int t = A.t_begin + blockIdx.x; t < A.t_end; t += gridDim.x) {
    const Tile T = A.tiles[t];
    const InstDesc& d = A.desc[T.inst];
    InstState& st = A.st[T.inst];
    if (st.status != kReady) continue;  // uniform
    Geo<DIM> g;
    g.init(d);
    const int cur = st.cur;
    const int i1 = (cur + 1) % d.nring, i2 = (cur + 2) % d.nring;
    const R* Uold = (const R*)d.U[i1];
    const R* Unew = (const R*)d.U[i2];
    const int nq = d.model == 1 ? 2 : 1;
    const R* mf[3] = {(const R*)d.flux_out[0], (const R*)d.flux_out[1], (const R*)d.flux_out[2]};
    R cu[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) cu[k] = R(st.coef_full[k]);
    const int ax = min(A.tx, g.na - T.x0);
    const int by = DIM == 3 ? min(A.ty, g.nb - T.y0) : 1;
    const bool owner = (int)threadIdx.x < ax * by;
    const int a = T.x0 + (owner ? (int)threadIdx.x % ax : 0);
    const int b = DIM == 3 ? T.y0 + (owner ? (int)threadIdx.x / ax : 0) : 0;
    int fl = 0;
    if (owner) {
      for (int s = 0; s < nq; ++s) {
        const R* q = (const R*)(s == 0 ? d.lam[i1] : d.beta[i1]);
        R* qn = (R*)(s == 0 ? d.lam[i2] : d.beta[i2]);
        for (int p = T.p0; p < T.p1; ++p) {
          const int64_t off = (int64_t)p * g.ps + (int64_t)b * g.na + a;
          const R qc = q[off];
          R rhoq = Uold[off] * qc;
#pragma unroll
          for (int dd = 0; dd < DIM; ++dd) {
            const int ia = dd == 0 ? 1 : 0;
            const int ib = (DIM == 3 && dd == 1) ? 1 : 0;
            const int ip = (DIM > 1 && dd == DIM - 1) ? 1 : 0;  // 1D has no marching axis
            // face arrays of this direction have one more entry along dd
            const int fa_n = dd == 0 ? g.na + 1 : g.na;
            const int fb_n = (DIM == 3 && dd == 1) ? g.nb + 1 : g.nb;
            const int64_t lo = ((int64_t)p * fb_n + b) * fa_n + a;
            const int64_t hi = ((int64_t)(p + ip) * fb_n + b + ib) * fa_n + a + ia;
            const R Flo = mf[dd][lo], Fhi = mf[dd][hi];
            const R qlo_l = fetch_scalar<R, DIM>(d, g, q, a - ia, b - ib, p - ip);
            const R qhi_r = fetch_scalar<R, DIM>(d, g, q, a + ia, b + ib, p + ip);
            const R Glo = Flo * (Flo >= R(0) ? qlo_l : qc);
            const R Ghi = Fhi * (Fhi >= R(0) ? qc : qhi_r);
            rhoq = rhoq - cu[dd] * (Ghi - Glo);
          }
          R frac;
          if (DIM == 3) {
            // the reference's interval check; FP32 roundoff needs a wider margin
            const R tol = Exact<R>::value ? R(1e-10) : R(1e-5);
            frac = rhoq / Unew[off];
            if (frac < -tol || frac > R(1) + tol) fl |= kFlagSpecies;
          } else {
            frac = rhoq / np_max(Unew[off], R(kFloor));
          }
          qn[off] = np_min(np_max(frac, R(0)), R(1));
        }
      }
    }
    fl = block_or(fl, red);
    if (threadIdx.x == 0 && fl) atomicOr(&A.t_flags[t], fl);
    __syncthreads();
  }
}

// gamma(lambda) of the current state into the per-cell gamma buffer.
template <typename R>
__global__ void gamma_kernel(StepArgs A) {
  for (int i = blockIdx.y; i < A.ninst; i += gridDim.y) {
    const InstDesc& d = A.desc[i];
    const InstState& st = A.st[i];
    if (!d.var_gamma || !d.gam) continue;
    const R* lam = (const R*)d.lam[(st.cur + A.src_off) % d.nring];
    R* gam = (R*)d.gam;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < d.ncell;
         k += (int64_t)gridDim.x * blockDim.x)
      gam[k] = gamma_of_lambda(lam[k]);
  }
}

#ifdef TFV_DEFINE_SHARED_KERNELS  // defined by exactly one translation unit
__global__ void __launch_bounds__(kFinalizeThreads) finalize_kernel(StepArgs A, int mode,
                                                                    int fp32,
                                                                    double* integrals_out) {
  // Grid (slices, instances).  A slice CTA reduces up to kFinalizeSlice tiles:
  // value k of the 23 partials (3 wave maxima, 15 boundary sums, 5 integrals)
  // is summed by kGroups threads over interleaved tiles, then in a fixed
  // order.  An instance with several slices publishes each slice's record;
  // the last slice to arrive combines the records in slice order (so the
  // result does not depend on which slice finished last) and commits.
  constexpr int NV = kPartVals;
  constexpr int kGroups = kFinalizeThreads / NV;
  __shared__ double vals[NV][kFinalizeSlice];  // this slice's partials, value-major
  __shared__ double acc[kFinalizeThreads];
  __shared__ double sh_v[NV];
  __shared__ int fred[kFinalizeThreads / 32];
  __shared__ int sh_f, sh_last;
  const int i = blockIdx.y;
  if (i >= A.ninst) return;
  const InstDesc& d = A.desc[i];
  InstState& st = A.st[i];
  if (mode == 0 && st.status != kReady) return;  // uniform over the instance's slices
  if (mode == 4 && st.status != kReady && st.status != kRetry) return;
  const int nslices = (d.ntiles + kFinalizeSlice - 1) / kFinalizeSlice;
  const int slice = blockIdx.x;
  if (slice >= nslices) return;
  const int nv = d.dim + 2;
  const bool want_s = mode == 0;
  const bool want_i = mode == 2 || mode == 3 || (mode == 0 && d.reactive);
  const int t0 = d.tile0 + slice * kFinalizeSlice;
  const int t1 = min(d.tile0 + d.ntiles, t0 + kFinalizeSlice);
  const int j = threadIdx.x;
  // one tile per thread: every load of the tile's record issued together
  int fl = 0;
  {
    const int t = t0 + j;
    const bool have = j < kFinalizeSlice && t < t1 && TFV_IN(32, t, A.ntiles);
    double w[3] = {0.0, 0.0, 0.0}, b[15], q[5];
#pragma unroll
    for (int k = 0; k < 15; ++k) b[k] = 0.0;
#pragma unroll
    for (int k = 0; k < 5; ++k) q[k] = 0.0;
    if (have) {
      fl = A.t_flags[t];
#pragma unroll
      for (int k = 0; k < 3; ++k) w[k] = A.t_wmax[(size_t)t * 3 + k];
      if (want_s) {
#pragma unroll
        for (int k = 0; k < 15; ++k) b[k] = A.t_bsum[(size_t)t * 15 + k];
      }
      if (want_i) {
#pragma unroll
        for (int k = 0; k < 5; ++k) q[k] = A.t_sum[(size_t)t * 5 + k];
      }
    }
    if (j < kFinalizeSlice) {
#pragma unroll
      for (int k = 0; k < 3; ++k) vals[k][j] = w[k];
#pragma unroll
      for (int k = 0; k < 15; ++k) vals[3 + k][j] = b[k];
#pragma unroll
      for (int k = 0; k < 5; ++k) vals[18 + k][j] = q[k];
    }
  }
  fl = block_or(fl, fred);  // includes a barrier: vals complete
  double v = 0.0;
  if (j < kGroups * NV) {
    const int k = j % NV, g = j / NV;
    const int m = t1 - t0;
    for (int r = g; r < m; r += kGroups) v = k < 3 ? fmax(v, vals[k][r]) : v + vals[k][r];
  }
  acc[j] = v;
  __syncthreads();
  if (j < NV) {
    double r = acc[j];
    for (int g = 1; g < kGroups; ++g) r = j < 3 ? fmax(r, acc[g * NV + j]) : r + acc[g * NV + j];
    sh_v[j] = r;
  }
  if (j == 0) sh_f = fl;
  __syncthreads();
  if (nslices > 1) {
    double* part = A.fin_part + ((size_t)i * A.fin_slices + slice) * (NV + 1);
    if (j < NV) part[j] = sh_v[j];
    if (j == 0) part[NV] = __int_as_double_bits(sh_f);
    __threadfence();
    __syncthreads();
    if (j == 0) sh_last = atomicAdd(&A.fin_cnt[i], 1) == nslices - 1;
    __syncthreads();
    if (!sh_last) return;
    __threadfence();
    const double* base = A.fin_part + (size_t)i * A.fin_slices * (NV + 1);
    if (j <= NV) {
      // slice records in slice order, loads issued eight at a time
      double r = j == NV ? 0.0 : __ldcg(base + j);
      int f = j == NV ? __double_bits_as_int(__ldcg(base + NV)) : 0;
      for (int q0 = 1; q0 < nslices; q0 += 8) {
        double x[8];
#pragma unroll
        for (int u = 0; u < 8; ++u)
          x[u] = q0 + u < nslices ? __ldcg(base + (size_t)(q0 + u) * (NV + 1) + j) : 0.0;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          if (q0 + u >= nslices) break;
          if (j == NV) f |= __double_bits_as_int(x[u]);
          else r = j < 3 ? fmax(r, x[u]) : r + x[u];
        }
      }
      if (j < NV) sh_v[j] = r;
      else sh_f = f;
    }
    if (j == 32) A.fin_cnt[i] = 0;  // ready for the next launch
    __syncthreads();
  }
  const double* sh_w = sh_v;
  const double* sh_s = sh_v + 3;
  const double* sh_i = sh_v + 18;
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  if (mode == 0) {
    // commit, one lane per conserved component
    const int f = sh_f;
    if (f & (kFlagNonphysical | kFlagSpecies | kFlagChemistry)) {
      if (lane == 0) {
        st.status = (f & kFlagNonphysical) ? kErrNonphysical
                    : (f & kFlagSpecies)   ? kErrSpecies
                                           : kErrChemistry;
        st.fb_word = 0;
      }
      return;
    }
    const double dt = st.dt;
    if (lane < nv) {
      double out = 0.0;
      for (int k = 0; k < d.dim; ++k) out += dt * d.vol / d.h[k] * sh_s[k * 5 + lane];
      st.boundary[lane] += out;
      if (d.reactive) st.source[lane] += d.vol * sh_i[lane];
    }
    const int fb = st.fb_word;
    __syncwarp();
    if (lane == 0) {
      st.cur = (st.cur + A.dst_off) % d.nring;
      const double tn = st.time + dt;
      st.time = tn < d.t_end ? tn : d.t_end;
      st.steps += 1;
      st.last_fallback = fb != 0;
      st.fallback_steps += fb != 0;
      st.fb_word = 0;
      st.retry = 0;
    }
    __syncwarp();
    plan_next_warp(d, st, sh_w, fp32, lane);
    return;
  }
  if (mode == 1 || mode == 3) {
    if (mode == 3 && lane < 5) st.initial[lane] = lane < nv ? sh_i[lane] * d.vol : 0.0;
    const int status = st.status;
    if (status != kReady && status != kDone) return;  // plan-only keeps a pending error
    __syncwarp();
    plan_next_warp(d, st, sh_w, fp32, lane);
    return;
  }
  if (lane != 0) return;
  if (mode == 2) {
    for (int c = 0; c < 5; ++c) integrals_out[i * 5 + c] = c < nv ? sh_i[c] * d.vol : 0.0;
    return;
  }
  if (mode == 4) {
    if (sh_f & kFlagChemistry) {
      st.status = kErrChemistry;
      return;
    }
    const double allowed = cfl_dt(d, sh_w);
    double dt = st.dt;
    if (dt <= allowed * (1 + 1e-12)) {
      st.status = kReady;
      return;
    }
    st.retry += 1;
    if (st.retry >= 60) {
      st.status = kErrReactive;
      return;
    }
    dt = (dt / 2 <= allowed) ? dt / 2 : allowed;
    if (fp32) dt = (double)(float)dt;
    set_dt(d, st, dt);
    st.status = kRetry;
    return;
  }
}

#endif  // TFV_DEFINE_SHARED_KERNELS

// --------------------------------------------------------------------------
// Stateless HLLC over n faces (python/cfdSolver/torchFlux.py:125-248).
// --------------------------------------------------------------------------
template <typename R, int NV>
__global__ void hllc_faces_kernel(int64_t n, const R* ul, const R* ur, const R* gl, const R* gr,
                                  R* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    R a[NV], b[NV], f[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) {
      a[c] = ul[c * n + i];
      b[c] = ur[c * n + i];
    }
    hllc<R, NV - 3>(a, b, gl[i], gr[i], f);
#pragma unroll
    for (int c = 0; c < NV; ++c) out[c * n + i] = f[c];
  }
}

}  // namespace tfv
