// 1D chain of the session step (python/cfdSolver/torchSession.py:413-445):
// one ghost cell (bc_creator), Sweby-bounded MUSCL with the sound-speed
// controlled w and the half-step predictor (muscl_wlim_calc), PVRS or
// Roe-Einfeldt interface wave speeds (wave_speed_estimate), HLLC with those
// speeds (hllc_flux_calc_for_muscl, "Variante 1" / "Variante_2"),
// conservative update with the whole-step Rusanov fallback
// (conservative_update_1d), and dt = min(delta_t_estimate, hydro_dt_1d).
//
// A 1D tile is a chunk of tx cells; one thread per cell.  Per-instance
// scratch (InstDesc::scratch) holds the interface wave speeds [3][n+1], the
// reconstructed half-step states [6][n] and the interface fluxes [3][n+1].
#pragma once

#include "tfv_kernels.cuh"

namespace tfv {

template <typename R>
struct Scratch1D {
  R* waves;  // s_L, s_*, s_R per face
  R* recon;  // left / right half-step states per cell (3 + 3 rows)
  R* flux;   // interface fluxes
  __device__ __forceinline__ Scratch1D(const InstDesc& d) {
    const int n = d.n[0];
    waves = (R*)d.scratch;
    recon = waves + 3 * (n + 1);
    flux = recon + 6 * n;
  }
};

// Padded cell k in [-1, n] (python/cfdSolver/torchSolver.py:164-186).
template <typename R>
__device__ __forceinline__ void cell1(const InstDesc& d, const R* U, int k, R* u) {
  const int n = d.n[0];
  int src = k;
  bool flip = false;
  if (k < 0) {
    src = d.bc[0] == kBcPeriodic ? n - 1 : 0;
    flip = d.bc[0] == kBcReflective;
  } else if (k >= n) {
    src = d.bc[0] == kBcPeriodic ? 0 : n - 1;
    flip = d.bc[0] == kBcReflective;
  }
  if (!TFV_IN(40, src, n)) {
    u[0] = u[1] = u[2] = R(0);
    return;
  }
  u[0] = U[src];
  u[1] = flip ? -U[n + src] : U[n + src];
  u[2] = U[2 * n + src];
}

// gamma of padded cell k: scalar_bc wraps for Periodic, copies the edge otherwise
// (python/cfdSolver/torchSolver.py:1121-1122).
template <typename R>
__device__ __forceinline__ R gamma1(const InstDesc& d, const R* gam, int k) {
  if (!gam) return desc_gamma(d, R(0));
  const int n = d.n[0];
  const int src = k < 0 ? (d.bc[0] == kBcPeriodic ? n - 1 : 0)
                        : (k >= n ? (d.bc[0] == kBcPeriodic ? 0 : n - 1) : k);
  return gam[src];
}

// uconsv_to_uprim (torchSolver.py:117-127)
template <typename R>
__device__ __forceinline__ void prim1(const R* u, R g, R& rho, R& v, R& p) {
  rho = np_max(u[0], R(kFloor));
  v = u[1] / rho;
  p = np_max((u[2] - (R(0.5) * rho) * (v * v)) * (g - R(1)), R(kFloor));
}

// sound_speed_calc (torchSolver.py:81-87)
template <typename R>
__device__ __forceinline__ R sound1(R rho, R p, R g) {
  return sqrt((g * np_max(p, R(0))) / np_max(rho, R(kFloor)));
}

// u_to_fu_calc (torchSolver.py:145-156)
template <typename R>
__device__ __forceinline__ void flux1(const R* u, R g, R* f) {
  R rho, v, p;
  prim1(u, g, rho, v, p);
  f[0] = rho * v;
  f[1] = rho * (v * v) + p;
  f[2] = v * (u[2] + p);
}

// Interface wave speeds between padded cells f-1 and f
// (python/cfdSolver/torchSolver.py:283-404).
template <typename R>
__device__ __forceinline__ void waves1(const InstDesc& d, const R* L, const R* Rr, R gl, R gr,
                                       R* s) {
  R rl, ul, pl, rr, ur, pr;
  prim1(L, gl, rl, ul, pl);
  prim1(Rr, gr, rr, ur, pr);
  const R al = sound1(rl, pl, gl), ar = sound1(rr, pr, gr);
  R sl, sr;
  if (d.wavespeed == 0) {  // Pressure Based (PVRS)
    const R rho_avg = R(0.5) * (rr + rl);
    const R a_avg = R(0.5) * (al + ar);
    const R ps = np_max(R(0), R(0.5) * (pl + pr) - ((R(0.5) * (ur - ul)) * rho_avg) * a_avg);
    const R ql = ps > pl ? sqrt(R(1) + ((gl + R(1)) / (R(2) * gl)) * (ps / pl - R(1))) : R(1);
    const R qr = ps > pr ? sqrt(R(1) + ((gr + R(1)) / (R(2) * gr)) * (ps / pr - R(1))) : R(1);
    sl = ul - al * ql;
    sr = ur + ar * qr;
  } else {  // Enthalpy Based (Roe-Einfeldt)
    const R el = rl * (R(0.5) * (ul * ul) + pl / ((gl - R(1)) * rl));
    const R er = rr * (R(0.5) * (ur * ur) + pr / ((gr - R(1)) * rr));
    const R sql = sqrt(rl), sqr = sqrt(rr);
    const R den = np_max(sql + sqr, R(kFloor));
    const R uavg = (sql * ul + sqr * ur) / den;
    const R havg = (sql * ((el + pl) / rl) + sqr * ((er + pr) / rr)) / den;
    const R gavg = R(0.5) * (gl + gr);
    const R aavg = sqrt(np_max((gavg - R(1)) * (havg - R(0.5) * (uavg * uavg)), R(1e-10)));
    sl = np_min(ul - al, uavg - aavg);
    sr = np_max(ur + ar, uavg + aavg);
  }
  const R den = guarded(rl * (sl - ul) - rr * (sr - ur), R(kGuard));
  R ss = (((pr - pl) + (rl * ul) * (sl - ul)) - (rr * ur) * (sr - ur)) / den;
  ss = np_min(np_max(ss, sl), sr);
  s[0] = sl;
  s[1] = ss;
  s[2] = sr;
}

// Sweby-bounded limited slope (python/cfdSolver/torchSolver.py:201-275).
template <typename R>
__device__ __forceinline__ R nan0(R x) { return isfinite(x) ? x : R(0); }

template <typename R>
__device__ __forceinline__ R limit1(R delta, R uw, R dw, R w, int limiter) {
  const R r = nan0(uw / dw);
  const R denom = (R(1) - w) + (R(1) + w) * r;
  const R eps_r = nan0(R(2) / (fabs(denom) < R(kFloor) ? R(kFloor) : denom));
  R eps = R(0);
  switch (limiter) {
    case 1:  // Albada
      if (r > R(0)) eps = np_min(nan0((r * (R(1) + r)) / (R(1) + r * r)), eps_r);
      break;
    case 2:  // MINBEE
      if (r > R(0) && r < R(1)) eps = r;
      if (r >= R(1)) eps = np_min(R(1), eps_r);
      break;
    case 3:  // Superbee
      if (r > R(0))
        eps = np_min(nan0(np_max(R(0), np_max(np_min(R(2) * r, R(1)), np_min(r, R(2))))), eps_r);
      break;
    case 4:  // Unos
      eps = np_min(np_max(R(0), np_min(np_min(R(2), R(2) * r), (R(2) + r) / R(3))), eps_r);
      break;
    default:  // VanLeer
      if (r > R(0)) eps = np_min(nan0((R(2) * r) / (R(1) + r)), eps_r);
      break;
  }
  eps = np_max(R(0), nan0(eps));
  const R slope = eps * delta;
  const R bound = R(2) * np_min(fabs(uw), fabs(dw));
  if (!(uw * dw > R(0))) return R(0);
  const R mag = np_min(fabs(slope), bound);
  return dw > R(0) ? mag : -mag;
}

// HLLC with precomputed S_L, S_R (python/cfdSolver/torchSolver.py:534-676).
template <typename R>
__device__ __forceinline__ void hllc1(const InstDesc& d, const R* UL, const R* UR, R gl, R gr,
                                      R sl, R sr, R* out) {
  R rl, vl, pl, rr, vr, pr;
  prim1(UL, gl, rl, vl, pl);
  prim1(UR, gr, rr, vr, pr);
  const R el = rl * (R(0.5) * (vl * vl) + pl / ((gl - R(1)) * rl));
  const R er = rr * (R(0.5) * (vr * vr) + pr / ((gr - R(1)) * rr));
  R fl[3], fr[3];
  flux1(UL, gl, fl);
  flux1(UR, gr, fr);
  const R den = guarded(rl * (sl - vl) - rr * (sr - vr), R(kGuard));
  R ss = (((pr - pl) + (rl * vl) * (sl - vl)) - (rr * vr) * (sr - vr)) / den;
  ss = np_min(np_max(ss, sl), sr);
  const R eps = R(kFloor);
  R fls[3], frs[3];
  if (d.variant == 0) {  // Variante 1 - Original
    const bool okl = fabs(sl - ss) > eps, okr = fabs(sr - ss) > eps;
    const R dl = okl ? sl - ss : -eps;
    const R dr = okr ? sr - ss : eps;
    const R dul = fabs(sl - vl) < eps ? -eps : sl - vl;
    const R dur = fabs(sr - vr) < eps ? eps : sr - vr;
    const R tl = el / rl + (ss - vl) * (ss + pl / (rl * dul));
    const R tr = er / rr + (ss - vr) * (ss + pr / (rr * dur));
    const R kl = rl * ((sl - vl) / dl), kr = rr * ((sr - vr) / dr);
    const R stl[3] = {kl * R(1), kl * ss, kl * tl};
    const R str[3] = {kr * R(1), kr * ss, kr * tr};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      fls[c] = fl[c] + sl * ((okl ? stl[c] : UL[c]) - UL[c]);
      frs[c] = fr[c] + sr * ((okr ? str[c] : UR[c]) - UR[c]);
    }
  } else {  // Variante_2
    const R ds[3] = {R(0), R(1), ss};
    const R sgl = (sl - ss + R(1e-30)) > R(0) ? R(1) : ((sl - ss + R(1e-30)) < R(0) ? R(-1) : R(0));
    const R sgr = (sr - ss + R(1e-30)) > R(0) ? R(1) : ((sr - ss + R(1e-30)) < R(0) ? R(-1) : R(0));
    const R dl = fabs(sl - ss) < eps ? sgl * eps : sl - ss;
    const R dr = fabs(sr - ss) < eps ? sgr * eps : sr - ss;
    const R ml = sl * (pl + (rl * (sl - vl)) * (ss - vl));
    const R mr = sr * (pr + (rr * (sr - vr)) * (ss - vr));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      fls[c] = (ss * (sl * UL[c] - fl[c]) + ml * ds[c]) / dl;
      frs[c] = (ss * (sr * UR[c] - fr[c]) + mr * ds[c]) / dr;
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    R v = R(0);
    if (sl > R(0)) v = fl[c];
    if (sl <= R(0) && ss > R(0)) v = fls[c];
    if (ss <= R(0) && sr >= R(0)) v = frs[c];
    if (sr < R(0)) v = fr[c];
    out[c] = v;
  }
}

// Interface states of face f of the reconstructed array: left = GL or the
// right half-state of cell f-1, right = GR or the left half-state of cell f
// (bc_creator applied to the interleaved states, torchSolver.py:494-508).
template <typename R>
__device__ __forceinline__ void face_states1(const InstDesc& d, const R* recon, int f, R* L,
                                             R* Rr) {
  const int n = d.n[0];
  auto rl = [&](int i, int c) { return recon[c * n + i]; };        // left half-state
  auto rr = [&](int i, int c) { return recon[(3 + c) * n + i]; };  // right half-state
  const bool per = d.bc[0] == kBcPeriodic, refl = d.bc[0] == kBcReflective;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (f == 0) L[c] = per ? rr(n - 1, c) : rl(0, c);
    else L[c] = rr(f - 1, c);
    if (f == n) Rr[c] = per ? rl(0, c) : rr(n - 1, c);
    else Rr[c] = rl(f, c);
  }
  if (f == 0 && refl) L[1] = -L[1];
  if (f == n && refl) Rr[1] = -Rr[1];
}

// Wave speeds of the state for the step and the next dt; per tile max |S|
// over its faces and max(|u| + a) over its cells, integrals, flags.
template <typename R, bool VARG>
// in_step: the pass inside a step (after the update or the second reaction
// half step): flags are ORed into the step's, the step's sums are kept;
// 2: the same, only for instances whose step was redone at first order;
// otherwise (bind, re-plan, integrals) the integrals of the state are written.
__global__ void __launch_bounds__(256) waves1d_kernel(StepArgs A, int in_step) {
  __shared__ double red[40];
  if (in_step == 2) {  // usually no instance took the fallback
    int any = 0;
    for (int k = threadIdx.x; k < A.ninst; k += blockDim.x)
      any |= (A.st[k].status == kReady && A.st[k].fb_word != 0);
    if (!__syncthreads_or(any)) return;
  }
  for (int t = A.t_begin + blockIdx.x; t < A.t_end; t += gridDim.x) {
    if (!TFV_IN(45, t, A.ntiles)) continue;
    const Tile T = A.tiles[t];
    if (!TFV_IN(46, T.inst, A.ninst)) continue;
    const InstDesc& d = A.desc[T.inst];
    const InstState& st = A.st[T.inst];
    if (in_step == 2 && (st.status != kReady || st.fb_word == 0)) continue;  // uniform
    const int n = d.n[0];
    const R* U = (const R*)d.U[(st.cur + A.src_off) % d.nring];
    const R* gam = VARG ? (const R*)d.gam : nullptr;
    Scratch1D<R> S(d);
    const int ax = min(A.tx, n - T.x0);
    const int i = T.x0 + (int)threadIdx.x;
    const bool owner = (int)threadIdx.x < ax;
    R ws = R(0), wh = R(0);
    double sum[3] = {0.0, 0.0, 0.0};
    bool bad = false;
    if (owner) {
      for (int f = i; f <= (i == n - 1 ? n : i); ++f) {  // face i (and face n by the last cell)
        R L[3], Rr[3], s[3];
        cell1(d, U, f - 1, L);
        cell1(d, U, f, Rr);
        waves1(d, L, Rr, gamma1(d, gam, f - 1), gamma1(d, gam, f), s);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          if (!TFV_IN(41, f, n + 1)) continue;
          if (!TFV_INSIDE(62, S.waves + k * (n + 1) + f, d.scratch, S.flux + 3 * (n + 1))) continue;
          S.waves[k * (n + 1) + f] = s[k];
          ws = fmax(ws, fabs(s[k]));
        }
      }
      R u[3];
      cell1(d, U, i, u);
      const R g = gamma1(d, gam, i);
      R rho, v, p;
      prim1(u, g, rho, v, p);
      wh = fabs(v) + sound1(rho, p, g);
      if (!in_step)
        for (int c = 0; c < 3; ++c) sum[c] = (double)u[c];
      bad = !physical_cell<R, 3>(u);
    }
    const int fl = block_or(bad ? kFlagNonphysical : 0, reinterpret_cast<int*>(red));
    const double mws = (double)block_max(ws, red);
    const double mwh = (double)block_max(wh, red);
    double sm[3] = {0.0, 0.0, 0.0};
    if (!in_step)  // uniform
      for (int c = 0; c < 3; ++c) sm[c] = block_sum(sum[c], red);
    if (threadIdx.x == 0) {
      A.t_wmax[(size_t)t * 3 + 0] = mws;
      A.t_wmax[(size_t)t * 3 + 1] = mwh;
      A.t_wmax[(size_t)t * 3 + 2] = 0.0;
      if (in_step) {
        A.t_flags[t] |= fl;
      } else {
        for (int c = 0; c < 3; ++c) A.t_sum[(size_t)t * 5 + c] = sm[c];
        A.t_flags[t] = fl;
      }
    }
    __syncthreads();
  }
}

// Limited half-step states (left ol, right orr) of a cell with state c0
// between neighbours cm and cp (python/cfdSolver/torchSolver.py:412-491).
template <typename R>
__device__ __forceinline__ R recon1_coef(const InstDesc& d, const InstState& st) {
  return -R(st.dt / (2.0 * d.h[0]));  // -(dt / (2 dx)) of the Hancock half step
}

// kcoef = recon1_coef(d, st), formed once per tile by the caller
template <typename R>
__device__ __forceinline__ void recon1_cells(const InstDesc& d, const R* c0, const R* cm,
                                             const R* cp, R g, R kcoef, R* ol, R* orr) {
  R w = R(0);
  if (d.controller == 0) {  // Sound Speed Controlled
    R rho, v, p;
    prim1(c0, g, rho, v, p);
    const R a = sound1(rho, p, g);
    const R mach = nan0(fabs(v) / np_max(a, R(kFloor)));
    w = np_min(np_max((R(1) - mach) / (R(1) + mach), R(-1)), R(1));
  }
  R ul[3], ur[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const R delta = R(0.5) * (cp[c] - cm[c]);
    const R lim = limit1(delta, c0[c] - cm[c], cp[c] - c0[c], w, d.limiter);
    ul[c] = c0[c] - R(0.5) * lim;
    ur[c] = c0[c] + R(0.5) * lim;
  }
  R fl[3], fr[3];
  flux1(ul, g, fl);
  flux1(ur, g, fr);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const R dfu = kcoef * (fr[c] - fl[c]);
    ol[c] = ul[c] + dfu;
    orr[c] = ur[c] + dfu;
  }
  R* outs[2] = {ol, orr};
  for (int sidx = 0; sidx < 2; ++sidx) {
    R* s = outs[sidx];
    const R p = (g - R(1)) * (s[2] - (R(0.5) * (s[1] * s[1])) / np_max(s[0], R(kFloor)));
    const bool badc = s[0] <= R(kFloor) || p <= R(kFloor) || !isfinite(s[0]) ||
                      !isfinite(s[1]) || !isfinite(s[2]);
    if (badc)
      for (int c = 0; c < 3; ++c) s[c] = c0[c];
  }
}

// recon1_cells of cell i read from the state array (one ghost cell by the
// boundary rule).
template <typename R>
__device__ __forceinline__ void recon1(const InstDesc& d, const InstState& st, const R* U,
                                       const R* gam, int i, R* ol, R* orr) {
  R c0[3], cm[3], cp[3];
  cell1(d, U, i, c0);
  cell1(d, U, i - 1, cm);
  cell1(d, U, i + 1, cp);
  recon1_cells<R>(d, c0, cm, cp, gamma1(d, gam, i), recon1_coef<R>(d, st), ol, orr);
}

// MUSCL reconstruction and half-step predictor per cell
// (python/cfdSolver/torchSolver.py:412-491).
template <typename R, bool VARG>
__global__ void __launch_bounds__(256) recon1d_kernel(StepArgs A) {
  for (int t = A.t_begin + blockIdx.x; t < A.t_end; t += gridDim.x) {
    if (!TFV_IN(45, t, A.ntiles)) continue;
    const Tile T = A.tiles[t];
    if (!TFV_IN(46, T.inst, A.ninst)) continue;
    const InstDesc& d = A.desc[T.inst];
    const InstState& st = A.st[T.inst];
    if (st.status != kReady) continue;
    const int n = d.n[0];
    const R* U = (const R*)d.U[(st.cur + A.src_off) % d.nring];
    const R* gam = VARG ? (const R*)d.gam : nullptr;
    Scratch1D<R> S(d);
    const int i = T.x0 + (int)threadIdx.x;
    if ((int)threadIdx.x >= min(A.tx, n - T.x0)) continue;
    R ol[3], orr[3];
    recon1<R>(d, st, U, gam, i, ol, orr);
    if (!TFV_IN(42, i, n)) continue;
    for (int c = 0; c < 3; ++c) {
      if (!TFV_INSIDE(63, S.recon + (3 + c) * n + i, d.scratch, S.flux + 3 * (n + 1)) ||
          !TFV_INSIDE(64, S.recon + c * n + i, A.ws_lo, A.ws_hi))
        continue;
      S.recon[c * n + i] = ol[c];
      S.recon[(3 + c) * n + i] = orr[c];
    }
  }
}

// Conservative update (second order: faces from the reconstruction; first
// order fallback: Rusanov on the padded cells), writing the face fluxes the
// species transport needs, flags and boundary sums
// (python/cfdSolver/torchSolver.py:692-700, 1054-1071).
template <typename R, bool VARG>
__device__ __forceinline__ void face_flux1(const InstDesc& d, const R* U, const R* gam,
                                           const Scratch1D<R>& S, int f, bool first_order,
                                           R* F) {
  const int n = d.n[0];
  const R gl = gamma1(d, gam, f - 1), gr = gamma1(d, gam, f);
  if (!first_order) {
    R L[3], Rr[3];
    if (!TFV_IN(43, f, n + 1)) {
      F[0] = F[1] = F[2] = R(0);
      return;
    }
    face_states1(d, S.recon, f, L, Rr);
    hllc1(d, L, Rr, gl, gr, S.waves[f], S.waves[2 * (n + 1) + f], F);
    return;
  }
  R L[3], Rr[3], pfl[3], pfr[3];
  cell1(d, U, f - 1, L);
  cell1(d, U, f, Rr);
  R rl, vl, pl, rr, vr, pr;
  prim1(L, gl, rl, vl, pl);
  prim1(Rr, gr, rr, vr, pr);
  const R alpha = np_max(fabs(vl) + sound1(rl, pl, gl), fabs(vr) + sound1(rr, pr, gr));
  flux1(L, gl, pfl);
  flux1(Rr, gr, pfr);
#pragma unroll
  for (int c = 0; c < 3; ++c) F[c] = R(0.5) * ((pfl[c] + pfr[c]) - alpha * (Rr[c] - L[c]));
}

template <typename R, bool VARG>
__global__ void __launch_bounds__(256) update1d_kernel(StepArgs A, int first_order) {
  __shared__ double red[40];
  if (first_order) {  // the fallback pass: usually no instance is flagged
    int any = 0;
    for (int k = threadIdx.x; k < A.ninst; k += blockDim.x)
      any |= (A.st[k].status == kReady && A.st[k].fb_word != 0);
    if (!__syncthreads_or(any)) return;
  }
  for (int t = A.t_begin + blockIdx.x; t < A.t_end; t += gridDim.x) {
    if (!TFV_IN(45, t, A.ntiles)) continue;
    const Tile T = A.tiles[t];
    if (!TFV_IN(46, T.inst, A.ninst)) continue;
    const InstDesc& d = A.desc[T.inst];
    InstState& st = A.st[T.inst];
    if (st.status != kReady) continue;
    if (first_order && st.fb_word == 0) continue;  // uniform
    const int n = d.n[0];
    const R* U = (const R*)d.U[(st.cur + A.src_off) % d.nring];
    R* Un = (R*)d.U[(st.cur + A.dst_off) % d.nring];
    const R* gam = VARG ? (const R*)d.gam : nullptr;
    Scratch1D<R> S(d);
    const int ax = min(A.tx, n - T.x0);
    const int i = T.x0 + (int)threadIdx.x;
    const bool owner = (int)threadIdx.x < ax;
    double bsum[3] = {0.0, 0.0, 0.0};
    bool bad = false;
    if (owner) {
      R Fm[3], Fp[3], u[3];
      face_flux1<R, VARG>(d, U, gam, S, i, first_order != 0, Fm);
      face_flux1<R, VARG>(d, U, gam, S, i + 1, first_order != 0, Fp);
      cell1(d, U, i, u);
      const R k = -R(st.coef_full[0]);
      R un[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) un[c] = u[c] + k * (Fp[c] - Fm[c]);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (!TFV_IN(44, i, n)) continue;
        if (!TFV_OUTSIDE(65, Un + c * n + i, A.ws_lo, A.ws_hi) ||
            !TFV_INSIDE(66, S.flux + c * (n + 1) + n, d.scratch, S.flux + 3 * (n + 1)))
          continue;
        Un[c * n + i] = un[c];
        S.flux[c * (n + 1) + i] = Fm[c];
        if (i == n - 1) S.flux[c * (n + 1) + n] = Fp[c];
        if (i == 0) bsum[c] -= (double)Fm[c];
        if (i == n - 1) bsum[c] += (double)Fp[c];
      }
      bad = !physical_cell<R, 3>(un);
    }
    const int fl = block_or(bad ? kFlagNonphysical : 0, reinterpret_cast<int*>(red));
    double sm[3];
    for (int c = 0; c < 3; ++c) sm[c] = block_sum(bsum[c], red);
    if (threadIdx.x == 0) {
      for (int c = 0; c < 3; ++c) A.t_bsum[(size_t)t * 15 + c] = sm[c];
      A.t_flags[t] = fl;
      if (fl && !first_order) atomicOr(&st.fb_word, fl);
    }
    __syncthreads();
  }
}


// Face flux at face f (0 <= f <= n) of the current state, evaluated from
// scratch: the two reconstructed interface states (bc_creator rules at the
// domain faces, torchSolver.py:494-508), the interface wave speeds
// (torchSolver.py:283-404) and HLLC with them (torchSolver.py:534-676).
template <typename R, bool VARG>
__device__ __forceinline__ void face_flux_direct1(const InstDesc& d, const InstState& st,
                                                  const R* U, const R* gam, int f, R* F) {
  const int n = d.n[0];
  const bool per = d.bc[0] == kBcPeriodic, refl = d.bc[0] == kBcReflective;
  R ol[3], orr[3], L[3], Rr[3];
  // left state: the right half-state of cell f-1 (at f == 0: periodic wraps
  // to cell n-1, otherwise the left half-state of cell 0)
  const int li = f == 0 ? (per ? n - 1 : 0) : f - 1;
  const bool l_right = f != 0 || per;
  recon1<R>(d, st, U, gam, li, ol, orr);
#pragma unroll
  for (int c = 0; c < 3; ++c) L[c] = l_right ? orr[c] : ol[c];
  // right state: the left half-state of cell f (at f == n: periodic wraps to
  // cell 0, otherwise the right half-state of cell n-1)
  const int ri = f == n ? (per ? 0 : n - 1) : f;
  const bool r_left = f != n || per;
  recon1<R>(d, st, U, gam, ri, ol, orr);
#pragma unroll
  for (int c = 0; c < 3; ++c) Rr[c] = r_left ? ol[c] : orr[c];
  if (f == 0 && refl) L[1] = -L[1];
  if (f == n && refl) Rr[1] = -Rr[1];
  R a[3], b[3], s[3];
  cell1(d, U, f - 1, a);
  cell1(d, U, f, b);
  const R gl = gamma1(d, gam, f - 1), gr = gamma1(d, gam, f);
  waves1(d, a, b, gl, gr, s);
  hllc1(d, L, Rr, gl, gr, s[0], s[2], F);
}

// Physical cell of padded index k in [-1, n] (cell1's ghost rule) and
// whether its momentum is mirrored.
__device__ __forceinline__ int phys1(const InstDesc& d, int k, bool& flip) {
  const int n = d.n[0];
  flip = false;
  if (k >= 0 && k < n) return k;
  flip = d.bc[0] == kBcReflective;
  if (k < 0) return d.bc[0] == kBcPeriodic ? n - 1 : 0;
  return d.bc[0] == kBcPeriodic ? 0 : n - 1;
}

// The whole inert 1D step of a tile in one kernel: faces, update, positivity
// flags, boundary sums, and the next dt's wave speeds of the new state.
// Shared memory holds the tile's state with a 3-cell halo; every cell is
// reconstructed once and every face's wave speeds and flux are evaluated once.
// The CTA also updates the cell on either side of its tile (the neighbouring
// tile's, or the ghost's source cell at a domain end), so that the interface
// wave speeds of the new state at its tile faces need no second pass.  Values
// are the same expressions as in the split kernels (recon1d, update1d,
// waves1d), so results are identical.  At a periodic domain end the wrapped
// neighbour lies outside the staged range and is evaluated from global memory.
template <typename R, bool VARG>
__global__ void __launch_bounds__(256) step1d_kernel(StepArgs A) {
  __shared__ double red[40];
  extern __shared__ __align__(16) unsigned char step1d_smem[];
  const int W = A.tx + 6;  // staged padded cells x0-3 .. x0+tx+2
  R* us = reinterpret_cast<R*>(step1d_smem);  // [3][W] state
  R* gs = us + 3 * W;                          // [W] gamma
  R* rc = gs + W;                              // [6][W] half-step states (l, r)
  R* fx = rc + 6 * W;                          // [3][W] flux at the face left of slot k
  R* un_s = fx + 3 * W;                        // [3][tx + 2] new state of the targets
  const int TS = A.tx + 2;
  for (int t = A.t_begin + blockIdx.x; t < A.t_end; t += gridDim.x) {
    if (!TFV_IN(45, t, A.ntiles)) continue;
    const Tile T = A.tiles[t];
    if (!TFV_IN(46, T.inst, A.ninst)) continue;
    const InstDesc& d = A.desc[T.inst];
    InstState& st = A.st[T.inst];
    if (st.status != kReady) continue;  // uniform
    const int n = d.n[0];
    const R* U = (const R*)d.U[(st.cur + A.src_off) % d.nring];
    R* Un = (R*)d.U[(st.cur + A.dst_off) % d.nring];
    const R* gam = VARG ? (const R*)d.gam : nullptr;
    const int ax = min(A.tx, n - T.x0);
    const int x0 = T.x0;
    const bool per = d.bc[0] == kBcPeriodic, refl = d.bc[0] == kBcReflective;
    const R kcoef = recon1_coef<R>(d, st);
    // slot k <-> padded cell x0 - 3 + k
    for (int k = threadIdx.x; k < ax + 6; k += blockDim.x) {
      const int pk = x0 - 3 + k;
      if (pk < -1 || pk > n) continue;
      R u[3];
      cell1(d, U, pk, u);
#pragma unroll
      for (int c = 0; c < 3; ++c) us[c * W + k] = u[c];
      gs[k] = gamma1(d, gam, pk);
    }
    __syncthreads();
    // half-step states of the cells x0-2 .. x0+ax+1 inside the domain
    for (int k = 1 + threadIdx.x; k < ax + 5; k += blockDim.x) {
      const int i = x0 - 3 + k;
      if (i < 0 || i >= n) continue;
      R c0[3], cm[3], cp[3], ol[3], orr[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        c0[c] = us[c * W + k];
        cm[c] = us[c * W + k - 1];
        cp[c] = us[c * W + k + 1];
      }
      recon1_cells<R>(d, c0, cm, cp, gs[k], kcoef, ol, orr);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        rc[c * W + k] = ol[c];
        rc[(3 + c) * W + k] = orr[c];
      }
    }
    __syncthreads();
    // faces x0-1 .. x0+ax+1 inside [0, n]; face f lies left of slot k = f - x0 + 3
    for (int k = 2 + threadIdx.x; k < ax + 5; k += blockDim.x) {
      const int f = x0 - 3 + k;
      if (f < 0 || f > n) continue;
      R L[3], Rr[3], ol[3], orr[3];
      if (f == 0 && per) {  // wraps to cell n-1: outside the staged range
        recon1<R>(d, st, U, gam, n - 1, ol, orr);
#pragma unroll
        for (int c = 0; c < 3; ++c) L[c] = orr[c];
      } else {
        // f == 0: left half-state of cell 0 (slot k); else right half of f-1
#pragma unroll
        for (int c = 0; c < 3; ++c) L[c] = f == 0 ? rc[c * W + k] : rc[(3 + c) * W + k - 1];
      }
      if (f == n && per) {  // wraps to cell 0
        recon1<R>(d, st, U, gam, 0, ol, orr);
#pragma unroll
        for (int c = 0; c < 3; ++c) Rr[c] = ol[c];
      } else {
        // f == n: right half-state of cell n-1 (slot k-1); else left half of f
#pragma unroll
        for (int c = 0; c < 3; ++c) Rr[c] = f == n ? rc[(3 + c) * W + k - 1] : rc[c * W + k];
      }
      if (f == 0 && refl) L[1] = -L[1];
      if (f == n && refl) Rr[1] = -Rr[1];
      R a[3], b[3], w3[3], F[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        a[c] = us[c * W + k - 1];
        b[c] = us[c * W + k];
      }
      waves1(d, a, b, gs[k - 1], gs[k], w3);
      hllc1(d, L, Rr, gs[k - 1], gs[k], w3[0], w3[2], F);
#pragma unroll
      for (int c = 0; c < 3; ++c) fx[c * W + k] = F[c];
    }
    __syncthreads();
    // targets: slot q <-> padded x0 + q - 1, q in [0, ax + 1]
    const R kk = -R(st.coef_full[0]);
    double bsum[3] = {0.0, 0.0, 0.0};
    bool bad = false;
    for (int q = threadIdx.x; q < ax + 2; q += blockDim.x) {
      bool flip;
      const int j = phys1(d, x0 + q - 1, flip);
      R Fm[3], Fp[3], u[3];
      if (j >= x0 - 1 && j <= x0 + ax) {  // the cell and its faces are staged
        const int k = j - x0 + 3;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          Fm[c] = fx[c * W + k];
          Fp[c] = fx[c * W + k + 1];
          u[c] = us[c * W + k];
        }
      } else {  // periodic wrap at a domain end
        face_flux_direct1<R, VARG>(d, st, U, gam, j, Fm);
        face_flux_direct1<R, VARG>(d, st, U, gam, j + 1, Fp);
        cell1(d, U, j, u);
      }
      R un[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) un[c] = u[c] + kk * (Fp[c] - Fm[c]);
#pragma unroll
      for (int c = 0; c < 3; ++c) un_s[c * TS + q] = un[c];
      if (q >= 1 && q <= ax) {  // a cell of this tile
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          if (!TFV_IN(44, j, n) || !TFV_OUTSIDE(65, Un + c * n + j, A.ws_lo, A.ws_hi)) continue;
          Un[c * n + j] = un[c];
          if (j == 0) bsum[c] -= (double)Fm[c];
          if (j == n - 1) bsum[c] += (double)Fp[c];
        }
        if (!physical_cell<R, 3>(un)) bad = true;
      }
    }
    __syncthreads();
    // the next dt: interface wave speeds and |u| + a of the new state
    R ws = R(0), wh = R(0);
    const int nf = ax + (x0 + ax == n ? 1 : 0);  // faces x0 .. x0+ax-1 (+ face n)
    for (int s = threadIdx.x; s < nf; s += blockDim.x) {
      const int f = x0 + s;
      bool fl_l, fl_r;
      phys1(d, f - 1, fl_l);
      phys1(d, f, fl_r);
      R L[3], Rr[3], w3[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        L[c] = un_s[c * TS + s];
        Rr[c] = un_s[c * TS + s + 1];
      }
      if (fl_l) L[1] = -L[1];
      if (fl_r) Rr[1] = -Rr[1];
      waves1(d, L, Rr, gamma1(d, gam, f - 1), gamma1(d, gam, f), w3);
#pragma unroll
      for (int k = 0; k < 3; ++k) ws = fmax(ws, fabs(w3[k]));
      if (s < ax) {
        R rho, v, p;
        const R g = gamma1(d, gam, f);
        R uc[3] = {un_s[0 * TS + s + 1], un_s[1 * TS + s + 1], un_s[2 * TS + s + 1]};
        prim1(uc, g, rho, v, p);
        wh = fmax(wh, fabs(v) + sound1(rho, p, g));
      }
    }
    const int fl = block_or(bad ? kFlagNonphysical : 0, reinterpret_cast<int*>(red));
    const double mws = (double)block_max(ws, red);
    const double mwh = (double)block_max(wh, red);
    double sm[3] = {0.0, 0.0, 0.0};
    if (x0 == 0 || x0 + ax == n)  // boundary faces only in the end tiles (uniform)
      for (int c = 0; c < 3; ++c) sm[c] = block_sum(bsum[c], red);
    if (threadIdx.x == 0) {
      A.t_wmax[(size_t)t * 3 + 0] = mws;
      A.t_wmax[(size_t)t * 3 + 1] = mwh;
      A.t_wmax[(size_t)t * 3 + 2] = 0.0;
      for (int c = 0; c < 3; ++c) A.t_bsum[(size_t)t * 15 + c] = sm[c];
      A.t_flags[t] = fl;
      if (fl) atomicOr(&st.fb_word, fl);
    }
    __syncthreads();
  }
}

}  // namespace tfv
