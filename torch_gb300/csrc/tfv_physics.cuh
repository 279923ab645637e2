// Device physics of TORCH's Cartesian finite-volume step, templated on the
// arithmetic type R.
//
// double — the reference-faithful path.  Every expression keeps the operation
//   order of the NumPy reference so that, compiled without FMA contraction
//   (-fmad=false), it reproduces the reference bit for bit: `a * b * c` in
//   Python is (a*b)*c, sums of squares over the component axis are
//   sequential, numpy.maximum/minimum propagate NaN, masks follow the
//   reference's precedence.
// float — the bulk FP32 path.  Same formulas, rearranged for throughput:
//   one reciprocal per density instead of one division per use, approximate
//   division and square root (MUFU), NaN-propagating min/max in one
//   instruction, a single finiteness test per state.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace tfv {

constexpr double kFloor = 1e-12;  // density / pressure floor
constexpr double kGuard = 1e-14;  // division guard (limiters, HLLC)

template <typename R>
struct Exact {
  static constexpr bool value = false;
};
template <>
struct Exact<double> {
  static constexpr bool value = true;
};

// numpy.maximum / numpy.minimum: NaN propagates, first operand wins ties.
__device__ __forceinline__ double np_max(double a, double b) { return (a >= b || a != a) ? a : b; }
__device__ __forceinline__ double np_min(double a, double b) { return (a <= b || a != a) ? a : b; }
__device__ __forceinline__ float np_max(float a, float b) {
  float r;
  asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float np_min(float a, float b) {
  float r;
  asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}

// numpy.maximum(a, numpy.maximum(b, c)) in one instruction: NaN if any
// operand is NaN (three-operand max, sm_100 and later).
__device__ __forceinline__ float np_max3(float a, float b, float c) {
  float r;
  asm("max.NaN.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// a / b: IEEE division (double) or the approximate single-precision one.
__device__ __forceinline__ double dv(double a, double b) { return a / b; }
__device__ __forceinline__ float dv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ float rcp(float b) { return __fdividef(1.0f, b); }

// np.where(abs(x) < g, g, x)
template <typename R>
__device__ __forceinline__ R guarded(R x, R g) { return (fabs(x) < g) ? g : x; }

template <typename R>
__device__ __forceinline__ bool finite_(R x) { return isfinite(x); }

// Constant gamma of an instance descriptor in the arithmetic type: single
// precision reads its float copy instead of converting the double per cell
// (a double-to-float conversion runs on the narrow FP64 pipe).
template <typename D>
__device__ __forceinline__ double desc_gamma(const D& d, double) { return d.gamma; }
template <typename D>
__device__ __forceinline__ float desc_gamma(const D& d, float) { return d.gamma_f; }

// --------------------------------------------------------------------------
// Limiters (LIM: 0 VanLeer, 1 Albada, 2 MINBEE, 3 Superbee, 4 Unos).
// 3D: python/cfdSolver/torchSolver3D.py:86-111.
// 2D: python/cfdSolver/torchSolver2D.py:124-168 (VanLeer/Albada zero for
//     r <= 0, Unos without the (1+2r)/3 bound).
// --------------------------------------------------------------------------
template <typename R, int DIM, int LIM>
__device__ __forceinline__ R limited_slope(R um, R uc, R up) {
  const R minus = uc - um;
  const R plus = up - uc;
  if constexpr (!Exact<R>::value && (LIM == 2 || LIM == 3)) {
    // single precision, MINBEE and Superbee: phi(r) * plus with r = minus /
    // plus, multiplied through by |plus| (no division): with s = sign(plus),
    // a = s * minus and b = |plus|, MINBEE is s * max(0, min(a, b)) and
    // Superbee s * max(0, max(min(2a, b), min(a, 2b))).  Equal to the
    // reference's form except where |plus| < 1e-14, whose guard changes the
    // result by less than 2e-14 (below single-precision resolution);
    // NaN still propagates through the NaN-propagating min / max.
    const R s = copysignf(1.0f, plus);
    const R a = minus * s;
    const R b = fabsf(plus);
    R t;
    if (LIM == 2)
      t = np_max(R(0), np_min(a, b));
    else
      t = np_max3(R(0), np_min(a + a, b), np_min(a, b + b));
    return t * s;
  }
  if constexpr (!Exact<R>::value && LIM == 0) {
    // single precision, VanLeer: with r = minus / plus > 0,
    // phi(r) * plus = 2 minus plus / (minus + plus); zero for r <= 0.  One
    // reciprocal instead of two; the guard of tiny |plus| makes a difference
    // below single-precision resolution; NaN inputs give NaN.
    const R mp = minus * plus;
    const R v = (mp + mp) * rcp(minus + plus);
    return mp > R(0) ? v : (mp == mp ? R(0) : mp);
  }
  const R r = dv(minus, guarded(plus, R(kGuard)));
  R phi;
  if (LIM == 1) {  // Albada
    const R pos = np_max(r, R(0));
    phi = dv(pos * pos + pos, pos * pos + R(1));
    if (DIM == 2 && !(r > R(0))) phi = R(0);
  } else if (LIM == 2) {  // MINBEE
    phi = np_max(R(0), np_min(r, R(1)));
  } else if (LIM == 3) {  // Superbee
    phi = np_max(R(0), np_max(np_min(R(2) * r, R(1)), np_min(r, R(2))));
  } else if (LIM == 4) {  // Unos
    if (DIM == 3)
      phi = np_max(R(0), np_min(np_min(np_min(R(2), R(2) * r), dv(R(2) + r, R(3))),
                                dv(R(1) + R(2) * r, R(3))));
    else
      phi = np_max(R(0), np_min(np_min(R(2), R(2) * r), dv(R(2) + r, R(3))));
  } else {  // VanLeer
    const R pos = np_max(r, R(0));
    phi = dv(R(2) * pos, R(1) + pos);
    if (DIM == 2 && !(r > R(0))) phi = R(0);
  }
  return phi * plus;
}

// --------------------------------------------------------------------------
// Predictor fluxes.
// 3D _flux: python/cfdSolver/torchSolver3D.py:77-83 with uconsv_to_uprim_3d
//   (:37-44, no floors).  m = normal momentum row (1..3).
// 2D euler_flux_x / euler_flux_y: python/cfdSolver/torchSolver2D.py:326-352
//   (rho and p floored).
// --------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void flux3(const R* u, R g, int m, R* f) {
  const R ssum = (u[1] * u[1] + u[2] * u[2]) + u[3] * u[3];
  R p, vel;
  if constexpr (Exact<R>::value) {
    const R rho = u[0];
    p = (g - R(1)) * (u[4] - (R(0.5) * ssum) / rho);
    vel = u[m] / rho;
  } else {
    const R irho = rcp(u[0]);
    p = (g - R(1)) * (u[4] - R(0.5) * ssum * irho);
    vel = u[m] * irho;
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) f[c] = u[c] * vel;
  if constexpr (!Exact<R>::value) f[0] = u[m];  // rho * (m / rho) is the momentum itself
  f[m] = f[m] + p;
  f[4] = vel * (u[4] + p);
}

template <typename R>
__device__ __forceinline__ void flux2(const R* u, R g, int normal, R* f) {
  const R rho = np_max(u[0], R(kFloor));
  R vx, vy;
  if constexpr (Exact<R>::value) {
    vx = u[1] / rho;
    vy = u[2] / rho;
  } else {
    const R irho = rcp(rho);
    vx = u[1] * irho;
    vy = u[2] * irho;
  }
  const R p = np_max((g - R(1)) * (u[3] - (R(0.5) * rho) * (vx * vx + vy * vy)), R(kFloor));
  if (normal == 0) {
    f[0] = rho * vx;
    f[1] = rho * (vx * vx) + p;
    f[2] = (rho * vx) * vy;
    f[3] = vx * (u[3] + p);
  } else {
    f[0] = rho * vy;
    f[1] = (rho * vx) * vy;
    f[2] = rho * (vy * vy) + p;
    f[3] = vy * (u[3] + p);
  }
}

// Physical-state test of one cell (python/cfdSolver/torchSolver.py:1038-1046).
template <typename R, int NV>
__device__ __forceinline__ bool physical_cell(const R* u) {
  R s = u[1] * u[1];
#pragma unroll
  for (int c = 2; c < NV - 1; ++c) s = s + u[c] * u[c];
  if constexpr (Exact<R>::value) {
    bool ok = true;
#pragma unroll
    for (int c = 0; c < NV; ++c) ok = ok && finite_(u[c]);
    return ok && (u[0] > R(kFloor)) && (u[NV - 1] - (R(0.5) * s) / u[0] > R(kFloor));
  } else {
    // one finiteness test: any NaN or infinity makes the sum non-finite
    R all = u[0];
#pragma unroll
    for (int c = 1; c < NV; ++c) all = all + u[c];
    // E - |m|^2 / (2 rho) > floor, multiplied through by rho > floor
    return finite_(all) && (u[0] > R(kFloor)) &&
           (u[NV - 1] * u[0] - R(0.5) * s > R(kFloor) * u[0]);
  }
}

// --------------------------------------------------------------------------
// HLLC in the normal basis: rows rho, m_n, m_t[NT], E
// (python/cfdSolver/torchFlux.py:125-248).  Only the star state of the side
// that can be selected is formed; values are identical to evaluating both.
// Where no wave-speed mask holds (NaN speeds) the result is NaN.
// --------------------------------------------------------------------------
template <typename R, int NT>
__device__ __forceinline__ void hllc(const R* ul, const R* ur, R gl, R gr, R* out) {
  constexpr int NV = NT + 3;
  constexpr int E = NV - 1;
  constexpr bool X = Exact<R>::value;
  const R g = R(0.5) * (gl + gr);
  const R rl = np_max(ul[0], R(kFloor));
  const R rr = np_max(ur[0], R(kFloor));
  R irl = R(0), irr = R(0);
  if constexpr (!X) {
    irl = rcp(rl);
    irr = rcp(rr);
  }
  const R unl = X ? ul[1] / rl : ul[1] * irl;
  const R unr = X ? ur[1] / rr : ur[1] * irr;
  R utl[NT], utr[NT];
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    utl[t] = X ? ul[2 + t] / rl : ul[2 + t] * irl;
    utr[t] = X ? ur[2 + t] / rr : ur[2 + t] * irr;
  }
  R stl = utl[0] * utl[0], str = utr[0] * utr[0];
#pragma unroll
  for (int t = 1; t < NT; ++t) {
    stl = stl + utl[t] * utl[t];
    str = str + utr[t] * utr[t];
  }
  const R kel = (R(0.5) * rl) * (unl * unl + stl);
  const R ker = (R(0.5) * rr) * (unr * unr + str);
  const R pl = np_max((gl - R(1)) * (ul[E] - kel), R(kFloor));
  const R pr = np_max((gr - R(1)) * (ur[E] - ker), R(kFloor));
  const R al = X ? sqrt((gl * pl) / rl) : sqrt(gl * pl * irl);
  const R ar = X ? sqrt((gr * pr) / rr) : sqrt(gr * pr * irr);

  R fl[NV], fr[NV];
  fl[0] = rl * unl;
  fl[1] = rl * (unl * unl) + pl;
  fr[0] = rr * unr;
  fr[1] = rr * (unr * unr) + pr;
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    fl[2 + t] = (rl * unl) * utl[t];
    fr[2 + t] = (rr * unr) * utr[t];
  }
  fl[E] = unl * (ul[E] + pl);
  fr[E] = unr * (ur[E] + pr);

  const R sql = sqrt(rl);
  const R sqr = sqrt(rr);
  const R inv = X ? R(1) / (sql + sqr) : rcp(sql + sqr);
  const R uroe = (sql * unl + sqr * unr) * inv;
  R vsum;
  {
    const R v0 = (sql * utl[0] + sqr * utr[0]) * inv;
    vsum = v0 * v0;
#pragma unroll
    for (int t = 1; t < NT; ++t) {
      const R vt = (sql * utl[t] + sqr * utr[t]) * inv;
      vsum = vsum + vt * vt;
    }
  }
  const R hl = X ? (ul[E] + pl) / rl : (ul[E] + pl) * irl;
  const R hr = X ? (ur[E] + pr) / rr : (ur[E] + pr) * irr;
  const R hroe = (sql * hl + sqr * hr) * inv;
  const R keroe = R(0.5) * (uroe * uroe + vsum);
  const R aroe = sqrt(np_max((g - R(1)) * (hroe - keroe), R(kFloor)));

  const R sL = np_min(unl - al, uroe - aroe);
  const R sR = np_max(unr + ar, uroe + aroe);
  const R den = guarded(rl * (sL - unl) - rr * (sR - unr), R(kGuard));
  const R ss = dv(((pr - pl) + (rl * unl) * (sL - unl)) - (rr * unr) * (sR - unr), den);

  // star state of the side whose star region can be selected
  const bool right = (ss <= R(0));
  const R rho = right ? rr : rl;
  const R un = right ? unr : unl;
  const R p = right ? pr : pl;
  const R s = right ? sR : sL;
  const R uE = right ? ur[E] : ul[E];
  const R dss = guarded(s - ss, R(kGuard));
  const R rho_s = np_max(rho * dv(s - un, dss), R(kFloor));
  const R dun = guarded(s - un, R(kGuard));
  R star[NV];
  star[0] = rho_s;
  star[1] = rho_s * ss;
#pragma unroll
  for (int t = 0; t < NT; ++t) star[2 + t] = rho_s * (right ? utr[t] : utl[t]);
  if constexpr (X) {
    star[E] = rho_s * (uE / rho + (ss - un) * (ss + p / (rho * dun)));
  } else {
    star[E] = rho_s * (uE * (right ? irr : irl) + (ss - un) * (ss + dv(p, rho * dun)));
  }
  const bool close = fabs(s - ss) < R(kFloor);

  const bool mr = (R(0) >= sR);
  const bool msr = (ss <= R(0)) && (R(0) <= sR);
  const bool msl = (sL <= R(0)) && (R(0) <= ss);
  const bool ml = (R(0) <= sL);
#pragma unroll
  for (int c = 0; c < NV; ++c) {
    const R uc = right ? ur[c] : ul[c];
    const R fc = right ? fr[c] : fl[c];
    const R fstar = close ? fc : fc + s * (star[c] - uc);
    R v = R(NAN);
    if (ml) v = fl[c];
    if (msl || msr) v = fstar;
    if (mr) v = fr[c];
    out[c] = v;
  }
}

// Rotation into the normal basis (python/cfdSolver/torchFlux.py:36-39):
// order = [0, normal] + other momenta ascending + [E].
template <int NV>
__device__ __forceinline__ void normal_order(int normal, int* order) {
  order[0] = 0;
  order[1] = normal;
  int k = 2;
#pragma unroll
  for (int m = 1; m < NV - 1; ++m)
    if (m != normal) order[k++] = m;
  order[NV - 1] = NV - 1;
}

// Single-precision HLLC of the fused step (same states, speeds and masks as
// hllc above).  Only one physical flux is formed: the region that the masks
// select (left, right, or the star state of the side `ss <= 0` picks, in the
// reference's precedence: right supersonic, then star, then left
// supersonic) reads one side's flux, so the other side's flux is never
// needed.  It also tests both input face states for the 3D predictor gate
// (density and internal energy density above the floor; NaN fails) and ORs
// the result into `gate`: every predicted face state the step consumes
// passes through here once.  NaN where no mask holds, as in hllc.
template <int NT>
__device__ __forceinline__ void hllc_gated(const float* ul, const float* ur, float gl, float gr,
                                           float* out, bool& gate) {
  constexpr int NV = NT + 3;
  constexpr int E = NV - 1;
  const float fl = float(kFloor);
  const float g = 0.5f * (gl + gr);
  // the density floors of the reference change nothing here: a face state
  // whose density is not above the floor fails the gate test below and the
  // step is redone to first order
  const float rl = ul[0];
  const float rr = ur[0];
  const float irl = rcp(rl), irr = rcp(rr);
  const float unl = ul[1] * irl, unr = ur[1] * irr;
  float utl[NT], utr[NT];
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    utl[t] = ul[2 + t] * irl;
    utr[t] = ur[2 + t] * irr;
  }
  float stl = utl[0] * utl[0], str = utr[0] * utr[0];
#pragma unroll
  for (int t = 1; t < NT; ++t) {
    stl = stl + utl[t] * utl[t];
    str = str + utr[t] * utr[t];
  }
  const float eil = ul[E] - (0.5f * rl) * (unl * unl + stl);  // internal energy density
  const float eir = ur[E] - (0.5f * rr) * (unr * unr + str);
  if (!(ul[0] > fl && eil > fl && ur[0] > fl && eir > fl)) gate = true;
  const float pl = np_max((gl - 1.0f) * eil, fl);
  const float pr = np_max((gr - 1.0f) * eir, fl);
  const float al = sqrtf(gl * pl * irl);
  const float ar = sqrtf(gr * pr * irr);
  const float sql = sqrtf(rl), sqr = sqrtf(rr);
  const float inv = rcp(sql + sqr);
  const float uroe = (sql * unl + sqr * unr) * inv;
  float vsum;
  {
    const float v0 = (sql * utl[0] + sqr * utr[0]) * inv;
    vsum = v0 * v0;
#pragma unroll
    for (int t = 1; t < NT; ++t) {
      const float vt = (sql * utl[t] + sqr * utr[t]) * inv;
      vsum = vsum + vt * vt;
    }
  }
  const float hl = (ul[E] + pl) * irl;
  const float hr = (ur[E] + pr) * irr;
  const float hroe = (sql * hl + sqr * hr) * inv;
  const float aroe = sqrtf(np_max((g - 1.0f) * (hroe - 0.5f * (uroe * uroe + vsum)), fl));
  const float sL = np_min(unl - al, uroe - aroe);
  const float sR = np_max(unr + ar, uroe + aroe);
  const float den = guarded(rl * (sL - unl) - rr * (sR - unr), float(kGuard));
  const float ss = dv(((pr - pl) + (rl * unl) * (sL - unl)) - (rr * unr) * (sR - unr), den);

  const bool mr = (0.0f >= sR);
  const bool mstar = ((ss <= 0.0f) && (0.0f <= sR)) || ((sL <= 0.0f) && (0.0f <= ss));
  const bool ml = (0.0f <= sL);
  // side whose flux the selected region reads
  const bool right = mr || (mstar && ss <= 0.0f);
  const float rho = right ? rr : rl;
  const float irho = right ? irr : irl;
  const float un = right ? unr : unl;
  const float p = right ? pr : pl;
  const float uE = right ? ur[E] : ul[E];
  float u[NV], f[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) u[c] = right ? ur[c] : ul[c];
  const float mn = rho * un;
  f[0] = mn;
  f[1] = mn * un + p;
#pragma unroll
  for (int t = 0; t < NT; ++t) f[2 + t] = mn * (right ? utr[t] : utl[t]);
  f[E] = un * (uE + p);
  const float s = right ? sR : sL;
  if (!mr && mstar && !(fabsf(s - ss) < fl)) {
    const float rho_s = np_max(rho * dv(s - un, guarded(s - ss, float(kGuard))), fl);
    const float dun = guarded(s - un, float(kGuard));
    float star[NV];
    star[0] = rho_s;
    star[1] = rho_s * ss;
#pragma unroll
    for (int t = 0; t < NT; ++t) star[2 + t] = rho_s * (right ? utr[t] : utl[t]);
    star[E] = rho_s * (uE * irho + (ss - un) * (ss + dv(p, rho * dun)));
#pragma unroll
    for (int c = 0; c < NV; ++c) f[c] = f[c] + s * (star[c] - u[c]);
  }
  // No NaN select for "no region": with face states that pass the gate test
  // above, sL, sR and ss are finite and one of the three regions always
  // holds; states that fail it flag the tile, and the flagged step is redone
  // to first order, so this flux is never committed.
#pragma unroll
  for (int c = 0; c < NV; ++c) out[c] = f[c];
}

template <int NV>
__device__ __forceinline__ void hllc_cartesian_gated(const float* L, const float* Rt, float gl,
                                                     float gr, int d, float* F, bool& gate) {
  int order[NV];
  normal_order<NV>(d + 1, order);
  float ul[NV], ur[NV], f[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) {
    ul[c] = L[order[c]];
    ur[c] = Rt[order[c]];
  }
  hllc_gated<NV - 3>(ul, ur, gl, gr, f, gate);
#pragma unroll
  for (int c = 0; c < NV; ++c) F[order[c]] = f[c];
}

// HLLC across a face along direction d (0=x,1=y,2=z) with Cartesian inputs
// and output (python/cfdSolver/torchFlux.py:6-77 without the batching).
template <typename R, int NV>
__device__ __forceinline__ void hllc_cartesian(const R* L, const R* Rt, R gl, R gr, int d,
                                               R* F) {
  int order[NV];
  normal_order<NV>(d + 1, order);
  R ul[NV], ur[NV], f[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) {
    ul[c] = L[order[c]];
    ur[c] = Rt[order[c]];
  }
  hllc<R, NV - 3>(ul, ur, gl, gr, f);
#pragma unroll
  for (int c = 0; c < NV; ++c) F[order[c]] = f[c];
}

}  // namespace tfv
