// Kernels of the metric / face-boundary finite-volume step: MUSCL
// reconstruction of primitives, Rusanov fluxes weighted by face areas,
// geometric sources of cylindrical / annular / spherical grids, SSPRK2
// stages, per-face boundary states, and the CFL rate.
//
// Reference: python/cfdSolver/torchFiniteVolume.py:16-276 (primitive,
// conservative, face_states, boundary_state, cfl_dt, limited, rhs, advance),
// python/cfdSolver/torchBoundaries.py:185-246 (ghost),
// python/cfdSolver/torchGeometry.py:95-204 (Metrics: volumes, areas,
// divergence, source).
//
// Geometry is separable: every volume and face area is an outer product of
// one-dimensional factors (torchGeometry.py:107-117), multiplied x, then y,
// then z.  The kernels keep only the factors and form each product in that
// order, which reproduces the reference's arrays exactly in double precision.
//
// Layout: a state is [nv][nz][ny][nx], x fastest.  Face arrays of direction
// d have n_d + 1 entries along axis d and the cell counts along the others.
// Double precision keeps the reference's operation order (with -fmad=false)
// so that results are bitwise the reference's except where pow enters
// (pressure outlet and stagnation inlet boundary states), whose CUDA and
// C-library roundings may differ in the last bit.
#pragma once

#include "tfv_kernels.cuh"
#include "tfv_metric.h"

namespace tfv {

constexpr int kMThreads = 256;

// Launch bounds of the column-marching kernels: the single-precision unit
// asks for three resident CTAs per SM (80 registers a thread: 24 warps
// instead of 16 hide the marching loads' latency); double precision leaves
// the register count to the compiler.
#if defined(TFV_MARCH_MIN_BLOCKS) && TFV_MARCH_MIN_BLOCKS > 0
#define TFV_MARCH_BOUNDS __launch_bounds__(kMThreads, TFV_MARCH_MIN_BLOCKS)
#else
#define TFV_MARCH_BOUNDS __launch_bounds__(kMThreads)
#endif
// The same for the one-thread-per-face kernel (x faces in single precision).
#if defined(TFV_FACE_MIN_BLOCKS) && TFV_FACE_MIN_BLOCKS > 0
#define TFV_FACE_BOUNDS __launch_bounds__(kMThreads, TFV_FACE_MIN_BLOCKS)
#else
#define TFV_FACE_BOUNDS __launch_bounds__(kMThreads)
#endif

template <typename R>
__device__ __forceinline__ R tpow(R a, R b);
template <>
__device__ __forceinline__ double tpow<double>(double a, double b) { return pow(a, b); }
template <>
__device__ __forceinline__ float tpow<float>(float a, float b) { return powf(a, b); }

// Read of an array that no thread of the running kernel writes (the
// non-coherent load path; lets loads move ahead of the kernel's stores).
template <typename T>
__device__ __forceinline__ T ro(const T* p) {
  return __ldg(p);
}

// cell coordinates of a linear index
struct MIdx {
  int i, j, k;
};
__device__ __forceinline__ MIdx cell_of(int64_t off, const int* n) {
  MIdx c;
  c.i = (int)(off % n[0]);
  const int64_t r = off / n[0];
  c.j = (int)(r % n[1]);
  c.k = (int)(r / n[1]);
  return c;
}
__device__ __forceinline__ uint32_t udiv(uint32_t n, const UDiv& v) {
  return (uint32_t)(((uint64_t)__umulhi(n, v.m) + n) >> v.l);
}
// (x, y) of index r = y * d + x, 0 <= x < d, by the invariant divisor of d
__device__ __forceinline__ void split32(uint32_t r, const UDiv& v, int& x, int& y) {
  const uint32_t q = udiv(r, v);
  x = (int)(r - q * v.d);
  y = (int)q;
}
template <typename R>
__device__ __forceinline__ MIdx cell_of(int64_t off, const MArgs<R>& A) {
  if (!A.idx32) return cell_of(off, A.n);
  MIdx c;
  int r;
  split32((uint32_t)off, A.dn0, c.i, r);
  split32((uint32_t)r, A.dn1, c.j, c.k);
  return c;
}
__device__ __forceinline__ int64_t off_of(int i, int j, int k, const int* n) {
  return ((int64_t)k * n[1] + j) * n[0] + i;
}

// volume of cell (i, j, k): factors multiplied x, y, z
template <typename R, int DIM>
__device__ __forceinline__ R volume(const MArgs<R>& A, const MIdx& c) {
  R v = ro(&A.vf[0][c.i]);
  if (DIM >= 2) v = v * ro(&A.vf[1][c.j]);
  if (DIM == 3) v = v * ro(&A.vf[2][c.k]);
  return v;
}

// area of face f along direction d at the transverse coordinates of c
template <typename R, int DIM>
__device__ __forceinline__ R area(const MArgs<R>& A, int d, int f, const MIdx& c) {
  const int idx[3] = {d == 0 ? f : c.i, d == 1 ? f : c.j, d == 2 ? f : c.k};
  R a = ro(&A.ff[d][0][idx[0]]);
  if (DIM >= 2) a = a * ro(&A.ff[d][1][idx[1]]);
  if (DIM == 3) a = a * ro(&A.ff[d][2][idx[2]]);
  return a;
}

// primitives and gamma of one cell (torchFiniteVolume.py:16-22)
template <typename R, int NV>
__device__ __forceinline__ void primitive_of(const R* u, R g, R* p) {
  R s = u[1] * u[1];
#pragma unroll
  for (int c = 2; c < NV - 1; ++c) s = s + u[c] * u[c];
  p[0] = u[0];
#pragma unroll
  for (int c = 1; c < NV - 1; ++c) p[c] = u[c] / u[0];
  p[NV - 1] = (g - R(1)) * (u[NV - 1] - (R(0.5) * s) / u[0]);
}

// conservative state of face primitives (torchFiniteVolume.py:25-29)
template <typename R, int NV>
__device__ __forceinline__ void conservative_of(const R* p, R g, R* u) {
  R s = p[1] * p[1];
#pragma unroll
  for (int c = 2; c < NV - 1; ++c) s = s + p[c] * p[c];
  u[0] = p[0];
#pragma unroll
  for (int c = 1; c < NV - 1; ++c) u[c] = p[c] * p[0];
  u[NV - 1] = p[NV - 1] / (g - R(1)) + (R(0.5) * p[0]) * s;
}

// A padded cell: primitives, gamma and fractions.
template <typename R, int NV>
struct MCell {
  R p[NV];
  R g;
  R q[2];
};

template <typename R, int NV>
__device__ __forceinline__ void load_cell(const MArgs<R>& A, int64_t off, MCell<R, NV>& c) {
#pragma unroll
  for (int v = 0; v < NV; ++v) c.p[v] = ro(&A.P[v * A.nc + off]);
  c.g = A.reactive ? ro(&A.G[off]) : A.gam;
  c.q[0] = A.nfrac > 0 ? ro(&A.Q[0][off]) : R(0);
  c.q[1] = A.nfrac > 1 ? ro(&A.Q[1][off]) : R(0);
}

// Boundary state built from the boundary cell (torchBoundaries.py:185-246).
// side -1 low face, +1 high face; d the direction.  Returns error bits.
template <typename R, int NV>
__device__ __forceinline__ int ghost_state(const MArgs<R>& A, const MFace<R>& F, int d, int side,
                                           MCell<R, NV>& c) {
  const int n = d + 1;
  const R gamma = c.g;  // the boundary cell's gamma
  if (F.type == kFaceWall) {
    c.p[n] = -c.p[n];
    return 0;
  }
  if (F.type == kFaceInflow || F.type == kFaceStagnation) {
    const R g = A.reactive ? F.gam : gamma;
    c.g = g;
    c.q[0] = F.lam;
    c.q[1] = F.beta;
    if (F.type == kFaceInflow) {
#pragma unroll
      for (int v = 0; v < NV; ++v) c.p[v] = F.prim[v];
      return 0;
    }
    const R sound = sqrt((gamma * c.p[NV - 1]) / c.p[0]);
    const R riemann = R(-side) * c.p[n] - (R(2) * sound) / (gamma - R(1));
    const R a0sq = (g * F.rgas) * F.t0;
    const R k = (g + R(1)) / (g - R(1));
    const R disc = riemann * riemann - k * ((R(0.5) * (g - R(1))) * (riemann * riemann) - a0sq);
    if (disc < R(0)) return kMErrReservoirSolution;
    R a = (-riemann + sqrt(disc)) / k;
    R speed = riemann + (R(2) * a) / (g - R(1));
    if (speed >= a) {  // choked
      a = sqrt((R(2) * a0sq) / (g + R(1)));
      speed = a;
    }
    if (speed < R(0) || a <= R(0)) return kMErrReservoirSupply;
#pragma unroll
    for (int v = 1; v < NV - 1; ++v) c.p[v] = R(0);
    c.p[n] = R(-side) * speed;
    c.p[NV - 1] = F.p0 * tpow((a * a) / a0sq, g / (g - R(1)));
    c.p[0] = (g * c.p[NV - 1]) / (a * a);
    return 0;
  }
  if (F.type == kFacePressureOutlet) {
    const R g = gamma;
    const R a = sqrt((g * c.p[NV - 1]) / c.p[0]);
    const R un = R(side) * c.p[n];
    const bool subsonic = un < a;
    const R pr = F.pressure;
    const R rho = c.p[0] * tpow(pr / c.p[NV - 1], R(1) / g);
    const R anew = sqrt((g * pr) / rho);
    const R velocity = un + (R(2) * (a - anew)) / (g - R(1));
    const bool back = subsonic && (velocity < R(0) || un < R(0));
    if (back && !F.has_backflow) return kMErrBackflow;
    if (subsonic) {
      c.p[0] = rho;
      c.p[NV - 1] = pr;
      c.p[n] = R(side) * velocity;
    }
    if (back) {
#pragma unroll
      for (int v = 0; v < NV; ++v) c.p[v] = F.prim[v];
      if (A.reactive) c.g = F.gam;
      c.q[0] = F.lam;
      c.q[1] = F.beta;
    }
    return 0;
  }
  return 0;  // outflow: the boundary cell itself
}

// Padded cell j (0..n+1) along direction D of the line through c
// (torchFiniteVolume.py:32-70).
template <typename R, int NV, int D>
__device__ __forceinline__ int padded_cell(const MArgs<R>& A, int j, const MIdx& c,
                                           MCell<R, NV>& out) {
  const int n = A.n[D];
  const bool periodic = A.periodic[D];
  int i = c.i, jj = c.j, k = c.k;
  int at;
  int side = 0;
  if (j == 0) {
    side = -1;
    at = periodic ? n - 1 : 0;
  } else if (j == n + 1) {
    side = 1;
    at = periodic ? 0 : n - 1;
  } else {
    at = j - 1;
  }
  if (D == 0) i = at;
  if (D == 1) jj = at;
  if (D == 2) k = at;
  load_cell<R, NV>(A, off_of(i, jj, k, A.n), out);
  if (side != 0 && !periodic) return ghost_state<R, NV>(A, A.face[2 * D + (side > 0)], D, side, out);
  return 0;
}

// limited (torchFiniteVolume.py:105-126)
template <typename R>
__device__ __forceinline__ R metric_limited(R minus, R plus, int lim) {
  const R r = minus / ((fabs(plus) < R(1e-14)) ? R(1e-14) : plus);
  const R pos = np_max(r, R(0));
  R phi;
  if (lim == 0) {
    phi = (R(2) * pos) / (R(1) + pos);
  } else if (lim == 1) {
    phi = (pos * pos + pos) / (pos * pos + R(1));
  } else if (lim == 2) {
    phi = np_max(R(0), np_min(r, R(1)));
  } else if (lim == 3) {
    phi = np_max(R(0), np_max(np_min(R(2) * r, R(1)), np_min(r, R(2))));
  } else {
    phi = np_max(R(0), np_min(np_min(R(2), R(2) * r),
                              np_min((R(2) + r) / R(3), (R(1) + R(2) * r) / R(3))));
  }
  return phi * plus;
}

// slope of padded cell j from its neighbours; zero when the reconstructed
// density or pressure could reach the floor (torchFiniteVolume.py:146-153)
template <typename R, int NV>
__device__ __forceinline__ void cell_slope(const MCell<R, NV>& m, const MCell<R, NV>& c,
                                           const MCell<R, NV>& p, int lim, R* s) {
#pragma unroll
  for (int v = 0; v < NV; ++v) s[v] = metric_limited(c.p[v] - m.p[v], p.p[v] - c.p[v], lim);
  const bool bad = (c.p[0] - R(0.5) * fabs(s[0])) <= R(1e-12) ||
                   (c.p[NV - 1] - R(0.5) * fabs(s[NV - 1])) <= R(1e-12);
  if (bad) {
#pragma unroll
    for (int v = 0; v < NV; ++v) s[v] = s[v] * R(0);
  }
}

// -- 1. primitives, gamma and geometric source --------------------------------
template <typename R, int DIM>
__global__ void __launch_bounds__(kMThreads) metric_prim_kernel(MArgs<R> A) {
  constexpr int NV = DIM + 2;
  __shared__ double red[32];
  double part[NV];
  // single precision: this thread's source sums with compensation (Kahan),
  // converted once; block and grid sums are double
  R ksum[NV], kcomp[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    part[v] = 0.0;
    ksum[v] = kcomp[v] = R(0);
  }
  // two cells of the thread's grid-stride sequence per iteration, both
  // loaded before either is processed (twice the loads in flight); they are
  // processed, and their source summed, in sequence order
  auto cell = [&](int64_t off, const R* u, R g) {
    R p[NV];
    primitive_of<R, NV>(u, g, p);
#pragma unroll
    for (int v = 0; v < NV; ++v) A.P[v * A.nc + off] = p[v];
    if (A.reactive) A.G[off] = g;
    A.S[off] = sqrt((g * p[NV - 1]) / p[0]);  // as cell_speed forms it
    R s[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) s[v] = R(0);
    if (A.geometry != kGeoCartesian) {  // torchGeometry.py:177-204
      const MIdx c = cell_of(off, A);
      const R vol = volume<R, DIM>(A, c);
      const R rho = p[0], pr = p[NV - 1];
      const R radial = (area<R, DIM>(A, 0, c.i + 1, c) - area<R, DIM>(A, 0, c.i, c)) / vol;
      s[1] = pr * radial;
      if (A.geometry == kGeoSpherical) {
        const R invr = radial / R(2);
        R sq = R(0);
        if (DIM >= 2) sq = p[2] * p[2];
        if (DIM == 3) sq = sq + p[3] * p[3];
        s[1] = s[1] + (rho * sq) * invr;
        if (DIM >= 2) {
          const R cot = (area<R, DIM>(A, 1, c.j + 1, c) - area<R, DIM>(A, 1, c.j, c)) / vol;
          s[2] = pr * cot - ((rho * p[1]) * p[2]) * invr;
          if (DIM == 3) {
            s[2] = s[2] + (rho * (p[3] * p[3])) * cot;
            s[3] = ((-rho) * p[3]) * (p[1] * invr + p[2] * cot);
          }
        }
      } else if (DIM >= 2 && !(A.geometry == kGeoCylindrical && DIM == 2)) {
        s[1] = s[1] + (rho * (p[2] * p[2])) * radial;
        s[2] = (((-rho) * p[1]) * p[2]) * radial;
      }
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        if constexpr (Exact<R>::value) {
          part[v] += s[v] * vol;
        } else {
          const R y = s[v] * vol - kcomp[v];
          const R t = ksum[v] + y;
          kcomp[v] = (t - ksum[v]) - y;
          ksum[v] = t;
        }
      }
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) A.K[v * A.nc + off] = s[v];
  };
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t off = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; off < A.nc;
       off += 2 * stride) {
    const int64_t off2 = off + stride;
    const bool two = off2 < A.nc;
    R u1[NV], u2[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      u1[v] = ro(&A.U[v * A.nc + off]);
      u2[v] = two ? ro(&A.U[v * A.nc + off2]) : R(1);
    }
    const R g1 = A.reactive ? gamma_of_lambda(ro(&A.Q[0][off])) : A.gam;
    const R g2 = A.reactive && two ? gamma_of_lambda(ro(&A.Q[0][off2])) : A.gam;
    cell(off, u1, g1);
    if (two) cell(off2, u2, g2);
  }
  if constexpr (!Exact<R>::value) {
#pragma unroll
    for (int v = 0; v < NV; ++v) part[v] = (double)ksum[v] - (double)kcomp[v];
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const double t = block_sum(part[v], red);
    if (threadIdx.x == 0) A.part[blockIdx.x * 8 + v] = t;
  }
}

// -- 2. Rusanov fluxes of one direction, weighted by the face areas ------------
// Rusanov flux of face f (padded cells f and f + 1 with their slopes),
// weighted by the face area, and the upwind fraction transport
// (torchFiniteVolume.py:160-226).
// The area-weighted flux (W[NV]) and fraction transport (T[2]) of face f.
template <typename R, int DIM, int D>
__device__ __forceinline__ void face_flux(const MArgs<R>& A, int f, const MIdx& c,
                                          const MCell<R, DIM + 2>& cl,
                                          const MCell<R, DIM + 2>& cr, const R* sl, const R* sr,
                                          R* W, R* T) {
  constexpr int NV = DIM + 2;
  constexpr int d = D;
  const int n = A.n[d];
  R left[NV], right[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    left[v] = cl.p[v] + R(0.5) * sl[v];
    right[v] = cr.p[v] - R(0.5) * sr[v];
  }
  R gl = cl.g, gr = cr.g;
  // walls mirror the interior face state (torchFiniteVolume.py:164-181)
  if (f == 0 && A.face[2 * d].type == kFaceWall) {  // face table in device memory
#pragma unroll
    for (int v = 0; v < NV; ++v) left[v] = right[v];
    gl = gr;
    left[d + 1] = -left[d + 1];
  }
  if (f == n && A.face[2 * d + 1].type == kFaceWall) {
#pragma unroll
    for (int v = 0; v < NV; ++v) right[v] = left[v];
    gr = gl;
    right[d + 1] = -right[d + 1];
  }
  // Rusanov (torchFiniteVolume.py:186-207)
  R ul[NV], ur[NV], fl[NV], fr[NV];
  conservative_of<R, NV>(left, gl, ul);
  conservative_of<R, NV>(right, gr, ur);
  const R vl = left[d + 1], vr = right[d + 1];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    fl[v] = ul[v] * vl;
    fr[v] = ur[v] * vr;
  }
  fl[d + 1] = fl[d + 1] + left[NV - 1];
  fr[d + 1] = fr[d + 1] + right[NV - 1];
  fl[NV - 1] = fl[NV - 1] + vl * left[NV - 1];
  fr[NV - 1] = fr[NV - 1] + vr * right[NV - 1];
  const R speed = np_max(fabs(vl) + sqrt((gl * left[NV - 1]) / left[0]),
                         fabs(vr) + sqrt((gr * right[NV - 1]) / right[0]));
  const R ar = area<R, DIM>(A, d, f, c);
  R flux0 = R(0);
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const R flux = ((fl[v] + fr[v]) - (ur[v] - ul[v]) * speed) * R(0.5);
    if (v == 0) flux0 = flux;
    W[v] = flux * ar;
  }
  // first-order upwind transport of the fractions (torchFiniteVolume.py:223-226)
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const R up = flux0 >= R(0) ? cl.q[q] : cr.q[q];
    T[q] = q < A.nfrac ? (flux0 * up) * ar : R(0);
  }
}

template <typename R, int DIM, int D>
__device__ __forceinline__ void emit_face(const MArgs<R>& A, int f, const MIdx& c, int64_t idx,
                                          const MCell<R, DIM + 2>& cl,
                                          const MCell<R, DIM + 2>& cr, const R* sl, const R* sr) {
  constexpr int NV = DIM + 2;
  const int64_t nf = A.nf[D];
  R W[NV], T[2];
  face_flux<R, DIM, D>(A, f, c, cl, cr, sl, sr, W, T);
#pragma unroll
  for (int v = 0; v < NV; ++v) A.W[D][v * nf + idx] = W[v];
#pragma unroll
  for (int q = 0; q < 2; ++q) if (q < A.nfrac) A.T[D][q * nf + idx] = T[q];
}

template <typename R, int DIM, int D>
__global__ void TFV_FACE_BOUNDS metric_face_kernel(MArgs<R> A) {
  constexpr int NV = DIM + 2;
  constexpr int d = D;
  const int n = A.n[d];
  const int64_t nf = A.nf[d];
  int err = 0;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nf;
       idx += (int64_t)gridDim.x * blockDim.x) {
    // face coordinates: f along d, the cell counts along the others
    MIdx c;
    int f;
    if (A.idx32) {
      int r;
      if (d == 0) {
        split32((uint32_t)idx, A.dn0f, f, r);
        split32((uint32_t)r, A.dn1, c.j, c.k);
        c.i = 0;
      } else if (d == 1) {
        split32((uint32_t)idx, A.dn0, c.i, r);
        split32((uint32_t)r, A.dn1f, f, c.k);
        c.j = 0;
      } else {
        split32((uint32_t)idx, A.dn0, c.i, r);
        split32((uint32_t)r, A.dn1, c.j, f);
        c.k = 0;
      }
    } else if (d == 0) {
      f = (int)(idx % (n + 1));
      const int64_t r = idx / (n + 1);
      c.j = (int)(r % A.n[1]);
      c.k = (int)(r / A.n[1]);
      c.i = 0;
    } else if (d == 1) {
      c.i = (int)(idx % A.n[0]);
      const int64_t r = idx / A.n[0];
      f = (int)(r % (n + 1));
      c.k = (int)(r / (n + 1));
      c.j = 0;
    } else {
      c.i = (int)(idx % A.n[0]);
      const int64_t r = idx / A.n[0];
      c.j = (int)(r % A.n[1]);
      f = (int)(r / A.n[1]);
      c.k = 0;
    }
    // padded cells f (left) and f + 1 (right) and their slopes
    MCell<R, NV> cl, cr;
    err |= padded_cell<R, NV, D>(A, f, c, cl);
    err |= padded_cell<R, NV, D>(A, f + 1, c, cr);
    R sl[NV], sr[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) sl[v] = sr[v] = R(0);
    if (!A.first_order) {
      const bool periodic = A.periodic[D];
      MCell<R, NV> m, p;
      // slope of padded cell f
      if (f >= 1) {
        err |= padded_cell<R, NV, D>(A, f - 1, c, m);
        cell_slope<R, NV>(m, cl, cr, A.limiter, sl);
      } else if (periodic) {  // the low ghost takes the last cell's slope
        MCell<R, NV> a, b, e;
        err |= padded_cell<R, NV, D>(A, n - 1, c, a);
        err |= padded_cell<R, NV, D>(A, n, c, b);
        err |= padded_cell<R, NV, D>(A, n + 1, c, e);
        cell_slope<R, NV>(a, b, e, A.limiter, sl);
      }
      // slope of padded cell f + 1
      if (f + 1 <= n) {
        err |= padded_cell<R, NV, D>(A, f + 2, c, p);
        cell_slope<R, NV>(cl, cr, p, A.limiter, sr);
      } else if (periodic) {  // the high ghost takes the first cell's slope
        MCell<R, NV> a, b, e;
        err |= padded_cell<R, NV, D>(A, 0, c, a);
        err |= padded_cell<R, NV, D>(A, 1, c, b);
        err |= padded_cell<R, NV, D>(A, 2, c, e);
        cell_slope<R, NV>(a, b, e, A.limiter, sr);
      }
    }
    emit_face<R, DIM, D>(A, f, c, idx, cl, cr, sl, sr);
  }
  if (err) atomicOr(A.err, err);
}

// face index of face f along d at cell coordinates c
__device__ __forceinline__ int64_t face_off(int d, int f, const MIdx& c, const int* n) {
  if (d == 0) return ((int64_t)c.k * n[1] + c.j) * (n[0] + 1) + f;
  if (d == 1) return ((int64_t)c.k * (n[1] + 1) + f) * n[0] + c.i;
  return ((int64_t)f * n[1] + c.j) * n[0] + c.i;
}

// Faces of direction D marched in chunks of `chunk` along D by one thread
// each (threads adjacent along x, or along y for the x faces of 2D / 3D
// grids): a sliding window of padded cells
// f, f + 1, f + 2 and the slope of each padded cell formed once, so a face
// costs one new cell load, one slope and one flux.  The values are those of
// metric_face_kernel.
template <typename R, int DIM, int D>
__global__ void TFV_MARCH_BOUNDS metric_face_march_kernel(MArgs<R> A) {
  const int chunk = A.chunk;
  constexpr int NV = DIM + 2;
  const int n = A.n[D];
  const int nchunks = (n + chunk) / chunk;  // faces 0..n
  const int64_t ntr = A.nc / n;             // cells of a plane normal to D
  const int64_t total = ntr * nchunks;
  const bool periodic = A.periodic[D];
  int err = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    int ch;
    MIdx c;
    if (D == 0 && A.xlanes) {  // threads adjacent along x: consecutive runs of a row
      int r;
      split32((uint32_t)t, A.dnch, ch, r);
      split32((uint32_t)r, A.dn1, c.j, c.k);
      c.i = 0;
    } else {
      const int64_t tr = t % ntr;
      ch = (int)(t / ntr);
      c.i = (int)(tr % A.n[0]);
      if (D == 0) {  // threads adjacent along y; each marches its own row
        c.i = 0;
        c.j = (int)(tr % A.n[1]);
        c.k = (int)(tr / A.n[1]);
      } else if (D == 1) {
        c.j = 0;
        c.k = (int)(tr / A.n[0]);
      } else {
        c.j = (int)(tr / A.n[0]);
        c.k = 0;
      }
    }
    const int f0 = ch * chunk;
    const int f1 = min(f0 + chunk, n + 1);
    MCell<R, NV> cl, cr, p;
    R sl[NV], sr[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) sl[v] = sr[v] = R(0);
    err |= padded_cell<R, NV, D>(A, f0, c, cl);
    err |= padded_cell<R, NV, D>(A, f0 + 1, c, cr);
    if (!A.first_order) {  // slope of padded cell f0
      if (f0 >= 1) {
        MCell<R, NV> m;
        err |= padded_cell<R, NV, D>(A, f0 - 1, c, m);
        cell_slope<R, NV>(m, cl, cr, A.limiter, sl);
      } else if (periodic) {
        MCell<R, NV> a, b, e;
        err |= padded_cell<R, NV, D>(A, n - 1, c, a);
        err |= padded_cell<R, NV, D>(A, n, c, b);
        err |= padded_cell<R, NV, D>(A, n + 1, c, e);
        cell_slope<R, NV>(a, b, e, A.limiter, sl);
      }
    }
    for (int f = f0; f < f1; ++f) {
      if (f + 2 <= n + 1) err |= padded_cell<R, NV, D>(A, f + 2, c, p);
      if (!A.first_order) {  // slope of padded cell f + 1
        if (f + 1 <= n) {
          cell_slope<R, NV>(cl, cr, p, A.limiter, sr);
        } else if (periodic) {
          MCell<R, NV> a, b, e;
          err |= padded_cell<R, NV, D>(A, 0, c, a);
          err |= padded_cell<R, NV, D>(A, 1, c, b);
          err |= padded_cell<R, NV, D>(A, 2, c, e);
          cell_slope<R, NV>(a, b, e, A.limiter, sr);
        } else {
#pragma unroll
          for (int v = 0; v < NV; ++v) sr[v] = R(0);
        }
      }
      emit_face<R, DIM, D>(A, f, c, face_off(D, f, c, A.n), cl, cr, sl, sr);
      cl = cr;
      cr = p;
#pragma unroll
      for (int v = 0; v < NV; ++v) sl[v] = sr[v];
    }
  }
  if (err) atomicOr(A.err, err);
}

// -- 3. divergence and the SSPRK2 stage combination ---------------------------
// stage 1: Uout = U + dt K, fractions (rho q + dt KQ) / rho_out, with KQ the
//          fraction divergence of the transport arrays T.
// stage 2: Uout = 0.5 (U0 + Us + dt K), fractions
//          0.5 (rho0 q0 + rho_s q_s + dt KQ) / rho_out  (torchFiniteVolume.py:234-276)
template <typename R, int DIM>
__global__ void __launch_bounds__(kMThreads) metric_update_kernel(MArgs<R> A, int stage) {
  constexpr int NV = DIM + 2;
  int err = 0;
  const R dt = R(A.dt);
  for (int64_t off = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; off < A.nc;
       off += (int64_t)gridDim.x * blockDim.x) {
    const MIdx c = cell_of(off, A);
    const R vol = volume<R, DIM>(A, c);
    R k[NV], kq[2] = {R(0), R(0)};
#pragma unroll
    for (int v = 0; v < NV; ++v) k[v] = ro(&A.K[v * A.nc + off]);
    const int cc[3] = {c.i, c.j, c.k};
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const int64_t lo = face_off(d, cc[d], c, A.n), hi = face_off(d, cc[d] + 1, c, A.n);
      const int64_t nf = A.nf[d];
#pragma unroll
      for (int v = 0; v < NV; ++v) k[v] = k[v] - (ro(&A.W[d][v * nf + hi]) - ro(&A.W[d][v * nf + lo])) / vol;
#pragma unroll
      for (int q = 0; q < 2; ++q) if (q < A.nfrac)
        kq[q] = kq[q] - (ro(&A.T[d][q * nf + hi]) - ro(&A.T[d][q * nf + lo])) / vol;
    }
    R out[NV], oq[2];
    if (stage == 1) {
#pragma unroll
      for (int v = 0; v < NV; ++v) out[v] = ro(&A.U[v * A.nc + off]) + dt * k[v];
      const R rho0 = ro(&A.U[off]);
#pragma unroll
      for (int q = 0; q < 2; ++q) if (q < A.nfrac)
        oq[q] = (rho0 * ro(&A.Q[q][off]) + dt * kq[q]) / out[0];
    } else {
#pragma unroll
      for (int v = 0; v < NV; ++v)
        out[v] = R(0.5) * ((ro(&A.U0[v * A.nc + off]) + ro(&A.Us[v * A.nc + off])) + dt * k[v]);
      const R rho0 = ro(&A.U0[off]), rhos = ro(&A.Us[off]);
#pragma unroll
      for (int q = 0; q < 2; ++q) if (q < A.nfrac)
        oq[q] = (R(0.5) * ((rho0 * ro(&A.Q0[q][off]) + rhos * ro(&A.Qs[q][off])) + dt * kq[q])) / out[0];
    }
    if (!physical_cell<R, NV>(out)) err |= kMErrNonphysical;
    // the reference's interval check (1e-12); single-precision roundoff of a
    // fraction of exactly 1 needs a wider margin
    const R tol = Exact<R>::value ? R(1e-12) : R(1e-5);
#pragma unroll
    for (int q = 0; q < 2; ++q) if (q < A.nfrac) {
      if (oq[q] < -tol || oq[q] > R(1) + tol) err |= kMErrFraction;
      oq[q] = np_min(np_max(oq[q], R(0)), R(1));  // np.clip
      A.Qout[q][off] = oq[q];
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) A.Uout[v * A.nc + off] = out[v];
  }
  if (err) atomicOr(A.err, err);
}

// -- 3b. last-direction faces fused with the stage update ---------------------
// The faces of the marching direction D = DIM - 1 (z in 3D, y in 2D) formed
// as metric_face_march_kernel forms them, each thread marching one column
// through a chunk of cells; with the low and high face of a cell in
// registers, the thread finishes that cell's divergence (x and y faces read
// from their arrays, then the D faces: the order of metric_update_kernel)
// and its SSPRK2 stage combination at once, so the D-face arrays are never
// written except on the two boundary planes (read by the outward sums) and
// the separate update pass is gone.  Values equal those of the separate
// kernels bit for bit (python/cfdSolver/torchFiniteVolume.py:160-276).
template <typename R, int DIM>
__device__ __forceinline__ int update_cell(const MArgs<R>& A, const MIdx& co, const R* wlo,
                                           const R* whi, int stage, R dt) {
  constexpr int NV = DIM + 2;
  constexpr int D = DIM - 1;
  int err = 0;
  const int64_t off = off_of(co.i, co.j, co.k, A.n);
  const R vol = volume<R, DIM>(A, co);
  // single precision divides by the volume as one reciprocal and products
  const R ivol = Exact<R>::value ? R(0) : R(1) / vol;
  auto pv = [&](R x) { return Exact<R>::value ? x / vol : x * ivol; };
  R k[NV], kq[2] = {R(0), R(0)};
#pragma unroll
  for (int v = 0; v < NV; ++v) k[v] = ro(&A.K[v * A.nc + off]);
  const int cc[3] = {co.i, co.j, co.k};
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    if (d == D) {
#pragma unroll
      for (int v = 0; v < NV; ++v) k[v] = k[v] - pv(whi[v] - wlo[v]);
#pragma unroll
      for (int q = 0; q < 2; ++q) if (q < A.nfrac) kq[q] = kq[q] - pv(whi[NV + q] - wlo[NV + q]);
    } else {
      const int64_t lo = face_off(d, cc[d], co, A.n), hi = face_off(d, cc[d] + 1, co, A.n);
      const int64_t nf = A.nf[d];
#pragma unroll
      for (int v = 0; v < NV; ++v) k[v] = k[v] - pv(ro(&A.W[d][v * nf + hi]) - ro(&A.W[d][v * nf + lo]));
#pragma unroll
      for (int q = 0; q < 2; ++q) if (q < A.nfrac)
        kq[q] = kq[q] - pv(ro(&A.T[d][q * nf + hi]) - ro(&A.T[d][q * nf + lo]));
    }
  }
  R out[NV], oq[2];
  if (stage == 1) {
#pragma unroll
    for (int v = 0; v < NV; ++v) out[v] = ro(&A.U[v * A.nc + off]) + dt * k[v];
    const R rho0 = ro(&A.U[off]);
#pragma unroll
    for (int q = 0; q < 2; ++q) if (q < A.nfrac) oq[q] = (rho0 * ro(&A.Q[q][off]) + dt * kq[q]) / out[0];
  } else {
#pragma unroll
    for (int v = 0; v < NV; ++v)
      out[v] = R(0.5) * ((ro(&A.U0[v * A.nc + off]) + ro(&A.Us[v * A.nc + off])) + dt * k[v]);
    const R rho0 = ro(&A.U0[off]), rhos = ro(&A.Us[off]);
#pragma unroll
    for (int q = 0; q < 2; ++q) if (q < A.nfrac)
      oq[q] = (R(0.5) * ((rho0 * ro(&A.Q0[q][off]) + rhos * ro(&A.Qs[q][off])) + dt * kq[q])) / out[0];
  }
  if (!physical_cell<R, NV>(out)) err |= kMErrNonphysical;
  const R tol = Exact<R>::value ? R(1e-12) : R(1e-5);
#pragma unroll
  for (int q = 0; q < 2; ++q) if (q < A.nfrac) {
    if (oq[q] < -tol || oq[q] > R(1) + tol) err |= kMErrFraction;
    oq[q] = np_min(np_max(oq[q], R(0)), R(1));  // np.clip
    A.Qout[q][off] = oq[q];
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) A.Uout[v * A.nc + off] = out[v];
  return err;
}

template <typename R, int DIM>
__global__ void TFV_MARCH_BOUNDS metric_march_update_kernel(MArgs<R> A, int stage) {
  constexpr int NV = DIM + 2;
  constexpr int D = DIM - 1;
  static_assert(DIM >= 2, "1D keeps the separate update");
  const int chunk = A.chunk;
  const int n = A.n[D];
  const int nchunks = (n + chunk - 1) / chunk;  // cells 0..n-1
  const int64_t ntr = A.nc / n;
  const int64_t total = ntr * nchunks;
  const int64_t nfd = A.nf[D];
  const bool periodic = A.periodic[D];
  const R dt = R(A.dt);
  int err = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t tr = t % ntr;
    const int ch = (int)(t / ntr);
    MIdx c;
    c.i = (int)(tr % A.n[0]);
    if (D == 1) {
      c.j = 0;
      c.k = (int)(tr / A.n[0]);
    } else {
      c.j = (int)(tr / A.n[0]);
      c.k = 0;
    }
    const int k0 = ch * chunk, k1 = min(k0 + chunk, n);  // cells k0..k1-1, faces k0..k1
    MCell<R, NV> cl, cr, p;
    R sl[NV], sr[NV], wlo[NV + 2];
#pragma unroll
    for (int v = 0; v < NV; ++v) sl[v] = sr[v] = R(0);
    err |= padded_cell<R, NV, D>(A, k0, c, cl);
    err |= padded_cell<R, NV, D>(A, k0 + 1, c, cr);
    if (!A.first_order) {  // slope of padded cell k0
      if (k0 >= 1) {
        MCell<R, NV> m;
        err |= padded_cell<R, NV, D>(A, k0 - 1, c, m);
        cell_slope<R, NV>(m, cl, cr, A.limiter, sl);
      } else if (periodic) {
        MCell<R, NV> a, b, e;
        err |= padded_cell<R, NV, D>(A, n - 1, c, a);
        err |= padded_cell<R, NV, D>(A, n, c, b);
        err |= padded_cell<R, NV, D>(A, n + 1, c, e);
        cell_slope<R, NV>(a, b, e, A.limiter, sl);
      }
    }
    for (int f = k0; f <= k1; ++f) {
      if (f + 2 <= n + 1) err |= padded_cell<R, NV, D>(A, f + 2, c, p);
      if (!A.first_order) {  // slope of padded cell f + 1
        if (f + 1 <= n) {
          cell_slope<R, NV>(cl, cr, p, A.limiter, sr);
        } else if (periodic) {
          MCell<R, NV> a, b, e;
          err |= padded_cell<R, NV, D>(A, 0, c, a);
          err |= padded_cell<R, NV, D>(A, 1, c, b);
          err |= padded_cell<R, NV, D>(A, 2, c, e);
          cell_slope<R, NV>(a, b, e, A.limiter, sr);
        } else {
#pragma unroll
          for (int v = 0; v < NV; ++v) sr[v] = R(0);
        }
      }
      R w[NV + 2];
      face_flux<R, DIM, D>(A, f, c, cl, cr, sl, sr, w, w + NV);
      if (f == 0 || f == n) {  // boundary planes: read by the outward sums
        const int64_t idx = face_off(D, f, c, A.n);
#pragma unroll
        for (int v = 0; v < NV; ++v) A.W[D][v * nfd + idx] = w[v];
      }
      if (f > k0) {  // cell f - 1: low face in wlo, high face in w
        MIdx co = c;
        if (D == 1) co.j = f - 1; else co.k = f - 1;
        err |= update_cell<R, DIM>(A, co, wlo, w, stage, dt);
      }
#pragma unroll
      for (int v = 0; v < NV + 2; ++v) wlo[v] = w[v];
      cl = cr;
      cr = p;
#pragma unroll
      for (int v = 0; v < NV; ++v) sl[v] = sr[v];
    }
  }
  if (err) atomicOr(A.err, err);
}

// -- 4. outward flux of the boundary planes ----------------------------------
// sum over the plane of (W_d[last face] - W_d[first face]) per component,
// directions in order (torchFiniteVolume.py:215-222).  Block partials into
// part[block][8]; slot 5.. unused.
template <typename R, int DIM>
__global__ void __launch_bounds__(kMThreads) metric_outward_kernel(MArgs<R> A) {
  constexpr int NV = DIM + 2;
  __shared__ double red[32];
  double acc[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) acc[v] = 0.0;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const int64_t plane = A.nc / A.n[d];
    const int64_t nf = A.nf[d];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < plane;
         t += (int64_t)gridDim.x * blockDim.x) {
      MIdx c;
      if (d == 0) {
        c.i = 0;
        c.j = (int)(t % A.n[1]);
        c.k = (int)(t / A.n[1]);
      } else if (d == 1) {
        c.i = (int)(t % A.n[0]);
        c.j = 0;
        c.k = (int)(t / A.n[0]);
      } else {
        c.i = (int)(t % A.n[0]);
        c.j = (int)(t / A.n[0]);
        c.k = 0;
      }
      const int64_t lo = face_off(d, 0, c, A.n), hi = face_off(d, A.n[d], c, A.n);
#pragma unroll
      for (int v = 0; v < NV; ++v) acc[v] += (double)(A.W[d][v * nf + hi] - A.W[d][v * nf + lo]);
    }
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const double t = block_sum(acc[v], red);
    if (threadIdx.x == 0) A.part[blockIdx.x * 8 + v] = t;
  }
}

// -- 5. CFL rate: sum over directions of max(area * face speed) / volume ------
// (torchFiniteVolume.py:74-102); reads the primitives of metric_prim_kernel.
template <typename R, int DIM>
__device__ __forceinline__ R cell_speed(const MCell<R, DIM + 2>& c, int d) {
  constexpr int NV = DIM + 2;
  return fabs(c.p[d + 1]) + sqrt((c.g * c.p[NV - 1]) / c.p[0]);
}

// rate of direction D at cell c (self: the cell's primitives, at offset off).
// The speed |u_D| + a of an interior cell reads a from the sound speeds the
// primitive pass stored (the same expression as cell_speed); boundary faces
// build the ghost state and form its speed.
template <typename R, int DIM, int D>
__device__ __forceinline__ R direction_rate(const MArgs<R>& A, const MIdx& c, int64_t off,
                                            const MCell<R, DIM + 2>& self, R vol, int& err) {
  constexpr int NV = DIM + 2;
  const int n = A.n[D];
  const int cd = D == 0 ? c.i : (D == 1 ? c.j : c.k);
  const int64_t stride = D == 0 ? 1 : (D == 1 ? (int64_t)A.n[0] : (int64_t)A.n[0] * A.n[1]);
  const R s = fabs(self.p[D + 1]) + ro(&A.S[off]);
  R fs_lo, fs_hi;
  MCell<R, NV> o;
  if (cd == 0) {  // boundary_state of the low face
    err |= padded_cell<R, NV, D>(A, 0, c, o);
    fs_lo = np_max(s, fabs(o.p[D + 1]) + sqrt((o.g * o.p[NV - 1]) / o.p[0]));
  } else {  // interior neighbour below
    const int64_t nb = off - stride;
    fs_lo = np_max(fabs(ro(&A.P[(D + 1) * A.nc + nb])) + ro(&A.S[nb]), s);
  }
  if (cd == n - 1) {
    err |= padded_cell<R, NV, D>(A, n + 1, c, o);
    fs_hi = np_max(s, fabs(o.p[D + 1]) + sqrt((o.g * o.p[NV - 1]) / o.p[0]));
  } else {  // interior neighbour above
    const int64_t nb = off + stride;
    fs_hi = np_max(s, fabs(ro(&A.P[(D + 1) * A.nc + nb])) + ro(&A.S[nb]));
  }
  return np_max(area<R, DIM>(A, D, cd, c) * fs_lo, area<R, DIM>(A, D, cd + 1, c) * fs_hi) / vol;
}

template <typename R, int DIM>
__global__ void __launch_bounds__(kMThreads) metric_rate_kernel(MArgs<R> A) {
  constexpr int NV = DIM + 2;
  __shared__ double red[32];
  R best = R(0);
  int err = 0;
  for (int64_t off = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; off < A.nc;
       off += (int64_t)gridDim.x * blockDim.x) {
    const MIdx c = cell_of(off, A);
    const R vol = volume<R, DIM>(A, c);
    MCell<R, NV> self;
    load_cell<R, NV>(A, off, self);
    R rate = direction_rate<R, DIM, 0>(A, c, off, self, vol, err);
    if constexpr (DIM >= 2) rate = rate + direction_rate<R, DIM, 1>(A, c, off, self, vol, err);
    if constexpr (DIM == 3) rate = rate + direction_rate<R, DIM, 2>(A, c, off, self, vol, err);
    if (!(rate == rate) || isinf(rate)) err |= kMErrRate;
    best = np_max(best, rate);
  }
  const R top = block_max(best, red);
  if (threadIdx.x == 0 && top > R(0)) {
    if constexpr (Exact<R>::value)
      atomicMax(A.rate_max, (unsigned long long)__double_as_longlong(top));
    else
      atomicMax(A.rate_max, (unsigned long long)__float_as_uint(top));
  }
  if (err) atomicOr(A.err, err);
}

// -- 6. Strang-split reaction halves --------------------------------------------
// mode 0: U (start) -> Uout, fractions Q -> Qout.
// mode 1: Uout holds the hydro state and is reacted in place; block partials
//   of ((old - start) + new - hydro) * volume (torchSession.py:559-568), with
//   old = U0 and start = Us.
template <typename R, int DIM>
__global__ void __launch_bounds__(kMThreads) metric_react_kernel(MArgs<R> A, int mode) {
  constexpr int NV = DIM + 2;
  __shared__ double red[32];
  double part[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) part[v] = 0.0;
  int err = 0;
  const bool znd = A.znd;
  const Chem<R> chem(A.chem);
  for (int64_t off = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; off < A.nc;
       off += (int64_t)gridDim.x * blockDim.x) {
    R u[NV], hyd[NV];
    const R* src = mode == 0 ? A.U : A.Uout;
#pragma unroll
    for (int v = 0; v < NV; ++v) u[v] = hyd[v] = src[v * A.nc + off];
    R lam = mode == 0 ? A.Q[0][off] : A.Qout[0][off];
    R beta = znd ? (mode == 0 ? A.Q[1][off] : A.Qout[1][off]) : R(1);
    if (!react_cell<R, DIM>(chem, u, lam, beta, znd, 0.5 * A.dt)) err |= kMErrChemistry;
    if (mode == 1) {
      const MIdx c = cell_of(off, A);
      const double vol = (double)volume<R, DIM>(A, c);
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const double old = A.U0[v * A.nc + off], start = A.Us[v * A.nc + off];
        part[v] += (((old - start) + (double)u[v]) - (double)hyd[v]) * vol;
      }
      if (!physical_cell<R, NV>(u)) err |= kMErrFinal;
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) A.Uout[v * A.nc + off] = u[v];
    A.Qout[0][off] = lam;
    if (znd) A.Qout[1][off] = beta;
  }
  if (mode == 1) {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const double t = block_sum(part[v], red);
      if (threadIdx.x == 0) A.part[blockIdx.x * 8 + v] = t;
    }
  }
  if (err) atomicOr(A.err, err);
}

// -- 7. integral of the state: sum of u * volume (metric) or of u (Cartesian) --
template <typename R, int DIM>
__global__ void __launch_bounds__(kMThreads) metric_integral_kernel(MArgs<R> A) {
  constexpr int NV = DIM + 2;
  __shared__ double red[32];
  double part[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) part[v] = 0.0;
  for (int64_t off = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; off < A.nc;
       off += (int64_t)gridDim.x * blockDim.x) {
    double w = 1.0;
    if (A.geometry != kGeoCartesian) w = (double)volume<R, DIM>(A, cell_of(off, A));
#pragma unroll
    for (int v = 0; v < NV; ++v) part[v] += (double)A.U[v * A.nc + off] * w;
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const double t = block_sum(part[v], red);
    if (threadIdx.x == 0) A.part[blockIdx.x * 8 + v] = t;
  }
}

// -- 8. stateless Rusanov over a list of faces ---------------------------------
// rows of the face states: rho, velocities (NV - 2), p; fluxes in the same
// component order (python/cfdSolver/torchFlux.py:80-99).
template <typename R, int NV>
__global__ void __launch_bounds__(kMThreads) rusanov_faces_kernel(
    int64_t n, int dir, const R* __restrict__ L, const R* __restrict__ Rt,
    const R* __restrict__ GL, const R* __restrict__ GR, R* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    R left[NV], right[NV], ul[NV], ur[NV], fl[NV], fr[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      left[v] = L[v * n + i];
      right[v] = Rt[v * n + i];
    }
    const R gl = GL[i], gr = GR[i];
    conservative_of<R, NV>(left, gl, ul);
    conservative_of<R, NV>(right, gr, ur);
    R vl = left[1], vr = right[1];
#pragma unroll
    for (int v = 1; v < NV - 1; ++v)
      if (v == dir + 1) {
        vl = left[v];
        vr = right[v];
      }
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      fl[v] = ul[v] * vl;
      fr[v] = ur[v] * vr;
    }
#pragma unroll
    for (int v = 1; v < NV - 1; ++v)
      if (v == dir + 1) {
        fl[v] = fl[v] + left[NV - 1];
        fr[v] = fr[v] + right[NV - 1];
      }
    fl[NV - 1] = fl[NV - 1] + vl * left[NV - 1];
    fr[NV - 1] = fr[NV - 1] + vr * right[NV - 1];
    const R speed = np_max(fabs(vl) + sqrt((gl * left[NV - 1]) / left[0]),
                           fabs(vr) + sqrt((gr * right[NV - 1]) / right[0]));
#pragma unroll
    for (int v = 0; v < NV; ++v) out[v * n + i] = R(0.5) * ((fl[v] + fr[v]) - speed * (ur[v] - ul[v]));
  }
}

// -- 9. block partials -> totals, in block order -------------------------------
namespace {
__global__ void __launch_bounds__(256) metric_reduce_kernel(const double* part, int nblocks,
                                                            int nv, double* out) {
  // fixed order: thread t sums partials t, t + 256, ...; then the block's
  // fixed shuffle tree and its warps in order (deterministic, independent of
  // timing; every partial is loaded by an independent, coalesced load)
  __shared__ double red[32];
  const int nb = min(nblocks, kMReduceBlocks);
  for (int v = 0; v < nv; ++v) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += part[b * 8 + v];
    const double t = block_sum(s, red);
    if (threadIdx.x == 0) out[v] = t;
    __syncthreads();  // red is reused by the next component
  }
}
}  // namespace

}  // namespace tfv
