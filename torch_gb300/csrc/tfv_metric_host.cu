// Host side of the metric / face-boundary session step (C ABI in
// include/tfv.h, tfv_metric_*): workspace layout, the transactional step of
// python/cfdSolver/torchSession.py:523-576 (CFL dt, Strang-split reaction
// halves, SSPRK2 with a first-order retry, up to 20 dt halvings) and the
// conservation balances.  Each step waits for the device three times (dt,
// end of each SSPRK2 stage); states are never copied to the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "tfv.h"
#include "tfv_launch.h"
#include "tfv_metric_launch.h"

using namespace tfv;

#define TFV_MCUDA(call)                                        \
  do {                                                         \
    cudaError_t e__ = (call);                                  \
    if (e__ != cudaSuccess) return host_cuda_fail(e__, #call); \
  } while (0)

namespace {

constexpr int kSlotSource1 = 0, kSlotOutward1 = 1, kSlotSource2 = 2, kSlotOutward2 = 3,
              kSlotReact = 4, kSlotIntegral = 5, kSlots = 6;

size_t mal(size_t x) { return (x + 255) / 256 * 256; }

}  // namespace

struct tfv_metric {
  int precision = 0;
  tfv_metric_config cfg{};
  int dim = 1, nv = 3, nfrac = 0;
  int64_t nc = 0, nf[3] = {0, 0, 0};
  std::vector<double> factors;  // host copy, layout of tfv_metric_factor_count
  size_t esz = 8;
  // workspace offsets (bytes)
  size_t off_state_a = 0, off_q_a[2] = {0, 0}, off_state_b = 0, off_q_b[2] = {0, 0};
  size_t off_p = 0, off_g = 0, off_s = 0, off_k = 0, off_w[3] = {0, 0, 0}, off_t[3] = {0, 0, 0};
  size_t off_faces = 0, off_fac = 0, off_part = 0, off_res = 0, off_rate = 0, off_err = 0, ws_size = 0;
  unsigned char* ws = nullptr;
  void* ring[2] = {nullptr, nullptr};
  void* lam[2] = {nullptr, nullptr};
  void* beta[2] = {nullptr, nullptr};
  cudaStream_t stream = nullptr;
  int sms = 132;
  bool bound = false;
  int cur = 0;
  // session scalars
  double time = 0.0, dt = 0.0;
  int64_t steps = 0;
  double initial[5] = {0, 0, 0, 0, 0}, boundary[5] = {0, 0, 0, 0, 0}, source[5] = {0, 0, 0, 0, 0};
  int fallback_steps = 0, last_fallback = 0, status = TFV_READY;
};

namespace {

int64_t factor_count(const tfv_metric_config& c) {
  int64_t total = 0;
  for (int a = 0; a < c.dim; ++a) total += c.n[a];
  for (int d = 0; d < c.dim; ++d)
    for (int a = 0; a < c.dim; ++a) total += c.n[a] + (a == d ? 1 : 0);
  return total;
}

int validate(const tfv_metric_config& c) {
  if (c.dim < 1 || c.dim > 3) return host_fail(TFV_EINVAL, "Invalid dimension");
  for (int a = 0; a < c.dim; ++a)
    if (c.n[a] < 2) return host_fail(TFV_EINVAL, "Require cells >= 2 along every axis");
  if (c.geometry < 0 || c.geometry > 3) return host_fail(TFV_EINVAL, "Unknown geometry");
  if (c.limiter < 0 || c.limiter > 4) return host_fail(TFV_EINVAL, "Unknown limiter");
  if (!(std::isfinite(c.cfl) && c.cfl > 0)) return host_fail(TFV_EINVAL, "Require CFL > 0");
  if (!(std::isfinite(c.t_end) && c.t_end >= 0)) return host_fail(TFV_EINVAL, "Require t_end >= 0");
  if (!(std::isfinite(c.gamma) && c.gamma > 1))
    return host_fail(TFV_EINVAL, "gamma must be finite and greater than one");
  if (c.max_steps < 1) return host_fail(TFV_EINVAL, "Invalid maximum steps");
  for (int f = 0; f < 2 * c.dim; ++f) {
    const int t = c.faces[f].type;
    if (t < TFV_FACE_OUTFLOW || t > TFV_FACE_STAGNATION_INLET)
      return host_fail(TFV_EINVAL, "Unknown face boundary type");
  }
  for (int d = 0; d < c.dim; ++d)
    if ((c.faces[2 * d].type == TFV_FACE_PERIODIC) != (c.faces[2 * d + 1].type == TFV_FACE_PERIODIC))
      return host_fail(TFV_EINVAL, "Periodic boundaries must be paired on an axis");
  return TFV_OK;
}

template <typename R>
MArgs<R> make_args(const tfv_metric* m) {
  MArgs<R> A;
  std::memset(&A, 0, sizeof(A));
  for (int a = 0; a < 3; ++a) A.n[a] = a < m->dim ? m->cfg.n[a] : 1;
  A.nc = m->nc;
  for (int d = 0; d < 3; ++d) A.nf[d] = m->nf[d];
  int64_t top = A.nc;
  for (int d = 0; d < 3; ++d) top = std::max<int64_t>(top, A.nf[d]);
  A.idx32 = top < (int64_t(1) << 31);
  A.dn0 = make_udiv((uint32_t)A.n[0]);
  A.dn1 = make_udiv((uint32_t)A.n[1]);
  A.dn0f = make_udiv((uint32_t)A.n[0] + 1);
  A.dn1f = make_udiv((uint32_t)A.n[1] + 1);
  A.nfrac = m->nfrac;
  A.reactive = m->cfg.reactive;
  A.limiter = m->cfg.limiter;
  A.geometry = m->cfg.geometry;
  A.znd = m->cfg.reactive && m->cfg.model == TFV_ZND;
  A.gamma = m->cfg.gamma;
  for (int d = 0; d < 3; ++d)
    A.periodic[d] = d < m->dim && m->cfg.faces[2 * d].type == TFV_FACE_PERIODIC;
  A.gam = (R)m->cfg.gamma;
  A.face = reinterpret_cast<const MFace<R>*>(m->ws + m->off_faces);
  A.chem.q = m->cfg.q;
  A.chem.ea = m->cfg.ea;
  A.chem.a = m->cfg.a;
  A.chem.closure = 0;
  A.chem.gamma = m->cfg.gamma;
  A.chem.gamma_f = (float)m->cfg.gamma;
  // factor arrays in the workspace: volume factors per axis, then face factors
  R* fac = reinterpret_cast<R*>(m->ws + m->off_fac);
  int64_t o = 0;
  for (int a = 0; a < m->dim; ++a) {
    A.vf[a] = fac + o;
    o += m->cfg.n[a];
  }
  for (int d = 0; d < m->dim; ++d)
    for (int a = 0; a < m->dim; ++a) {
      A.ff[d][a] = fac + o;
      o += m->cfg.n[a] + (a == d ? 1 : 0);
    }
  A.P = reinterpret_cast<R*>(m->ws + m->off_p);
  A.G = reinterpret_cast<R*>(m->ws + m->off_g);
  A.S = reinterpret_cast<R*>(m->ws + m->off_s);
  A.K = reinterpret_cast<R*>(m->ws + m->off_k);
  for (int d = 0; d < 3; ++d) {
    A.W[d] = reinterpret_cast<R*>(m->ws + m->off_w[d]);
    A.T[d] = reinterpret_cast<R*>(m->ws + m->off_t[d]);
  }
  A.part = reinterpret_cast<double*>(m->ws + m->off_part);
  A.rate_max = reinterpret_cast<unsigned long long*>(m->ws + m->off_rate);
  A.err = reinterpret_cast<int32_t*>(m->ws + m->off_err);
  return A;
}

int grid_for(const tfv_metric* m, int64_t n) {
  const int64_t blocks = (n + 255) / 256;
  return (int)std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)m->sms * 8));
}
int reduce_grid(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, kMReduceBlocks));
}

// A state (or fractions) view: ring slot or workspace buffer.
struct View {
  void* u;
  void* q[2];
};

template <typename R>
struct Driver {
  tfv_metric* m;
  MArgs<R> A;
  double* res;        // device [kSlots][8]
  double* part;
  cudaStream_t s;
  // state whose primitives, gamma and source are in P, G, K (and whose
  // source sum is in res[prim_slot]); a right-hand side of that state reuses them
  const void* prim_state = nullptr;
  int prim_slot = -1;

  cudaError_t launch(int op, int arg, int grid) {
    return sizeof(R) == 8
               ? metric_launch_f64(op, m->dim, reinterpret_cast<const MArgs<double>&>(A), arg, grid, s)
               : metric_launch_f32(op, m->dim, reinterpret_cast<const MArgs<float>&>(A), arg, grid, s);
  }
  void set_input(const View& v) {
    A.U = (const R*)v.u;
    A.Q[0] = (const R*)v.q[0];
    A.Q[1] = (const R*)v.q[1];
  }
  int reduce(int slot, int nblocks) {
    TFV_MCUDA(metric_reduce(part, nblocks, m->nv, res + slot * 8, s));
    return TFV_OK;
  }
  // primitives + source of the state v (source partials -> slot)
  int prim(const View& v, int slot) {
    set_input(v);
    const int g = reduce_grid(m->nc);
    TFV_MCUDA(launch(kMOpPrim, 0, g));
    prim_state = v.u;
    prim_slot = slot;
    return reduce(slot, g);
  }
  // one SSPRK2 right-hand side: K, the face fluxes, the source and outward
  // sums.  stage > 0 (2D / 3D grids): the last direction's faces are fused
  // with that stage's update into A.Uout (A.U / A.U0 / A.Us set by the caller)
  int rhs(const View& v, bool first_order, int slot_source, int slot_outward, int stage = 0) {
    A.first_order = first_order ? 1 : 0;
    if (prim_state == v.u && prim_slot >= 0) {  // primitives of v already computed (dt pass)
      set_input(v);
      if (prim_slot != slot_source)
        TFV_MCUDA(cudaMemcpyAsync(res + slot_source * 8, res + prim_slot * 8, 8 * sizeof(double),
                                  cudaMemcpyDeviceToDevice, s));
    } else {
      int r = prim(v, slot_source);
      if (r) return r;
    }
    const bool fused = stage > 0 && m->dim >= 2;
    for (int d = 0; d < m->dim; ++d) {
      // y and z faces (and the x faces of double-precision 2D / 3D grids): one
      // thread per run of A.chunk faces (cells, when fused with the update),
      // the run as long as keeps eight 256-thread CTAs per SM busy; other x
      // faces: one thread per face
      const bool last_fused = fused && d == m->dim - 1;
      int64_t work = m->nf[0];
      A.xlanes = 0;
      if (d == 0 && m->dim >= 2 && m->esz == 4 && A.idx32) {
        // single-precision x faces: runs of kMXRun faces, threads adjacent
        // along x (their loads stay within a few lines of one row)
        A.chunk = kMXRun;
        const int nchunks = (m->cfg.n[0] + kMXRun) / kMXRun;  // faces 0..n
        A.dnch = make_udiv((uint32_t)nchunks);
        A.xlanes = 1;
        work = (m->nc / m->cfg.n[0]) * nchunks;
      } else if (d > 0 || (m->dim >= 2 && m->esz == 8)) {
        const int64_t lines = m->nc / m->cfg.n[d];
        const int64_t runs = m->cfg.n[d] + (last_fused ? 0 : 1);
        const int64_t target = (int64_t)m->sms * 8 * 256;
        A.chunk = (int)std::max<int64_t>(
            4, std::min<int64_t>(kMChunk, (runs * lines + target - 1) / target));
        work = lines * ((runs + A.chunk - 1) / A.chunk);
      }
      if (last_fused)
        TFV_MCUDA(launch(kMOpMarchUpdate, stage, grid_for(m, work)));
      else
        TFV_MCUDA(launch(kMOpFace, d, grid_for(m, work)));
    }
    int64_t plane = 0;
    for (int d = 0; d < m->dim; ++d) plane = std::max<int64_t>(plane, m->nc / m->cfg.n[d]);
    const int g = reduce_grid(plane);
    TFV_MCUDA(launch(kMOpOutward, 0, g));
    return reduce(slot_outward, g);
  }
  // largest CFL rate of the state v; sets *rate (NaN when not finite) and err bits
  int rate(const View& v, double* out, int32_t* err) {
    TFV_MCUDA(cudaMemsetAsync(A.rate_max, 0, sizeof(unsigned long long), s));
    TFV_MCUDA(cudaMemsetAsync(A.err, 0, sizeof(int32_t), s));
    int r = prim(v, kSlotIntegral);
    if (r) return r;
    // the rate's block maxima combine by an atomic max (order-free), so its
    // grid is sized for occupancy, not for the fixed reduction partition
    TFV_MCUDA(launch(kMOpRate, 0, grid_for(m, m->nc)));
    unsigned long long bits = 0;
    TFV_MCUDA(cudaMemcpyAsync(&bits, A.rate_max, sizeof(bits), cudaMemcpyDeviceToHost, s));
    TFV_MCUDA(cudaMemcpyAsync(err, A.err, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    TFV_MCUDA(cudaStreamSynchronize(s));
    double v_;
    if (sizeof(R) == 8) {
      std::memcpy(&v_, &bits, sizeof(double));
    } else {
      float f;
      const uint32_t b32 = (uint32_t)bits;
      std::memcpy(&f, &b32, sizeof(float));
      v_ = (double)f;
    }
    *out = (*err & kMErrRate) ? NAN : v_;
    return TFV_OK;
  }
  int boundary_error(int32_t err) {
    if (err & kMErrReservoirSolution)
      return host_fail(TFV_EINVAL, "No subsonic reservoir-inlet solution");
    if (err & kMErrReservoirSupply)
      return host_fail(TFV_EINVAL, "Reservoir cannot supply inflow against the interior pressure");
    if (err & kMErrBackflow)
      return host_fail(TFV_EINVAL,
                       "Pressure outlet backflow requires an explicit backflow primitive state");
    return TFV_OK;
  }
};

template <typename R>
int metric_step(tfv_metric* m) {
  const tfv_metric_config& c = m->cfg;
  if (m->time == c.t_end) return TFV_OK;
  if (m->steps >= c.max_steps)
    return host_fail(TFV_ENUMERIC, "Maximum steps reached before requested final time");
  Driver<R> D;
  D.m = m;
  D.A = make_args<R>(m);
  D.res = reinterpret_cast<double*>(m->ws + m->off_res);
  D.part = reinterpret_cast<double*>(m->ws + m->off_part);
  D.s = m->stream;
  const int nxt = 1 - m->cur;
  View start{m->ring[m->cur], {m->lam[m->cur], m->beta[m->cur]}};
  View next{m->ring[nxt], {m->lam[nxt], m->beta[nxt]}};
  View heated{m->ws + m->off_state_a, {m->ws + m->off_q_a[0], m->ws + m->off_q_a[1]}};
  View stage{m->ws + m->off_state_b, {m->ws + m->off_q_b[0], m->ws + m->off_q_b[1]}};
  double rate = 0.0;
  int32_t err = 0;
  int r = D.rate(start, &rate, &err);
  if (r) return r;
  if ((r = D.boundary_error(err))) return r;
  double dt = std::min(c.cfl / rate, c.t_end - m->time);
  const int nb = reduce_grid(m->nc);
  for (int retry = 0; retry < 20; ++retry) {
    if (!std::isfinite(dt) || dt <= 0 || m->time + dt == m->time)
      return host_fail(TFV_ENUMERIC, "Integration stalled before requested final time");
    View old = start;
    D.A.dt = dt;
    if (c.reactive) {  // first reaction half, then the CFL check of the heated state
      TFV_MCUDA(cudaMemsetAsync(D.A.err, 0, sizeof(int32_t), D.s));
      D.set_input(start);
      D.A.Uout = (R*)heated.u;
      D.A.Qout[0] = (R*)heated.q[0];
      D.A.Qout[1] = (R*)heated.q[1];
      TFV_MCUDA(D.launch(kMOpReact, 0, grid_for(m, m->nc)));
      int32_t rerr = 0;
      TFV_MCUDA(cudaMemcpyAsync(&rerr, D.A.err, sizeof(int32_t), cudaMemcpyDeviceToHost, D.s));
      TFV_MCUDA(cudaStreamSynchronize(D.s));
      if (rerr & kMErrChemistry)
        return host_fail(TFV_EINVAL, "Reaction input outside the valid range (lambda, beta or state)");
      double hrate = 0.0;
      if ((r = D.rate(heated, &hrate, &err))) return r;
      if ((r = D.boundary_error(err))) return r;
      const double allowed = c.cfl / hrate;
      if (dt > allowed * (1 + 1e-12)) {
        dt = std::min(dt / 2, allowed);
        continue;
      }
      old = heated;
    }
    // SSPRK2, then the same at first order (torchFiniteVolume.py:234-276)
    int used = -1;
    // single-precision 2D / 3D: the last direction's faces and the stage
    // update are one kernel (double precision, bound by its FP64 pipe, ran
    // slower so: it keeps the separate update pass)
    const bool fused = m->dim >= 2 && m->esz == 4;
    // Both stages are enqueued before the host looks at either: stage 2
    // reports into its own error word, and when stage 1 failed (checked
    // first, as the reference orders it) the stage-2 results are discarded.
    int32_t* const err1 = D.A.err;
    for (int fo = 0; fo < 2 && used < 0; ++fo) {
      TFV_MCUDA(cudaMemsetAsync(err1, 0, 2 * sizeof(int32_t), D.s));
      D.A.err = err1;
      D.A.Uout = (R*)stage.u;
      D.A.Qout[0] = (R*)stage.q[0];
      D.A.Qout[1] = (R*)stage.q[1];
      if ((r = D.rhs(old, fo == 1, kSlotSource1, kSlotOutward1, fused ? 1 : 0))) return r;
      if (!fused) {
        D.set_input(old);
        TFV_MCUDA(D.launch(kMOpUpdate, 1, grid_for(m, m->nc)));
      }
      D.A.err = err1 + 1;
      D.A.U0 = (const R*)old.u;
      D.A.Q0[0] = (const R*)old.q[0];
      D.A.Q0[1] = (const R*)old.q[1];
      D.A.Us = (const R*)stage.u;
      D.A.Qs[0] = (const R*)stage.q[0];
      D.A.Qs[1] = (const R*)stage.q[1];
      D.A.Uout = (R*)next.u;
      D.A.Qout[0] = (R*)next.q[0];
      D.A.Qout[1] = (R*)next.q[1];
      const int r2 = D.rhs(stage, fo == 1, kSlotSource2, kSlotOutward2, fused ? 2 : 0);
      D.A.err = err1;
      if (r2) return r2;
      if (!fused) {
        D.A.err = err1 + 1;
        const cudaError_t e = D.launch(kMOpUpdate, 2, grid_for(m, m->nc));
        D.A.err = err1;
        TFV_MCUDA(e);
      }
      int32_t e12[2] = {0, 0};
      TFV_MCUDA(cudaMemcpyAsync(e12, err1, sizeof(e12), cudaMemcpyDeviceToHost, D.s));
      TFV_MCUDA(cudaStreamSynchronize(D.s));
      if ((r = D.boundary_error(e12[0]))) return r;
      if (e12[0] & (kMErrNonphysical | kMErrFraction)) continue;
      if ((r = D.boundary_error(e12[1]))) return r;
      if (e12[1] & (kMErrNonphysical | kMErrFraction)) continue;
      used = fo;
    }
    if (used < 0) {  // lost positivity at both orders: halve dt
      dt /= 2;
      continue;
    }
    double sums[kSlots * 8];
    if (c.reactive) {  // closing reaction half in place, source of both halves
      TFV_MCUDA(cudaMemsetAsync(D.A.err, 0, sizeof(int32_t), D.s));
      D.A.U0 = (const R*)old.u;
      D.A.Us = (const R*)start.u;
      D.A.Uout = (R*)next.u;
      D.A.Qout[0] = (R*)next.q[0];
      D.A.Qout[1] = (R*)next.q[1];
      TFV_MCUDA(D.launch(kMOpReact, 1, nb));
      if ((r = D.reduce(kSlotReact, nb))) return r;
    }
    int32_t e3 = 0;
    TFV_MCUDA(cudaMemcpyAsync(&e3, D.A.err, sizeof(int32_t), cudaMemcpyDeviceToHost, D.s));
    TFV_MCUDA(cudaMemcpyAsync(sums, D.res, sizeof(sums), cudaMemcpyDeviceToHost, D.s));
    TFV_MCUDA(cudaStreamSynchronize(D.s));
    if (c.reactive && (e3 & kMErrChemistry))
      return host_fail(TFV_EINVAL, "Reaction input outside the valid range (lambda, beta or state)");
    if (c.reactive && (e3 & kMErrFinal))
      return host_fail(TFV_ENUMERIC, "Reaction produced a nonphysical state");
    // commit (torchSession.py:566-576)
    for (int v = 0; v < m->nv; ++v) {
      m->boundary[v] += (0.5 * dt) * (sums[kSlotOutward1 * 8 + v] + sums[kSlotOutward2 * 8 + v]);
      double src = (0.5 * dt) * (sums[kSlotSource1 * 8 + v] + sums[kSlotSource2 * 8 + v]);
      if (c.reactive) src += sums[kSlotReact * 8 + v];
      m->source[v] += src;
    }
    m->cur = nxt;
    m->time = std::min(m->time + dt, c.t_end);
    m->steps += 1;
    m->dt = dt;
    m->last_fallback = used;
    m->fallback_steps += used;
    m->status = m->time == c.t_end ? TFV_DONE : TFV_READY;
    return TFV_OK;
  }
  return host_fail(TFV_ENUMERIC, "Could not find a positive metric/face step");
}

template <typename R>
int upload_faces(tfv_metric* m) {
  MFace<R> faces[6];
  std::memset(faces, 0, sizeof(faces));
  for (int f = 0; f < 6; ++f) {
    const tfv_metric_face& s = m->cfg.faces[f];
    MFace<R>& F = faces[f];
    F.type = f < 2 * m->dim ? s.type : kFaceOutflow;
    F.has_backflow = s.has_backflow;
    for (int v = 0; v < 5; ++v) F.prim[v] = (R)s.primitive[v];
    F.lam = (R)s.lambda_;
    F.beta = (R)s.beta;
    F.gam = (R)((4.5 - s.lambda_) / (3.5 - s.lambda_));  // gamma_calc (torchSolver.py:71-82)
    F.pressure = (R)s.pressure;
    F.p0 = (R)s.total_pressure;
    F.t0 = (R)s.total_temperature;
    F.rgas = (R)s.gas_constant;
  }
  TFV_MCUDA(cudaMemcpyAsync(m->ws + m->off_faces, faces, sizeof(faces), cudaMemcpyHostToDevice,
                            m->stream));
  TFV_MCUDA(cudaStreamSynchronize(m->stream));
  return TFV_OK;
}

template <typename R>
int metric_integrals(tfv_metric* m, double* out) {
  Driver<R> D;
  D.m = m;
  D.A = make_args<R>(m);
  D.res = reinterpret_cast<double*>(m->ws + m->off_res);
  D.part = reinterpret_cast<double*>(m->ws + m->off_part);
  D.s = m->stream;
  View v{m->ring[m->cur], {m->lam[m->cur], m->beta[m->cur]}};
  D.set_input(v);
  const int g = reduce_grid(m->nc);
  TFV_MCUDA(D.launch(kMOpIntegral, 0, g));
  int r = D.reduce(kSlotIntegral, g);
  if (r) return r;
  double sums[8];
  TFV_MCUDA(cudaMemcpyAsync(sums, D.res + kSlotIntegral * 8, sizeof(sums), cudaMemcpyDeviceToHost,
                            D.s));
  TFV_MCUDA(cudaStreamSynchronize(D.s));
  double cell = 1.0;  // Cartesian: sums times the cell volume (torchSession.py:284-294)
  if (m->cfg.geometry == TFV_GEO_CARTESIAN)
    for (int a = 0; a < m->dim; ++a) cell *= m->cfg.lengths[a] / m->cfg.n[a];
  for (int v = 0; v < m->nv; ++v) out[v] = m->cfg.geometry == TFV_GEO_CARTESIAN ? sums[v] * cell : sums[v];
  return TFV_OK;
}

}  // namespace

extern "C" {

int64_t tfv_metric_factor_count(const tfv_metric_config* cfg) {
  return cfg ? factor_count(*cfg) : -1;
}

int tfv_metric_create(int32_t precision, const tfv_metric_config* cfg, const double* factors,
                      tfv_metric** out) {
  if (!cfg || !factors || !out) return host_fail(TFV_EINVAL, "invalid arguments");
  if (precision != TFV_FP64 && precision != TFV_FP32)
    return host_fail(TFV_EINVAL, "precision must be fp64 or fp32");
  int r = validate(*cfg);
  if (r) return r;
  tfv_metric* m = new tfv_metric();
  m->precision = precision;
  m->cfg = *cfg;
  m->dim = cfg->dim;
  m->nv = cfg->dim + 2;
  m->nfrac = cfg->reactive ? (cfg->model == TFV_ZND ? 2 : 1) : 0;
  m->nc = 1;
  for (int a = 0; a < m->dim; ++a) m->nc *= cfg->n[a];
  for (int d = 0; d < 3; ++d) m->nf[d] = d < m->dim ? m->nc / cfg->n[d] * (cfg->n[d] + 1) : 0;
  m->factors.assign(factors, factors + factor_count(*cfg));
  for (double f : m->factors)
    if (!std::isfinite(f)) {
      delete m;
      return host_fail(TFV_EINVAL, "Invalid cell volumes");
    }
  m->esz = precision == TFV_FP64 ? 8 : 4;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += mal(bytes);
    return at;
  };
  const size_t st = m->esz * m->nv * m->nc, sc = m->esz * m->nc;
  if (cfg->reactive) {
    m->off_state_a = take(st);
    m->off_q_a[0] = take(sc);
    m->off_q_a[1] = take(sc);
  }
  m->off_state_b = take(st);
  m->off_q_b[0] = take(sc);
  m->off_q_b[1] = take(sc);
  m->off_p = take(st);
  m->off_g = take(sc);
  m->off_s = take(sc);
  m->off_k = take(st);
  for (int d = 0; d < m->dim; ++d) {
    m->off_w[d] = take(m->esz * m->nv * m->nf[d]);
    m->off_t[d] = take(m->esz * 2 * m->nf[d]);
  }
  m->off_faces = take(sizeof(MFace<double>) * 6);
  m->off_fac = take(m->esz * m->factors.size());
  m->off_part = take(sizeof(double) * kMReduceBlocks * 8);
  m->off_res = take(sizeof(double) * kSlots * 8);
  m->off_rate = take(sizeof(unsigned long long));
  m->off_err = take(2 * sizeof(int32_t));  // error words of the two SSPRK2 stages
  m->ws_size = o;
  *out = m;
  return TFV_OK;
}

int tfv_metric_workspace_size(tfv_metric* m, size_t* bytes) {
  if (!m || !bytes) return host_fail(TFV_EINVAL, "invalid arguments");
  *bytes = m->ws_size;
  return TFV_OK;
}

int tfv_metric_bind(tfv_metric* m, void* workspace, void* const* states, void* const* lams,
                    void* const* betas, void* stream) {
  if (!m || !workspace || !states || !states[0] || !states[1])
    return host_fail(TFV_EINVAL, "invalid arguments");
  if ((reinterpret_cast<uintptr_t>(workspace) & 255) != 0)
    return host_fail(TFV_EINVAL, "workspace must be 256-byte aligned");
  if (m->cfg.reactive && (!lams || !lams[0] || !lams[1]))
    return host_fail(TFV_EINVAL, "reactive sessions need lambda buffers");
  if (m->nfrac == 2 && (!betas || !betas[0] || !betas[1]))
    return host_fail(TFV_EINVAL, "ZND sessions need beta buffers");
  m->ws = static_cast<unsigned char*>(workspace);
  for (int i = 0; i < 2; ++i) {
    m->ring[i] = states[i];
    m->lam[i] = m->nfrac > 0 ? lams[i] : nullptr;
    m->beta[i] = m->nfrac > 1 ? betas[i] : nullptr;
  }
  m->stream = static_cast<cudaStream_t>(stream);
  int dev = 0;
  TFV_MCUDA(cudaGetDevice(&dev));
  TFV_MCUDA(cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, dev));
  // face table and factors in the workspace, in the arithmetic type
  int r0 = m->precision == TFV_FP64 ? upload_faces<double>(m) : upload_faces<float>(m);
  if (r0) return r0;
  if (m->precision == TFV_FP64) {
    TFV_MCUDA(cudaMemcpyAsync(m->ws + m->off_fac, m->factors.data(),
                              sizeof(double) * m->factors.size(), cudaMemcpyHostToDevice, m->stream));
    TFV_MCUDA(cudaStreamSynchronize(m->stream));
  } else {
    std::vector<float> f(m->factors.begin(), m->factors.end());
    TFV_MCUDA(cudaMemcpyAsync(m->ws + m->off_fac, f.data(), sizeof(float) * f.size(),
                              cudaMemcpyHostToDevice, m->stream));
    TFV_MCUDA(cudaStreamSynchronize(m->stream));
  }
  m->cur = 0;
  m->time = 0.0;
  m->steps = 0;
  m->fallback_steps = m->last_fallback = 0;
  std::memset(m->boundary, 0, sizeof(m->boundary));
  std::memset(m->source, 0, sizeof(m->source));
  m->bound = true;
  double integral[5] = {0, 0, 0, 0, 0};
  int r = m->precision == TFV_FP64 ? metric_integrals<double>(m, integral)
                                   : metric_integrals<float>(m, integral);
  if (r) return r;
  std::memcpy(m->initial, integral, sizeof(integral));
  m->status = m->time == m->cfg.t_end ? TFV_DONE : TFV_READY;
  return TFV_OK;
}

int tfv_metric_advance(tfv_metric* m, int32_t nsteps) {
  if (!m || !m->bound) return host_fail(TFV_EINVAL, "session not bound");
  for (int32_t k = 0; k < nsteps && m->time != m->cfg.t_end; ++k) {
    const int r = m->precision == TFV_FP64 ? metric_step<double>(m) : metric_step<float>(m);
    if (r) return r;
  }
  return TFV_OK;
}

int tfv_metric_report(tfv_metric* m, tfv_report* out) {
  if (!m || !out) return host_fail(TFV_EINVAL, "invalid arguments");
  std::memset(out, 0, sizeof(*out));
  out->time = m->time;
  out->dt = m->dt;
  for (int v = 0; v < 5; ++v) {
    out->initial_integral[v] = m->initial[v];
    out->boundary_integral[v] = m->boundary[v];
    out->source_integral[v] = m->source[v];
  }
  out->steps = m->steps;
  out->status = m->status;
  out->current = m->cur;
  out->fallback_steps = m->fallback_steps;
  out->last_fallback = m->last_fallback;
  return TFV_OK;
}

int tfv_metric_integrals(tfv_metric* m, double* out) {
  if (!m || !out || !m->bound) return host_fail(TFV_EINVAL, "invalid arguments");
  return m->precision == TFV_FP64 ? metric_integrals<double>(m, out)
                                  : metric_integrals<float>(m, out);
}

int tfv_metric_restore(tfv_metric* m, const tfv_report* r) {
  if (!m || !r || !m->bound) return host_fail(TFV_EINVAL, "invalid arguments");
  m->time = r->time;
  m->steps = r->steps;
  for (int v = 0; v < 5; ++v) {
    m->initial[v] = r->initial_integral[v];
    m->boundary[v] = r->boundary_integral[v];
    m->source[v] = r->source_integral[v];
  }
  m->fallback_steps = r->fallback_steps;
  m->last_fallback = r->last_fallback;
  m->status = m->time == m->cfg.t_end ? TFV_DONE : TFV_READY;
  return TFV_OK;
}

int tfv_metric_set_current(tfv_metric* m, int32_t slot) {
  if (!m || (slot != 0 && slot != 1)) return host_fail(TFV_EINVAL, "invalid arguments");
  m->cur = slot;
  return TFV_OK;
}

int tfv_rusanov_flux(int32_t precision, int32_t nv, int64_t n, int32_t direction,
                     const void* left, const void* right, const void* gl, const void* gr,
                     void* out, void* stream) {
  if (nv < 3 || nv > 5 || n < 0 || !left || !right || !gl || !gr || !out)
    return host_fail(TFV_EINVAL, "Rusanov requires matching (3..5, m) face states");
  if (direction < 0 || direction > nv - 3) return host_fail(TFV_EINVAL, "Invalid normal direction");
  if (precision != TFV_FP64 && precision != TFV_FP32)
    return host_fail(TFV_EINVAL, "precision must be fp64 or fp32");
  if (n == 0) return TFV_OK;
  int dev = 0, sms = 132;
  TFV_MCUDA(cudaGetDevice(&dev));
  TFV_MCUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sms * 8));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  TFV_MCUDA(precision == TFV_FP64
                ? rusanov_launch_f64(nv, n, direction, left, right, gl, gr, out, grid, s)
                : rusanov_launch_f32(nv, n, direction, left, right, gl, gr, out, grid, s));
  return TFV_OK;
}

int tfv_metric_destroy(tfv_metric* m) {
  delete m;
  return TFV_OK;
}

}  // extern "C"
