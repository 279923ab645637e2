// Host side of the C ABI declared in include/tfv.h: validation, tile tables,
// workspace layout, step sequencing and CUDA-graph capture.  The library
// never allocates device memory: the caller passes a workspace and the state
// buffers.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <functional>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "tfv.h"
#include "tfv_launch.h"
#include "tfv_types.h"

using namespace tfv;

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& msg) {
  g_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  g_error = std::string(where) + ": " + cudaGetErrorString(e);
  return TFV_ECUDA;
}

#define TFV_CUDA(call)                                   \
  do {                                                   \
    cudaError_t e__ = (call);                            \
    if (e__ != cudaSuccess) return cuda_fail(e__, #call); \
  } while (0)

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

namespace tfv {
int host_fail(int code, const char* msg) { return fail(code, msg); }
int host_cuda_fail(cudaError_t e, const char* where) { return cuda_fail(e, where); }
}  // namespace tfv

struct tfv_batch {
  int dim = 0, precision = 0, n = 0;
  std::vector<tfv_config> cfg;
  tfv_tile tile{};
  bool varg = false;
  bool own_gamma = false;  // the per-cell gamma buffer lives in the workspace
  bool reactive = false;
  int nring = 2;
  std::vector<InstDesc> desc;
  std::vector<Tile> tiles;
  struct Group {
    int limiter, t_begin, t_end;
  };
  std::vector<Group> groups;  // contiguous tile ranges sharing a limiter
  std::vector<InstState> st;
  // workspace layout (bytes)
  size_t off_desc = 0, off_st = 0, off_tiles = 0, off_bsum = 0, off_wmax = 0, off_sum = 0,
         off_flags = 0, off_int = 0, off_gam = 0, off_tmaps = 0, total = 0;
  std::vector<CUtensorMap> tmaps;  // [n][4]: ring buffers 0..2, gamma
  size_t gam_bytes = 0;
  size_t off_mflux = 0, mflux_bytes = 0, off_scratch = 0, off_fin = 0, off_cnt = 0;
  int fin_slices = 1;
  int sms = 0;  // SMs of the bound device
  unsigned char* ws = nullptr;
  cudaStream_t stream = nullptr;
  StepArgs args{};
  int block = 0, grid = 0;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  bool bound = false;
};

namespace {

bool valid_bc(int bc, int dim, int axis) {
  if (bc == TFV_BC_OPEN || bc == TFV_BC_REFLECTIVE || bc == TFV_BC_PERIODIC) return true;
  return bc == TFV_BC_INFLOW && dim == 2 && axis == 1;
}

// Construction-time checks of Simulation (python/cfdSolver/torchSession.py:
// 190-254; validate_grid, torchSolver.py:1074-1088, without its CFL <= 0.5
// bound, which the Python layer enforces unless told otherwise).
int validate(const tfv_config& c, int dim) {
  if (c.dim != dim) return fail(TFV_EINVAL, "instance dimension differs from the batch");
  for (int k = 0; k < dim; ++k) {
    if (c.counts[k] < 2) return fail(TFV_EINVAL, "Require cells >= 2 along every axis");
    if (!(std::isfinite(c.lengths[k]) && c.lengths[k] > 0))
      return fail(TFV_EINVAL, "Require length > 0");
    if (!valid_bc(c.bc[k], dim, k)) return fail(TFV_EINVAL, "Unsupported session boundary");
  }
  if (!(std::isfinite(c.cfl) && c.cfl > 0)) return fail(TFV_EINVAL, "Require CFL > 0");
  if (!(std::isfinite(c.t_end) && c.t_end >= 0)) return fail(TFV_EINVAL, "Require t_end >= 0");
  if (!(std::isfinite(c.gamma) && c.gamma > 1))
    return fail(TFV_EINVAL, "gamma must be finite and greater than one");
  if (c.limiter < 0 || c.limiter > 4) return fail(TFV_EINVAL, "Unknown limiter");
  if (c.max_steps < 1) return fail(TFV_EINVAL, "Invalid maximum steps");
  if (c.reactive && dim != 1 && false) return fail(TFV_EINVAL, "reactive");
  return TFV_OK;
}

void build_tiles(tfv_batch* b) {
  b->tiles.clear();
  b->groups.clear();
  const int tx = b->tile.tx, ty = b->dim == 3 ? b->tile.ty : 1, ch = b->tile.chunk;
  // instances ordered by limiter so that each limiter's tiles are contiguous
  std::vector<int> order(b->n);
  for (int i = 0; i < b->n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return b->cfg[x].limiter < b->cfg[y].limiter; });
  for (int i : order) {
    const tfv_config& c = b->cfg[i];
    InstDesc& d = b->desc[i];
    d.tile0 = (int)b->tiles.size();
    const int na = c.counts[0];
    const int nb = b->dim == 3 ? c.counts[1] : 1;
    const int np = b->dim == 3 ? c.counts[2] : (b->dim == 2 ? c.counts[1] : 1);
    for (int p = 0; p < np; p += ch)
      for (int y = 0; y < nb; y += ty)
        for (int x = 0; x < na; x += tx) {
          Tile t{};
          t.inst = i;
          t.x0 = x;
          t.y0 = y;
          t.p0 = p;
          t.p1 = std::min(np, p + ch);
          b->tiles.push_back(t);
        }
    d.ntiles = (int)b->tiles.size() - d.tile0;
    if (b->groups.empty() || b->groups.back().limiter != c.limiter)
      b->groups.push_back({c.limiter, d.tile0, d.tile0});
    b->groups.back().t_end = (int)b->tiles.size();
  }
}

// Resident step-kernel CTAs on the current device (SMs x CTAs per SM), or 0
// when no device is available or the launch is persistent.
int resident_slots(const tfv_batch* b) {
  if (b->dim == 1 || b->tile.persistent_ctas > 0) return 0;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();  // no device here: keep the plain tiling
    return 0;
  }
  const bool f64 = b->precision == TFV_FP64;
  int per_sm = 0;
  if (b->dim == 3)
    per_sm = f64 ? occupancy3_f64(b->varg, b->tile.tx, b->tile.ty)
                 : occupancy3_f32(b->varg, b->tile.tx, b->tile.ty);
  else
    per_sm = f64 ? occupancy2_f64(b->varg, b->tile.tx) : occupancy2_f32(b->varg, b->tile.tx);
  cudaGetLastError();
  return per_sm > 0 ? per_sm * sms : 0;
}

// Completion time of `dur` dispatched in order onto `slots` resident CTAs
// (each block starts on the first slot that frees up).
double dispatch_makespan(const std::vector<double>& dur, int slots) {
  std::vector<double> heap(static_cast<size_t>(slots), 0.0);
  double end = 0.0;
  for (double d : dur) {
    std::pop_heap(heap.begin(), heap.end(), std::greater<double>());
    heap.back() += d;
    end = std::max(end, heap.back());
    std::push_heap(heap.begin(), heap.end(), std::greater<double>());
  }
  return end;
}

// Wave-quantisation fix: when a launch's tiles leave its last wave of
// resident CTAs partly idle, split the final `slots` tiles along the
// marching axis into halves, so that the tail is made of short tiles.  The
// split is kept only where the dispatch model predicts a shorter launch.
void split_tail(tfv_batch* b) {
  const int slots = resident_slots(b);
  if (slots <= 0 || b->dim == 1) return;
  const int tx = b->tile.tx, ty = b->dim == 3 ? b->tile.ty : 1;
  auto weight = [&](const Tile& t) {
    const InstDesc& d = b->desc[t.inst];
    const int ax = std::min(tx, d.n[0] - t.x0);
    const int by = b->dim == 3 ? std::min(ty, d.n[1] - t.y0) : 1;
    const double area = 0.3 + 0.7 * double(ax * by) / double(tx * ty);
    return area * (double(t.p1 - t.p0) + 2.0);  // + the chunk's extra plane and fixed cost
  };
  std::vector<Tile> out;
  out.reserve(b->tiles.size() + slots);
  for (const auto& g : b->groups) {
    std::vector<double> plain, split;
    const int first_split = std::max(g.t_begin, g.t_end - slots);
    for (int t = g.t_begin; t < g.t_end; ++t) {
      const Tile& T = b->tiles[t];
      plain.push_back(weight(T));
      if (t >= first_split && T.p1 - T.p0 >= 8) {
        Tile a = T, c = T;
        a.p1 = c.p0 = T.p0 + (T.p1 - T.p0) / 2;
        split.push_back(weight(a));
        split.push_back(weight(c));
      } else {
        split.push_back(weight(T));
      }
    }
    const bool use = dispatch_makespan(split, slots) < 0.99 * dispatch_makespan(plain, slots);
    for (int t = g.t_begin; t < g.t_end; ++t) {
      const Tile& T = b->tiles[t];
      if (use && t >= first_split && T.p1 - T.p0 >= 8) {
        Tile a = T, c = T;
        a.p1 = c.p0 = T.p0 + (T.p1 - T.p0) / 2;
        out.push_back(a);
        out.push_back(c);
      } else {
        out.push_back(T);
      }
    }
  }
  if (out.size() == b->tiles.size()) return;
  b->tiles.swap(out);
  // tiles of an instance stay contiguous: recompute ranges and groups
  for (int i = 0; i < b->n; ++i) b->desc[i].ntiles = 0;
  b->groups.clear();
  for (int t = 0; t < (int)b->tiles.size(); ++t) {
    InstDesc& d = b->desc[b->tiles[t].inst];
    if (d.ntiles == 0) d.tile0 = t;
    ++d.ntiles;
    const int lim = b->cfg[b->tiles[t].inst].limiter;
    if (b->groups.empty() || b->groups.back().limiter != lim) b->groups.push_back({lim, t, t});
    b->groups.back().t_end = t + 1;
  }
}

void fill_desc(tfv_batch* b, int i) {
  const tfv_config& c = b->cfg[i];
  InstDesc& d = b->desc[i];
  std::memset(&d, 0, sizeof(d));
  d.dim = b->dim;
  d.nring = b->nring;
  double vol = 1.0;
  d.ncell = 1;
  for (int k = 0; k < 3; ++k) {
    d.n[k] = k < b->dim ? c.counts[k] : 1;
    d.bc[k] = k < b->dim ? c.bc[k] : TFV_BC_OPEN;
    d.h[k] = k < b->dim ? (c.spacing[k] > 0 ? c.spacing[k] : c.lengths[k] / c.counts[k]) : 1.0;
    if (k < b->dim) {
      vol *= d.h[k];
      d.ncell *= c.counts[k];
    }
  }
  d.vol = vol;
  d.limiter = c.limiter;
  d.reactive = c.reactive;
  d.model = c.kinetic_model;
  d.closure = c.closure;
  d.var_gamma = b->varg;
  d.controller = c.controller;
  d.variant = c.variant;
  d.wavespeed = c.wavespeed;
  d.max_steps = c.max_steps;
  d.cfl = c.cfl;
  d.gamma = c.gamma;
  d.gamma_f = (float)c.gamma;
  d.t_end = c.t_end;
  d.q = c.q_heat;
  d.ea = c.activation;
  d.a = c.pre_exponential;
  // conservative 2D inlet with gamma = 1.4 (python/cfdSolver/torchSolver2D.py:227-243)
  const double rho = std::max(c.inlet_primitive[0], 1e-12);
  const double u = c.inlet_primitive[1], v = c.inlet_primitive[2];
  const double p = std::max(c.inlet_primitive[3], 1e-12);
  d.inlet[0] = rho;
  d.inlet[1] = rho * u;
  d.inlet[2] = rho * v;
  d.inlet[3] = p / (1.4 - 1.0) + (0.5 * rho) * (u * u + v * v);
}

size_t real_size(int precision) { return precision == TFV_FP64 ? 8 : 4; }

void layout(tfv_batch* b) {
  size_t o = 0;
  const size_t nt = b->tiles.size();
  b->off_desc = o;
  o = align_up(o + sizeof(InstDesc) * b->n, 256);
  b->off_st = o;
  o = align_up(o + sizeof(InstState) * b->n, 256);
  b->off_tiles = o;
  o = align_up(o + sizeof(Tile) * nt, 256);
  b->off_bsum = o;
  o = align_up(o + sizeof(double) * 15 * nt, 256);
  b->off_wmax = o;
  o = align_up(o + sizeof(double) * 3 * nt, 256);
  b->off_sum = o;
  o = align_up(o + sizeof(double) * 5 * nt, 256);
  b->off_flags = o;
  o = align_up(o + sizeof(int32_t) * nt, 256);
  b->off_int = o;
  o = align_up(o + sizeof(double) * 5 * b->n, 256);
  b->fin_slices = 1;
  for (int i = 0; i < b->n; ++i)
    b->fin_slices =
        std::max(b->fin_slices, (b->desc[i].ntiles + kFinalizeSlice - 1) / kFinalizeSlice);
  b->off_fin = o;  // finalize slice records [n][fin_slices][24] and counters [n]
  o = align_up(o + sizeof(double) * 24 * b->fin_slices * b->n, 256);
  b->off_cnt = o;
  o = align_up(o + sizeof(int32_t) * b->n, 256);
  b->off_tmaps = o;
  o = align_up(o + sizeof(CUtensorMap) * 4 * b->n, 256);
  b->off_gam = o;
  b->gam_bytes = 0;
  if (b->varg && b->own_gamma) {
    for (int i = 0; i < b->n; ++i) b->gam_bytes += align_up(real_size(b->precision) * b->desc[i].ncell, 256);
  }
  o += b->gam_bytes;
  o = align_up(o, 256);
  b->off_mflux = o;
  b->mflux_bytes = 0;
  if (b->reactive && b->dim > 1) {  // face mass fluxes of the hydro step, read by the species transport
    for (int i = 0; i < b->n; ++i) {
      const InstDesc& d = b->desc[i];
      for (int k = 0; k < b->dim; ++k)
        b->mflux_bytes += align_up(real_size(b->precision) * (d.ncell / d.n[k]) * (d.n[k] + 1), 256);
    }
  }
  o += b->mflux_bytes;
  o = align_up(o, 256);
  b->off_scratch = o;  // 1D: waves [3][n+1], reconstruction [6][n], fluxes [3][n+1]
  if (b->dim == 1)
    for (int i = 0; i < b->n; ++i) o += align_up(real_size(b->precision) * (12 * b->desc[i].ncell + 6), 256);
  b->total = align_up(o, 256);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no -lcuda).
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// Tensor map of one state buffer (scalar=false: dims x, y, [z], component)
// or of the per-cell gamma buffer (scalar=true), with the box the step
// kernel stages per plane: x from x0 - 16 bytes over tx + 32 bytes, y over
// ty + 4 cells, one plane.  False when the grid does not allow tensor copies.
bool encode_map(CUtensorMap* m, const tfv_batch* b, const InstDesc& d, void* base, bool scalar) {
  auto fn = encode_fn();
  if (!fn || !base) return false;
  const int es = b->precision == TFV_FP64 ? 8 : 4;
  const int xo = 16 / es;
  const int tx = b->tile.tx, ty = b->dim == 3 ? b->tile.ty : 1;
  if ((d.n[0] * es) % 16 != 0 || reinterpret_cast<uintptr_t>(base) % 16 != 0 || tx % xo != 0 ||
      tx + 2 * xo > 256 || ty + 4 > 256)
    return false;
  const int nv = b->dim + 2;
  cuuint64_t dims[4], strides[3];
  cuuint32_t box[4], estr[4] = {1, 1, 1, 1};
  cuuint32_t rank;
  const cuuint64_t nx = d.n[0], ny = d.n[1], nz = d.n[2];
  if (b->dim == 3) {
    dims[0] = nx; dims[1] = ny; dims[2] = nz; dims[3] = nv;
    strides[0] = nx * es; strides[1] = nx * ny * es; strides[2] = nx * ny * nz * es;
    box[0] = tx + 2 * xo; box[1] = ty + 4; box[2] = 1; box[3] = nv;
    rank = scalar ? 3 : 4;
  } else {
    dims[0] = nx; dims[1] = ny; dims[2] = nv;
    strides[0] = nx * es; strides[1] = nx * ny * es;
    box[0] = tx + 2 * xo; box[1] = 1; box[2] = nv;
    rank = scalar ? 2 : 3;
  }
  const CUresult r = fn(m, es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                        rank, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

int grid_for(const tfv_batch* b, int ntiles) {
  return b->tile.persistent_ctas > 0 ? std::min<int>(b->tile.persistent_ctas, ntiles) : ntiles;
}

#if TFV_CHECKED
// Checked build: every bound batch is registered; after each launch the whole
// device is waited for and every registered batch's descriptor and tile table
// in device memory are compared with the host copies, so that a write into
// another batch's workspace names the launch that made it.
std::mutex g_live_mutex;
std::vector<tfv_batch*> g_live;
bool g_corrupt = false;  // a registered batch's tables changed: refuse further launches

void live_add(tfv_batch* b) {
  std::lock_guard<std::mutex> lock(g_live_mutex);
  g_live.push_back(b);
}
void live_remove(tfv_batch* b) {
  std::lock_guard<std::mutex> lock(g_live_mutex);
  g_live.erase(std::remove(g_live.begin(), g_live.end(), b), g_live.end());
}

void integrity(const tfv_batch* by, int op) {
  std::lock_guard<std::mutex> lock(g_live_mutex);
  for (tfv_batch* b : g_live) {
    if (!b->bound || b->ws == nullptr) continue;
    std::vector<unsigned char> dev(sizeof(InstDesc) * b->n);
    if (cudaMemcpy(dev.data(), b->ws + b->off_desc, dev.size(), cudaMemcpyDeviceToHost) !=
        cudaSuccess)
      return;
    const unsigned char* host = reinterpret_cast<const unsigned char*>(b->desc.data());
    for (size_t k = 0; k < dev.size(); ++k)
      if (dev[k] != host[k]) {
        std::fprintf(stderr,
                     "tfv-checked: descriptor of batch %p (dim %d n %d ws %p) changed at byte %zu "
                     "after op %d of batch %p (dim %d n %d ws %p)\n",
                     (void*)b, b->dim, b->n, (void*)b->ws, k, op, (const void*)by, by->dim, by->n,
                     (void*)by->ws);
        b->bound = false;  // report once
        g_corrupt = true;
        break;
      }
    if (!b->bound) continue;
    std::vector<unsigned char> tdev(sizeof(Tile) * b->tiles.size());
    if (cudaMemcpy(tdev.data(), b->ws + b->off_tiles, tdev.size(), cudaMemcpyDeviceToHost) !=
        cudaSuccess)
      return;
    if (std::memcmp(tdev.data(), b->tiles.data(), tdev.size()) != 0) {
      std::fprintf(stderr,
                   "tfv-checked: tile table of batch %p (dim %d n %d ws %p) changed after op %d of "
                   "batch %p (dim %d n %d ws %p)\n",
                   (void*)b, b->dim, b->n, (void*)b->ws, op, (const void*)by, by->dim, by->n,
                   (void*)by->ws);
      b->bound = false;
      g_corrupt = true;
    }
  }
}

// Wait for each launch, report the first index violation the kernels
// recorded (and a fault, naming the launch that raised it).
cudaError_t checked_sync(const tfv_batch* b, int op, int lim, int t0, int t1, cudaError_t e) {
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    std::fprintf(stderr, "tfv-checked: fault after op %d lim %d tiles [%d,%d) dim %d prec %d n %d: %s\n",
                 op, lim, t0, t1, b->dim, b->precision, b->n, cudaGetErrorString(e));
    return e;
  }
  cudaError_t (*readers[3])(unsigned long long*) = {check_read_f64, check_read_f32_3d,
                                                    check_read_f32_2d};
  for (auto rd : readers) {
    unsigned long long rec[4] = {0, 0, 0, 0};
    e = rd(rec);
    if (e != cudaSuccess) return e;
    if (rec[0])
      std::fprintf(stderr,
                   "tfv-checked: violation op %d lim %d tiles [%d,%d) dim %d prec %d n %d: site %llu "
                   "block %llu index %lld extent %lld\n",
                   op, lim, t0, t1, b->dim, b->precision, b->n, rec[0], rec[1], (long long)rec[2],
                   (long long)rec[3]);
  }
  integrity(b, op);
  return g_corrupt ? cudaErrorNotPermitted : cudaSuccess;
}
#endif

cudaError_t launch_range_unchecked(tfv_batch* b, int op, int lim, int t0, int t1, int src_off,
                                   int dst_off);

cudaError_t launch_range(tfv_batch* b, int op, int lim, int t0, int t1, int src_off, int dst_off) {
#if TFV_CHECKED
  if (g_corrupt) return cudaErrorNotPermitted;
#endif
  cudaError_t e = launch_range_unchecked(b, op, lim, t0, t1, src_off, dst_off);
#if TFV_CHECKED
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(b->stream, &cs);
  if (cs == cudaStreamCaptureStatusNone) e = checked_sync(b, op, lim, t0, t1, e);
#endif
  return e;
}

cudaError_t launch_range_unchecked(tfv_batch* b, int op, int lim, int t0, int t1, int src_off,
                                   int dst_off) {
  if (t1 <= t0) return cudaSuccess;
  StepArgs A = b->args;
  A.src_off = src_off;
  A.dst_off = dst_off;
  A.t_begin = t0;
  A.t_end = t1;
  // the fallback usually exits at once (no tile flagged): two CTAs per SM
  // walk the tiles instead of one CTA per tile
  const int grid = op == kOpFallback ? std::min(grid_for(b, t1 - t0), std::max(2 * b->sms, 1))
                                     : grid_for(b, t1 - t0);
  if (b->precision == TFV_FP64) {
    if (b->dim == 1) return launch_step1_f64(op, b->varg, lim, A, grid, b->block, b->stream);
    return b->dim == 3 ? launch_step3_f64(op, b->varg, lim, A, grid, b->block, b->stream)
                       : launch_step2_f64(op, b->varg, lim, A, grid, b->block, b->stream);
  }
  if (b->dim == 1) return launch_step1_f32(op, b->varg, lim, A, grid, b->block, b->stream);
  return b->dim == 3 ? launch_step3_f32(op, b->varg, lim, A, grid, b->block, b->stream)
                     : launch_step2_f32(op, b->varg, lim, A, grid, b->block, b->stream);
}

// The step kernel is instantiated per limiter: one launch per limiter group.
cudaError_t launch(tfv_batch* b, int op, int src_off, int dst_off) {
  if (op == kOpHydro) {
    for (const auto& g : b->groups) {
      cudaError_t e = launch_range(b, op, g.limiter, g.t_begin, g.t_end, src_off, dst_off);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  return launch_range(b, op, 0, 0, (int)b->tiles.size(), src_off, dst_off);
}

cudaError_t finalize(tfv_batch* b, int mode, int dst_off) {
#if TFV_CHECKED
  if (g_corrupt) return cudaErrorNotPermitted;
#endif
  StepArgs A = b->args;
  A.dst_off = dst_off;
  cudaError_t e = launch_finalize(A, mode, b->precision == TFV_FP32,
                                  reinterpret_cast<double*>(b->ws + b->off_int), b->stream);
#if TFV_CHECKED
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(b->stream, &cs);
  if (cs == cudaStreamCaptureStatusNone) e = checked_sync(b, 100 + mode, 0, 0, b->n, e);
#endif
  return e;
}

// Enqueue one complete step for every READY instance.  Reactive steps
// (python/cfdSolver/torchSession.py:401-517): half reaction from the start
// state (ring cur -> cur+1) and the CFL check, which may halve dt and leave
// the instance in RETRY (the next enqueued step retries from the start
// state); hydro on the heated state (cur+1 -> cur+2) with its mass fluxes;
// species transport; second half reaction (cur+2 -> cur+1) with the source
// sums; commit (cur <- cur+1).
cudaError_t enqueue_step(tfv_batch* b) {
  if (b->dim == 1) {  // the 1D chain: wave speeds of the new state plan the next dt
    cudaError_t e = cudaSuccess;
    if (b->reactive) {
      e = launch(b, kOpReact1, 0, 1);
      if (e == cudaSuccess) e = launch(b, kOpWavesStep, 1, 1);
      if (e == cudaSuccess) e = finalize(b, 4, 1);
      if (e == cudaSuccess) e = launch(b, kOpHydro, 1, 2);
      if (e == cudaSuccess) e = launch(b, kOpFallback, 1, 2);
      if (e == cudaSuccess) e = launch(b, kOpSpecies, 1, 2);
      if (e == cudaSuccess) e = launch(b, kOpReact2, 2, 1);
      // the next dt is planned with gamma of the new composition (SI closure)
      if (e == cudaSuccess && b->own_gamma) e = launch(b, kOpGamma, 1, 1);
      if (e == cudaSuccess) e = launch(b, kOpWavesStep, 1, 1);
    } else {
      // fused step (faces, update, next-dt wave speeds); the first-order
      // fallback and its wave pass run only for flagged instances
      e = launch(b, kOpStep1d, 0, 1);
      if (e == cudaSuccess) e = launch(b, kOpFallback, 0, 1);
      if (e == cudaSuccess) e = launch(b, kOpWavesFallback, 1, 1);
    }
    if (e == cudaSuccess) e = finalize(b, 0, 1);
    return e;
  }
  if (b->reactive) {
    cudaError_t e = launch(b, kOpReact1, 0, 1);
    if (e == cudaSuccess) e = finalize(b, 4, 1);
    if (e == cudaSuccess) e = launch(b, kOpHydro, 1, 2);
    if (e == cudaSuccess) e = launch(b, kOpFallback, 1, 2);
    if (e == cudaSuccess) e = launch(b, kOpSpecies, 1, 2);
    if (e == cudaSuccess) e = launch(b, kOpReact2, 2, 1);
    if (e == cudaSuccess) e = finalize(b, 0, 1);
    return e;
  }
  cudaError_t e = launch(b, kOpHydro, 0, 1);
  if (e != cudaSuccess) return e;
  e = launch(b, kOpFallback, 0, 1);
  if (e != cudaSuccess) return e;
  return finalize(b, 0, 1);
}

int check_bound(const tfv_batch* b) {
  if (!b) return fail(TFV_EINVAL, "null batch");
  if (!b->bound) return fail(TFV_EINVAL, "batch is not bound to memory");
  return TFV_OK;
}

}  // namespace

extern "C" {

const char* tfv_version(void) {
#if TFV_CHECKED
  return "tfv 0.1 (sm_103a, checked)";
#else
  return "tfv 0.1 (sm_103a)";
#endif
}

const char* tfv_last_error(void) { return g_error.c_str(); }

static int create_internal(int32_t dim, int32_t precision, int32_t n, const tfv_config* cfgs,
                           const tfv_tile* tile, bool varg, tfv_batch** out);

int tfv_batch_create(int32_t dim, int32_t precision, int32_t n, const tfv_config* cfgs,
                     const tfv_tile* tile, tfv_batch** out) {
  return create_internal(dim, precision, n, cfgs, tile, false, out);
}

static int create_internal(int32_t dim, int32_t precision, int32_t n, const tfv_config* cfgs,
                           const tfv_tile* tile, bool varg, tfv_batch** out) {
  if (!out || !cfgs || n < 1) return fail(TFV_EINVAL, "invalid arguments");
  if (dim < 1 || dim > 3) return fail(TFV_EINVAL, "dimension must be 1, 2 or 3");
  if (precision != TFV_FP64 && precision != TFV_FP32) return fail(TFV_EINVAL, "bad precision");
  for (int i = 0; i < n; ++i) {
    const int r = validate(cfgs[i], dim);
    if (r != TFV_OK) return r;
    if (cfgs[i].reactive != cfgs[0].reactive || cfgs[i].closure != cfgs[0].closure)
      return fail(TFV_EINVAL, "a batch holds only reactive or only inert instances of one closure");
    if (cfgs[i].reactive) {
      const tfv_config& c = cfgs[i];
      if (!(std::isfinite(c.q_heat) && std::isfinite(c.activation) &&
            std::isfinite(c.pre_exponential)) ||
          c.q_heat < 0 || c.activation < 0 || c.pre_exponential < 0)
        return fail(TFV_EINVAL, "Reaction time and constants must be finite and nonnegative");
      if (c.kinetic_model != TFV_ARRHENIUS && c.kinetic_model != TFV_ZND)
        return fail(TFV_EINVAL, "Unknown limiter or chemistry model");
      if (c.closure != TFV_CLOSURE_SI && c.closure != TFV_CLOSURE_NONDIM)
        return fail(TFV_EINVAL, "Unknown chemistry closure");
    }
  }
  tfv_batch* b = new tfv_batch();
  b->dim = dim;
  b->precision = precision;
  b->n = n;
  b->cfg.assign(cfgs, cfgs + n);
  if (tile) {
    b->tile = *tile;
  } else {
    // 3D: 32 x 4 (FP64, one CTA per SM) or 16 x 16 (FP32, three CTAs per SM;
    // the fastest measured shape at 256^3)
    // 2D FP32: rows of 124 cells in 128 threads (the two ring cells on the
    // spare lanes: no warp does a second cell stage or face per row), 32-row
    // chunks (4096^2: 31.9 G cell-updates/s against 29.8 for 128 x 32; 64-row
    // chunks reach 32.5 there but leave small grids too few tiles: the
    // autotuner tries them per batch)
    const bool f32 = precision == TFV_FP32;
    b->tile.tx = dim == 3 ? (f32 ? 16 : 32) : (dim == 2 ? (f32 ? 124 : 128) : 256);
    b->tile.ty = dim == 3 ? (f32 ? 16 : 4) : 1;
    // 3D FP32: 40-plane chunks (256^3: 1.065 ms per step kernel against 1.105
    // with 32 and 1.085 with 48, measured)
    b->tile.chunk = dim == 3 && f32 ? 40 : 32;
    b->tile.persistent_ctas = 0;
    b->tile.tma = 1;
  }
  if (dim != 3) b->tile.ty = 1;
  {
    // per-thread work items of the step kernel: ring cells <= 3, faces <= 4
    const int tx = b->tile.tx, ty = b->tile.ty, nt = tx * ty;
    const int ring = dim == 3 ? 2 * tx + 2 * ty + 4 : 2;
    const int faces = (tx + 1) * ty + (dim == 3 ? tx * (ty + 1) : 0);
    if (ring > 3 * nt || faces > 4 * nt) {
      delete b;
      return fail(TFV_EINVAL, "tile shape leaves too much ring or face work per thread");
    }
  }
  if (b->tile.tx < 4 || b->tile.ty < 1 || b->tile.chunk < 1 || b->tile.tx * b->tile.ty > 256 ||
      step_threads(dim, precision == TFV_FP64, b->tile.tx, b->tile.ty) % 32 != 0) {
    delete b;
    return fail(TFV_EINVAL,
                "tile shape must have tx >= 4, ty >= 1, chunk >= 1, at most 256 cells, and "
                "tx*ty a multiple of 32 (single precision: tx*ty plus its ring cells within "
                "whole warps of at most 256 threads)");
  }
  b->reactive = cfgs[0].reactive != 0;
  // reactive SI closure: gamma(lambda) per cell, computed into the workspace
  b->own_gamma = b->reactive && cfgs[0].closure == TFV_CLOSURE_SI;
  b->varg = varg || b->own_gamma;
  b->nring = b->reactive ? 3 : 2;
  b->desc.resize(n);
  for (int i = 0; i < n; ++i) fill_desc(b, i);
  build_tiles(b);
  split_tail(b);
  layout(b);
  b->st.assign(n, InstState{});
  *out = b;
  return TFV_OK;
}

int tfv_batch_workspace_size(const tfv_batch* b, size_t* bytes) {
  if (!b || !bytes) return fail(TFV_EINVAL, "invalid arguments");
  *bytes = b->total;
  return TFV_OK;
}

int tfv_batch_ring_size(const tfv_batch* b, int32_t* nring) {
  if (!b || !nring) return fail(TFV_EINVAL, "invalid arguments");
  *nring = b->nring;
  return TFV_OK;
}

int tfv_batch_bind(tfv_batch* b, void* workspace, void* const* states, void* const* lams,
                   void* const* betas, void* stream) {
  if (!b || !workspace || !states) return fail(TFV_EINVAL, "invalid arguments");
  if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0)
    return fail(TFV_EINVAL, "workspace must be 256-byte aligned");
  {
    // the workspace and every state / composition buffer must be disjoint
    struct Range {
      uintptr_t lo, hi;
    };
    std::vector<Range> r;
    const uintptr_t w = reinterpret_cast<uintptr_t>(workspace);
    r.push_back({w, w + b->total});
    const size_t rs = real_size(b->precision);
    for (int i = 0; i < b->n; ++i) {
      const size_t cells = static_cast<size_t>(b->desc[i].ncell);
      for (int k = 0; k < b->nring; ++k) {
        const void* u = states[i * b->nring + k];
        if (u) r.push_back({reinterpret_cast<uintptr_t>(u),
                            reinterpret_cast<uintptr_t>(u) + rs * (b->dim + 2) * cells});
        const void* l = lams ? lams[i * b->nring + k] : nullptr;
        if (l) r.push_back({reinterpret_cast<uintptr_t>(l), reinterpret_cast<uintptr_t>(l) + rs * cells});
        const void* e = betas ? betas[i * b->nring + k] : nullptr;
        if (e) r.push_back({reinterpret_cast<uintptr_t>(e), reinterpret_cast<uintptr_t>(e) + rs * cells});
      }
    }
    std::sort(r.begin(), r.end(), [](const Range& x, const Range& y) { return x.lo < y.lo; });
    for (size_t k = 1; k < r.size(); ++k)
      if (r[k].lo < r[k - 1].hi)
        return fail(TFV_EINVAL, "state, composition and workspace buffers must not overlap");
  }
  b->ws = static_cast<unsigned char*>(workspace);
  b->stream = static_cast<cudaStream_t>(stream);
  {
    int dev = 0;
    TFV_CUDA(cudaGetDevice(&dev));
    TFV_CUDA(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev));
  }
  for (int i = 0; i < b->n; ++i) {
    InstDesc& d = b->desc[i];
    for (int k = 0; k < b->nring; ++k) {
      d.U[k] = states[i * b->nring + k];
      if (!d.U[k]) return fail(TFV_EINVAL, "null state buffer");
      d.lam[k] = lams ? lams[i * b->nring + k] : nullptr;
      d.beta[k] = betas ? betas[i * b->nring + k] : nullptr;
    }
    d.has_flux_out = 0;
    d.flux_nv = b->dim + 2;
    if (b->reactive && (!d.lam[0] || !d.lam[1] || !d.lam[2]))
      return fail(TFV_EINVAL, "reactive instances need lambda ring buffers");
    if (b->reactive && b->cfg[i].kinetic_model == TFV_ZND && (!d.beta[0] || !d.beta[1] || !d.beta[2]))
      return fail(TFV_EINVAL, "ZND instances need beta ring buffers");
  }
  {
    size_t og = b->off_gam, om = b->off_mflux;
    for (int i = 0; i < b->n; ++i) {
      InstDesc& d = b->desc[i];
      if (b->own_gamma) {
        d.gam = b->ws + og;
        og += align_up(real_size(b->precision) * d.ncell, 256);
      }
      if (b->dim == 1) {  // the 1D scratch; its flux rows feed the species transport
        size_t off = b->off_scratch;
        for (int j = 0; j < i; ++j)
          off += align_up(real_size(b->precision) * (12 * b->desc[j].ncell + 6), 256);
        d.scratch = b->ws + off;
        d.flux_out[0] = static_cast<unsigned char*>(d.scratch) +
                        real_size(b->precision) * (3 * (d.ncell + 1) + 6 * d.ncell);
        d.flux_out[1] = d.flux_out[2] = nullptr;
        d.has_flux_out = 0;
      } else if (b->reactive) {
        for (int k = 0; k < 3; ++k) d.flux_out[k] = nullptr;
        for (int k = 0; k < b->dim; ++k) {
          d.flux_out[k] = b->ws + om;
          om += align_up(real_size(b->precision) * (d.ncell / d.n[k]) * (d.n[k] + 1), 256);
        }
        d.has_flux_out = 1;
        d.flux_nv = 1;
      }
    }
  }
  b->tmaps.assign((size_t)b->n * 4, CUtensorMap{});
  for (int i = 0; i < b->n; ++i) {
    InstDesc& d = b->desc[i];
    bool ok = b->tile.tma != 0 && b->dim > 1;
    for (int k = 0; k < b->nring && ok; ++k) ok = encode_map(&b->tmaps[i * 4 + k], b, d, d.U[k], false);
    if (ok && b->varg) ok = encode_map(&b->tmaps[i * 4 + 3], b, d, d.gam, true);
    d.tma = ok ? 1 : 0;
  }
  for (int i = 0; i < b->n; ++i) {
    InstState& s = b->st[i];
    std::memset(&s, 0, sizeof(s));
    s.status = TFV_READY;
  }
  StepArgs& A = b->args;
  A.desc = reinterpret_cast<const InstDesc*>(b->ws + b->off_desc);
  A.st = reinterpret_cast<InstState*>(b->ws + b->off_st);
  A.tiles = reinterpret_cast<const Tile*>(b->ws + b->off_tiles);
  A.ntiles = (int)b->tiles.size();
  A.tx = b->tile.tx;
  A.ty = b->tile.ty;
  A.ninst = b->n;
  A.t_bsum = reinterpret_cast<double*>(b->ws + b->off_bsum);
  A.t_wmax = reinterpret_cast<double*>(b->ws + b->off_wmax);
  A.t_sum = reinterpret_cast<double*>(b->ws + b->off_sum);
  A.t_flags = reinterpret_cast<int32_t*>(b->ws + b->off_flags);
  A.tmaps = b->ws + b->off_tmaps;
  A.fin_part = reinterpret_cast<double*>(b->ws + b->off_fin);
  A.fin_cnt = reinterpret_cast<int32_t*>(b->ws + b->off_cnt);
  A.fin_slices = b->fin_slices;
  A.ws_lo = b->ws;
  A.ws_hi = b->ws + b->total;
  // every kernel of the batch runs whole warps (the block reductions shuffle
  // over full warps); lanes past a tile's cells own nothing
  b->block = step_threads(b->dim, b->precision == TFV_FP64, b->tile.tx, b->tile.ty);
  b->grid = grid_for(b, A.ntiles);
  TFV_CUDA(cudaMemcpyAsync(b->ws + b->off_desc, b->desc.data(), sizeof(InstDesc) * b->n,
                           cudaMemcpyHostToDevice, b->stream));
  TFV_CUDA(cudaMemcpyAsync(b->ws + b->off_st, b->st.data(), sizeof(InstState) * b->n,
                           cudaMemcpyHostToDevice, b->stream));
  TFV_CUDA(cudaMemcpyAsync(b->ws + b->off_tiles, b->tiles.data(), sizeof(Tile) * b->tiles.size(),
                           cudaMemcpyHostToDevice, b->stream));
  TFV_CUDA(cudaMemsetAsync(b->ws + b->off_cnt, 0, sizeof(int32_t) * b->n, b->stream));
  TFV_CUDA(cudaMemcpyAsync(b->ws + b->off_tmaps, b->tmaps.data(),
                           sizeof(CUtensorMap) * b->tmaps.size(), cudaMemcpyHostToDevice,
                           b->stream));
  // initial integrals and first dt
  if (b->own_gamma) TFV_CUDA(launch(b, kOpGamma, 0, 0));
  TFV_CUDA(launch(b, kOpWaves, 0, 0));
  TFV_CUDA(finalize(b, 3, 0));
  TFV_CUDA(cudaStreamSynchronize(b->stream));
  b->bound = true;
#if TFV_CHECKED
  live_remove(b);
  live_add(b);
  std::fprintf(stderr, "tfv-checked: bind batch %p dim %d n %d ws [%p, +%zu) stream %p\n", (void*)b,
               b->dim, b->n, (void*)b->ws, b->total, (void*)b->stream);
  for (int i = 0; i < b->n; ++i)
    std::fprintf(stderr, "tfv-checked:   inst %d cells %lld U %p %p %p scratch %p\n", i,
                 (long long)b->desc[i].ncell, b->desc[i].U[0], b->desc[i].U[1], b->desc[i].U[2],
                 b->desc[i].scratch);
#endif
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return TFV_OK;
}

int tfv_batch_use_graph(tfv_batch* b, int32_t steps_per_graph) {
  int r = check_bound(b);
  if (r) return r;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  b->graph_steps = 0;
  if (steps_per_graph <= 0) return TFV_OK;
  cudaGraph_t g = nullptr;
  TFV_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < steps_per_graph && e == cudaSuccess; ++k) e = enqueue_step(b);
  cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
  if (e != cudaSuccess) return cuda_fail(e, "capture");
  if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  b->graph_steps = steps_per_graph;
  return TFV_OK;
}

int tfv_batch_advance(tfv_batch* b, int32_t nsteps) {
  int r = check_bound(b);
  if (r) return r;
  int k = 0;
  if (b->graph && b->graph_steps > 0) {
    for (; k + b->graph_steps <= nsteps; k += b->graph_steps)
      TFV_CUDA(cudaGraphLaunch(b->graph, b->stream));
  }
  for (; k < nsteps; ++k) TFV_CUDA(enqueue_step(b));
  return TFV_OK;
}

int tfv_batch_report(tfv_batch* b, tfv_report* out) {
  int r = check_bound(b);
  if (r) return r;
  TFV_CUDA(cudaMemcpyAsync(b->st.data(), b->ws + b->off_st, sizeof(InstState) * b->n,
                           cudaMemcpyDeviceToHost, b->stream));
  TFV_CUDA(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < b->n; ++i) {
    const InstState& s = b->st[i];
    tfv_report& o = out[i];
    std::memset(&o, 0, sizeof(o));
    o.time = s.time;
    o.dt = s.dt;
    for (int c = 0; c < 5; ++c) {
      o.initial_integral[c] = s.initial[c];
      o.boundary_integral[c] = s.boundary[c];
      o.source_integral[c] = s.source[c];
    }
    o.steps = s.steps;
    o.status = s.status;
    o.current = s.cur;
    o.fallback_steps = s.fallback_steps;
    o.last_fallback = s.last_fallback;
  }
  return TFV_OK;
}

int tfv_batch_integrals(tfv_batch* b, double* out) {
  int r = check_bound(b);
  if (r) return r;
  if (b->own_gamma) TFV_CUDA(launch(b, kOpGamma, 0, 0));
  TFV_CUDA(launch(b, kOpWaves, 0, 0));
  TFV_CUDA(finalize(b, 2, 0));
  TFV_CUDA(cudaMemcpyAsync(out, b->ws + b->off_int, sizeof(double) * 5 * b->n,
                           cudaMemcpyDeviceToHost, b->stream));
  TFV_CUDA(cudaStreamSynchronize(b->stream));
  return TFV_OK;
}

int tfv_batch_replan(tfv_batch* b) {
  int r = check_bound(b);
  if (r) return r;
  if (b->own_gamma) TFV_CUDA(launch(b, kOpGamma, 0, 0));
  TFV_CUDA(launch(b, kOpWavesPlan, 0, 0));
  TFV_CUDA(finalize(b, 1, 0));
  return TFV_OK;
}

int tfv_batch_restore(tfv_batch* b, const tfv_report* reports) {
  int r = check_bound(b);
  if (r) return r;
  if (!reports) return fail(TFV_EINVAL, "invalid arguments");
  TFV_CUDA(cudaMemcpyAsync(b->st.data(), b->ws + b->off_st, sizeof(InstState) * b->n,
                           cudaMemcpyDeviceToHost, b->stream));
  TFV_CUDA(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < b->n; ++i) {
    const tfv_report& o = reports[i];
    if (!(o.steps > 0 || o.time > 0 || o.initial_integral[0] != 0)) continue;
    InstState& s = b->st[i];
    s.time = o.time;
    s.steps = o.steps;
    for (int c = 0; c < 5; ++c) {
      s.initial[c] = o.initial_integral[c];
      s.boundary[c] = o.boundary_integral[c];
      s.source[c] = o.source_integral[c];
    }
    s.fallback_steps = o.fallback_steps;
    s.last_fallback = o.last_fallback;
    s.cur = 0;
    s.fb_word = 0;
    s.retry = 0;
    // terminal statuses persist; READY / RETRY are re-planned
    s.status = (o.status == TFV_READY || o.status == TFV_RETRY) ? TFV_READY : o.status;
  }
  TFV_CUDA(cudaMemcpyAsync(b->ws + b->off_st, b->st.data(), sizeof(InstState) * b->n,
                           cudaMemcpyHostToDevice, b->stream));
  if (b->own_gamma) TFV_CUDA(launch(b, kOpGamma, 0, 0));
  TFV_CUDA(launch(b, kOpWavesPlan, 0, 0));
  TFV_CUDA(finalize(b, 1, 0));
  TFV_CUDA(cudaStreamSynchronize(b->stream));
  return TFV_OK;
}

int tfv_batch_set_flux_outputs(tfv_batch* b, int32_t inst, void* fx, void* fy, void* fz) {
  int r = check_bound(b);
  if (r) return r;
  if (inst < 0 || inst >= b->n) return fail(TFV_EINVAL, "instance out of range");
  if (b->reactive)
    return fail(TFV_EINVAL, "reactive batches use the flux buffers for species transport");
  InstDesc& d = b->desc[inst];
  d.flux_out[0] = fx;
  d.flux_out[1] = fy;
  d.flux_out[2] = fz;
  d.has_flux_out = (fx || fy || fz) ? 1 : 0;
  TFV_CUDA(cudaMemcpyAsync(b->ws + b->off_desc + sizeof(InstDesc) * inst, &d, sizeof(InstDesc),
                           cudaMemcpyHostToDevice, b->stream));
  TFV_CUDA(cudaStreamSynchronize(b->stream));
  return TFV_OK;
}

int tfv_batch_profile(tfv_batch* b, int32_t nsteps, float* ms_step, float* ms_fallback,
                      float* ms_finalize) {
  int r = check_bound(b);
  if (r) return r;
  cudaEvent_t ev[4];
  for (auto& e : ev) TFV_CUDA(cudaEventCreate(&e));
  float acc[3] = {0.f, 0.f, 0.f};
  for (int k = 0; k < nsteps; ++k) {
    TFV_CUDA(cudaEventRecord(ev[0], b->stream));
    TFV_CUDA(launch(b, kOpHydro, 0, 1));
    TFV_CUDA(cudaEventRecord(ev[1], b->stream));
    TFV_CUDA(launch(b, kOpFallback, 0, 1));
    TFV_CUDA(cudaEventRecord(ev[2], b->stream));
    TFV_CUDA(finalize(b, 0, 1));
    TFV_CUDA(cudaEventRecord(ev[3], b->stream));
    TFV_CUDA(cudaEventSynchronize(ev[3]));
    for (int i = 0; i < 3; ++i) {
      float ms = 0.f;
      TFV_CUDA(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
      acc[i] += ms;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (ms_step) *ms_step = acc[0];
  if (ms_fallback) *ms_fallback = acc[1];
  if (ms_finalize) *ms_finalize = acc[2];
  return TFV_OK;
}

int tfv_batch_destroy(tfv_batch* b) {
  if (!b) return TFV_OK;
#if TFV_CHECKED
  live_remove(b);
#endif
  if (b->graph) cudaGraphExecDestroy(b->graph);
  delete b;
  return TFV_OK;
}

int tfv_hllc_flux(int32_t precision, int32_t nv, int64_t n, const void* ul, const void* ur,
                  const void* gl, const void* gr, void* out, void* stream) {
  if ((nv != 4 && nv != 5) || n < 0 || !ul || !ur || !gl || !gr || !out)
    return fail(TFV_EINVAL, "HLLC requires matching (4,m) or (5,m) states");
  if (n == 0) return TFV_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = precision == TFV_FP64 ? launch_hllc_f64(nv, n, ul, ur, gl, gr, out, s)
                                        : launch_hllc_f32(nv, n, ul, ur, gl, gr, out, s);
  if (e != cudaSuccess) return cuda_fail(e, "hllc kernel");
  return TFV_OK;
}

static tfv_config single_step_config(const tfv_config* cfg) {
  tfv_config c = *cfg;
  c.t_end = 1e300;
  c.max_steps = INT64_MAX;
  c.reactive = 0;
  return c;
}

int tfv_step_workspace_size(const tfv_config* cfg, int32_t precision, size_t* bytes) {
  if (!cfg || !bytes) return fail(TFV_EINVAL, "invalid arguments");
  tfv_config c = single_step_config(cfg);
  tfv_batch* b = nullptr;
  const int r = create_internal(cfg->dim, precision, 1, &c, nullptr, true, &b);
  if (r) return r;
  *bytes = b->total;
  tfv_batch_destroy(b);
  return TFV_OK;
}

int tfv_hydro_step(const tfv_config* cfg, int32_t precision, const void* state_in,
                   void* state_out, const void* gamma_cells, double dt, void* fx, void* fy,
                   void* fz, void* workspace, int32_t* used_fallback, void* stream) {
  if (!cfg || !state_in || !state_out || !workspace) return fail(TFV_EINVAL, "invalid arguments");
  if (!(std::isfinite(dt) && dt >= 0)) return fail(TFV_EINVAL, "dt must be finite and >= 0");
  tfv_config c = single_step_config(cfg);
  tfv_batch* b = nullptr;
  int r = create_internal(cfg->dim, precision, 1, &c, nullptr, gamma_cells != nullptr, &b);
  if (r) return r;
  b->desc[0].gam = const_cast<void*>(gamma_cells);
  void* ring[2] = {const_cast<void*>(state_in), state_out};
  r = tfv_batch_bind(b, workspace, ring, nullptr, nullptr, stream);
  if (!r) r = tfv_batch_set_flux_outputs(b, 0, fx, fy, fz);
  if (!r) {
    // the step uses the caller's dt instead of the planned one
    InstState s = b->st[0];
    s.dt = dt;
    for (int k = 0; k < 3; ++k) {
      s.coef_half[k] = (0.5 * dt) / b->desc[0].h[k];
      s.coef_full[k] = dt / b->desc[0].h[k];
    }
    s.status = TFV_READY;
    cudaError_t e = cudaMemcpyAsync(b->ws + b->off_st, &s, sizeof(s), cudaMemcpyHostToDevice,
                                    b->stream);
    if (e == cudaSuccess) e = enqueue_step(b);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&s, b->ws + b->off_st, sizeof(s),
                                              cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) {
      r = cuda_fail(e, "tfv_hydro_step");
    } else {
      if (used_fallback) *used_fallback = s.last_fallback;
      if (s.status == TFV_ERR_NONPHYSICAL)
        r = fail(TFV_ENUMERIC, "Hydrodynamic update produced a nonphysical state");
    }
  }
  tfv_batch_destroy(b);
  return r;
}

}  // extern "C"

// --------------------------------------------------------------------------
// tfv_hydro_step_static: the stateless step with its scratch in a fixed array
// of this library's device memory, for callers that cannot allocate.
// --------------------------------------------------------------------------
namespace {

constexpr size_t kStaticScratchBytes = size_t(1) << 20;  // 1 MiB on every device
__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// Device address of g_static_scratch in the current device's context.  Host
// code may not use the symbol itself (it names a host-side shadow).  The
// address is looked up on every call, with the device current: the lookup is
// a table read in the CUDA runtime, and a cached address would go stale when
// the context is torn down and re-created (cudaDeviceReset).
int static_scratch(void** out) {
  void* p = nullptr;
  TFV_CUDA(cudaGetSymbolAddress(&p, g_static_scratch));
  if (!p) return fail(TFV_ECUDA, "cudaGetSymbolAddress returned a null address");
  *out = p;
  return TFV_OK;
}

}  // namespace

extern "C" int tfv_hydro_step_static(const tfv_config* cfg, int32_t precision,
                                     const void* state_in, void* state_out,
                                     const void* gamma_cells, double dt, void* fx, void* fy,
                                     void* fz, int32_t* used_fallback, void* stream) {
  if (!cfg) return fail(TFV_EINVAL, "invalid arguments");
  size_t need = 0;
  int r = tfv_step_workspace_size(cfg, precision, &need);
  if (r) return r;
  if (need > kStaticScratchBytes)
    return fail(TFV_EINVAL, "this grid needs " + std::to_string(need) +
                                " bytes of step scratch but tfv_hydro_step_static holds " +
                                std::to_string(kStaticScratchBytes) +
                                "; use tfv_hydro_step with a workspace");
  void* ws = nullptr;
  r = static_scratch(&ws);
  if (r) return r;
  return tfv_hydro_step(cfg, precision, state_in, state_out, gamma_cells, dt, fx, fy, fz, ws,
                        used_fallback, stream);
}
