"""GPU versions of TORCH's stateless step functions.

Same signatures and exceptions as the reference functions they replace:
  hllc_flux              python/cfdSolver/torchFlux.py:125-248
  hllc_flux_grid         python/cfdSolver/torchFlux.py:6-77
  muscl_hancock_step_2d  python/cfdSolver/torchSolver2D.py:274-466
  muscl_hancock_step_3d  python/cfdSolver/torchSolver3D.py:206-222
Inputs may be NumPy arrays (results come back as float64 NumPy arrays, like
the reference) or CUDA tensors (results stay on the GPU).  ``execution`` is
accepted for signature compatibility; the GPU replaces the CPU workers.
"""

import ctypes as C

import numpy as np
import torch

from . import _lib
from .session import make_config

_2D_LIMITER_ALIASES = {"vanleer": "VanLeer", "van_leer": "VanLeer", "albada": "Albada",
                       "vanalbada": "Albada", "van_albada": "Albada", "minbee": "MINBEE",
                       "minmod": "MINBEE", "superbee": "Superbee", "unos": "Unos"}


def _device():
    return torch.device("cuda", torch.cuda.current_device())


def _as_device(x, dtype, device):
    return torch.as_tensor(np.array(x, copy=True) if isinstance(x, np.ndarray) else x,
                           dtype=dtype, device=device).contiguous()


def _out(t, host):
    return t.cpu().numpy() if host else t


def hllc_flux(u_l, u_r, gamma=1.4, wave_speed_mode="Pressure Based", gamma_right=None,
              precision="fp64"):
    """Normal HLLC flux with one or two tangential momenta (4 or 5 rows)."""
    host = isinstance(u_l, np.ndarray)
    if u_l.ndim != 2 or tuple(u_l.shape) != tuple(u_r.shape) or u_l.shape[0] not in (4, 5):
        raise ValueError("HLLC requires matching (4,m) or (5,m) states")
    dtype = torch.float64 if precision == "fp64" else torch.float32
    dev = u_l.device if isinstance(u_l, torch.Tensor) else _device()
    ul = _as_device(u_l, dtype, dev)
    ur = _as_device(u_r, dtype, dev)
    m = ul.shape[1]
    gl = torch.as_tensor(np.broadcast_to(gamma, (m,)).copy() if not isinstance(gamma, torch.Tensor)
                         else gamma, dtype=dtype, device=dev).expand(m).contiguous()
    gr_src = gamma if gamma_right is None else gamma_right
    gr = torch.as_tensor(np.broadcast_to(gr_src, (m,)).copy() if not isinstance(gr_src, torch.Tensor)
                         else gr_src, dtype=dtype, device=dev).expand(m).contiguous()
    out = torch.empty_like(ul)
    lib = _lib.load()
    stream = torch.cuda.current_stream(dev)
    _lib.check(lib.tfv_hllc_flux(_lib.TFV_FP64 if dtype == torch.float64 else _lib.TFV_FP32,
                                 ul.shape[0], m, _lib.ptr(ul), _lib.ptr(ur), _lib.ptr(gl),
                                 _lib.ptr(gr), _lib.ptr(out), _lib.stream_ptr(stream)))
    stream.synchronize()
    return _out(out.to(torch.float64) if host else out, host)


def hllc_flux_grid(left, right, gamma, gamma_right=None, *, direction=0, batch_size=8192,
                   execution=None, precision="fp64"):
    """Grid faces in Cartesian component order; rotation into the normal basis
    as torchFlux.py:36-39.  ``batch_size`` is validated and otherwise unused."""
    if left.shape != right.shape or left.ndim < 2 or left.shape[0] not in (4, 5):
        raise ValueError("HLLC requires matching four/five-component grids")
    if direction not in range(left.shape[0] - 2):
        raise ValueError("Invalid normal direction")
    if not isinstance(batch_size, int) or isinstance(batch_size, bool) or batch_size < 1:
        raise ValueError("HLLC batch size must be a positive integer")
    nv = left.shape[0]
    normal = direction + 1
    order = [0, normal] + [m for m in range(1, nv - 1) if m != normal] + [nv - 1]
    host = isinstance(left, np.ndarray)
    lib_ = np if host else torch
    gl = np.broadcast_to(gamma, left.shape[1:]) if host else torch.as_tensor(gamma).expand(
        left.shape[1:])
    gr = gl if gamma_right is None else (np.broadcast_to(gamma_right, left.shape[1:]) if host
                                         else torch.as_tensor(gamma_right).expand(left.shape[1:]))
    ul = left[order].reshape(nv, -1)
    ur = right[order].reshape(nv, -1)
    val = hllc_flux(ul, ur, gl.reshape(-1), gamma_right=gr.reshape(-1), precision=precision)
    out = lib_.empty_like(left) if host else torch.empty_like(val.reshape(left.shape))
    out[order] = val.reshape((nv,) + tuple(left.shape[1:]))
    return out


def rusanov_flux(left, right, gl, gr, direction, precision="fp64"):
    """Normal Rusanov flux from primitive face states (rho, velocities, p)
    with every tangential momentum (python/cfdSolver/torchFlux.py:80-99).
    ``left``/``right``: (dim+2, ...) arrays; ``gl``/``gr``: gamma per face
    (scalars broadcast)."""
    host = isinstance(left, np.ndarray)
    if tuple(left.shape) != tuple(right.shape) or left.ndim < 1 or left.shape[0] not in (3, 4, 5):
        raise ValueError("Rusanov requires matching (dim+2, ...) face states")
    if direction not in range(left.shape[0] - 2):
        raise ValueError("Invalid normal direction")
    dtype = torch.float64 if precision == "fp64" else torch.float32
    dev = left.device if isinstance(left, torch.Tensor) else _device()
    nv = left.shape[0]
    shape = tuple(left.shape)
    lt = _as_device(left, dtype, dev).reshape(nv, -1).contiguous()
    rt = _as_device(right, dtype, dev).reshape(nv, -1).contiguous()
    m = lt.shape[1]

    def per_face(g):
        if isinstance(g, torch.Tensor):
            return g.to(device=dev, dtype=dtype).expand(shape[1:]).reshape(-1).contiguous()
        return torch.as_tensor(np.broadcast_to(np.asarray(g, dtype=float), shape[1:]).reshape(-1)
                               .copy(), dtype=dtype, device=dev)

    g_l, g_r = per_face(gl), per_face(gr)
    out = torch.empty_like(lt)
    lib = _lib.load()
    stream = torch.cuda.current_stream(dev)
    _lib.check(lib.tfv_rusanov_flux(_lib.TFV_FP64 if dtype == torch.float64 else _lib.TFV_FP32,
                                    nv, m, int(direction), _lib.ptr(lt), _lib.ptr(rt),
                                    _lib.ptr(g_l), _lib.ptr(g_r), _lib.ptr(out),
                                    _lib.stream_ptr(stream)))
    out = out.reshape(shape)
    # device inputs: the result stays on the device, ordered on the current
    # stream (no host round trip); host inputs: copied back
    return _out(out.to(torch.float64) if host else out, host)


def rusanov_flux_grid(left, right, gl, gr, direction, execution=None, precision="fp64"):
    """rusanov_flux over a grid of faces in one launch
    (python/cfdSolver/torchFlux.py:102-122: the reference batches 8,192 faces
    per CPU task; ``execution`` is accepted and unused)."""
    return rusanov_flux(left, right, gl, gr, direction, precision=precision)


def _step(dim, state, spacing, dt, gamma, limiter, bcs, return_fluxes, inlet_primitive,
          precision):
    host = isinstance(state, np.ndarray)
    dtype = torch.float64 if precision == "fp64" else torch.float32
    dev = state.device if isinstance(state, torch.Tensor) else _device()
    u = _as_device(state, dtype, dev)
    shape = tuple(u.shape)
    counts = list(shape[1:][::-1])
    lengths = [spacing[k] * counts[k] for k in range(dim)]
    cfg = make_config(dim, counts, lengths, bcs, t_end=1.0, cfl=0.4, gamma=1.4, limiter=limiter,
                      max_steps=1, inlet_primitive=inlet_primitive)
    for k in range(dim):
        cfg.spacing[k] = float(spacing[k])  # the caller's dx, dy, dz exactly
    if np.ndim(gamma) == 0 and not isinstance(gamma, torch.Tensor):
        cfg.gamma = float(gamma)
        gcell = None
    else:
        gcell = _as_device(np.broadcast_to(gamma, shape[1:]) if not isinstance(gamma, torch.Tensor)
                           else gamma.expand(shape[1:]), dtype, dev)
    out = torch.empty_like(u)
    fl = [None, None, None]
    if return_fluxes:
        for k in range(dim):
            fshape = list(shape)
            fshape[dim - k] += 1
            fl[k] = torch.empty(fshape, dtype=dtype, device=dev)
    ws = C.c_size_t()
    lib = _lib.load()
    prec = _lib.TFV_FP64 if dtype == torch.float64 else _lib.TFV_FP32
    _lib.check(lib.tfv_step_workspace_size(C.byref(cfg), prec, C.byref(ws)))
    work = torch.empty(ws.value + 256, dtype=torch.uint8, device=dev)
    wp = work.data_ptr() + ((-work.data_ptr()) % 256)
    used = C.c_int32()
    stream = torch.cuda.current_stream(dev)
    code = lib.tfv_hydro_step(C.byref(cfg), prec, _lib.ptr(u), _lib.ptr(out), _lib.ptr(gcell),
                              float(dt), _lib.ptr(fl[0]), _lib.ptr(fl[1]), _lib.ptr(fl[2]),
                              C.c_void_p(wp), C.byref(used), _lib.stream_ptr(stream))
    _lib.check(code)
    res = [out] + [f for f in fl[:dim]] if return_fluxes else [out]
    res = [_out(r.to(torch.float64) if host else r, host) for r in res]
    return tuple(res) if return_fluxes else res[0]


def muscl_hancock_step_2d(u_inner, dx, dy, dt, gamma=1.4, limiter="VanLeer", bc_x="Periodic",
                          bc_y="Open", return_fluxes=False, inlet_primitive=None, execution=None,
                          precision="fp64"):
    """One unsplit 2D MUSCL-Hancock step; returns u_next (and flux_x, flux_y)."""
    lim = _2D_LIMITER_ALIASES.get(str(limiter).lower(), "VanLeer")
    if str(bc_x).lower() == "inflow":
        raise ValueError(f"Unknown x boundary: {bc_x}")
    if str(bc_y).lower() == "inflow":
        inlet = np.asarray([1.0, 0.0, 100.0, 101325.0] if inlet_primitive is None
                           else inlet_primitive, dtype=float)
        if (inlet.shape != (4,) or not np.isfinite(inlet).all() or inlet[0] <= 0
                or inlet[3] <= 0 or inlet[2] < 0):
            raise ValueError("Inlet requires [rho>0, u, v>=0, p>0] in SI")
    return _step(2, u_inner, (dx, dy), dt, gamma, lim, (bc_x, bc_y), return_fluxes,
                 inlet_primitive, precision)


def muscl_hancock_step_3d(state, dx, dy, dz, dt, gamma=1.4, limiter="VanLeer", bc_x="Open",
                          bc_y="Open", bc_z="Open", return_fluxes=False, precision="fp64"):
    """One unsplit 3D MUSCL-Hancock step; returns result (and fx, fy, fz)."""
    if limiter not in _lib.LIMITERS:
        raise ValueError(f"Unknown limiter: {limiter}")
    return _step(3, state, (dx, dy, dz), dt, gamma, limiter, (bc_x, bc_y, bc_z), return_fluxes,
                 None, precision)
