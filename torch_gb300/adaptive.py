"""GPU leaf-face fluxes for TORCH's adaptive (AMR) sessions.

TORCH's adaptive solver (python/cfdSolver/torchAdaptive.py) keeps its dyadic
leaf mesh, the face reconstruction and the conservative accumulation on the
host.  Its right-hand side (torchAdaptive.py:115-153) evaluates the Rusanov
flux of every leaf face in batches of up to 8,192 faces through the module
attribute ``rusanov`` (torchFlux.rusanov_flux, torchFlux.py:80-99), once per
SSPRK2 stage.  The mesh stays on the host here as well; the drop-in is that
flux call.  ``leaf_fluxes`` evaluates one batch on the GPU (tfv_rusanov_flux)
from the host arrays the adaptive solver holds: the four inputs are packed
into one pinned staging buffer, copied to the device once, and the fluxes
come back through one pinned buffer.  ``gpu_leaf_fluxes(module)`` installs
it as the module's ``rusanov`` for the duration of a ``with`` block:

    from cfdSolver import torchAdaptive
    with torch_gb300.adaptive.gpu_leaf_fluxes(torchAdaptive):
        session.step()

In double precision the GPU flux is bit-identical to the reference's, so an
adaptive session advanced this way follows the reference's trajectory bit for
bit.  Callers whose face states are already on the GPU use
``torch_gb300.rusanov_flux`` with device tensors instead: no copies and no
synchronisation.
"""

import contextlib

import numpy as np
import torch

from . import _lib

_STAGING = {}  # (device index, kind) -> pinned host buffer, grown on demand


def _pinned(dev, kind, n):
    key = (dev.index, kind)
    buf = _STAGING.get(key)
    if buf is None or buf.numel() < n:
        buf = torch.empty(max(n, 1 << 16), dtype=torch.float64, pin_memory=True)
        _STAGING[key] = buf
    return buf[:n]


def leaf_fluxes(left, right, gl, gr, direction, precision="fp64"):
    """Rusanov fluxes of one batch of leaf faces (the reference's
    ``rusanov(left, right, gl, gr, direction)``): ``left``/``right`` are
    (dim+2, m) primitive face states on the host, ``gl``/``gr`` per-face gamma
    (or scalars); returns the (dim+2, m) fluxes as a NumPy array."""
    left = np.asarray(left, dtype=np.float64)
    right = np.asarray(right, dtype=np.float64)
    if left.shape != right.shape or left.ndim != 2 or left.shape[0] not in (3, 4, 5):
        raise ValueError("Rusanov requires matching (dim+2, ...) face states")
    nv, m = left.shape
    if direction not in range(nv - 2):
        raise ValueError("Invalid normal direction")
    if m == 0:
        return np.empty((nv, 0))
    dev = torch.device("cuda", torch.cuda.current_device())
    stage = _pinned(dev, "in", (2 * nv + 2) * m).view(2 * nv + 2, m)
    host = stage.numpy()
    host[:nv] = left
    host[nv:2 * nv] = right
    host[2 * nv] = np.broadcast_to(gl, (m,))
    host[2 * nv + 1] = np.broadcast_to(gr, (m,))
    stream = torch.cuda.current_stream(dev)
    d = stage.to(dev, non_blocking=True)
    if precision == "fp32":
        d = d.float()
    out = torch.empty((nv, m), dtype=d.dtype, device=dev)
    lib = _lib.load()
    _lib.check(lib.tfv_rusanov_flux(_lib.TFV_FP64 if d.dtype == torch.float64 else _lib.TFV_FP32,
                                    nv, m, int(direction), _lib.ptr(d[0]), _lib.ptr(d[nv]),
                                    _lib.ptr(d[2 * nv]), _lib.ptr(d[2 * nv + 1]), _lib.ptr(out),
                                    _lib.stream_ptr(stream)))
    back = _pinned(dev, "out", nv * m).view(nv, m)
    back.copy_(out, non_blocking=True)
    stream.synchronize()  # the staging buffers are reused by the next batch
    return back.numpy().copy()


@contextlib.contextmanager
def gpu_leaf_fluxes(module, precision="fp64"):
    """Route the leaf-face Rusanov batches of an adaptive solver module (the
    reference's ``cfdSolver.torchAdaptive``, whose right-hand side calls the
    module attribute ``rusanov``) to the GPU inside the block."""
    original = module.rusanov

    def rusanov(left, right, gl, gr, direction):
        return leaf_fluxes(left, right, gl, gr, direction, precision)

    module.rusanov = rusanov
    try:
        yield
    finally:
        module.rusanov = original
