"""Many independent grids advanced together on one GPU.

A ``Grid`` owns one grid's device buffers (state ring, composition rings) and
its last scalars; a ``Batch`` advances a set of grids of one dimension and
precision with one launch per stage for all of them (the tile table spans
every grid; each grid keeps its own CFL dt, time, status and integrals).
Grids can leave a batch and join another one between steps without copies:
their current ring buffer becomes buffer 0 of the next batch and their
scalars are restored (``tfv_batch_restore``).  This is the engine of the
batched mode and of the serving loop; TORCH itself has no batched sessions.
"""

import ctypes as C

import numpy as np
import torch

from . import _lib
from .session import _dtype, make_config, prim_to_cons

_BYTES = {"fp64": 8, "fp32": 4}


class Grid:
    """Device state of one Cartesian grid plus its configuration."""

    def __init__(self, primitive, lengths, *, precision="fp32", device=None, t_end, cfl=0.4,
                 gamma=1.4, boundaries=None, limiter="VanLeer", max_steps=10 ** 9,
                 reactive=False, kinetic_model="arrhenius", lambda_init=None, beta_init=None,
                 chemistry=None, inlet_primitive=None, controller="Sound Speed Controlled",
                 variant="Variante 1 - Original", wavespeed="Pressure Based", tag=None):
        primitive = np.asarray(primitive, dtype=float)
        self.dim = primitive.ndim - 1
        self.precision = precision
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self.counts = list(primitive.shape[1:][::-1])
        self.cells = int(np.prod(self.counts))
        boundaries = list(boundaries) if boundaries is not None else ["Open"] * self.dim
        chem = dict(chemistry or {})
        closure = chem.pop("closure", "si")
        self.cfg = make_config(self.dim, self.counts, list(np.atleast_1d(lengths)), boundaries,
                               t_end=t_end, cfl=cfl, gamma=gamma, limiter=limiter,
                               max_steps=max_steps, reactive=reactive,
                               kinetic_model=kinetic_model, closure=closure, chemistry=chem,
                               inlet_primitive=inlet_primitive, controller=controller,
                               variant=variant, wavespeed=wavespeed)
        self.reactive = bool(reactive)
        self.nring = 3 if reactive else 2
        shape = tuple(self.counts[::-1])
        lam = None
        if reactive:
            lam = np.ones(shape) if lambda_init is None else np.asarray(lambda_init, float)
        beta = None
        if reactive and kinetic_model == "znd":
            beta = np.ones(shape) if beta_init is None else np.asarray(beta_init, float)
        g = gamma if not (reactive and closure == "si") else (4.5 - lam) / (3.5 - lam)
        state = prim_to_cons(primitive, g)
        dt = _dtype(precision)
        with torch.cuda.device(self.device):
            self.ring = [torch.as_tensor(state, dtype=dt, device=self.device).contiguous()]
            self.ring += [torch.empty_like(self.ring[0]) for _ in range(self.nring - 1)]
            self.lam_ring = self.beta_ring = None
            if lam is not None:
                self.lam_ring = [torch.as_tensor(lam, dtype=dt, device=self.device).contiguous()]
                self.lam_ring += [torch.empty_like(self.lam_ring[0]) for _ in range(2)]
            if beta is not None:
                self.beta_ring = [torch.as_tensor(beta, dtype=dt, device=self.device).contiguous()]
                self.beta_ring += [torch.empty_like(self.beta_ring[0]) for _ in range(2)]
        self.report = None  # last tfv_report; None before the first batch
        self.tag = tag

    @property
    def nbytes(self):
        """Device bytes held by this grid (state and composition rings)."""
        per = _BYTES[self.precision] * self.cells
        n = self.nring * (self.dim + 2) * per
        if self.lam_ring is not None:
            n += 3 * per
        if self.beta_ring is not None:
            n += 3 * per
        return n

    def rotate_current_first(self):
        """Make the current ring buffer index 0 (list rotation, no copy)."""
        if self.report is None or self.report.current == 0:
            return
        k = self.report.current

        def rot(ring):
            return None if ring is None else ring[k:] + ring[:k]

        self.ring, self.lam_ring, self.beta_ring = rot(self.ring), rot(self.lam_ring), rot(
            self.beta_ring)
        self.report.current = 0

    @property
    def current(self):
        return self.ring[self.report.current if self.report is not None else 0]

    @property
    def status(self):
        return self.report.status if self.report is not None else _lib.READY

    @property
    def done(self):
        return self.report is not None and self.report.status != _lib.READY and \
            self.report.status != _lib.RETRY

    @property
    def time(self):
        return self.report.time if self.report is not None else 0.0

    @property
    def steps(self):
        return self.report.steps if self.report is not None else 0

    def state_host(self):
        return self.current.detach().to("cpu", torch.float64).numpy()


class Batch:
    """Advance a list of grids of one dimension and precision together."""

    def __init__(self, grids, tile=None, stream=None, graph_steps=0):
        if not grids:
            raise ValueError("a batch needs at least one grid")
        dims = {g.dim for g in grids}
        precs = {g.precision for g in grids}
        if len(dims) != 1 or len(precs) != 1:
            raise ValueError("a batch holds grids of one dimension and precision")
        self.grids = list(grids)
        self.dim = dims.pop()
        self.precision = precs.pop()
        self.device = grids[0].device
        self.lib = _lib.load()
        self.stream = stream or torch.cuda.Stream(self.device)
        for g in self.grids:
            g.rotate_current_first()
        cfgs = (_lib.Config * len(grids))(*[g.cfg for g in grids])
        handle = C.c_void_p()
        t = None
        if tile is not None:
            vals = list(tile) + [0, 1][len(tile) - 3:] if len(tile) < 5 else list(tile)
            t = _lib.Tile(*vals[:5])
        _lib.check(self.lib.tfv_batch_create(
            self.dim, _lib.TFV_FP64 if self.precision == "fp64" else _lib.TFV_FP32, len(grids),
            cfgs, C.byref(t) if t is not None else None, C.byref(handle)))
        self.handle = handle
        ws = C.c_size_t()
        _lib.check(self.lib.tfv_batch_workspace_size(handle, C.byref(ws)))
        self.workspace = torch.empty(ws.value + 256, dtype=torch.uint8, device=self.device)
        wp = self.workspace.data_ptr() + ((-self.workspace.data_ptr()) % 256)

        def ptrs(rings):
            flat = [r.data_ptr() for ring in rings for r in ring]
            return (C.c_void_p * len(flat))(*flat)

        states = ptrs([g.ring for g in self.grids])
        lams = ptrs([g.lam_ring for g in self.grids]) if all(
            g.lam_ring is not None for g in self.grids) else None
        betas = ptrs([g.beta_ring for g in self.grids]) if all(
            g.beta_ring is not None for g in self.grids) else None
        torch.cuda.current_stream(self.device).synchronize()
        _lib.check(self.lib.tfv_batch_bind(handle, C.c_void_p(wp), states, lams, betas,
                                           _lib.stream_ptr(self.stream)))
        prior = [g.report for g in self.grids]
        if any(r is not None for r in prior):
            reps = (_lib.Report * len(grids))()
            for i, r in enumerate(prior):
                if r is not None:
                    C.memmove(C.byref(reps[i]), C.byref(r), C.sizeof(_lib.Report))
            _lib.check(self.lib.tfv_batch_restore(handle, reps))
        self.reports = (_lib.Report * len(grids))()
        self._ev = None
        self._pending = 0
        self.refresh()
        if graph_steps:
            _lib.check(self.lib.tfv_batch_use_graph(handle, int(graph_steps)))

    def advance(self, nsteps):
        _lib.check(self.lib.tfv_batch_advance(self.handle, int(nsteps)))

    def advance_async(self, nsteps):
        """Enqueue `nsteps` steps bracketed by timing events; `idle()` tells
        when they are done and `last_ms()` how long they took."""
        if self._ev is None:
            self._ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        self._ev[0].record(self.stream)
        self.advance(nsteps)
        self._ev[1].record(self.stream)
        self._pending = int(nsteps)

    def idle(self):
        return self._pending == 0 or self._ev[1].query()

    def last_ms(self):
        """(milliseconds, steps) of the last advance_async, once idle."""
        if self._pending == 0:
            return None
        ms = self._ev[0].elapsed_time(self._ev[1])
        k = self._pending
        self._pending = 0
        return ms, k

    def refresh(self):
        _lib.check(self.lib.tfv_batch_report(self.handle, self.reports))
        for g, r in zip(self.grids, self.reports):
            if g.report is None:
                g.report = _lib.Report()
            C.memmove(C.byref(g.report), C.byref(r), C.sizeof(_lib.Report))
        return self.reports

    def all_done(self):
        return all(g.done for g in self.grids)

    def close(self):
        if getattr(self, "handle", None):
            self.stream.synchronize()
            self.lib.tfv_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
