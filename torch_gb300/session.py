"""GPU drop-in for TORCH's ``Simulation`` session.

Mirrors python/cfdSolver/torchSession.py:19-694: same constructor keywords,
state layout ``(dim+2, nz, ny, nx)`` x fastest, properties, transactional
``step()``, checkpoints and exception types.  Cartesian grids run the
MUSCL-Hancock + HLLC engine (``tfv_batch_*``); cylindrical, annular and
spherical grids and grids with per-face boundaries run the metric engine
(``tfv_metric_*``, torch_gb300/metric.py), as the reference's
``uses_metric_kernel`` selects.  The state lives on the GPU; ``state``,
``lam`` and ``beta`` materialise as host float64 arrays on access so that
host-side consumers (checkpoint writers, plots) keep working.

Extensions (off by default): ``precision="fp32"`` runs the bulk step in FP32
with FP64 time and conservation sums; ``strict_cfl=False`` accepts CFL > 0.5
(rejected by the reference's validate_grid, torchSolver.py:1074-1088);
``chemistry=`` selects the nondimensional Arrhenius closure.
"""

import ctypes as C
import uuid

import numpy as np
import torch

from . import _lib
from . import metric

LIMITERS = ("VanLeer", "Albada", "MINBEE", "Superbee", "Unos")
DEFAULT_INLET = [1.0, 0.0, 100.0, 101325.0]
SI_CHEMISTRY = dict(q_heat=141584000.0, activation_energy=17.15 * 4184.0,
                    pre_exponential=1.76e5)


def _validate_grid(length, cells, cfl, end_time, strict_cfl):
    """validate_grid (python/cfdSolver/torchSolver.py:1074-1088)."""
    cfl_ok = 0 < cfl <= 0.5 if strict_cfl else 0 < cfl <= 1.0
    if (not isinstance(cells, (int, np.integer)) or not np.isfinite([length, cfl, end_time]).all()
            or length <= 0 or cells < 2 or not cfl_ok or end_time < 0):
        raise ValueError("Require length > 0, cells >= 2, 0 < CFL <= 0.5 and final time >= 0")


def _physical(state):
    """physical_state (python/cfdSolver/torchSolver.py:1038-1046)."""
    return bool(np.isfinite(state).all() and np.all(state[0] > 1e-12) and np.all(
        state[-1] - 0.5 * np.sum(state[1:-1] ** 2, axis=0) / state[0] > 1e-12))


def prim_to_cons(primitive, gamma):
    """Session primitive -> conservative conversion (torchSession.py:145-150)."""
    state = primitive.copy()
    state[1:-1] *= primitive[0]
    state[-1] = primitive[-1] / (gamma - 1) + 0.5 * primitive[0] * np.sum(
        primitive[1:-1] ** 2, axis=0)
    return state


def make_config(dim, counts, lengths, boundaries, *, t_end, cfl, gamma, limiter, max_steps,
                reactive=False, kinetic_model="arrhenius", closure="si", chemistry=None,
                inlet_primitive=None, controller="Sound Speed Controlled",
                variant="Variante 1 - Original", wavespeed="Pressure Based"):
    cfg = _lib.Config()
    cfg.dim = dim
    for k in range(3):
        cfg.counts[k] = int(counts[k]) if k < dim else 1
        cfg.lengths[k] = float(lengths[k]) if k < dim else 1.0
        cfg.bc[k] = _lib.bc_code(boundaries[k]) if k < dim else 0
    cfg.limiter = _lib.LIMITERS[limiter]
    cfg.gamma = float(gamma)
    cfg.cfl = float(cfl)
    cfg.t_end = float(t_end)
    cfg.max_steps = int(max_steps)
    cfg.reactive = int(bool(reactive))
    cfg.kinetic_model = _lib.MODELS[kinetic_model]
    cfg.closure = _lib.CLOSURES[closure]
    chem = dict(SI_CHEMISTRY)
    chem.update(chemistry or {})
    cfg.q_heat = chem["q_heat"]
    cfg.activation = chem["activation_energy"]
    cfg.pre_exponential = chem["pre_exponential"]
    inlet = DEFAULT_INLET if inlet_primitive is None else inlet_primitive
    for k in range(4):
        cfg.inlet_primitive[k] = float(inlet[k])
    cfg.controller = _lib.CONTROLLERS[controller]
    cfg.variant = _lib.VARIANTS[variant]
    cfg.wavespeed = _lib.WAVESPEEDS[wavespeed]
    return cfg


def validate_config(c, strict_cfl=True):
    """Session configuration checks (torchSession.py:190-254), Cartesian."""
    dim = c["dimension"]
    if not isinstance(dim, (int, np.integer)) or dim not in (1, 2, 3) or isinstance(dim, bool):
        raise ValueError("Invalid dimension")
    for key in ("counts_xyz", "lengths_xyz", "boundaries_xyz"):
        if len(c[key]) != dim:
            raise ValueError("Incomplete mesh/boundary metadata")
    for length, n in zip(c["lengths_xyz"], c["counts_xyz"]):
        _validate_grid(length, n, c["cfl"], c["t_end"], strict_cfl)
    metric.validate_geometry(c)
    if c.get("geometry", "cartesian") != "cartesian" or "face_boundaries" in c:
        c["face_boundaries"] = metric.normalize_faces(c, c.get("face_boundaries"))
        if (c["controller"], c["variant"], c["wavespeed"]) != (
                "Sound Speed Controlled", "Variante 1 - Original", "Pressure Based"):
            raise ValueError("Metric/face sessions use MUSCL-Rusanov/SSPRK2; legacy HLLC "
                             "switches are unsupported")
    if not np.isfinite(c["gamma"]) or c["gamma"] <= 1:
        raise ValueError("gamma must be finite and greater than one")
    if c["limiter"] not in LIMITERS or c["kinetic_model"] not in ("arrhenius", "znd"):
        raise ValueError("Unknown limiter or chemistry model")
    if (not isinstance(c["max_steps"], (int, np.integer)) or isinstance(c["max_steps"], bool)
            or c["max_steps"] < 1):
        raise ValueError("Invalid maximum steps")
    for axis, boundary in enumerate(c["boundaries_xyz"]):
        if boundary not in ("Open", "Reflective", "Periodic") and not (
                dim == 2 and axis == 1 and boundary == "Inflow"):
            raise ValueError("Unsupported session boundary")
    if c["controller"] not in _lib.CONTROLLERS or c["variant"] not in _lib.VARIANTS or \
            c["wavespeed"] not in _lib.WAVESPEEDS:
        raise ValueError("Unknown solver option")
    if dim == 2 and "Inflow" in c["boundaries_xyz"]:
        inlet = np.asarray(c["inlet_primitive"])
        if (inlet.shape != (4,) or not np.isfinite(inlet).all() or inlet[0] <= 0
                or inlet[3] <= 0 or inlet[2] < 0):
            raise ValueError("Invalid inlet primitives")


def _dtype(precision):
    if precision not in ("fp64", "fp32"):
        raise ValueError("precision must be 'fp64' or 'fp32'")
    return torch.float64 if precision == "fp64" else torch.float32


class _Engine:
    """One batch handle with its device memory (ring buffers and workspace)."""

    def __init__(self, dim, precision, cfgs, states, device, tile=None, stream=None, lams=None,
                 betas=None):
        lib = _lib.load()
        self.lib = lib
        self.dim = dim
        self.n = len(cfgs)
        self.precision = precision
        self.dtype = _dtype(precision)
        self.device = device
        # a dedicated stream: graph capture is not allowed on the legacy default stream
        self.stream = stream or torch.cuda.Stream(device)
        arr = (_lib.Config * self.n)(*cfgs)
        handle = C.c_void_p()
        t = None
        if tile is not None:
            # (tx, ty, chunk[, persistent_ctas[, tma]]); tensor-copy staging on by default
            vals = list(tile) + [0, 1][len(tile) - 3:] if len(tile) < 5 else list(tile)
            t = _lib.Tile(*vals[:5])
        _lib.check(lib.tfv_batch_create(dim, _lib.TFV_FP64 if precision == "fp64" else _lib.TFV_FP32,
                                        self.n, arr, C.byref(t) if t is not None else None,
                                        C.byref(handle)))
        self.handle = handle
        ws = C.c_size_t()
        _lib.check(lib.tfv_batch_workspace_size(handle, C.byref(ws)))
        nring = C.c_int32()
        _lib.check(lib.tfv_batch_ring_size(handle, C.byref(nring)))
        self.nring = nring.value
        self.workspace = torch.empty(ws.value + 256, dtype=torch.uint8, device=device)
        off = (-self.workspace.data_ptr()) % 256
        self.ws_ptr = self.workspace.data_ptr() + off
        def make_rings(arrays):
            rings, ptrs = [], []
            for a in arrays:
                ring = [torch.as_tensor(np.asarray(a), dtype=self.dtype).to(device).contiguous()]
                for _ in range(self.nring - 1):
                    ring.append(torch.empty_like(ring[0]))
                rings.append(ring)
                ptrs.extend(r.data_ptr() for r in ring)
            return rings, (C.c_void_p * len(ptrs))(*ptrs) if ptrs else None

        with torch.cuda.stream(self.stream):
            self.rings, parr = make_rings(states)
            self.lam_rings, larr = make_rings(lams) if lams is not None else ([], None)
            self.beta_rings, barr = make_rings(betas) if betas is not None else ([], None)
        self.stream.synchronize()
        _lib.check(lib.tfv_batch_bind(handle, C.c_void_p(self.ws_ptr), parr, larr, barr,
                                      _lib.stream_ptr(self.stream)))
        self.reports = (_lib.Report * self.n)()
        self.refresh()

    def advance(self, nsteps):
        _lib.check(self.lib.tfv_batch_advance(self.handle, int(nsteps)))

    def restore(self, reports):
        """Carry time, steps, integrals and fallback counters of an earlier run
        into this freshly bound engine (its current states are ring slot 0)."""
        arr = (_lib.Report * self.n)(*reports)
        _lib.check(self.lib.tfv_batch_restore(self.handle, arr))
        self.refresh()

    def profile(self, nsteps):
        """Milliseconds (step kernel, fallback, finalize) summed over nsteps."""
        out = [C.c_float(), C.c_float(), C.c_float()]
        _lib.check(self.lib.tfv_batch_profile(self.handle, int(nsteps), *[C.byref(v) for v in out]))
        return [v.value for v in out]

    def use_graph(self, steps):
        _lib.check(self.lib.tfv_batch_use_graph(self.handle, int(steps)))

    def refresh(self):
        _lib.check(self.lib.tfv_batch_report(self.handle, self.reports))
        return self.reports

    def integrals(self):
        out = (C.c_double * (5 * self.n))()
        _lib.check(self.lib.tfv_batch_integrals(self.handle, out))
        return np.array(out[:]).reshape(self.n, 5)

    def current(self, i=0):
        return self.rings[i][self.reports[i].current]

    def current_lam(self, i=0):
        return self.lam_rings[i][self.reports[i].current] if self.lam_rings else None

    def current_beta(self, i=0):
        return self.beta_rings[i][self.reports[i].current] if self.beta_rings else None

    def replan(self):
        _lib.check(self.lib.tfv_batch_replan(self.handle))
        self.refresh()

    def replan_async(self):
        """Recompute dt from the current buffers without waiting."""
        _lib.check(self.lib.tfv_batch_replan(self.handle))

    def set_flux_outputs(self, i, fx, fy, fz):
        _lib.check(self.lib.tfv_batch_set_flux_outputs(self.handle, i, _lib.ptr(fx), _lib.ptr(fy),
                                                       _lib.ptr(fz)))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.tfv_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Simulation:
    """Cartesian simulation session resumable between steps, on one GPU."""

    def __init__(self, primitive, lengths, *, t_end, cfl=0.4, gamma=1.4, boundaries=None,
                 limiter="VanLeer", reactive=False, kinetic_model="arrhenius", lambda_init=None,
                 beta_init=None, inlet_primitive=None, controller="Sound Speed Controlled",
                 variant="Variante 1 - Original", wavespeed="Pressure Based", max_steps=100000,
                 geometry="cartesian", origins=None, face_boundaries=None, workers=1,
                 precision="fp64", device=None, strict_cfl=True, chemistry=None, tile=None,
                 graph_steps=0):
        primitive = np.array(primitive, dtype=float, copy=True)
        dim = primitive.ndim - 1
        if dim not in (1, 2, 3) or primitive.shape[0] != dim + 2:
            raise ValueError("Require primitives with shape (dimension+2, ... reversed spatial axes)")
        lengths = list(np.atleast_1d(lengths))
        counts = list(primitive.shape[1:][::-1])
        if len(lengths) != dim:
            raise ValueError("Lengths must be in x,y,z order, one per active axis")
        boundaries = list(boundaries) if boundaries is not None else ["Open"] * dim
        uses_metric = geometry != "cartesian" or face_boundaries is not None
        chem = dict(chemistry or {})
        closure = chem.pop("closure", "si")
        if closure not in _lib.CLOSURES:
            raise ValueError("Unknown chemistry closure")
        if uses_metric and closure != "si":
            raise ValueError("Metric/face sessions use the SI chemistry closure")
        self.config = dict(
            dimension=dim, counts_xyz=counts, lengths_xyz=lengths, boundaries_xyz=boundaries,
            t_end=t_end, cfl=cfl, gamma=gamma, limiter=limiter, reactive=bool(reactive),
            kinetic_model=kinetic_model,
            inlet_primitive=list(DEFAULT_INLET if inlet_primitive is None else inlet_primitive),
            controller=controller, variant=variant, wavespeed=wavespeed, max_steps=max_steps,
            geometry=geometry, origins_xyz=(list(np.atleast_1d(origins)) if origins is not None
                                            else [0.0] * dim))
        if uses_metric:  # walls implied at a radial origin and at poles (torchSession.py:89-121)
            self.config["face_boundaries"] = metric.normalize_faces(
                self.config, metric.default_face_spec(self.config, face_boundaries))
        self._strict_cfl = strict_cfl
        self._closure = closure
        self._chem = chem
        self._validate_config()
        if not np.isfinite(primitive).all() or np.any(primitive[[0, -1]] <= 0):
            raise ValueError("Initial density and pressure must be positive and primitives finite")
        lam0 = self._fraction(lambda_init, "lambda") if reactive else None
        beta0 = self._fraction(beta_init, "beta") if reactive and kinetic_model == "znd" else None
        if (not reactive and lambda_init is not None) or (beta_init is not None and beta0 is None):
            raise ValueError("Composition requires reactive chemistry; beta requires ZND")
        self._lam0 = lam0
        g = self._gamma_of(lam0)
        state = prim_to_cons(primitive, g)
        if not _physical(state):
            raise ValueError("Nonphysical initial conservative state")
        self.precision = precision
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        if uses_metric:
            self._engine = metric.MetricEngine(self.config, self.config["face_boundaries"], state,
                                               lam0, beta0, precision, self.device,
                                               dict(SI_CHEMISTRY, **chem))
        else:
            cfg = make_config(dim, counts, lengths, boundaries, t_end=t_end, cfl=cfl, gamma=gamma,
                              limiter=limiter, max_steps=max_steps, reactive=reactive,
                              kinetic_model=kinetic_model, closure=closure, chemistry=chem,
                              inlet_primitive=inlet_primitive, controller=controller,
                              variant=variant, wavespeed=wavespeed)
            self._engine = _Engine(dim, precision, [cfg], [state], self.device, tile=tile,
                                   lams=None if lam0 is None else [lam0],
                                   betas=None if beta0 is None else [beta0])
        if graph_steps:
            self._engine.use_graph(graph_steps)
        self.run_id = str(uuid.uuid4())
        self._workers = 1
        self.set_workers(workers)

    def _fraction(self, values, name):
        """Composition arrays (torchSession.py:256-271)."""
        shape = tuple(self.config["counts_xyz"][::-1])
        result = np.ones(shape) if values is None else np.array(values, dtype=float, copy=True)
        if (result.shape != shape or not np.isfinite(result).all()
                or np.any((result < 0) | (result > 1))):
            raise ValueError(f"{name} must have the spatial shape and values in [0,1]")
        return result

    def _gamma_of(self, lam):
        if self.config["reactive"] and self._closure == "si" and lam is not None:
            return (4.5 - lam) / (3.5 - lam)
        return self.config["gamma"]

    def _validate_config(self):
        validate_config(self.config, self._strict_cfl)

    # -- workers: the GPU replaces the CPU flux pool (torchExecution.py) ----
    @property
    def workers(self):
        return self._workers

    def set_workers(self, workers):
        if not isinstance(workers, int) or isinstance(workers, bool) or not 1 <= workers <= 64:
            raise ValueError("Workers must be an integer from 1 to 64")
        self._workers = workers
        return self

    def close(self):
        pass

    # -- state access --------------------------------------------------------
    @property
    def _report(self):
        return self._engine.reports[0]

    @property
    def state(self):
        self._engine.stream.synchronize()
        return self._engine.current().detach().to("cpu", torch.float64).numpy()

    @state.setter
    def state(self, value):
        value = np.array(value, dtype=float)
        cur = self._engine.current()
        if value.shape != tuple(cur.shape):
            raise ValueError("state shape mismatch")
        with torch.cuda.stream(self._engine.stream):
            cur.copy_(torch.as_tensor(value, dtype=cur.dtype))
        self._engine.replan()

    @property
    def device_state(self):
        """The current state buffer on the GPU (no copy), ready to read."""
        self._engine.stream.synchronize()
        return self._engine.current()

    @property
    def time(self):
        return self._report.time

    @property
    def steps(self):
        return self._report.steps

    @property
    def dt(self):
        return self._report.dt

    @property
    def initial_integral(self):
        return np.array(self._report.initial_integral[:self.config["dimension"] + 2])

    @property
    def boundary_integral(self):
        return np.array(self._report.boundary_integral[:self.config["dimension"] + 2])

    @property
    def source_integral(self):
        return np.array(self._report.source_integral[:self.config["dimension"] + 2])

    @property
    def fallback_steps(self):
        return self._report.fallback_steps

    @property
    def gamma(self):
        return self._gamma_of(self.lam)

    @property
    def lam(self):
        if not self.config["reactive"]:
            return None
        self._engine.stream.synchronize()
        return self._engine.current_lam().detach().to("cpu", torch.float64).numpy()

    @property
    def beta(self):
        t = self._engine.current_beta()
        if t is None:
            return None
        self._engine.stream.synchronize()
        return t.detach().to("cpu", torch.float64).numpy()

    @property
    def spacing(self):
        return np.array(self.config["lengths_xyz"]) / self.config["counts_xyz"]

    @property
    def integral(self):
        return self._engine.integrals()[0, :self.config["dimension"] + 2]

    @property
    def uses_metric_kernel(self):
        """torchSession.py:303-308"""
        return self.config.get("geometry", "cartesian") != "cartesian" or \
            "face_boundaries" in self.config

    @property
    def primitive(self):
        s = self.state
        p = s.copy()
        p[1:-1] /= s[0]
        p[-1] = (self.gamma - 1) * (s[-1] - 0.5 * np.sum(s[1:-1] ** 2, axis=0) / s[0])
        return p

    @property
    def balance_residual(self):
        return (self.integral - self.initial_integral + self.boundary_integral
                - self.source_integral)

    @property
    def completed(self):
        return self.time == self.config["t_end"]

    # -- stepping ------------------------------------------------------------
    def _raise_pending(self):
        status = self._report.status
        if status in (_lib.READY, _lib.DONE, _lib.RETRY):
            return
        if status == _lib.ERR_CHEMISTRY:  # the reference's reaction step raises ValueError
            raise ValueError(_lib.STATUS_MESSAGES[status])
        raise RuntimeError(_lib.STATUS_MESSAGES.get(status, _lib.STATUS[status]))

    def step(self):
        """Advance one complete split step; failed steps leave session data intact."""
        if self.completed:
            return
        self._raise_pending()  # max steps / stall found when this step was planned
        before = self.steps
        for _ in range(61):  # a reactive step may take up to 60 dt halvings
            self._engine.advance(1)
            self._engine.refresh()
            if self._report.status != _lib.RETRY:
                break
        if self.steps == before:
            self._raise_pending()  # the step itself failed; nothing was committed

    def advance(self, nsteps):
        """Enqueue ``nsteps`` steps without waiting (stops at t_end or on error)."""
        self._engine.advance(nsteps)

    def synchronize(self):
        self._engine.refresh()
        self._raise_pending()

    def run(self, *, step_limit=None, checkpoint=None, checkpoint_every=0, output_prefix=None,
            output_every=1, formats=("vtk", "xdmf"), chunk=64):
        """Advance to t_end or by `step_limit` steps (torchSession.py:578-632).
        With `checkpoint`, a checkpoint is written whenever the step count
        reaches a multiple of `checkpoint_every` and once at the end; with
        `output_prefix`, a VTK / XDMF frame at the start, at every multiple of
        `output_every` and at the end (torch_gb300/output.py: the state is
        copied to pinned host memory on the session's stream and a host thread
        writes the files while the GPU keeps stepping).  Steps are enqueued in
        chunks that stop at those multiples, so no numerical step is
        shortened."""
        for value in (step_limit, checkpoint_every, output_every):
            if value is not None and (not isinstance(value, int) or value < 0):
                raise ValueError("Step intervals must be nonnegative integers")
        if checkpoint_every and not checkpoint:
            raise ValueError("checkpoint_every requires a checkpoint destination")
        if output_prefix and output_every < 1:
            raise ValueError("output_every must be positive")
        writer = None
        if output_prefix:  # frames are copied off the GPU and written by a host thread
            from .output import AsyncWriter
            writer = AsyncWriter(output_prefix, self, formats)
        try:
            remaining = step_limit
            while not self.completed and (remaining is None or remaining > 0):
                self._raise_pending()
                k = chunk if remaining is None else min(chunk, remaining)
                if checkpoint and checkpoint_every:
                    k = min(k, checkpoint_every - self.steps % checkpoint_every)
                if writer:
                    k = min(k, output_every - self.steps % output_every)
                before = self.steps
                self._engine.advance(k)
                self._engine.refresh()
                if remaining is not None:
                    remaining -= self.steps - before
                self._raise_pending()
                if (checkpoint and checkpoint_every and self.steps != before
                        and self.steps % checkpoint_every == 0):
                    self.save(checkpoint)
                if writer and self.steps != before and self.steps % output_every == 0:
                    writer.append(self)
            if checkpoint:
                self.save(checkpoint)
            if writer:
                writer.append(self)
        finally:
            if writer:
                writer.close()
        return self

    # -- checkpoint interchange (torchSession.py:634-651) ----------------------
    def save(self, path):
        """Write a TORCH checkpoint (schema 2) of this session; the reference's
        read_checkpoint accepts it."""
        from . import checkpoint
        return checkpoint.write(path, self)

    @classmethod
    def load(cls, path, *, t_end=None, **options):
        """Resume a TORCH checkpoint on the GPU, optionally with a later end
        time (torchSession.py:640-651).  `options` are the GPU extensions
        accepted by `from_session`."""
        from . import checkpoint
        snap = checkpoint.read(path)
        if t_end is not None:
            if not np.isfinite(t_end) or t_end < snap.time:
                raise ValueError("New end time must be finite and not precede checkpoint")
            snap.config["t_end"] = t_end
        return cls.from_session(snap, **options)

    @classmethod
    def from_session(cls, session, **options):
        """A GPU session that continues `session`: any object with the
        reference session's attributes (config, state, lam, beta, time, steps,
        initial/boundary/source integrals, run_id), such as the reference's
        own Simulation or a checkpoint Snapshot.  The conservative state and
        composition are taken exactly; `options` adds GPU extensions
        (precision, strict_cfl, chemistry, tile, graph_steps, device)."""
        c = session.config
        state = np.array(session.state, dtype=float)
        reactive = bool(c["reactive"])
        lam = np.array(session.lam, dtype=float) if reactive else None
        znd = reactive and c["kinetic_model"] == "znd"
        beta = np.array(session.beta, dtype=float) if znd else None
        closure = dict(options.get("chemistry") or {}).get("closure", "si")
        gamma = (4.5 - lam) / (3.5 - lam) if reactive and closure == "si" else c["gamma"]
        primitive = state.copy()
        primitive[1:-1] /= state[0]
        primitive[-1] = (gamma - 1) * (state[-1] - 0.5 * np.sum(state[1:-1] ** 2, axis=0)
                                       / state[0])
        kw = dict(t_end=c["t_end"], cfl=c["cfl"], gamma=c["gamma"],
                  boundaries=list(c["boundaries_xyz"]), limiter=c["limiter"], reactive=reactive,
                  kinetic_model=c["kinetic_model"], lambda_init=lam, beta_init=beta,
                  inlet_primitive=c.get("inlet_primitive"),
                  controller=c.get("controller", "Sound Speed Controlled"),
                  variant=c.get("variant", "Variante 1 - Original"),
                  wavespeed=c.get("wavespeed", "Pressure Based"), max_steps=c["max_steps"],
                  origins=c.get("origins_xyz"), geometry=c.get("geometry", "cartesian"),
                  face_boundaries=c.get("face_boundaries"))
        kw.update(options)
        sim = cls(primitive, list(c["lengths_xyz"]), **kw)
        sim.state = state  # exact conservative values, not a round trip through primitives
        report = _lib.Report()
        report.time = float(session.time)
        report.steps = int(session.steps)
        for field, name in ((report.initial_integral, "initial_integral"),
                            (report.boundary_integral, "boundary_integral"),
                            (report.source_integral, "source_integral")):
            for k, v in enumerate(np.asarray(getattr(session, name), dtype=float)):
                field[k] = v
        report.fallback_steps = int(getattr(session, "fallback_steps", 0))
        report.status = _lib.READY
        sim._engine.restore([report])
        sim.run_id = getattr(session, "run_id", None) or sim.run_id
        return sim
