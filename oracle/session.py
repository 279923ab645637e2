"""Oracle session: the reference ``Simulation.step()`` loop restated on top of
``oracle.fv`` (TEST INFRASTRUCTURE ONLY; see ``oracle/__init__.py``).

Follows python/cfdSolver/torchSession.py:24-158 (construction),
:285-327 (integrals), :333-372 (dt, reaction) and :374-522 (transactional step)
for Cartesian sessions.  Two documented extensions, both off by default:

* ``strict_cfl=False`` accepts CFL > 0.5, which ``validate_grid`` rejects
  (torchSolver.py:1074-1088); the step arithmetic is unchanged.
* ``chemistry={"closure": "nondimensional", ...}`` selects the restated
  nondimensional Arrhenius closure (constant gamma, T = p/rho); parity for it
  is unpinned because the reference has no such closure.
"""

import numpy as np

from . import fv


class OracleSimulation:
    def __init__(self, primitive, lengths, *, t_end, cfl=0.4, gamma=1.4,
                 boundaries=None, limiter="VanLeer", reactive=False,
                 kinetic_model="arrhenius", lambda_init=None, beta_init=None,
                 inlet_primitive=None, controller="Sound Speed Controlled",
                 variant="Variante 1 - Original", wavespeed="Pressure Based",
                 max_steps=100000, strict_cfl=True, chemistry=None):
        primitive = np.array(primitive, dtype=float, copy=True)
        dim = primitive.ndim - 1
        if dim not in (1, 2, 3) or primitive.shape[0] != dim + 2:
            raise ValueError("Require primitives with shape (dimension+2, ...)")
        lengths = [float(v) for v in np.atleast_1d(lengths)]
        counts = list(primitive.shape[1:][::-1])
        boundaries = list(boundaries) if boundaries is not None else ["Open"] * dim
        if len(lengths) != dim or len(boundaries) != dim:
            raise ValueError("Lengths/boundaries must be in x,y,z order")
        for length, n in zip(lengths, counts):
            bad_cfl = not 0 < cfl <= (0.5 if strict_cfl else 1.0)
            if length <= 0 or n < 2 or bad_cfl or t_end < 0:
                raise ValueError("Require length > 0, cells >= 2, valid CFL, t_end >= 0")
        chem = dict(chemistry or {})
        self.closure = chem.pop("closure", "si")
        self.chem = dict(fv.SI_CHEMISTRY)
        self.chem.update(chem)
        self.config = dict(dimension=dim, counts_xyz=counts, lengths_xyz=lengths,
                           boundaries_xyz=boundaries, t_end=t_end, cfl=cfl,
                           gamma=gamma, limiter=limiter, reactive=bool(reactive),
                           kinetic_model=kinetic_model,
                           inlet_primitive=list(fv.DEFAULT_INLET if inlet_primitive is None
                                                else inlet_primitive),
                           controller=controller, variant=variant,
                           wavespeed=wavespeed, max_steps=max_steps)
        shape = tuple(counts[::-1])
        self.lam = (np.ones(shape) if lambda_init is None
                    else np.array(lambda_init, dtype=float)) if reactive else None
        self.beta = ((np.ones(shape) if beta_init is None else np.array(beta_init, dtype=float))
                     if reactive and kinetic_model == "znd" else None)
        self.state = fv.prim_to_cons(primitive, self.gamma)
        if not fv.physical(self.state):
            raise ValueError("Nonphysical initial conservative state")
        self.time, self.steps = 0.0, 0
        self.initial_integral = self.integral.copy()
        self.boundary_integral = np.zeros(dim + 2)
        self.source_integral = np.zeros(dim + 2)
        self.fallback_steps = 0

    # -- properties (torchSession.py:273-331) --------------------------------
    def gamma_of(self, lam):
        if not self.config["reactive"] or self.closure != "si":
            return self.config["gamma"]
        return fv.gamma_of_lambda(lam)

    @property
    def gamma(self):
        return self.gamma_of(self.lam)

    @property
    def spacing(self):
        return np.array(self.config["lengths_xyz"]) / self.config["counts_xyz"]

    @property
    def integral(self):
        d = self.config["dimension"]
        return self.state.reshape(d + 2, -1).sum(axis=1) * np.prod(self.spacing)

    @property
    def balance_residual(self):
        return (self.integral - self.initial_integral + self.boundary_integral
                - self.source_integral)

    @property
    def completed(self):
        return self.time == self.config["t_end"]

    # -- dt and reaction (torchSession.py:333-372) ---------------------------
    def _dt(self, state, gamma):
        c = self.config
        h = self.spacing
        bc = c["boundaries_xyz"]
        if c["dimension"] == 1:
            return fv.dt_1d(state, gamma, h[0], c["cfl"], bc[0], c["wavespeed"])
        if c["dimension"] == 2:
            return fv.dt_2d(state, h, c["cfl"], gamma, bc[0], bc[1], c["inlet_primitive"])
        return fv.dt_3d(state, h, c["cfl"], gamma)

    def _reaction(self, state, lam, beta, dt):
        model = self.config["kinetic_model"]
        kw = dict(self.chem, closure=self.closure, gamma=self.config["gamma"])
        if self.config["dimension"] == 1:
            lam, state, beta = fv.react_1d(lam, dt, state, model, beta, **kw)
            return state, lam, beta if model == "znd" else None
        return fv.reaction_nd(state, lam, beta, dt, model, **kw)

    # -- step (torchSession.py:374-522) --------------------------------------
    def step(self):
        if self.completed:
            return
        c = self.config
        dim = c["dimension"]
        h = self.spacing
        bc = c["boundaries_xyz"]
        if self.steps >= c["max_steps"]:
            raise RuntimeError("Maximum steps reached before requested final time")
        dt = min(self._dt(self.state, self.gamma), c["t_end"] - self.time)
        if not np.isfinite(dt) or dt <= 0 or self.time + dt == self.time:
            raise RuntimeError("Integration stalled before requested final time")
        start = self.state
        old, lam, beta = start, self.lam, self.beta
        if c["reactive"]:
            for _ in range(60):
                old, lam, beta = self._reaction(start, self.lam, self.beta, dt / 2)
                allowed = self._dt(old, self.gamma_of(lam))
                if dt <= allowed * (1 + 1e-12):
                    break
                dt = min(dt / 2, allowed)
            else:
                raise RuntimeError("Could not find stable reactive step")
        gamma = self.gamma_of(lam)
        if dim == 1:
            state, flux, used = fv.step_1d(old, dt, h[0], gamma, c["cfl"], c["limiter"],
                                           c["controller"], c["variant"], c["wavespeed"],
                                           bc[0])
            fluxes = [flux]
            if c["reactive"]:
                lam = fv.advect_1d(lam, old, state, flux[0], dt / h[0], bc[0])
                if beta is not None:
                    beta = fv.advect_1d(beta, old, state, flux[0], dt / h[0], bc[0])
        elif dim == 2:
            state, fx, fy, used = fv.hydro_2d(old, h[0], h[1], dt, gamma, c["limiter"],
                                              bc[0], bc[1], c["inlet_primitive"])
            fluxes = [fx, fy]
            if c["reactive"]:
                lam = fv.advect_2d(lam, old, state, fx[0], fy[0], dt / h[0], dt / h[1], *bc)
                if beta is not None:
                    beta = fv.advect_2d(beta, old, state, fx[0], fy[0], dt / h[0],
                                        dt / h[1], *bc)
        else:
            state, fluxes, used = fv.hydro_3d(old, gamma, h, dt, c["limiter"], bc)
            if c["reactive"]:
                lam = fv.advect_3d(lam, old, state, fluxes, dt, h, bc)
                if beta is not None:
                    beta = fv.advect_3d(beta, old, state, fluxes, dt, h, bc)
        outward = np.zeros(dim + 2)
        volume = np.prod(h)
        for direction, flux in enumerate(fluxes):
            axis = dim - direction
            faces = np.take(flux, -1, axis=axis) - np.take(flux, 0, axis=axis)
            outward += dt * volume / h[direction] * faces.reshape(dim + 2, -1).sum(axis=1)
        source = np.zeros(dim + 2)
        if c["reactive"]:
            hydro = state
            state, lam, beta = self._reaction(hydro, lam, beta, dt / 2)
            source = volume * (old - start + state - hydro).reshape(dim + 2, -1).sum(axis=1)
        if not fv.physical(state):
            raise RuntimeError("Reaction produced a nonphysical state")
        self.state, self.lam, self.beta = state, lam, beta
        self.boundary_integral += outward
        self.source_integral += source
        self.time = min(self.time + dt, c["t_end"])
        self.steps += 1
        self.fallback_steps += int(used)
        self.last_dt = dt

    def run(self, step_limit=None):
        count = 0
        while not self.completed and (step_limit is None or count < step_limit):
            self.step()
            count += 1
        return self
