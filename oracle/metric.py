"""Oracle for the metric / face-boundary finite-volume step (TEST
INFRASTRUCTURE ONLY: imported by tests, smoke() and bench.py's CPU legs,
never by the product path).

Restates, in NumPy and with the reference's operation order, the second
solver of TORCH: MUSCL reconstruction of primitives with limited slopes,
Rusanov fluxes weighted by face areas, SSPRK2 stages with a first-order
retry, geometric source terms of cylindrical / annular / spherical grids, and
per-face boundary states (outflow, wall, periodic, inflow, pressure outlet,
stagnation inlet).

* geometry factors and sources: python/cfdSolver/torchGeometry.py:34-204
* face boundaries: python/cfdSolver/torchBoundaries.py:18-246
* reconstruction, flux, update, dt: python/cfdSolver/torchFiniteVolume.py:16-276
* the session's metric step: python/cfdSolver/torchSession.py:523-576

Pinned against the reference's own sessions (tests/golden/metric.npz, made by
tests/golden/make_golden.py) in tests/test_oracle_golden.py.
"""

import numpy as np

from . import fv

GEOMETRIES = ("cartesian", "cylindrical", "annular", "spherical")
FACE_TYPES = ("outflow", "wall", "periodic", "inflow", "pressure_outlet", "stagnation_inlet")


# -- geometry (torchGeometry.py:34-204) ----------------------------------------
def axes(c):
    dim = c["dimension"]
    return [np.linspace(o, o + l, n + 1) for o, l, n in
            zip(c.get("origins_xyz", [0.0] * dim), c["lengths_xyz"], c["counts_xyz"])]


def factors(c):
    """One-dimensional factors, x first: (volume factors, face factors per
    direction).  Volumes and face areas are their outer products."""
    dim, g = c["dimension"], c.get("geometry", "cartesian")
    ax = axes(c)
    widths = [np.diff(a) for a in ax]
    n = c["counts_xyz"]
    if g == "cartesian":
        vol = widths
        face = [[np.ones(n[a] + 1) if a == d else widths[a] for a in range(dim)]
                for d in range(dim)]
        return vol, face
    r = ax[0]
    dr, shell2 = np.diff(r), np.diff(r ** 2) / 2
    if g == "spherical":
        shell3 = np.diff(r ** 3) / 3
        if dim == 1:
            return [4 * np.pi * shell3], [[4 * np.pi * r ** 2]]
        theta = ax[1]
        solid = -np.diff(np.cos(theta))
        azimuth = widths[2] if dim == 3 else np.array([2 * np.pi])
        k = 1 if dim == 3 else 2 * np.pi
        extra = [azimuth] if dim == 3 else []
        vol = [k * shell3, solid] + extra
        face = [[k * r ** 2, solid] + extra, [k * shell2, np.sin(theta)] + extra]
        if dim == 3:
            face.append([shell2, widths[1], np.ones(n[2] + 1)])
        return vol, face
    if dim == 1:
        return [2 * np.pi * shell2], [[2 * np.pi * r]]
    if g == "cylindrical" and dim == 2:
        return ([2 * np.pi * shell2, widths[1]],
                [[2 * np.pi * r, widths[1]], [2 * np.pi * shell2, np.ones(n[1] + 1)]])
    vol = [shell2, widths[1]] + widths[2:]
    face = [[r, widths[1]] + widths[2:], [dr, np.ones(n[1] + 1)] + widths[2:]]
    if dim == 3:
        face.append([shell2, widths[1], np.ones(n[2] + 1)])
    return vol, face


def outer(fs):
    """Outer product in (z, y, x) layout, multiplied x, then y, then z."""
    dim = len(fs)
    out = np.ones(tuple(len(f) for f in fs)[::-1])
    for d, f in enumerate(fs):
        shape = [1] * dim
        shape[dim - 1 - d] = len(f)
        out *= np.asarray(f).reshape(shape)
    return out


class Metric:
    def __init__(self, c):
        self.config = c
        dim = c["dimension"]
        vol, face = factors(c)
        self.volumes = outer(vol)
        self.areas = [outer(f) for f in face]
        self.divergence = [np.diff(a, axis=dim - 1 - d) / self.volumes
                           for d, a in enumerate(self.areas)]

    def source(self, p):
        c = self.config
        dim, g = c["dimension"], c.get("geometry", "cartesian")
        out = np.zeros_like(p)
        if g == "cartesian":
            return out
        rho, pr = p[0], p[-1]
        radial = self.divergence[0]
        out[1] = pr * radial
        if g == "spherical":
            invr = radial / 2
            out[1] += rho * np.sum(p[2:-1] ** 2, axis=0) * invr
            if dim >= 2:
                cot = self.divergence[1]
                out[2] = pr * cot - rho * p[1] * p[2] * invr
                if dim == 3:
                    out[2] += rho * p[3] ** 2 * cot
                    out[3] = -rho * p[3] * (p[1] * invr + p[2] * cot)
        elif dim >= 2 and not (g == "cylindrical" and dim == 2):
            out[1] += rho * p[2] ** 2 * radial
            out[2] = -rho * p[1] * p[2] * radial
        return out


# -- face boundaries (torchBoundaries.py:18-246) -------------------------------
def default_faces(c):
    """Faces implied by boundaries_xyz (torchBoundaries.py:20-35)."""
    kinds = {"Open": "outflow", "Reflective": "wall", "Periodic": "periodic",
             "Inflow": "inflow"}
    out = []
    for name in c["boundaries_xyz"]:
        low = dict(type=kinds[name])
        if low["type"] == "inflow":
            low["primitive"] = list(c["inlet_primitive"])
        out += [low, dict(type="outflow") if low["type"] == "inflow" else dict(low)]
    return out


def ghost(p, gamma, fractions, face, direction, side, reactive):
    """Boundary-plane state from the boundary cells' primitives; side -1 is
    the low face, +1 the high face."""
    p = p.copy()
    g = np.array(gamma, copy=True)
    qs = [np.array(q, copy=True) for q in fractions]
    kind = face["type"]
    n = direction + 1
    if kind == "wall":
        p[n] *= -1
    elif kind in ("inflow", "stagnation_inlet"):
        g[...] = fv.gamma_of_lambda(face.get("lambda", 1.0)) if reactive else gamma
        for q, key in zip(qs, ("lambda", "beta")):
            q[...] = face.get(key, 1.0)
        if kind == "inflow":
            p[...] = np.asarray(face["primitive"]).reshape((-1,) + (1,) * (p.ndim - 1))
        else:
            interior = p.copy()
            sound = np.sqrt(gamma * interior[-1] / interior[0])
            riemann = -side * interior[n] - 2 * sound / (gamma - 1)
            a0sq = g * face["gas_constant"] * face["total_temperature"]
            k = (g + 1) / (g - 1)
            disc = riemann ** 2 - k * (0.5 * (g - 1) * riemann ** 2 - a0sq)
            if np.any(disc < 0):
                raise ValueError("No subsonic reservoir-inlet solution")
            a = (-riemann + np.sqrt(disc)) / k
            speed = riemann + 2 * a / (g - 1)
            choked = speed >= a
            a = np.where(choked, np.sqrt(2 * a0sq / (g + 1)), a)
            speed = np.where(choked, a, speed)
            if np.any(speed < 0) or np.any(a <= 0):
                raise ValueError("Reservoir cannot supply inflow against the interior pressure")
            p[1:-1] = 0
            p[n] = -side * speed
            p[-1] = face["total_pressure"] * (a * a / a0sq) ** (g / (g - 1))
            p[0] = g * p[-1] / (a * a)
    elif kind == "pressure_outlet":
        a = np.sqrt(g * p[-1] / p[0])
        un = side * p[n]
        subsonic = un < a
        rho = p[0] * (face["pressure"] / p[-1]) ** (1 / g)
        anew = np.sqrt(g * face["pressure"] / rho)
        velocity = un + 2 * (a - anew) / (g - 1)
        back = subsonic & ((velocity < 0) | (un < 0))
        if np.any(back) and "backflow" not in face:
            raise ValueError("Pressure outlet backflow requires an explicit backflow "
                             "primitive state")
        p[0] = np.where(subsonic, rho, p[0])
        p[-1] = np.where(subsonic, face["pressure"], p[-1])
        p[n] = np.where(subsonic, side * velocity, p[n])
        if np.any(back):
            p = np.where(back[None], np.asarray(face["backflow"]).reshape(
                (-1,) + (1,) * (p.ndim - 1)), p)
            if reactive:
                g = np.where(back, fv.gamma_of_lambda(face.get("lambda", 1.0)), g)
            for q, key in zip(qs, ("lambda", "beta")):
                q[...] = np.where(back, face.get(key, 1.0), q)
    return p, g, qs


def boundary_plane(p, gamma, fractions, c, faces, d, side):
    axis = c["dimension"] - 1 - d
    face = faces[2 * d + (side == 1)]
    index = 0 if side == -1 else -1
    if face["type"] == "periodic":
        index = -1 if side == -1 else 0
    pf = np.take(p, index, axis=axis + 1)
    gf = np.take(gamma, index, axis=axis)
    qf = [np.take(q, index, axis=axis) for q in fractions]
    if face["type"] != "periodic":
        pf, gf, qf = ghost(pf, gf, qf, face, d, side, c["reactive"])
    return pf, gf, qf


def padded(p, gamma, fractions, c, faces, d):
    """Primitives, gamma and fractions with one boundary plane on each side."""
    axis = c["dimension"] - 1 - d
    lo = boundary_plane(p, gamma, fractions, c, faces, d, -1)
    hi = boundary_plane(p, gamma, fractions, c, faces, d, 1)
    pp = np.concatenate((np.expand_dims(lo[0], axis + 1), p,
                         np.expand_dims(hi[0], axis + 1)), axis=axis + 1)
    gg = np.concatenate((np.expand_dims(lo[1], axis), gamma, np.expand_dims(hi[1], axis)),
                        axis=axis)
    qq = [np.concatenate((np.expand_dims(a, axis), q, np.expand_dims(b, axis)), axis=axis)
          for q, a, b in zip(fractions, lo[2], hi[2])]
    return pp, gg, qq


def _pairs(a, axis):
    lo = [slice(None)] * a.ndim
    hi = list(lo)
    lo[axis], hi[axis] = slice(None, -1), slice(1, None)
    return a[tuple(lo)], a[tuple(hi)]


# -- reconstruction, flux and update (torchFiniteVolume.py:16-276) -------------
def primitive(state, gamma):
    p = state.copy()
    p[1:-1] /= state[0]
    p[-1] = (gamma - 1) * (state[-1] - 0.5 * np.sum(state[1:-1] ** 2, axis=0) / state[0])
    return p


def conservative(p, gamma):
    u = p.copy()
    u[1:-1] *= p[0]
    u[-1] = p[-1] / (gamma - 1) + 0.5 * p[0] * np.sum(p[1:-1] ** 2, axis=0)
    return u


def limited(minus, plus, name):
    r = minus / np.where(abs(plus) < 1e-14, 1e-14, plus)
    pos = np.maximum(r, 0.0)
    if name == "VanLeer":
        phi = 2 * pos / (1 + pos)
    elif name == "Albada":
        phi = (pos * pos + pos) / (pos * pos + 1)
    elif name == "MINBEE":
        phi = np.maximum(0, np.minimum(r, 1))
    elif name == "Superbee":
        phi = np.maximum(0, np.maximum(np.minimum(2 * r, 1), np.minimum(r, 2)))
    else:  # Unos
        phi = np.maximum(0, np.minimum(np.minimum(2, 2 * r),
                                       np.minimum((2 + r) / 3, (1 + 2 * r) / 3)))
    return phi * plus


def _gamma_field(c, fractions, shape):
    return np.broadcast_to(fv.gamma_of_lambda(fractions[0]) if c["reactive"] else c["gamma"],
                           shape)


def rusanov(left, right, gl, gr, d):
    """Rusanov flux along direction d from primitive face states, in the
    reference's buffer-reuse order (torchFiniteVolume.py:187-207)."""
    ul, ur = conservative(left, gl), conservative(right, gr)
    fl, fr = ul * left[d + 1], ur * right[d + 1]
    fl[d + 1] += left[-1]
    fr[d + 1] += right[-1]
    fl[-1] += left[d + 1] * left[-1]
    fr[-1] += right[d + 1] * right[-1]
    speed = np.maximum(abs(left[d + 1]) + np.sqrt(gl * left[-1] / left[0]),
                       abs(right[d + 1]) + np.sqrt(gr * right[-1] / right[0]))
    ur -= ul
    ur *= speed[None]
    fl += fr
    fl -= ur
    fl *= 0.5
    return fl


def rhs(state, fractions, c, metric, faces, first_order=False):
    """(d state/dt, d(rho q)/dt per fraction, outward face integral, source
    integral) of one stage."""
    dim = c["dimension"]
    gamma = _gamma_field(c, fractions, state.shape[1:])
    p = primitive(state, gamma)
    source = metric.source(p)
    change = source.copy()
    species = [np.zeros_like(q) for q in fractions]
    outward = np.zeros(dim + 2)
    for d, area in enumerate(metric.areas):
        axis = dim - 1 - d
        pp, gg, qq = padded(p, gamma, fractions, c, faces, d)
        slope = np.zeros_like(pp)
        mid = [slice(None)] * (dim + 1)
        mid[axis + 1] = slice(1, -1)
        lo, hi = list(mid), list(mid)
        lo[axis + 1], hi[axis + 1] = slice(None, -2), slice(2, None)
        if not first_order:
            slope[tuple(mid)] = limited(pp[tuple(mid)] - pp[tuple(lo)],
                                        pp[tuple(hi)] - pp[tuple(mid)], c["limiter"])
            bad = np.any((pp[[0, -1]] - 0.5 * abs(slope[[0, -1]])) <= 1e-12, axis=0)
            slope *= (~bad)[None]
            if faces[2 * d]["type"] == "periodic":
                for target, src in ((0, -2), (-1, 1)):
                    sl = [slice(None)] * (dim + 1)
                    sl[axis + 1] = target
                    slope[tuple(sl)] = np.take(slope, src, axis=axis + 1)
        pl, pr = _pairs(pp, axis + 1)
        sl, sr = _pairs(slope, axis + 1)
        left, right = pl + 0.5 * sl, pr - 0.5 * sr
        gl, gr = _pairs(gg, axis)
        gl, gr = gl.copy(), gr.copy()
        for end, side in ((0, 0), (-1, 1)):
            if faces[2 * d + side]["type"] != "wall":
                continue
            idx = [slice(None)] * (dim + 1)
            idx[axis + 1] = end
            sidx = tuple(idx[1:])
            if side == 0:
                left[tuple(idx)] = right[tuple(idx)]
                gl[sidx] = gr[sidx]
                idx[0] = d + 1
                left[tuple(idx)] *= -1
            else:
                right[tuple(idx)] = left[tuple(idx)]
                gr[sidx] = gl[sidx]
                idx[0] = d + 1
                right[tuple(idx)] *= -1
        flux = rusanov(left, right, gl, gr, d)
        weighted = flux * area[None]
        change -= np.diff(weighted, axis=axis + 1) / metric.volumes[None]
        outward += (np.take(weighted, -1, axis=axis + 1)
                    - np.take(weighted, 0, axis=axis + 1)).reshape(dim + 2, -1).sum(axis=1)
        for j, q in enumerate(qq):
            ql, qr = _pairs(q, axis)
            transport = flux[0] * np.where(flux[0] >= 0, ql, qr) * area
            species[j] -= np.diff(transport, axis=axis) / metric.volumes
    integrated = (source * metric.volumes[None]).reshape(dim + 2, -1).sum(axis=1)
    return change, species, outward, integrated


def advance(state, lam, beta, dt, c, metric, faces):
    """SSPRK2 with a first-order retry (torchFiniteVolume.py:234-276).
    Returns (state, lam, beta, boundary integral, source integral, used
    first order)."""
    fractions = [q for q in (lam, beta) if q is not None]
    for first_order in (False, True):
        conserved = [state[0] * q for q in fractions]
        k1, q1, b1, s1 = rhs(state, fractions, c, metric, faces, first_order)
        stage = state + dt * k1
        if not fv.physical(stage):
            continue
        stage_q = [(q + dt * k) / stage[0] for q, k in zip(conserved, q1)]
        if any(np.any((q < -1e-12) | (q > 1 + 1e-12)) for q in stage_q):
            continue
        stage_q = [np.clip(q, 0, 1) for q in stage_q]
        k2, q2, b2, s2 = rhs(stage, stage_q, c, metric, faces, first_order)
        result = 0.5 * (state + stage + dt * k2)
        if not fv.physical(result):
            continue
        final_q = [(0.5 * (q + stage[0] * f + dt * k)) / result[0]
                   for q, f, k in zip(conserved, stage_q, q2)]
        if any(np.any((q < -1e-12) | (q > 1 + 1e-12)) for q in final_q):
            continue
        final_q = [np.clip(q, 0, 1) for q in final_q]
        return (result, final_q[0] if final_q else None,
                final_q[1] if len(final_q) > 1 else None,
                0.5 * dt * (b1 + b2), 0.5 * dt * (s1 + s2), first_order)
    raise RuntimeError("Metric/face update lost positivity; reduce CFL")


def cfl_dt(state, lam, c, metric, faces):
    """CFL / max over cells of sum_d max(area * face speed)/volume
    (torchFiniteVolume.py:74-102)."""
    dim = c["dimension"]
    gamma = np.broadcast_to(fv.gamma_of_lambda(lam) if c["reactive"] else c["gamma"],
                            state.shape[1:])
    p = primitive(state, gamma)
    sound = np.sqrt(gamma * p[-1] / p[0])
    rate = np.zeros(state.shape[1:])
    for d, area in enumerate(metric.areas):
        axis = dim - 1 - d
        speed = abs(p[d + 1]) + sound
        face_speed = np.empty_like(area)
        mid = [slice(None)] * dim
        mid[axis] = slice(1, -1)
        face_speed[tuple(mid)] = np.maximum(*_pairs(speed, axis))
        for index, side in ((0, -1), (-1, 1)):
            pf, gf, _ = boundary_plane(p, gamma, [], c, faces, d, side)
            edge = [slice(None)] * dim
            edge[axis] = index
            face_speed[tuple(edge)] = np.maximum(np.take(speed, index, axis=axis),
                                                 abs(pf[d + 1]) + np.sqrt(gf * pf[-1] / pf[0]))
        rate += np.maximum(*_pairs(area * face_speed, axis)) / metric.volumes
    return c["cfl"] / np.max(rate)


class OracleMetricSimulation:
    """The reference session's metric branch (torchSession.py:523-576) over
    this module: dt from cfl_dt, Strang-split reaction halves around the
    SSPRK2 hydro step, up to 20 dt halvings."""

    def __init__(self, primitive_init, lengths, *, t_end, cfl=0.4, gamma=1.4, limiter="VanLeer",
                 reactive=False, kinetic_model="arrhenius", lambda_init=None, beta_init=None,
                 geometry="cartesian", origins=None, faces=None, max_steps=100000):
        p0 = np.array(primitive_init, dtype=float)
        dim = p0.ndim - 1
        self.config = dict(dimension=dim, counts_xyz=list(p0.shape[1:][::-1]),
                           lengths_xyz=[float(v) for v in np.atleast_1d(lengths)],
                           t_end=t_end, cfl=cfl, gamma=gamma, limiter=limiter,
                           reactive=bool(reactive), kinetic_model=kinetic_model,
                           max_steps=max_steps, geometry=geometry,
                           origins_xyz=list(np.atleast_1d(origins)) if origins is not None
                           else [0.0] * dim)
        self.faces = faces
        self.metric = Metric(self.config)
        shape = p0.shape[1:]
        self.lam = (np.ones(shape) if lambda_init is None else np.array(lambda_init, float)) \
            if reactive else None
        self.beta = (np.ones(shape) if beta_init is None else np.array(beta_init, float)) \
            if reactive and kinetic_model == "znd" else None
        self.chem = dict(fv.SI_CHEMISTRY)
        self.state = conservative(p0, self.gamma)
        self.time, self.steps, self.fallback_steps = 0.0, 0, 0
        self.initial_integral = self.integral.copy()
        self.boundary_integral = np.zeros(dim + 2)
        self.source_integral = np.zeros(dim + 2)

    @property
    def gamma(self):
        return fv.gamma_of_lambda(self.lam) if self.config["reactive"] else self.config["gamma"]

    @property
    def integral(self):
        """torchSession.py:284-294: Cartesian grids use sums times the cell
        volume, metric grids per-cell volumes."""
        c = self.config
        d = c["dimension"]
        if c["geometry"] == "cartesian":
            h = np.array(c["lengths_xyz"]) / c["counts_xyz"]
            return self.state.reshape(d + 2, -1).sum(axis=1) * np.prod(h)
        return (self.state * self.metric.volumes[None]).reshape(d + 2, -1).sum(axis=1)

    @property
    def completed(self):
        return self.time == self.config["t_end"]

    def _reaction(self, state, lam, beta, dt):
        model = self.config["kinetic_model"]
        kw = dict(self.chem, closure="si", gamma=self.config["gamma"])
        if self.config["dimension"] == 1:
            lam, state, beta = fv.react_1d(lam, dt, state, model, beta, **kw)
            return state, lam, beta if model == "znd" else None
        return fv.reaction_nd(state, lam, beta, dt, model, **kw)

    def step(self):
        if self.completed:
            return
        c = self.config
        if self.steps >= c["max_steps"]:
            raise RuntimeError("Maximum steps reached before requested final time")
        start = self.state
        dt = min(cfl_dt(start, self.lam, c, self.metric, self.faces), c["t_end"] - self.time)
        for _ in range(20):
            if not np.isfinite(dt) or dt <= 0 or self.time + dt == self.time:
                raise RuntimeError("Integration stalled before requested final time")
            old, lam, beta = start, self.lam, self.beta
            if c["reactive"]:
                old, lam, beta = self._reaction(start, self.lam, self.beta, dt / 2)
                allowed = cfl_dt(old, lam, c, self.metric, self.faces)
                if dt > allowed * (1 + 1e-12):
                    dt = min(dt / 2, allowed)
                    continue
            try:
                hydro, lam, beta, boundary, source, used = advance(
                    old, lam, beta, dt, c, self.metric, self.faces)
            except RuntimeError:
                dt /= 2
                continue
            state = hydro
            if c["reactive"]:
                state, lam, beta = self._reaction(hydro, lam, beta, dt / 2)
                source += ((old - start + state - hydro) * self.metric.volumes[None]).reshape(
                    c["dimension"] + 2, -1).sum(axis=1)
            if not fv.physical(state):
                raise RuntimeError("Reaction produced a nonphysical state")
            self.state, self.lam, self.beta = state, lam, beta
            self.boundary_integral += boundary
            self.source_integral += source
            self.time = min(self.time + dt, c["t_end"])
            self.steps += 1
            self.fallback_steps += int(used)
            self.last_dt = dt
            return
        raise RuntimeError("Could not find a positive metric/face step")
