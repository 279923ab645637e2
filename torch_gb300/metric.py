"""Metric / face-boundary sessions on the GPU (host side).

TORCH runs a second finite-volume scheme for cylindrical, annular and
spherical grids and for any grid with per-face boundaries
(python/cfdSolver/torchSession.py:303-308, 523-576): MUSCL reconstruction of
primitives with limited slopes, area-weighted Rusanov fluxes, geometric
source terms, SSPRK2 with a first-order retry and Strang-split chemistry
(python/cfdSolver/torchFiniteVolume.py).  This module holds its host logic:

* geometry checks and the one-dimensional metric factors whose outer
  products are the cell volumes and face areas
  (python/cfdSolver/torchGeometry.py:45-170), computed with the same NumPy
  operations so the GPU sees the reference's exact factors;
* face-boundary normalisation and validation
  (python/cfdSolver/torchBoundaries.py:18-171);
* ``MetricEngine``: the ctypes handle of ``tfv_metric_*`` with its state
  slots and workspace, exposing the interface the session uses.
"""

import ctypes as C

import numpy as np
import torch

from . import _lib

GEOMETRIES = ("cartesian", "cylindrical", "annular", "spherical")
TYPES = ("outflow", "wall", "periodic", "inflow", "pressure_outlet", "stagnation_inlet")


# -- geometry (torchGeometry.py:34-93) ------------------------------------------
def axes(c):
    dim = c["dimension"]
    return [np.linspace(o, o + l, n + 1) for o, l, n in
            zip(c.get("origins_xyz", [0.0] * dim), c["lengths_xyz"], c["counts_xyz"])]


def validate_geometry(c):
    dim, g = c["dimension"], c.get("geometry", "cartesian")
    if g not in GEOMETRIES:
        raise ValueError("Unknown geometry")
    origin = np.asarray(c.get("origins_xyz", [0.0] * dim), dtype=float)
    if origin.shape != (dim,) or not np.isfinite(origin).all():
        raise ValueError("One finite origin per logical coordinate is required")
    if g == "cartesian":
        return
    if origin[0] < 0 or (g == "annular" and origin[0] <= 0):
        raise ValueError("Radius must be nonnegative; an annulus needs a positive inner radius")
    if g == "cylindrical" and dim == 3 and origin[0] == 0:
        raise ValueError("3D cylindrical grids require a positive inner radius")
    if g == "spherical" and dim >= 2:
        if origin[1] < 0 or origin[1] + c["lengths_xyz"][1] > np.pi + 1e-14:
            raise ValueError("Spherical theta must lie in [0, pi]")
        if dim == 3 and (origin[0] == 0 or origin[1] <= 0
                         or origin[1] + c["lengths_xyz"][1] >= np.pi):
            raise ValueError("3D spherical grids require r>0 and 0<theta<pi (shell/wedge)")
    angular = azimuth_axis(c)
    angular = [] if angular is None else [angular]
    if any(c["lengths_xyz"][a] > 2 * np.pi + 1e-14 for a in angular):
        raise ValueError("Azimuthal extent cannot exceed 2*pi")
    if any(c["lengths_xyz"][a] / c["counts_xyz"][a] >= np.pi for a in angular):
        raise ValueError("Azimuthal cells must span less than pi radians")


def azimuth_axis(c):
    dim, g = c["dimension"], c.get("geometry", "cartesian")
    if g == "spherical" and dim == 3:
        return 2
    if (g == "annular" and dim >= 2) or (g == "cylindrical" and dim == 3):
        return 1
    return None


def factors(c):
    """One-dimensional metric factors (x first): the volume factor of each
    axis and, per direction, the face factor of each axis
    (torchGeometry.py:95-170)."""
    dim, g = c["dimension"], c.get("geometry", "cartesian")
    ax = axes(c)
    widths = [np.diff(a) for a in ax]
    n = c["counts_xyz"]
    if g == "cartesian":
        return widths, [[np.ones(n[a] + 1) if a == d else widths[a] for a in range(dim)]
                        for d in range(dim)]
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
        face = [[k * r ** 2, solid] + extra, [k * shell2, np.sin(theta)] + extra]
        if dim == 3:
            face.append([shell2, widths[1], np.ones(n[2] + 1)])
        return [k * shell3, solid] + extra, face
    if dim == 1:
        return [2 * np.pi * shell2], [[2 * np.pi * r]]
    if g == "cylindrical" and dim == 2:
        return ([2 * np.pi * shell2, widths[1]],
                [[2 * np.pi * r, widths[1]], [2 * np.pi * shell2, np.ones(n[1] + 1)]])
    face = [[r, widths[1]] + widths[2:], [dr, np.ones(n[1] + 1)] + widths[2:]]
    if dim == 3:
        face.append([shell2, widths[1], np.ones(n[2] + 1)])
    return [shell2, widths[1]] + widths[2:], face


def flat_factors(c):
    """Factors in the order tfv_metric_create reads them (volume factors of
    each axis, then the face factors of each direction and axis); rejects
    grids whose cell volumes are not finite and positive."""
    vol, face = factors(c)
    dim = c["dimension"]
    out = [np.asarray(v, dtype=float) for v in vol[:dim]]
    for d in range(dim):
        out += [np.asarray(f, dtype=float) for f in face[d][:dim]]
    flat = np.concatenate(out)
    volumes = np.ones(tuple(c["counts_xyz"][::-1]))
    for d, f in enumerate(vol[:dim]):
        shape = [1] * dim
        shape[dim - 1 - d] = len(f)
        volumes = volumes * np.asarray(f).reshape(shape)
    if not np.isfinite(volumes).all() or np.any(volumes <= 0):
        raise ValueError("Invalid cell volumes")
    return flat


# -- face boundaries (torchBoundaries.py:18-171) ---------------------------------
def normalize_faces(c, specification=None, _base=False):
    """One dict per face (x_min, x_max, y_min, ...) with validated parameters."""
    dim = c["dimension"]
    if specification is None:
        kinds = {"Open": "outflow", "Reflective": "wall", "Periodic": "periodic",
                 "Inflow": "inflow"}
        result = []
        for name in c["boundaries_xyz"]:
            kind = kinds[name]
            low = dict(type=kind)
            if kind == "inflow":
                low["primitive"] = list(c["inlet_primitive"])
            result.extend([low, dict(type="outflow") if kind == "inflow" else low.copy()])
    elif isinstance(specification, dict):
        expected = [a + side for a in "xyz"[:dim] for side in ("_min", "_max")]
        if set(specification) - set(expected):
            raise ValueError("Face keys must use logical x_min,x_max,y_min,...")
        result = normalize_faces(c, _base=True)
        for i, name in enumerate(expected):
            if name in specification:
                value = specification[name]
                result[i] = dict(type=value) if isinstance(value, str) else dict(value)
    else:
        result = [dict(v) for v in specification]
    if _base:
        return result
    if len(result) != 2 * dim:
        raise ValueError("Require one boundary per face")
    for i, face in enumerate(result):
        kind = face.get("type")
        if kind not in TYPES:
            raise ValueError("Unknown face boundary type")
        allowed = {"type", "lambda", "beta"}
        if kind == "inflow":
            allowed |= {"primitive"}
        if kind == "pressure_outlet":
            allowed |= {"pressure", "backflow"}
        if kind == "stagnation_inlet":
            allowed |= {"total_pressure", "total_temperature", "gas_constant"}
        if set(face) - allowed:
            raise ValueError("Unknown boundary parameters")
        for key in ("lambda", "beta"):
            value = face.get(key, 1.0)
            if not np.isscalar(value) or not np.isfinite(value) or not 0 <= value <= 1:
                raise ValueError("Boundary fractions must lie in [0,1]")
        for key in ("primitive", "backflow"):
            if key in face:
                p = np.asarray(face[key], dtype=float)
                if p.shape != (dim + 2,) or not np.isfinite(p).all() or np.any(p[[0, -1]] <= 0):
                    raise ValueError("Invalid boundary primitive state")
                sign = -1 if i % 2 == 0 else 1
                if p[i // 2 + 1] * sign >= 0:
                    raise ValueError("Inlet/backflow velocity must point into the domain")
                face[key] = p.tolist()
        if kind == "inflow" and "primitive" not in face:
            raise ValueError("Inflow requires primitive state")
        needed = ({"pressure"} if kind == "pressure_outlet" else
                  {"total_pressure", "total_temperature", "gas_constant"}
                  if kind == "stagnation_inlet" else set())
        for key in needed:
            if key == "gas_constant":
                face.setdefault(key, 287.0)
            if (key not in face or not np.isscalar(face[key]) or not np.isfinite(face[key])
                    or face[key] <= 0):
                raise ValueError("Boundary pressures, temperatures and gas constant must be "
                                 "positive")
    for d in range(dim):
        if (result[2 * d]["type"] == "periodic") != (result[2 * d + 1]["type"] == "periodic"):
            raise ValueError("Periodic boundaries must be paired on an axis")
    g = c.get("geometry", "cartesian")
    origin = c.get("origins_xyz", [0.0] * dim)
    if g != "cartesian":
        if any(f["type"] == "periodic" for f in result[:2]):
            raise ValueError("Radius cannot be periodic")
        if origin[0] == 0 and result[0]["type"] != "wall":
            raise ValueError("The radial origin requires a reflective wall")
        if g == "spherical" and dim >= 2:
            poles = ((2, origin[1] == 0),
                     (3, np.isclose(origin[1] + c["lengths_xyz"][1], np.pi, atol=1e-14, rtol=0)))
            for i, at_pole in poles:
                if at_pole and result[i]["type"] != "wall":
                    raise ValueError("A spherical pole requires a reflective wall")
            if any(f["type"] == "periodic" for f in result[2:4]):
                raise ValueError("Polar theta cannot be periodic")
        a = azimuth_axis(c)
        if a is not None and result[2 * a]["type"] == "periodic" and not np.isclose(
                c["lengths_xyz"][a], 2 * np.pi, atol=1e-14, rtol=0):
            raise ValueError("Azimuthal periodicity requires a complete 2*pi domain")
    return result


def default_face_spec(c, face_boundaries):
    """Walls implied at a radial origin and at spherical poles when the
    session gives only Open boundaries (torchSession.py:96-118)."""
    dim, g = c["dimension"], c["geometry"]
    lengths, origin = c["lengths_xyz"], c["origins_xyz"]
    if (list(c["boundaries_xyz"]) == ["Open"] * dim and g != "cartesian"
            and (face_boundaries is None or isinstance(face_boundaries, dict))):
        provided = face_boundaries or {}
        face_boundaries = {}
        if origin[0] == 0:
            face_boundaries["x_min"] = "wall"
        if g == "spherical" and dim >= 2:
            if origin[1] == 0:
                face_boundaries["y_min"] = "wall"
            if np.isclose(origin[1] + lengths[1], np.pi, rtol=0, atol=1e-14):
                face_boundaries["y_max"] = "wall"
        face_boundaries.update(provided)
    return face_boundaries


def face_structs(faces, dim):
    out = (_lib.MetricFace * 6)()
    for i, face in enumerate(faces):
        f = out[i]
        f.type = _lib.FACE_TYPES[face["type"]]
        state = face.get("primitive", face.get("backflow"))
        f.has_backflow = int("backflow" in face)
        if state is not None:
            for v, value in enumerate(state):
                f.primitive[v] = float(value)
        f.lambda_ = float(face.get("lambda", 1.0))
        f.beta = float(face.get("beta", 1.0))
        f.pressure = float(face.get("pressure", 0.0))
        f.total_pressure = float(face.get("total_pressure", 0.0))
        f.total_temperature = float(face.get("total_temperature", 0.0))
        f.gas_constant = float(face.get("gas_constant", 287.0))
    for i in range(len(faces), 6):
        out[i].type = _lib.FACE_TYPES["outflow"]
    return out


# -- engine ---------------------------------------------------------------------
class MetricEngine:
    """One metric session on the GPU: two state slots (and fraction slots),
    the workspace and the ``tfv_metric`` handle.  Same surface as the
    Cartesian engine the session drives (reports, refresh, advance, current,
    integrals)."""

    def __init__(self, config, faces, state, lam, beta, precision, device, chemistry):
        lib = _lib.load()
        self.lib = lib
        self.n = 1
        c = config
        dim = c["dimension"]
        self.dim = dim
        self.dtype = torch.float64 if precision == "fp64" else torch.float32
        self.device = device
        self.stream = torch.cuda.Stream(device)
        cfg = _lib.MetricConfig()
        cfg.dim = dim
        for a in range(dim):
            cfg.n[a] = int(c["counts_xyz"][a])
            cfg.lengths[a] = float(c["lengths_xyz"][a])
        cfg.geometry = _lib.GEOMETRIES[c["geometry"]]
        cfg.limiter = _lib.LIMITERS[c["limiter"]]
        cfg.reactive = int(bool(c["reactive"]))
        cfg.model = _lib.MODELS[c["kinetic_model"]]
        cfg.cfl, cfg.gamma, cfg.t_end = float(c["cfl"]), float(c["gamma"]), float(c["t_end"])
        cfg.max_steps = int(c["max_steps"])
        cfg.q = float(chemistry["q_heat"])
        cfg.ea = float(chemistry["activation_energy"])
        cfg.a = float(chemistry["pre_exponential"])
        cfg.faces = face_structs(faces, dim)
        flat = np.ascontiguousarray(flat_factors(c), dtype=np.float64)
        if lib.tfv_metric_factor_count(C.byref(cfg)) != flat.size:
            raise RuntimeError("metric factor layout mismatch")
        handle = C.c_void_p()
        _lib.check(lib.tfv_metric_create(_lib.TFV_FP64 if precision == "fp64" else _lib.TFV_FP32,
                                         C.byref(cfg), flat.ctypes.data_as(C.POINTER(C.c_double)),
                                         C.byref(handle)))
        self.handle = handle
        ws = C.c_size_t()
        _lib.check(lib.tfv_metric_workspace_size(handle, C.byref(ws)))
        self.workspace = torch.empty(ws.value + 256, dtype=torch.uint8, device=device)
        self.ws_ptr = self.workspace.data_ptr() + (-self.workspace.data_ptr()) % 256

        def ring(a):
            if a is None:
                return [], None
            first = torch.as_tensor(np.asarray(a), dtype=self.dtype).to(device).contiguous()
            slots = [first, torch.empty_like(first)]
            return slots, (C.c_void_p * 2)(*[t.data_ptr() for t in slots])

        with torch.cuda.stream(self.stream):
            self.rings, sp = ring(state)
            self.lam_rings, lp = ring(lam)
            self.beta_rings, bp = ring(beta)
        self.stream.synchronize()
        self.rings = [self.rings]  # per-instance list, as the Cartesian engine
        _lib.check(lib.tfv_metric_bind(handle, C.c_void_p(self.ws_ptr), sp, lp, bp,
                                       _lib.stream_ptr(self.stream)))
        self.reports = (_lib.Report * 1)()
        self.refresh()

    def advance(self, nsteps):
        _lib.check(self.lib.tfv_metric_advance(self.handle, int(nsteps)))

    def refresh(self):
        _lib.check(self.lib.tfv_metric_report(self.handle, self.reports))
        return self.reports

    def integrals(self):
        out = (C.c_double * 5)()
        _lib.check(self.lib.tfv_metric_integrals(self.handle, out))
        return np.array(out[:]).reshape(1, 5)

    def current(self, i=0):
        return self.rings[0][self.reports[0].current]

    def current_lam(self, i=0):
        return self.lam_rings[self.reports[0].current] if self.lam_rings else None

    def current_beta(self, i=0):
        return self.beta_rings[self.reports[0].current] if self.beta_rings else None

    def replan(self):
        """dt is computed at the start of every metric step: nothing to plan."""
        self.stream.synchronize()
        self.refresh()

    replan_async = replan

    def restore(self, reports):
        _lib.check(self.lib.tfv_metric_restore(self.handle, C.byref(reports[0])))
        self.refresh()

    def use_graph(self, steps):
        """Metric steps synchronise with the host inside each step (dt,
        SSPRK2 stage checks): there is nothing to capture."""

    def close(self):
        if getattr(self, "handle", None):
            self.lib.tfv_metric_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
