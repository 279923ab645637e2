"""Generate golden vectors by running the TORCH reference itself.

Run where the reference source tree is available, naming its root (the
directory that holds ``python/cfdSolver``) with ``--reference`` or
``$TORCH_REFERENCE``:

    python tests/golden/make_golden.py --reference PATH [checkpoint|metric|rusanov|output|adaptive]

The reference package ``cfdSolver`` imports matplotlib at package level, so it
is loaded through a bare namespace module whose ``__path__`` points at the
source directory; the solver modules themselves need only NumPy.  Every case
uses small seeded inputs.  Outputs go to ``tests/golden/*.npz`` next to this
script and are committed; tests read them without the reference.
"""

import json
import os
import sys
import types
import importlib
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent
REF = None  # <reference root>/python, set by main()


def load_reference():
    pkg = types.ModuleType("cfdSolver")
    pkg.__path__ = [str(REF / "cfdSolver")]
    sys.modules["cfdSolver"] = pkg
    names = ("torchSolver", "torchSolver2D", "torchSolver3D", "torchFlux",
             "torchSession", "torchExecution")
    return types.SimpleNamespace(**{n: importlib.import_module("cfdSolver." + n)
                                    for n in names})


LIMITERS = ("VanLeer", "Albada", "MINBEE", "Superbee", "Unos")


def blob_primitive(rng, dim, shape, jump=True):
    """Seeded smooth field plus a discontinuous blob, positive rho and p."""
    coords = np.meshgrid(*[(np.arange(n) + 0.5) / n for n in shape], indexing="ij")
    r2 = sum((c - 0.45) ** 2 for c in coords)
    p = np.empty((dim + 2,) + shape)
    p[0] = 1.0 + 0.3 * rng.random(shape)
    for m in range(1, dim + 1):
        p[m] = 0.4 * (rng.random(shape) - 0.5)
    p[-1] = 1.0 + 0.3 * rng.random(shape)
    if jump:
        inside = r2 <= 0.3 ** 2
        p[0] = np.where(inside, p[0] * 4.0, p[0])
        p[-1] = np.where(inside, p[-1] * 6.0, p[-1])
    return p


def hllc_cases(R, rng):
    out = {}
    for nv in (4, 5):
        n = 1500
        p_l = np.empty((nv, n))
        p_r = np.empty((nv, n))
        for p in (p_l, p_r):
            p[0] = 0.05 + 3 * rng.random(n)
            p[1:-1] = 4 * (rng.random((nv - 2, n)) - 0.5)
            p[-1] = 0.01 + 5 * rng.random(n)
        # identical states, contacts and strong shocks
        p_r[:, :100] = p_l[:, :100]
        p_r[1, 100:200] = p_l[1, 100:200]
        p_r[-1, 100:200] = p_l[-1, 100:200]
        p_l[-1, 200:300] *= 1e4
        gl = 1.15 + 0.3 * rng.random(n)
        gr = np.where(rng.random(n) < 0.5, gl, 1.15 + 0.3 * rng.random(n))
        cons = []
        for p, g in ((p_l, gl), (p_r, gr)):
            u = p.copy()
            u[1:-1] *= p[0]
            u[-1] = p[-1] / (g - 1) + 0.5 * p[0] * np.sum(p[1:-1] ** 2, axis=0)
            cons.append(u)
        out[f"ul{nv}"], out[f"ur{nv}"] = cons
        out[f"gl{nv}"], out[f"gr{nv}"] = gl, gr
        out[f"flux{nv}"] = R.torchFlux.hllc_flux(cons[0], cons[1], gl, gamma_right=gr)
    np.savez_compressed(OUT / "hllc.npz", **out)


def step3d_cases(R, rng):
    out = {}
    bc_sets = [("Open", "Open", "Open"), ("Reflective", "Periodic", "Open"),
               ("Periodic", "Reflective", "Reflective")]
    k = 0
    for limiter in LIMITERS:
        for bcs in bc_sets:
            shape = (5, 6, 7)  # nz, ny, nx
            prim = blob_primitive(rng, 3, shape)
            gamma = 1.4 if k % 2 == 0 else 1.2 + 0.2 * rng.random(shape)
            state = R.torchSolver3D.uprim_to_uconsv_3d(prim, gamma)
            h = (1 / 7, 1.3 / 6, 0.9 / 5)
            dt = 0.2 * min(h) / 4.0
            res, fluxes = R.torchSolver3D._hydro(state, gamma, h, dt, limiter, bcs[::-1])
            out[f"c{k}_state"] = state
            out[f"c{k}_gamma"] = np.broadcast_to(gamma, shape).copy()
            out[f"c{k}_meta"] = np.array([*h, dt])
            out[f"c{k}_limiter"] = np.array(limiter)
            out[f"c{k}_bcs"] = np.array(bcs)
            out[f"c{k}_result"] = res
            for d, f in enumerate(fluxes):
                out[f"c{k}_flux{d}"] = f
            k += 1
    # rough seeded field: the second-order step is nonphysical, so the whole
    # step is redone at first order (Rusanov)
    shape = (4, 4, 6)
    p = np.empty((5,) + shape)
    p[0] = 10 ** rng.uniform(-3, 1, shape)
    p[1:4] = rng.uniform(-3, 3, (3,) + shape)
    p[4] = 10 ** rng.uniform(-4, 1, shape)
    state = R.torchSolver3D.uprim_to_uconsv_3d(p)
    h = (1 / 6, 1 / 4, 1 / 4)
    q = R.torchSolver3D.uconsv_to_uprim_3d(state)
    sound = np.sqrt(1.4 * q[4] / q[0])
    dt = 0.4 / sum(np.max(abs(q[m]) + sound) / d for m, d in enumerate(h, 1))
    res, fluxes = R.torchSolver3D._hydro(state, 1.4, h, dt, "Superbee",
                                         ("Reflective", "Periodic", "Open"))
    out[f"c{k}_state"] = state
    out[f"c{k}_gamma"] = np.full(state.shape[1:], 1.4)
    out[f"c{k}_meta"] = np.array([*h, dt])
    out[f"c{k}_limiter"] = np.array("Superbee")
    out[f"c{k}_bcs"] = np.array(("Open", "Periodic", "Reflective"))
    out[f"c{k}_result"] = res
    for d, f in enumerate(fluxes):
        out[f"c{k}_flux{d}"] = f
    out["count"] = np.array(k + 1)
    np.savez_compressed(OUT / "step3d.npz", **out)


def step2d_cases(R, rng):
    out = {}
    bc_sets = [("Open", "Open"), ("Reflective", "Periodic"), ("Periodic", "Reflective"),
               ("Open", "Inflow")]
    k = 0
    for limiter in LIMITERS:
        for bc_x, bc_y in bc_sets:
            shape = (9, 11)
            prim = blob_primitive(rng, 2, shape)
            gamma = 1.4 if k % 2 == 0 else 1.2 + 0.2 * rng.random(shape)
            state = R.torchSolver2D.uprim_to_uconsv_2d(prim, gamma)
            dx, dy = 1 / 11, 1.2 / 9
            dt = 0.05 * min(dx, dy)
            inlet = [1.1, 0.1, 0.6, 1.3]
            res, fx, fy = R.torchSolver2D.muscl_hancock_step_2d(
                state, dx, dy, dt, gamma, limiter, bc_x, bc_y, return_fluxes=True,
                inlet_primitive=inlet)
            out[f"c{k}_state"] = state
            out[f"c{k}_gamma"] = np.broadcast_to(gamma, shape).copy()
            out[f"c{k}_meta"] = np.array([dx, dy, dt])
            out[f"c{k}_limiter"] = np.array(limiter)
            out[f"c{k}_bcs"] = np.array((bc_x, bc_y))
            out[f"c{k}_inlet"] = np.array(inlet)
            out[f"c{k}_result"] = res
            out[f"c{k}_flux0"] = fx
            out[f"c{k}_flux1"] = fy
            k += 1
    # rough seeded field whose second-order update is nonphysical: the step is
    # redone with the first-order LLF fluxes
    shape = (6, 8)
    p = np.empty((4,) + shape)
    p[0] = 10 ** rng.uniform(-3, 1, shape)
    p[1:3] = rng.uniform(-3, 3, (2,) + shape)
    p[3] = 10 ** rng.uniform(-4, 1, shape)
    state = R.torchSolver2D.uprim_to_uconsv_2d(p, 1.4)
    dx, dy = 1 / 8, 1 / 6
    padded = R.torchSolver2D.apply_boundary_conditions_2d(state, "Open", "Reflective")
    gp = R.torchSolver2D.pad_scalar_2d(np.full(shape, 1.4), "Open", "Reflective", 1.4)
    dt = R.torchSolver2D.compute_cfl_dt_2d(
        R.torchSolver2D.uconsv_to_uprim_2d(padded, gp), dx, dy, 0.4, gp)
    res, fx, fy = R.torchSolver2D.muscl_hancock_step_2d(
        state, dx, dy, dt, 1.4, "Superbee", "Open", "Reflective", return_fluxes=True)
    out[f"c{k}_state"] = state
    out[f"c{k}_gamma"] = np.full(state.shape[1:], 1.4)
    out[f"c{k}_meta"] = np.array([dx, dy, dt])
    out[f"c{k}_limiter"] = np.array("Superbee")
    out[f"c{k}_bcs"] = np.array(("Open", "Reflective"))
    out[f"c{k}_inlet"] = np.array([1.0, 0.0, 100.0, 101325.0])
    out[f"c{k}_result"] = res
    out[f"c{k}_flux0"] = fx
    out[f"c{k}_flux1"] = fy
    out["count"] = np.array(k + 1)
    np.savez_compressed(OUT / "step2d.npz", **out)


def chemistry_cases(R, rng):
    out = {}
    n = 500
    for model in ("arrhenius", "znd"):
        lam = rng.random(n)
        beta = rng.random(n)
        rho = 0.5 + rng.random(n)
        u = 100 * (rng.random(n) - 0.5)
        p = 101325 * (1 + 40 * rng.random(n))
        g = R.torchSolver.gamma_calc(lam)
        state = np.vstack((rho, rho * u, p / (g - 1) + 0.5 * rho * u * u))
        dt = 2e-6
        lam_new, st, beta_new = R.torchSolver.new_lambda_n_e_calc(lam, dt, state, model, beta)
        out[f"{model}_lam"], out[f"{model}_beta"], out[f"{model}_state"] = lam, beta, state
        out[f"{model}_out_lam"], out[f"{model}_out_state"] = lam_new, st
        out[f"{model}_out_beta"] = beta_new
    out["dt"] = np.array(2e-6)
    # 3D reaction step
    shape = (3, 4, 5)
    prim = np.empty((5,) + shape)
    prim[0] = 0.5 + rng.random(shape)
    prim[1:4] = 50 * (rng.random((3,) + shape) - 0.5)
    prim[4] = 101325 * (1 + 20 * rng.random(shape))
    lam = rng.random(shape)
    beta = rng.random(shape)
    state = R.torchSolver3D.uprim_to_uconsv_3d(prim, R.torchSolver.gamma_calc(lam))
    res, l3, b3 = R.torchSolver3D.reaction_step_3d(state, lam, beta, 3e-6, "znd")
    out.update(r3_state=state, r3_lam=lam, r3_beta=beta, r3_out=res, r3_out_lam=l3,
               r3_out_beta=b3)
    np.savez_compressed(OUT / "chemistry.npz", **out)


def session_setups(R):
    """The session cases of sessions.npz and checkpoint.npz, freshly built."""
    S = R.torchSession.Simulation
    cases = {}
    cases["s2d_explosion"] = S.preset("2d_explosion", [24, 20], t_end=0.05,
                                      limiter="VanLeer")
    p3 = R.torchSolver3D.get_3d_preset("3d_explosion", 10, 9, 8)["primitive"]
    cases["s3d_explosion"] = S(p3, [1, 1, 1], t_end=0.05, limiter="Superbee",
                               boundaries=["Reflective"] * 3)
    cases["s3d_open_albada"] = S(p3, [1.0, 0.9, 0.8], t_end=0.02, limiter="Albada",
                                 boundaries=["Open", "Periodic", "Reflective"])
    p1 = np.empty((3, 64))
    p1[:, :32] = np.array([1.0, 0.0, 1.0])[:, None]
    p1[:, 32:] = np.array([0.125, 0.0, 0.1])[:, None]
    cases["s1d_sod"] = S(p1, [1.0], t_end=0.1, limiter="VanLeer")
    cases["s1d_sod_superbee_reflective"] = S(p1, [1.0], t_end=0.05, limiter="Superbee",
                                             boundaries=["Reflective"])
    # reactive 3D (SI kinetics): ignition preset on a tiny grid
    pi = R.torchSolver3D.get_3d_preset("3d_ignition", 6, 5, 4)["primitive"]
    cases["s3d_ignition_znd"] = S(pi, [1, 1, 1], t_end=2e-6, reactive=True,
                                  kinetic_model="znd", limiter="VanLeer")
    cases["s3d_ignition_arr"] = S(pi, [1, 1, 1], t_end=2e-6, reactive=True,
                                  kinetic_model="arrhenius", limiter="MINBEE",
                                  boundaries=["Reflective", "Open", "Periodic"])
    p2 = np.ones((4, 10, 12))
    p2[1:3] = 0.0
    p2[3] = np.where(np.arange(12) < 6, 3e6, 101325.0)[None, :]
    cases["s2d_reactive"] = S(p2, [1, 1], t_end=1e-6, reactive=True, limiter="Superbee",
                              boundaries=["Periodic", "Inflow"],
                              inlet_primitive=[1.0, 0.0, 100.0, 101325.0])
    p1r = np.empty((3, 40))
    p1r[:, :20] = np.array([1.0, 0.0, 5e6])[:, None]
    p1r[:, 20:] = np.array([0.5, 0.0, 101325.0])[:, None]
    cases["s1d_reactive_znd"] = S(p1r, [1.0], t_end=2e-6, reactive=True,
                                  kinetic_model="znd")
    return cases


def session_cases(R, rng):
    """Multi-step Simulation.step() trajectories (state, time, integrals)."""
    out = {}
    cases = session_setups(R)
    for name, s in cases.items():
        out[f"{name}_state0"] = s.state.copy()
        if s.lam is not None:
            out[f"{name}_lam0"] = s.lam.copy()
        if s.beta is not None:
            out[f"{name}_beta0"] = s.beta.copy()
        for _ in range(8):
            if s.completed:
                break
            s.step()
        out[f"{name}_state"] = s.state
        if s.lam is not None:
            out[f"{name}_lam"] = s.lam
        if s.beta is not None:
            out[f"{name}_beta"] = s.beta
        out[f"{name}_scalars"] = np.array([s.time, s.steps])
        out[f"{name}_boundary"] = s.boundary_integral
        out[f"{name}_source"] = s.source_integral
        out[f"{name}_initial"] = s.initial_integral
    np.savez_compressed(OUT / "sessions.npz", **out)


class _RecordingHDF5(types.ModuleType):
    """Stand-in for h5py (absent here) under the reference's checkpoint writer
    and reader: datasets are kept as NumPy arrays in an .npz container, so the
    reference's own write_checkpoint / read_checkpoint run unchanged."""

    class File:
        def __init__(self, path, mode="r"):
            self.path, self.mode = Path(path), mode
            self.data = {}
            if mode == "r":
                with np.load(self.path) as z:
                    self.data = {k.replace("|", "/"): z[k] for k in z.files}

        def __enter__(self):
            return self

        def __exit__(self, *exc):
            if self.mode == "w" and exc[0] is None:
                with open(self.path, "wb") as f:
                    np.savez(f, **{k.replace("/", "|"): v for k, v in self.data.items()})

        def create_dataset(self, name, data, **options):
            self.data[name] = np.array(data)

        def flush(self):
            pass

        def __getitem__(self, name):
            if name in self.data:
                return self.data[name]
            prefix = name + "/"
            members = [k[len(prefix):] for k in self.data if k.startswith(prefix)]
            if not members:
                raise KeyError(name)
            return members


def checkpoint_cases(R):
    """Reference checkpoints taken after 4 steps (write_checkpoint's metadata
    bytes and datasets), accepted by the reference's read_checkpoint, and the
    reference's state after 4 more steps from there."""
    import tempfile
    sys.modules["h5py"] = _RecordingHDF5("h5py")
    io = importlib.import_module("cfdSolver.torchIO")
    cases = session_setups(R)
    metric = metric_setups(R)
    for name in ("m2d_cylindrical_origin", "m3d_cartesian_faces", "m2d_spherical_reactive"):
        cases[name] = metric[name]
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name in ("s3d_explosion", "s3d_open_albada", "s2d_explosion", "s1d_sod",
                     "s3d_ignition_znd", "s3d_ignition_arr", "s2d_reactive",
                     "s1d_reactive_znd", "m2d_cylindrical_origin", "m3d_cartesian_faces",
                     "m2d_spherical_reactive"):
            s = cases[name]
            # a later end time so that all 8 steps run (the session reads it each step)
            s.config["t_end"] = 1e-3 if s.config["reactive"] else 1.0
            for _ in range(4):
                s.step()
            path = Path(tmp) / (name + ".h5")
            io.write_checkpoint(path, s)
            with _RecordingHDF5.File(path) as f:
                for key, value in f.data.items():
                    out[f"{name}|{key}"] = value
            back = io.read_checkpoint(path)
            assert back.steps == s.steps == 4 and np.array_equal(back.state, s.state)
            for _ in range(4):
                back.step()
            out[f"{name}|final/state"] = back.state
            for key in ("lam", "beta"):
                if getattr(back, key) is not None:
                    out[f"{name}|final/{key}"] = getattr(back, key)
            out[f"{name}|final/scalars"] = np.array([back.time, back.steps])
            out[f"{name}|final/initial"] = back.initial_integral
            out[f"{name}|final/boundary"] = back.boundary_integral
            out[f"{name}|final/source"] = back.source_integral
    np.savez_compressed(OUT / "checkpoint.npz", **out)


def metric_setups(R):
    """Metric / face-boundary sessions: every geometry and dimension with the
    inflow / pressure-outlet faces of python/tests/testGeometry.py:27-65, and
    walls at radial origins and poles, a stagnation inlet, a full periodic
    azimuth, all limiters, reactive shells."""
    S = R.torchSession.Simulation
    limiters = ("VanLeer", "Albada", "MINBEE", "Superbee", "Unos")
    cases = {}

    def centres(origin, lengths, counts):
        c = [o + (np.arange(n) + 0.5) * l / n for o, l, n in zip(origin, lengths, counts)]
        return np.meshgrid(*c[::-1], indexing="ij")[::-1]

    k = 0
    for dim in (1, 2, 3):
        for geometry in ("cartesian", "cylindrical", "annular", "spherical"):
            for reactive in (False, True):
                if reactive and geometry in ("cartesian", "cylindrical"):
                    continue
                counts = [12, 6, 4][:dim]
                origin = [0.4, 0.3, 0.2][:dim] if geometry != "cartesian" else [0.1] * dim
                lengths = [0.8, 0.6, 0.4][:dim]
                g = centres(origin, lengths, counts)
                p = np.ones((dim + 2, *counts[::-1]))
                p[0] = 1 + 0.05 * np.sin(3 * g[0])
                if dim > 1:
                    p[0] += 0.03 * np.cos(2 * g[1])
                if dim == 3:
                    p[0] += 0.01 * g[2]
                p[1:-1] = 0.15
                p[-1] = np.where(g[0] < 0.8, 1e6, 101325.0) if reactive else 1.0 + 0.3 * (g[0] < 0.8)
                pr = 101325.0 if reactive else 1.0
                faces = {
                    "x_min": {"type": "inflow",
                              "primitive": [1.0, 0.15] + [0.15] * (dim - 1) + [pr]},
                    "x_max": {"type": "pressure_outlet", "pressure": pr,
                              "backflow": [1.0, -0.1] + [0.0] * (dim - 1) + [pr]},
                }
                name = f"m{dim}d_{geometry}" + ("_reactive" if reactive else "")
                model = "znd" if reactive and dim != 2 else "arrhenius"
                cases[name] = S(p, lengths, geometry=geometry, origins=origin,
                                t_end=2e-5 if reactive else 0.025, reactive=reactive,
                                kinetic_model=model, limiter=limiters[k % 5],
                                face_boundaries=faces)
                k += 1
    # radial origin (default wall) and both spherical poles, at rest with a pressure bump
    for dim, geometry in ((2, "cylindrical"), (2, "spherical"), (1, "spherical")):
        counts = [10, 8][:dim]
        lengths = [1.0, np.pi][:dim]
        g = centres([0.0] * dim, lengths, counts)
        p = np.ones((dim + 2, *counts[::-1]))
        p[1:-1] = 0.0
        p[-1] = 1.0 + 0.5 * np.exp(-10 * (g[0] - 0.5) ** 2)
        cases[f"m{dim}d_{geometry}_origin"] = S(p, lengths, geometry=geometry,
                                                 origins=[0.0] * dim, t_end=0.05,
                                                 limiter="Superbee")
    # full periodic azimuth, stagnation inlet inside, subsonic outlet outside
    counts = [12, 16]
    g = centres([0.5, 0.0], [1.0, 2 * np.pi], counts)
    p = np.ones((4, *counts[::-1]))
    p[1] = 0.1
    p[2] = 0.2 * np.sin(g[1])
    p[3] = 1.0 - 0.05 * g[0]
    cases["m2d_annular_stagnation"] = S(
        p, [1.0, 2 * np.pi], geometry="annular", origins=[0.5, 0.0], t_end=0.05,
        limiter="Albada", boundaries=["Open", "Periodic"],
        face_boundaries={"x_min": {"type": "stagnation_inlet", "total_pressure": 1.2,
                                   "total_temperature": 1.2 / 287.0},
                         "x_max": {"type": "pressure_outlet", "pressure": 0.9}})
    # Cartesian 3D with a wall, periodic pair and outflow faces
    counts = [8, 6, 5]
    g = centres([0.0] * 3, [1.0] * 3, counts)
    p = np.ones((5, *counts[::-1]))
    p[0] += 0.2 * np.sin(2 * np.pi * g[1])
    p[1] = 0.3
    p[2] = -0.2
    p[3] = 0.1
    p[4] = 1 + 0.5 * (g[0] < 0.5)
    cases["m3d_cartesian_faces"] = S(
        p, [1.0] * 3, t_end=0.05, limiter="Unos", boundaries=["Open", "Periodic", "Open"],
        face_boundaries={"x_min": "wall", "z_max": "wall"})
    return cases


def metric_cases(R):
    """Reference metric / face-boundary sessions: one-stage right-hand sides
    (second and first order) and cfl_dt at the initial state, then a few
    complete steps (state, composition, times, balances)."""
    fvm = importlib.import_module("cfdSolver.torchFiniteVolume")
    out = {}
    for name, s in metric_setups(R).items():
        c = s.config
        out[f"{name}|config"] = np.frombuffer(json.dumps(c).encode(), dtype=np.uint8)
        out[f"{name}|state0"] = s.state.copy()
        fractions = [q for q in (s.lam, s.beta) if q is not None]
        for q, key in zip(fractions, ("lam0", "beta0")):
            out[f"{name}|{key}"] = q.copy()
        out[f"{name}|dt0"] = np.array([fvm.cfl_dt(s.state, s.lam, c, s.metrics)])
        for order in (0, 1):
            change, species, outward, source = fvm.rhs(s.state, fractions, c, s.metrics,
                                                       first_order=bool(order))
            out[f"{name}|rhs{order}/change"] = change
            for j, sp in enumerate(species):
                out[f"{name}|rhs{order}/species{j}"] = sp
            out[f"{name}|rhs{order}/outward"] = outward
            out[f"{name}|rhs{order}/source"] = source
        times = []
        for _ in range(4):
            if s.completed:
                break
            s.step()
            times.append(s.time)
        out[f"{name}|times"] = np.array(times)
        out[f"{name}|state"] = s.state
        if s.lam is not None:
            out[f"{name}|lam"] = s.lam
        if s.beta is not None:
            out[f"{name}|beta"] = s.beta
        out[f"{name}|initial"] = s.initial_integral
        out[f"{name}|boundary"] = s.boundary_integral
        out[f"{name}|source"] = s.source_integral
    np.savez_compressed(OUT / "metric.npz", **out)


def rusanov_cases(R):
    """The reference's rusanov_flux (torchFlux.py:80-99) on seeded random
    faces in 1D/2D/3D along every direction with per-face gamma, and the
    leaf-face batches an adaptive session hands to it (torchAdaptive.py:
    115-135), recorded from two steps of a refined 2D cylindrical blast."""
    flux = importlib.import_module("cfdSolver.torchFlux")
    rng = np.random.default_rng(11)
    out = {}
    for dim in (1, 2, 3):
        nv = dim + 2
        for d in range(dim):
            n = 256
            left = np.empty((nv, n))
            right = np.empty((nv, n))
            for a in (left, right):
                a[0] = 10 ** rng.uniform(-2, 1, n)
                a[1:-1] = rng.uniform(-3, 3, (dim, n))
                a[-1] = 10 ** rng.uniform(-2, 2, n)
            gl = rng.uniform(1.1, 1.67, n)
            gr = rng.uniform(1.1, 1.67, n)
            key = f"random{dim}d_dir{d}"
            out[f"{key}|left"], out[f"{key}|right"] = left, right
            out[f"{key}|gl"], out[f"{key}|gr"] = gl, gr
            out[f"{key}|flux"] = flux.rusanov_flux(left, right, gl, gr, d)
    adaptive = importlib.import_module("cfdSolver.torchAdaptive")
    S = R.torchSession.Simulation
    counts = [12, 8]
    p = np.ones((4, *counts[::-1]))
    p[1:-1] = 0.0
    r = 0.2 + (np.arange(counts[0]) + 0.5) / counts[0]
    p[-1] = np.where(r < 0.5, 4.0, 1.0)[None, :]
    s = S(p, [1.0, 1.0], geometry="cylindrical", origins=[0.2, 0.0], t_end=0.05)
    a = s.to_adaptive(max_level=2)
    a.regrid(refine=a.mesh.centers[:, 0] < 0.7, coarsen=False)
    calls = []
    original = adaptive.rusanov

    def recording(left, right, gl, gr, k):
        value = original(left, right, gl, gr, k)
        calls.append((left.copy(), right.copy(), np.array(gl, copy=True),
                      np.array(gr, copy=True), k, value))
        return value

    adaptive.rusanov = recording
    try:
        for _ in range(2):
            a.step()
    finally:
        adaptive.rusanov = original
    for i, (left, right, gl, gr, k, value) in enumerate(calls[:4]):
        key = f"amr{i}"
        out[f"{key}|left"], out[f"{key}|right"] = left, right
        out[f"{key}|gl"], out[f"{key}|gr"] = gl, gr
        out[f"{key}|dir"] = np.array([k])
        out[f"{key}|flux"] = value
    np.savez_compressed(OUT / "rusanov.npz", **out)


def adaptive_sessions(S):
    """The two adaptive sessions of the adaptive trajectories (also built by
    tests/test_gpu_adaptive.py): a 2D Cartesian explosion on a 32^2 root grid
    with two refinement levels, and the refined 2D cylindrical blast of the
    leaf-face batches above."""
    n = 32
    c = (np.arange(n) + 0.5) / n
    Y, X = np.meshgrid(c, c, indexing="ij")
    inside = (X - 0.5) ** 2 + (Y - 0.5) ** 2 <= 0.2 ** 2
    p = np.zeros((4, n, n))
    p[0] = np.where(inside, 1.0, 0.125)
    p[3] = np.where(inside, 1.0, 0.1)
    explosion = S(p, [1.0, 1.0], t_end=0.2).to_adaptive(max_level=2)
    counts = [12, 8]
    q = np.ones((4, *counts[::-1]))
    q[1:-1] = 0.0
    r = 0.2 + (np.arange(counts[0]) + 0.5) / counts[0]
    q[-1] = np.where(r < 0.5, 4.0, 1.0)[None, :]
    s = S(q, [1.0, 1.0], geometry="cylindrical", origins=[0.2, 0.0], t_end=0.05)
    blast = s.to_adaptive(max_level=2)
    blast.regrid(refine=blast.mesh.centers[:, 0] < 0.7, coarsen=False)
    return {"explosion2d": (explosion, 8), "cylindrical_blast": (blast, 4)}


def adaptive_cases(R):
    """Trajectories of the reference's AdaptiveSimulation (torchAdaptive.py:
    346-492) with its own CPU Rusanov fluxes: every step's time, leaf count
    and boundary integral, and the final leaf keys and state."""
    out = {}
    for name, (a, steps) in adaptive_sessions(R.torchSession.Simulation).items():
        times, leaves, bnd = [], [], []
        for _ in range(steps):
            a.step()
            times.append(a.time)
            leaves.append(len(a.mesh.keys))
            bnd.append(a.boundary_integral.copy())
        out[f"{name}|time"] = np.array(times)
        out[f"{name}|leaves"] = np.array(leaves)
        out[f"{name}|boundary"] = np.array(bnd)
        out[f"{name}|keys"] = np.array(a.mesh.keys)
        out[f"{name}|state"] = a.state
        out[f"{name}|steps"] = np.array([a.steps])
    np.savez_compressed(OUT / "adaptive.npz", **out)


def output_cases(R):
    """The reference's field output (torchIO.py:122-733): VTK rectilinear and
    structured snapshots, XDMF snapshots with their HDF5 heavy data, and the
    temporal series (frames, .pvd, .xdmf, manifest) of short runs.  Every
    file is recorded as bytes (HDF5 files as their datasets), with the session
    attributes at each frame, so the GPU session's writers can be compared
    byte for byte."""
    import tempfile
    sys.modules["h5py"] = _RecordingHDF5("h5py")
    io = importlib.import_module("cfdSolver.torchIO")
    S = R.torchSession.Simulation
    out = {}

    def snap(key, s):
        out[f"{key}|state"] = s.state.copy()
        for name in ("lam", "beta"):
            if getattr(s, name) is not None:
                out[f"{key}|{name}"] = getattr(s, name).copy()
        out[f"{key}|scalars"] = np.array([s.time, s.steps])
        out[f"{key}|integrals"] = np.stack((s.initial_integral, s.boundary_integral,
                                            s.source_integral))
        out[f"{key}|config"] = np.frombuffer(json.dumps(s.config).encode(), dtype=np.uint8)
        out[f"{key}|run_id"] = np.frombuffer(s.run_id.encode(), dtype=np.uint8)

    def files(key, folder):
        for f in sorted(Path(folder).iterdir()):
            if f.suffix == ".h5":
                with _RecordingHDF5.File(f) as h:
                    for name, value in h.data.items():
                        out[f"{key}|file/{f.name}/{name}"] = value
            else:
                out[f"{key}|file/{f.name}"] = np.frombuffer(f.read_bytes(), dtype=np.uint8)

    rng = np.random.default_rng(5)
    p2 = np.ones((4, 4, 6))
    p2[0] += 0.3 * rng.random((4, 6))
    p2[1:3] = 0.1 * rng.standard_normal((2, 4, 6))
    p2[3] += rng.random((4, 6))
    cases = {
        "vtr2d": S(p2, [1.0, 0.8], t_end=0.05, limiter="MINBEE"),
        "vts2d_znd": S(np.stack((p2[0], p2[1], p2[2], 1e5 * p2[3])), [1.0, 1.0],
                       geometry="spherical", origins=[0.5, 0.5], t_end=2e-5, reactive=True,
                       kinetic_model="znd"),
    }
    p1 = np.ones((3, 7))
    p1[0] += np.linspace(0, 0.5, 7)
    cases["vtr1d"] = S(p1, [1.0], t_end=0.05)
    p3 = np.ones((5, 3, 4, 5))
    p3[1] = 0.2
    cases["vts3d_annular"] = S(p3, [1.0, 1.0, 0.5], geometry="annular",
                               origins=[0.5, 0.0, 0.0], t_end=0.05)
    with tempfile.TemporaryDirectory() as tmp:
        for key, s in cases.items():
            folder = Path(tmp) / key
            folder.mkdir()
            recorded = []
            original = io.TemporalWriter.append

            def append(self, session, _orig=original, _rec=recorded):
                _rec.append(len(_rec))
                snap(f"{key}/frame{len(_rec) - 1}", session)
                return _orig(self, session)

            io.TemporalWriter.append = append
            try:
                s.run(step_limit=3, output_prefix=folder / "series", output_every=2,
                      formats=("vtk",) if key.startswith("vts2d") else ("vtk", "xdmf"))
            finally:
                io.TemporalWriter.append = original
            out[f"{key}|frames"] = np.array([len(recorded)])
            single = Path(tmp) / (key + "_single")
            single.mkdir()
            snap(f"{key}/single", s)
            io.write_vtk(single / ("snap" + (".vts" if "vts" in key else ".vtr")), s)
            io.write_xdmf(single / "snap.xdmf", s)
            files(f"{key}/series", folder)
            files(f"{key}/single", single)
    np.savez_compressed(OUT / "output.npz", **out)


def large_cfl_case(R):
    """2D explosion at CFL 0.8 (rejected by Simulation): dt from the session
    formula, step function called directly, 12 steps on a 40x40 grid."""
    two = R.torchSolver2D
    n = 40
    x = (np.arange(n) + 0.5) * 2.0 / n
    X, Y = np.meshgrid(x, x)
    inside = np.hypot(X - 1, Y - 1) <= 0.4
    prim = np.stack((np.where(inside, 1.0, 0.125), 0 * X, 0 * X, np.where(inside, 1.0, 0.1)))
    state = prim.copy()
    state[1:-1] *= prim[0]
    state[-1] = prim[-1] / 0.4 + 0.5 * prim[0] * np.sum(prim[1:-1] ** 2, axis=0)
    h = (2.0 / n, 2.0 / n)
    out = dict(state0=state.copy())
    dts = []
    for _ in range(12):
        padded = two.apply_boundary_conditions_2d(state, "Open", "Open")
        gp = two.pad_scalar_2d(np.broadcast_to(1.4, state.shape[1:]), "Open", "Open", 1.4)
        dt = two.compute_cfl_dt_2d(two.uconsv_to_uprim_2d(padded, gp), *h, 0.8, gp)
        state = two.muscl_hancock_step_2d(state, *h, dt, 1.4, "VanLeer", "Open", "Open")
        dts.append(dt)
    out.update(state=state, dts=np.array(dts))
    np.savez_compressed(OUT / "cfl08_2d.npz", **out)


def exact_riemann_cases():
    """The reference's exact Riemann solver (torchAnalysis.exact_riemann_sod)
    on Sod and on shock / rarefaction pairs with nonzero velocities.  The
    module imports matplotlib at top level; a stub module stands in for it."""
    for name in ("matplotlib", "matplotlib.pyplot"):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["matplotlib"].use = lambda *a, **k: None
    analysis = importlib.import_module("cfdSolver.torchAnalysis")
    cases = {
        "sod": dict(),
        "sod_t02": dict(t=0.2),
        "strong": dict(t=0.012, rho_l=1.0, u_l=0.0, p_l=1000.0, rho_r=1.0, u_r=0.0, p_r=0.01),
        "two_rarefactions": dict(t=0.15, rho_l=1.0, u_l=-2.0, p_l=0.4, rho_r=1.0, u_r=2.0,
                                 p_r=0.4),
        "collision": dict(t=0.035, rho_l=5.99924, u_l=19.5975, p_l=460.894, rho_r=5.99242,
                          u_r=-6.19633, p_r=46.095, x0=0.4),
    }
    out = {}
    x = (np.arange(200) + 0.5) / 200
    for name, kw in cases.items():
        kw = dict(kw)
        kw.setdefault("t", 0.08)
        rho, u, p = analysis.exact_riemann_sod(x, **kw)
        out[f"{name}_x"] = x
        out[f"{name}_rho"], out[f"{name}_u"], out[f"{name}_p"] = rho, u, p
        out[f"{name}_args"] = np.array([kw.get(k, d) for k, d in (
            ("t", 0.2), ("x0", 0.5), ("gamma", 1.4), ("rho_l", 1.0), ("u_l", 0.0),
            ("p_l", 1.0), ("rho_r", 0.125), ("u_r", 0.0), ("p_r", 0.1))])
    np.savez_compressed(OUT / "exact_riemann.npz", **out)


def main():
    import argparse

    global REF
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--reference", default=os.environ.get("TORCH_REFERENCE"),
                    help="root of the TORCH source tree (default: $TORCH_REFERENCE)")
    ap.add_argument("case", nargs="?",
                    choices=["checkpoint", "metric", "rusanov", "output", "adaptive"],
                    help="regenerate this fixture alone")
    args = ap.parse_args()
    if not args.reference:
        ap.error("name the reference source tree with --reference or $TORCH_REFERENCE")
    REF = Path(args.reference) / "python"
    if not (REF / "cfdSolver").is_dir():
        ap.error(f"{REF / 'cfdSolver'} is not a directory")
    R = load_reference()
    single = {"checkpoint": checkpoint_cases, "metric": metric_cases,
              "rusanov": rusanov_cases, "output": output_cases,
              "adaptive": adaptive_cases}
    if args.case:
        single[args.case](R)
        return
    rng = np.random.default_rng(20261203)
    hllc_cases(R, rng)
    step3d_cases(R, rng)
    step2d_cases(R, rng)
    chemistry_cases(R, rng)
    session_cases(R, rng)
    large_cfl_case(R)
    exact_riemann_cases()
    checkpoint_cases(R)
    metric_cases(R)
    rusanov_cases(R)
    output_cases(R)
    adaptive_cases(R)
    for f in sorted(OUT.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
