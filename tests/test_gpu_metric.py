"""GPU parity of the metric / face-boundary session step against the
reference's own sessions (tests/golden/metric.npz: cylindrical, annular,
spherical and Cartesian grids in 1D/2D/3D with inflow, pressure-outlet,
stagnation-inlet, wall and periodic faces, all limiters, reactive shells) and
against the oracle (oracle/metric.py) for the paths the golden cases do not
reach: first-order retries, dt halving, boundary errors.

Tolerances, stated per case: double precision is bitwise where no boundary
state needs pow; the pressure outlet and the stagnation inlet call pow, whose
CUDA rounding may differ from the C library's in the last bit, so those cases
are compared at a relative 1e-11; reactive cases at 1e-10 (exp, as in the
Cartesian reactive tests).  Single precision: L1 density error against double
precision below 1e-5."""

import json
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import torch_gb300  # noqa: E402
from oracle import fv  # noqa: E402
from oracle import metric as M  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden"


def golden():
    g = np.load(GOLDEN / "metric.npz")
    names = sorted({k.split("|")[0] for k in g.files})
    return g, names


G, NAMES = golden()


def uses_pow(config):
    return any(f["type"] in ("pressure_outlet", "stagnation_inlet")
               for f in config["face_boundaries"])


def start(name, **options):
    c = json.loads(bytes(G[f"{name}|config"]).decode())
    lam = G[f"{name}|lam0"] if f"{name}|lam0" in G.files else None
    beta = G[f"{name}|beta0"] if f"{name}|beta0" in G.files else None
    dim = c["dimension"]
    snap = SimpleNamespace(config=c, state=G[f"{name}|state0"], lam=lam, beta=beta, time=0.0,
                           steps=0, initial_integral=G[f"{name}|initial"],
                           boundary_integral=np.zeros(dim + 2),
                           source_integral=np.zeros(dim + 2), run_id="golden")
    return torch_gb300.Simulation.from_session(snap, **options), c


@pytest.mark.parametrize("name", NAMES)
def test_metric_sessions_match_reference(name):
    sim, c = start(name)
    assert sim.uses_metric_kernel
    times = G[f"{name}|times"]
    got = []
    for _ in range(len(times)):
        sim.step()
        got.append(sim.time)
    if c["reactive"]:
        rtol = 1e-10
    elif uses_pow(c):
        rtol = 1e-11
    else:
        rtol = 0.0
    state = G[f"{name}|state"]
    if rtol == 0.0:
        np.testing.assert_array_equal(got, times)
        np.testing.assert_array_equal(sim.state, state)
    else:
        np.testing.assert_allclose(got, times, rtol=rtol, atol=0)
        np.testing.assert_allclose(sim.state, state, rtol=rtol, atol=rtol * np.abs(state).max())
    for key in ("lam", "beta"):
        if f"{name}|{key}" in G.files:
            np.testing.assert_allclose(getattr(sim, key), G[f"{name}|{key}"], rtol=1e-10,
                                       atol=1e-13)
    scale = max(1.0, np.abs(G[f"{name}|initial"]).max())
    np.testing.assert_allclose(sim.boundary_integral, G[f"{name}|boundary"], rtol=1e-9,
                               atol=1e-12 * scale)
    np.testing.assert_allclose(sim.source_integral, G[f"{name}|source"], rtol=1e-9,
                               atol=1e-12 * scale)
    np.testing.assert_array_equal(sim.initial_integral, G[f"{name}|initial"])
    assert sim.steps == len(times)


def oracle_pair(p, lengths, faces_spec=None, **kw):
    sim = torch_gb300.Simulation(p, lengths, face_boundaries=faces_spec, **kw)
    c = sim.config
    ref = M.OracleMetricSimulation(
        p, lengths, t_end=c["t_end"], cfl=c["cfl"], gamma=c["gamma"], limiter=c["limiter"],
        reactive=c["reactive"], kinetic_model=c["kinetic_model"],
        lambda_init=kw.get("lambda_init"), beta_init=kw.get("beta_init"),
        geometry=c["geometry"], origins=c["origins_xyz"], faces=c["face_boundaries"])
    ref.state = sim.state.copy()  # the conversion from primitives is the session's
    ref.initial_integral = ref.integral.copy()
    return sim, ref


def test_first_order_retry_matches_oracle():
    """A rough spherical shell whose second-order stages lose positivity:
    the GPU takes the same first-order retries as the oracle."""
    rng = np.random.default_rng(3)
    shape = (6, 10)
    p = np.empty((4,) + shape)
    p[0] = 10 ** rng.uniform(-3, 1, shape)
    p[1:3] = rng.uniform(-4, 4, (2,) + shape)
    p[3] = 10 ** rng.uniform(-4, 1, shape)
    sim, ref = oracle_pair(p, [1.0, 1.0], geometry="spherical", origins=[0.5, 0.8], t_end=1.0,
                           limiter="Superbee", cfl=0.5)
    for _ in range(6):
        ref.step()
        sim.step()
        np.testing.assert_array_equal(sim.state, ref.state)
        assert sim.time == ref.time
    assert ref.fallback_steps > 0 and sim.fallback_steps == ref.fallback_steps


def test_periodic_annulus_and_walls_match_oracle_bitwise():
    n = (16, 8)
    r = 0.5 + (np.arange(n[1]) + 0.5) / n[1]
    th = (np.arange(n[0]) + 0.5) * 2 * np.pi / n[0]
    R, T = np.meshgrid(r, th, indexing="xy")
    p = np.stack((1 + 0.2 * np.cos(T), 0.1 * np.sin(T), 0.3 + 0 * R, 1 + 0.1 * R))
    for lim in ("VanLeer", "Albada", "MINBEE", "Superbee", "Unos"):
        sim, ref = oracle_pair(p, [1.0, 2 * np.pi], geometry="annular", origins=[0.5, 0.0],
                               t_end=0.2, limiter=lim, boundaries=["Reflective", "Periodic"])
        for _ in range(5):
            ref.step()
            sim.step()
        np.testing.assert_array_equal(sim.state, ref.state, err_msg=lim)
        assert sim.time == ref.time


def test_boundary_errors_raise_value_error_and_keep_the_state():
    p = np.ones((3, 16))
    p[1] = -3.0  # strong outflow through the inlet face
    sim = torch_gb300.Simulation(
        p, [1.0], t_end=0.1, geometry="cylindrical", origins=[0.5],
        face_boundaries={"x_min": {"type": "stagnation_inlet", "total_pressure": 1.0,
                                   "total_temperature": 1.0 / 287.0}})
    before = sim.state
    with pytest.raises(ValueError):
        sim.step()
    np.testing.assert_array_equal(sim.state, before)
    assert sim.steps == 0
    q = np.ones((3, 16))
    q[1] = -0.5  # flow entering through a subsonic outlet without a backflow state
    sim = torch_gb300.Simulation(q, [1.0], t_end=0.1, geometry="spherical", origins=[0.5],
                                 face_boundaries={"x_max": {"type": "pressure_outlet",
                                                            "pressure": 1.0}})
    with pytest.raises(ValueError, match="backflow"):
        sim.step()


def test_uniform_rest_preserved_at_radial_origin_and_poles():
    """python/tests/testGeometry.py:112-138."""
    for dim in (1, 2, 3):
        for geometry in ("cartesian", "cylindrical", "annular", "spherical"):
            origin = [0.3] * dim if dim == 3 or geometry == "annular" else [0.0] * dim
            lengths = ([1.0, np.pi, 0.5][:dim] if geometry == "spherical" and dim < 3
                       else [0.5] * dim)
            p = np.ones((dim + 2, *([6] * dim)))
            p[1:-1] = 0
            s = torch_gb300.Simulation(p, lengths, geometry=geometry, origins=origin, t_end=0.02,
                                       face_boundaries={} if geometry == "cartesian" else None)
            old = s.state.copy()
            s.run()
            np.testing.assert_allclose(s.state, old, rtol=0, atol=3e-14)
            np.testing.assert_allclose(s.balance_residual, 0, atol=3e-14)


def test_fp32_metric_session_tracks_fp64():
    name = "m3d_spherical"
    s64, _ = start(name)
    s32, _ = start(name, precision="fp32")
    for _ in range(4):
        s64.step()
        s32.step()
    assert abs(s32.time - s64.time) <= 1e-6 * s64.time
    assert np.mean(np.abs(s32.state[0] - s64.state[0])) < 1e-5
    assert np.max(np.abs(s32.balance_residual)) < 1e-5 * np.abs(s32.initial_integral).max()


def test_metric_checkpoint_restart_is_exact(fake_h5py, tmp_path):
    name = "m2d_annular_reactive"
    continuous, _ = start(name)
    continuous.run(step_limit=4)
    a, _ = start(name)
    a.run(step_limit=2, checkpoint=tmp_path / "c.h5")
    b = torch_gb300.Simulation.load(tmp_path / "c.h5").run(step_limit=2)
    for key in ("state", "lam", "boundary_integral", "source_integral"):
        np.testing.assert_array_equal(getattr(b, key), getattr(continuous, key))
    assert (b.steps, b.time) == (continuous.steps, continuous.time)


def test_inflow_and_pressure_outlet_on_every_face():
    """A uniform stream entering through an inflow face and leaving through
    a pressure outlet stays uniform (python/tests/testGeometry.py:341-380)."""
    for dim in (1, 2, 3):
        for direction in range(dim):
            for side in (-1, 1):
                p = np.ones((dim + 2, *([5] * dim)))
                p[1:-1] = 0
                p[direction + 1] = -side * 0.2
                values = [1.0] + [0.0] * dim + [1.0]
                values[direction + 1] = -side * 0.2
                faces = {a + edge: "periodic" for a in "xyz"[:dim] for edge in ("_min", "_max")}
                axis = "xyz"[direction]
                faces[axis + ("_min" if side == -1 else "_max")] = dict(
                    type="inflow", primitive=values, **{"lambda": 0.6})
                faces[axis + ("_max" if side == -1 else "_min")] = dict(
                    type="pressure_outlet", pressure=1.0)
                for reactive in (False, True):
                    s = torch_gb300.Simulation(
                        p, [1.0] * dim, t_end=0.02, face_boundaries=faces, reactive=reactive,
                        lambda_init=np.full(p.shape[1:], 0.6) if reactive else None)
                    initial = s.state.copy()
                    s.run()
                    np.testing.assert_allclose(s.state, initial, atol=1e-14, rtol=1e-14)
                    np.testing.assert_allclose(s.balance_residual, 0, atol=1e-13)


def test_metric_max_steps_raise_and_keep_the_state():
    sim, _ = start("m2d_cylindrical_origin", max_steps=2)
    sim.step()
    sim.step()
    before, time = sim.state, sim.time
    with pytest.raises(RuntimeError, match="Maximum steps"):
        sim.step()
    np.testing.assert_array_equal(sim.state, before)
    assert sim.time == time and sim.steps == 2


def test_reactive_metric_fp32_tracks_fp64():
    name = "m3d_spherical_reactive"
    s64, _ = start(name)
    s32, _ = start(name, precision="fp32")
    for _ in range(3):
        s64.step()
        s32.step()
    rel = np.abs(s32.state - s64.state) / np.abs(s64.state).max(axis=(1, 2, 3))[:, None, None, None]
    assert rel.mean() < 1e-5
    assert np.mean(np.abs(s32.lam - s64.lam)) < 1e-5
    assert abs(s32.time - s64.time) <= 1e-5 * s64.time
