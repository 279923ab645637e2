"""Metric / face-boundary path on the host: the oracle (oracle/metric.py) is
pinned bit for bit to the reference's own sessions (tests/golden/metric.npz:
one-stage right-hand sides at second and first order, the CFL dt, and four
complete steps), the product's host logic (geometry factors, face
normalisation, validation) reproduces the reference's configuration, and the
configurations the reference rejects are rejected
(python/tests/testGeometry.py:520-552)."""

import json
from pathlib import Path

import numpy as np
import pytest

from oracle import fv
from oracle import metric as M
from torch_gb300 import metric, session

GOLDEN = Path(__file__).resolve().parent / "golden"
G = np.load(GOLDEN / "metric.npz")
NAMES = sorted({k.split("|")[0] for k in G.files})


def config(name):
    return json.loads(bytes(G[f"{name}|config"]).decode())


def fractions(name):
    return [G[f"{name}|{k}"] for k in ("lam0", "beta0") if f"{name}|{k}" in G.files]


@pytest.mark.parametrize("name", NAMES)
def test_oracle_rhs_and_dt_match_reference(name):
    c = config(name)
    met = M.Metric(c)
    state = G[f"{name}|state0"]
    fr = fractions(name)
    assert M.cfl_dt(state, fr[0] if fr else None, c, met, c["face_boundaries"]) == \
        G[f"{name}|dt0"][0]
    for order in (0, 1):
        change, species, outward, source = M.rhs(state, fr, c, met, c["face_boundaries"],
                                                 bool(order))
        np.testing.assert_array_equal(change, G[f"{name}|rhs{order}/change"])
        for j, sp in enumerate(species):
            np.testing.assert_array_equal(sp, G[f"{name}|rhs{order}/species{j}"])
        np.testing.assert_array_equal(outward, G[f"{name}|rhs{order}/outward"])
        np.testing.assert_array_equal(source, G[f"{name}|rhs{order}/source"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_sessions_match_reference(name):
    c = config(name)
    fr = fractions(name)
    lam0 = fr[0] if fr else None
    beta0 = fr[1] if len(fr) > 1 else None
    gamma = fv.gamma_of_lambda(lam0) if c["reactive"] else c["gamma"]
    state0 = G[f"{name}|state0"]
    s = M.OracleMetricSimulation(
        M.primitive(state0, gamma), c["lengths_xyz"], t_end=c["t_end"], cfl=c["cfl"],
        gamma=c["gamma"], limiter=c["limiter"], reactive=c["reactive"],
        kinetic_model=c["kinetic_model"], lambda_init=lam0, beta_init=beta0,
        geometry=c["geometry"], origins=c["origins_xyz"], faces=c["face_boundaries"])
    s.state = state0.copy()
    s.initial_integral = s.integral.copy()
    times = []
    for _ in range(len(G[f"{name}|times"])):
        s.step()
        times.append(s.time)
    np.testing.assert_array_equal(times, G[f"{name}|times"])
    np.testing.assert_array_equal(s.state, G[f"{name}|state"])
    if lam0 is not None:
        np.testing.assert_array_equal(s.lam, G[f"{name}|lam"])
    if beta0 is not None:
        np.testing.assert_array_equal(s.beta, G[f"{name}|beta"])
    np.testing.assert_array_equal(s.initial_integral, G[f"{name}|initial"])
    np.testing.assert_array_equal(s.source_integral, G[f"{name}|source"])
    np.testing.assert_allclose(s.boundary_integral, G[f"{name}|boundary"], rtol=1e-12,
                               atol=1e-15)


@pytest.mark.parametrize("name", NAMES)
def test_host_logic_reproduces_reference_configuration(name):
    c = config(name)
    mine = dict(c)
    session.validate_config(mine)
    assert mine["face_boundaries"] == c["face_boundaries"]
    vol, face = metric.factors(c)
    ov, of = M.factors(c)
    for a, b in zip(vol, ov):
        np.testing.assert_array_equal(a, b)
    for fa, fb in zip(face, of):
        for a, b in zip(fa, fb):
            np.testing.assert_array_equal(a, b)
    flat = metric.flat_factors(c)
    dim = c["dimension"]
    n = c["counts_xyz"]
    assert flat.size == sum(n[:dim]) + sum(n[a] + (a == d) for d in range(dim)
                                           for a in range(dim))


def test_invalid_geometries_and_incomplete_boundaries_rejected():
    import torch_gb300
    p = np.ones((4, 4, 4))
    p[1:-1] = 0
    for opts in (
        dict(geometry="unknown"),
        dict(geometry="annular"),
        dict(geometry="spherical", lengths=[1.0, 4.0]),
        dict(face_boundaries={"x_min": "periodic"}),
        dict(face_boundaries={"bad": "wall"}),
        dict(face_boundaries={"x_min": {"type": "inflow", "primitive": [1.0, -1.0, 0.0, 1.0]}}),
        dict(geometry="annular", origins=[0.5, 0.0], lengths=[1.0, 2 * np.pi],
             face_boundaries={"x_min": "periodic", "x_max": "periodic"}),
        dict(geometry="annular", origins=[0.5, 0.0], lengths=[1.0, 3.0],
             boundaries=["Open", "Periodic"]),
        dict(face_boundaries={"x_max": {"type": "pressure_outlet"}}),
        dict(face_boundaries={"x_min": {"type": "wall", "pressure": 1.0}}),
        dict(geometry="cylindrical", controller="w=0"),
    ):
        kwargs = dict(opts)
        lengths = kwargs.pop("lengths", [1.0, 1.0])
        with pytest.raises(ValueError):
            torch_gb300.Simulation(p, lengths, t_end=0.01, **kwargs)
    p3 = np.ones((5, 4, 4, 4))
    p3[1:-1] = 0
    for geo in ("spherical", "cylindrical"):
        with pytest.raises(ValueError):
            torch_gb300.Simulation(p3, [1.0, 1.0, 1.0], geometry=geo, t_end=0.01)


def test_default_walls_at_origin_and_poles():
    c = dict(dimension=2, counts_xyz=[4, 4], lengths_xyz=[1.0, np.pi], boundaries_xyz=["Open"] * 2,
             geometry="spherical", origins_xyz=[0.0, 0.0], inlet_primitive=[1, 0, 100, 101325])
    faces = metric.normalize_faces(c, metric.default_face_spec(c, None))
    assert [f["type"] for f in faces] == ["wall", "outflow", "wall", "wall"]
    faces = metric.normalize_faces(c, metric.default_face_spec(c, {"x_max": "wall"}))
    assert [f["type"] for f in faces] == ["wall", "wall", "wall", "wall"]
    with pytest.raises(ValueError, match="pole"):
        metric.normalize_faces(c, {"y_min": "outflow", "x_min": "wall"})
