"""Host-side session logic (validation, conversions) — no GPU needed: every
check here raises before device memory is touched."""

import numpy as np
import pytest

from torch_gb300.session import Simulation, prim_to_cons, _physical
from oracle import fv


def uniform(shape=(4, 4, 4)):
    p = np.ones((len(shape) + 2,) + shape)
    p[1:-1] = 0.1
    return p


@pytest.mark.parametrize("kw,match", [
    (dict(cfl=0.6), "CFL"),                       # torchSolver.py:1080 rejects CFL > 0.5
    (dict(limiter="bad"), "limiter"),
    (dict(gamma=1.0), "gamma"),
    (dict(boundaries=["Open", "Inflow", "Open"]), "boundary"),
    (dict(max_steps=0), "maximum steps"),
    (dict(max_steps=True), "maximum steps"),
    (dict(t_end=-1.0), "final time"),
])
def test_session_validation_matches_reference(kw, match):
    args = dict(t_end=0.1)
    args.update(kw)
    with pytest.raises(ValueError, match=match):
        Simulation(uniform(), [1, 1, 1], **args)


def test_bad_primitives_and_shapes():
    p = uniform()
    p[0, 0, 0, 0] = -1.0
    with pytest.raises(ValueError):
        Simulation(p, [1, 1, 1], t_end=0.1)
    with pytest.raises(ValueError):
        Simulation(uniform(), [1, 1], t_end=0.1)
    with pytest.raises(ValueError):
        Simulation(np.ones((3, 4, 4)), [1, 1], t_end=0.1)
    with pytest.raises(ValueError, match="Inlet|inlet"):
        Simulation(uniform((6, 6)), [1, 1], t_end=0.1, boundaries=["Open", "Inflow"],
                   inlet_primitive=[1.0, 0.0, -1.0, 1.0])


def test_large_cfl_needs_explicit_opt_in():
    with pytest.raises(ValueError):
        Simulation(uniform((6, 6)), [1, 1], t_end=0.1, cfl=0.8)


def test_conversion_matches_oracle_bitwise():
    rng = np.random.default_rng(3)
    p = 0.5 + rng.random((5, 3, 4, 5))
    np.testing.assert_array_equal(prim_to_cons(p, 1.4), fv.prim_to_cons(p, 1.4))
    assert _physical(prim_to_cons(p, 1.4)) == fv.physical(fv.prim_to_cons(p, 1.4))


def test_served_request_stream_mix_and_determinism():
    from torch_gb300.serve import served_requests

    a = served_requests(rate=100.0, count=400, seed=7)
    b = served_requests(rate=100.0, count=400, seed=7)
    assert [(r.dim, r.n, r.arrival) for r in a] == [(r.dim, r.n, r.arrival) for r in b]
    dims = np.array([r.dim for r in a])
    assert abs(np.mean(dims == 1) - 0.4) < 0.08 and abs(np.mean(dims == 3) - 0.2) < 0.06
    assert all(1e3 <= r.n <= 1e5 for r in a if r.dim == 1)
    assert all(128 <= r.n <= 1024 for r in a if r.dim == 2)
    assert all(64 <= r.n <= 256 for r in a if r.dim == 3)
    assert all(0.1 <= r.t_end <= 0.3 for r in a)
    gaps = np.diff([0.0] + [r.arrival for r in a])
    assert abs(gaps.mean() - 0.01) < 0.002  # Poisson at 100 requests/s
    p = a[0].primitive()
    assert p.shape[0] == a[0].dim + 2 and np.all(p[0] > 0) and np.all(p[-1] > 0)
