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
