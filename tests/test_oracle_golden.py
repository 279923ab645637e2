"""Pin the oracle (NumPy restatement) against vectors produced by the
reference itself (tests/golden/make_golden.py).  CPU only."""

from pathlib import Path

import numpy as np
import pytest

from oracle import fv
from oracle.session import OracleSimulation

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name):
    return np.load(GOLDEN / name, allow_pickle=False)


def test_hllc_bit_exact():
    g = load("hllc.npz")
    for nv in (4, 5):
        got = fv.hllc(g[f"ul{nv}"], g[f"ur{nv}"], g[f"gl{nv}"], g[f"gr{nv}"])
        np.testing.assert_array_equal(got, g[f"flux{nv}"])


def test_step3d_bit_exact_all_limiters_and_boundaries():
    g = load("step3d.npz")
    fallback_seen = False
    for k in range(int(g["count"])):
        hx, hy, hz, dt = g[f"c{k}_meta"]
        res, fluxes, used = fv.hydro_3d(g[f"c{k}_state"], g[f"c{k}_gamma"], (hx, hy, hz),
                                        dt, str(g[f"c{k}_limiter"]),
                                        [str(b) for b in g[f"c{k}_bcs"]])
        fallback_seen |= used
        np.testing.assert_array_equal(res, g[f"c{k}_result"])
        for d in range(3):
            np.testing.assert_array_equal(fluxes[d], g[f"c{k}_flux{d}"])
    assert fallback_seen, "the strong-shock case must exercise the first-order fallback"


def test_step2d_bit_exact_all_limiters_and_boundaries():
    g = load("step2d.npz")
    fallback_seen = False
    for k in range(int(g["count"])):
        dx, dy, dt = g[f"c{k}_meta"]
        bcs = [str(b) for b in g[f"c{k}_bcs"]]
        res, fx, fy, used = fv.hydro_2d(g[f"c{k}_state"], dx, dy, dt, g[f"c{k}_gamma"],
                                        str(g[f"c{k}_limiter"]), bcs[0], bcs[1],
                                        list(g[f"c{k}_inlet"]))
        fallback_seen |= used
        np.testing.assert_array_equal(res, g[f"c{k}_result"])
        np.testing.assert_array_equal(fx, g[f"c{k}_flux0"])
        np.testing.assert_array_equal(fy, g[f"c{k}_flux1"])
    assert fallback_seen, "the strong-shock case must exercise the LLF fallback"


def test_chemistry_bit_exact():
    g = load("chemistry.npz")
    dt = float(g["dt"])
    for model in ("arrhenius", "znd"):
        lam, st, beta = fv.react_1d(g[f"{model}_lam"], dt, g[f"{model}_state"], model,
                                    g[f"{model}_beta"])
        np.testing.assert_array_equal(lam, g[f"{model}_out_lam"])
        np.testing.assert_array_equal(st, g[f"{model}_out_state"])
        np.testing.assert_array_equal(beta, g[f"{model}_out_beta"])
    res, lam, beta = fv.reaction_nd(g["r3_state"], g["r3_lam"], g["r3_beta"], 3e-6, "znd")
    np.testing.assert_array_equal(res, g["r3_out"])
    np.testing.assert_array_equal(lam, g["r3_out_lam"])
    np.testing.assert_array_equal(beta, g["r3_out_beta"])


def _session(name, prim_state, **kw):
    return kw


SESSION_SETUPS = {
    "s2d_explosion": dict(lengths=[1, 1], t_end=0.05, limiter="VanLeer"),
    "s3d_explosion": dict(lengths=[1, 1, 1], t_end=0.05, limiter="Superbee",
                          boundaries=["Reflective"] * 3),
    "s3d_open_albada": dict(lengths=[1.0, 0.9, 0.8], t_end=0.02, limiter="Albada",
                            boundaries=["Open", "Periodic", "Reflective"]),
    "s1d_sod": dict(lengths=[1.0], t_end=0.1, limiter="VanLeer"),
    "s1d_sod_superbee_reflective": dict(lengths=[1.0], t_end=0.05, limiter="Superbee",
                                        boundaries=["Reflective"]),
    "s3d_ignition_znd": dict(lengths=[1, 1, 1], t_end=2e-6, reactive=True,
                             kinetic_model="znd", limiter="VanLeer"),
    "s3d_ignition_arr": dict(lengths=[1, 1, 1], t_end=2e-6, reactive=True,
                             kinetic_model="arrhenius", limiter="MINBEE",
                             boundaries=["Reflective", "Open", "Periodic"]),
    "s2d_reactive": dict(lengths=[1, 1], t_end=1e-6, reactive=True, limiter="Superbee",
                         boundaries=["Periodic", "Inflow"],
                         inlet_primitive=[1.0, 0.0, 100.0, 101325.0]),
    "s1d_reactive_znd": dict(lengths=[1.0], t_end=2e-6, reactive=True, kinetic_model="znd"),
}


def primitive_from_state(state, gamma):
    p = state.copy()
    p[1:-1] /= state[0]
    p[-1] = (gamma - 1) * (state[-1] - 0.5 * np.sum(state[1:-1] ** 2, axis=0) / state[0])
    return p


@pytest.mark.parametrize("name", sorted(SESSION_SETUPS))
def test_session_trajectories_match_reference(name):
    g = load("sessions.npz")
    kw = dict(SESSION_SETUPS[name])
    lengths = kw.pop("lengths")
    state0 = g[f"{name}_state0"]
    lam0 = g[f"{name}_lam0"] if f"{name}_lam0" in g else None
    beta0 = g[f"{name}_beta0"] if f"{name}_beta0" in g else None
    gamma0 = fv.gamma_of_lambda(lam0) if kw.get("reactive") else 1.4
    s = OracleSimulation(primitive_from_state(state0, gamma0), lengths, lambda_init=lam0,
                         beta_init=beta0, **kw)
    # the session rebuilds the conservative state from primitives; start from
    # the reference's exact conservative state instead
    s.state = state0.copy()
    s.initial_integral = s.integral.copy()
    steps = int(g[f"{name}_scalars"][1])
    for _ in range(steps):
        s.step()
    exact = True  # the oracle uses NumPy exp like the reference: bit-exact
    cmp = (np.testing.assert_array_equal if exact
           else lambda a, b: np.testing.assert_allclose(a, b, rtol=1e-12, atol=0))
    cmp(s.state, g[f"{name}_state"])
    assert s.time == pytest.approx(g[f"{name}_scalars"][0], rel=1e-13)
    if lam0 is not None:
        cmp(s.lam, g[f"{name}_lam"])
    if beta0 is not None:
        cmp(s.beta, g[f"{name}_beta"])
    np.testing.assert_allclose(s.boundary_integral, g[f"{name}_boundary"], rtol=1e-10,
                               atol=1e-13 * max(1.0, np.abs(g[f"{name}_initial"]).max()))
    np.testing.assert_allclose(s.source_integral, g[f"{name}_source"], rtol=1e-10, atol=1e-6)


def test_large_cfl_2d_trajectory_matches_reference():
    g = load("cfl08_2d.npz")
    state = g["state0"].copy()
    h = (2.0 / 40, 2.0 / 40)
    for k in range(12):
        dt = fv.dt_2d(state, h, 0.8, 1.4, "Open", "Open")
        assert dt == g["dts"][k]
        state = fv.hydro_2d(state, h[0], h[1], dt, 1.4, "VanLeer", "Open", "Open")[0]
    np.testing.assert_array_equal(state, g["state"])


def test_exact_riemann_solver_matches_reference():
    """The oracle's exact Riemann solver (used by the Sod parity tests)
    against the reference's exact_riemann_sod on Sod, a strong shock, two
    rarefactions and a shock collision."""
    from oracle import exact_riemann

    g = np.load(GOLDEN / "exact_riemann.npz")
    names = sorted({k.rsplit("_", 1)[0] for k in g.files if k.endswith("_args")})
    assert len(names) == 5
    for name in names:
        t, x0, gamma, rl, ul, pl, rr, ur, pr = g[f"{name}_args"]
        rho, u, p = exact_riemann.sample((rl, ul, pl), (rr, ur, pr), g[f"{name}_x"], t, x0, gamma)
        for got, key in ((rho, "rho"), (u, "u"), (p, "p")):
            want = g[f"{name}_{key}"]
            np.testing.assert_allclose(got, want, rtol=1e-6, atol=1e-7 * np.abs(want).max(),
                                       err_msg=f"{name} {key}")
