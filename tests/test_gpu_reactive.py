"""GPU parity of the reactive step (Strang-split Arrhenius / ZND source,
species transport, reactive dt halving) against the reference's golden
trajectories and the oracle.  The chemistry uses exp, whose last bit differs
between CUDA and NumPy, so reactive FP64 results are compared at a stated
relative tolerance of 1e-10 instead of bitwise."""

from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import torch_gb300  # noqa: E402
from oracle import fv  # noqa: E402
from oracle.session import OracleSimulation  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden"
RTOL = 1e-10


def close(a, b, what):
    scale = np.maximum(np.abs(b), 1e-300)
    err = np.max(np.abs(a - b) / scale)
    assert err <= RTOL or np.allclose(a, b, rtol=RTOL, atol=1e-12 * np.abs(b).max()), (what, err)


def prim_of(state, gamma):
    p = state.copy()
    p[1:-1] /= state[0]
    p[-1] = (gamma - 1) * (state[-1] - 0.5 * np.sum(state[1:-1] ** 2, axis=0) / state[0])
    return p


GOLDEN_CASES = {
    "s3d_ignition_znd": dict(lengths=[1, 1, 1], t_end=2e-6, reactive=True, kinetic_model="znd",
                             limiter="VanLeer"),
    "s3d_ignition_arr": dict(lengths=[1, 1, 1], t_end=2e-6, reactive=True,
                             kinetic_model="arrhenius", limiter="MINBEE",
                             boundaries=["Reflective", "Open", "Periodic"]),
    "s2d_reactive": dict(lengths=[1, 1], t_end=1e-6, reactive=True, limiter="Superbee",
                         boundaries=["Periodic", "Inflow"],
                         inlet_primitive=[1.0, 0.0, 100.0, 101325.0]),
}


@pytest.mark.parametrize("name", sorted(GOLDEN_CASES))
def test_reactive_sessions_match_reference(name):
    g = np.load(GOLDEN / "sessions.npz")
    kw = dict(GOLDEN_CASES[name])
    lengths = kw.pop("lengths")
    state0 = g[f"{name}_state0"]
    lam0 = g[f"{name}_lam0"]
    beta0 = g[f"{name}_beta0"] if f"{name}_beta0" in g else None
    gpu = torch_gb300.Simulation(prim_of(state0, fv.gamma_of_lambda(lam0)), lengths,
                                 lambda_init=lam0, beta_init=beta0, **kw)
    gpu.state = state0
    steps = int(g[f"{name}_scalars"][1])
    for _ in range(steps):
        gpu.step()
    assert gpu.steps == steps
    close(gpu.state, g[f"{name}_state"], "state")
    close(gpu.lam, g[f"{name}_lam"], "lambda")
    if beta0 is not None:
        close(gpu.beta, g[f"{name}_beta"], "beta")
    assert abs(gpu.time - g[f"{name}_scalars"][0]) <= 1e-12 * g[f"{name}_scalars"][0]
    np.testing.assert_allclose(gpu.source_integral, g[f"{name}_source"], rtol=1e-8, atol=1e-6)


def test_reactive_dt_halving_matches_oracle():
    """Fast SI ZND kinetics (A = 1.76e8) force CFL halvings of the reactive
    step; the GPU session takes the same dt sequence as the oracle."""
    p = np.ones((5, 6, 6, 8))
    p[1:4] = 0.0
    p[4] = np.where(np.arange(8) < 4, 1e6, 101325.0)
    kw = dict(t_end=1e-3, reactive=True, kinetic_model="znd", chemistry=dict(pre_exponential=1.76e8),
              limiter="VanLeer")
    ref = OracleSimulation(p, [1, 1, 1], **kw)
    gpu = torch_gb300.Simulation(p, [1, 1, 1], **kw)
    calls = [0]
    react = ref._reaction

    def counted(*a, **k):
        calls[0] += 1
        return react(*a, **k)

    ref._reaction = counted
    for _ in range(6):
        ref.step()
        gpu.step()
        assert abs(gpu.time - ref.time) <= 1e-12 * ref.time
    assert calls[0] > 2 * 6, "the case must exercise dt halvings"
    close(gpu.state, ref.state, "state")
    close(gpu.lam, ref.lam, "lambda")
    close(gpu.beta, ref.beta, "beta")
    assert np.max(np.abs(gpu.balance_residual) / np.abs(gpu.initial_integral).max()) < 1e-12


def ignition_3d(n):
    """Nondimensional ignition: rho = 1, T = 1 + 2 exp(-r^2 / (2 * 0.05^2)),
    p = rho T, at rest, lambda = 1."""
    c = (np.arange(n) + 0.5) / n
    Z, Y, X = np.meshgrid(c, c, c, indexing="ij")
    r2 = (X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2
    p = np.zeros((5, n, n, n))
    p[0] = 1.0
    p[4] = 1.0 + 2.0 * np.exp(-r2 / (2 * 0.05 ** 2))
    return p


NONDIM = dict(closure="nondimensional", q_heat=20.0, activation_energy=25.0, pre_exponential=1e3)


def test_nondimensional_ignition_matches_oracle():
    p = ignition_3d(16)
    kw = dict(t_end=1.0, cfl=0.4, gamma=1.2, reactive=True, limiter="Albada",
              chemistry=dict(NONDIM))
    ref = OracleSimulation(p, [1, 1, 1], **kw)
    gpu = torch_gb300.Simulation(p, [1, 1, 1], **kw)
    for _ in range(8):
        ref.step()
        gpu.step()
    close(gpu.state, ref.state, "state")
    close(gpu.lam, ref.lam, "lambda")
    close(gpu.source_integral, ref.source_integral, "source")
    assert np.max(np.abs(gpu.balance_residual) / np.abs(gpu.initial_integral).max()) < 1e-12


def test_nondimensional_ignition_fp32_against_fp64():
    """FP32 bulk with FP64 sums: L1 density error <= 1e-5 after 20 steps."""
    p = ignition_3d(32)
    kw = dict(t_end=1.0, cfl=0.4, gamma=1.2, reactive=True, limiter="Albada",
              chemistry=dict(NONDIM))
    s64 = torch_gb300.Simulation(p, [1, 1, 1], **kw)
    s32 = torch_gb300.Simulation(p, [1, 1, 1], precision="fp32", **kw)
    s64.run(step_limit=20)
    s32.run(step_limit=20)
    assert np.mean(np.abs(s32.state[0] - s64.state[0])) <= 1e-5
    assert np.mean(np.abs(s32.lam - s64.lam)) <= 1e-5
    assert np.max(np.abs(s32.balance_residual) / np.abs(s32.initial_integral).max()) < 1e-6
