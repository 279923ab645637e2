"""GPU parity: the CUDA path (through the C ABI) against the reference's golden
vectors and the oracle.  FP64 results must be bit-identical to the reference
(the kernels keep NumPy's operation order and are built without FMA
contraction); FP32 results are checked against FP64 within the stated L1
tolerance."""

from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import torch_gb300  # noqa: E402
from torch_gb300 import stepfn  # noqa: E402
from oracle import fv  # noqa: E402
from oracle.session import OracleSimulation  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name):
    return np.load(GOLDEN / name, allow_pickle=False)


def test_hllc_matches_reference_bitwise():
    g = load("hllc.npz")
    for nv in (4, 5):
        got = stepfn.hllc_flux(g[f"ul{nv}"], g[f"ur{nv}"], g[f"gl{nv}"],
                               gamma_right=g[f"gr{nv}"])
        np.testing.assert_array_equal(got, g[f"flux{nv}"])


def test_step3d_matches_reference_bitwise():
    g = load("step3d.npz")
    for k in range(int(g["count"])):
        hx, hy, hz, dt = g[f"c{k}_meta"]
        bcs = [str(b) for b in g[f"c{k}_bcs"]]
        res, fx, fy, fz = stepfn.muscl_hancock_step_3d(
            g[f"c{k}_state"], hx, hy, hz, dt, g[f"c{k}_gamma"], str(g[f"c{k}_limiter"]),
            *bcs, return_fluxes=True)
        np.testing.assert_array_equal(res, g[f"c{k}_result"], err_msg=f"case {k}")
        for d, f in enumerate((fx, fy, fz)):
            np.testing.assert_array_equal(f, g[f"c{k}_flux{d}"], err_msg=f"case {k} flux {d}")


def test_step2d_matches_reference_bitwise():
    g = load("step2d.npz")
    for k in range(int(g["count"])):
        dx, dy, dt = g[f"c{k}_meta"]
        bcs = [str(b) for b in g[f"c{k}_bcs"]]
        res, fx, fy = stepfn.muscl_hancock_step_2d(
            g[f"c{k}_state"], dx, dy, dt, g[f"c{k}_gamma"], str(g[f"c{k}_limiter"]), *bcs,
            return_fluxes=True, inlet_primitive=list(g[f"c{k}_inlet"]))
        np.testing.assert_array_equal(res, g[f"c{k}_result"], err_msg=f"case {k}")
        np.testing.assert_array_equal(fx, g[f"c{k}_flux0"], err_msg=f"case {k} fx")
        np.testing.assert_array_equal(fy, g[f"c{k}_flux1"], err_msg=f"case {k} fy")


def _rough_state(rng, dim, shape):
    p = np.empty((dim + 2,) + shape)
    p[0] = 0.5 + rng.random(shape)
    p[1:-1] = 0.6 * (rng.random((dim,) + shape) - 0.5)
    p[-1] = 0.5 + rng.random(shape)
    return fv.prim_to_cons(p, 1.4)


@pytest.mark.parametrize("shape", [(2, 2, 2), (3, 5, 2), (11, 19, 37), (9, 70, 33)])
@pytest.mark.parametrize("bcs", [("Open", "Reflective", "Periodic"),
                                 ("Periodic", "Open", "Reflective")])
def test_step3d_partial_tiles_and_tiny_grids(shape, bcs):
    rng = np.random.default_rng(sum(shape))
    state = _rough_state(rng, 3, shape)
    h = (0.7 / shape[2], 1.1 / shape[1], 0.9 / shape[0])
    dt = 0.5 * fv.dt_3d(state, h, 0.4, 1.4)
    for limiter in ("Superbee", "Unos"):
        want, fl, _ = fv.hydro_3d(state, 1.4, h, dt, limiter, bcs)
        got = stepfn.muscl_hancock_step_3d(state, *h, dt, 1.4, limiter, *bcs, return_fluxes=True)
        np.testing.assert_array_equal(got[0], want)
        for d in range(3):
            np.testing.assert_array_equal(got[1 + d], fl[d])


@pytest.mark.parametrize("shape", [(2, 2), (7, 3), (130, 67), (33, 260)])
@pytest.mark.parametrize("bcs", [("Open", "Inflow"), ("Periodic", "Reflective")])
def test_step2d_partial_tiles_and_tiny_grids(shape, bcs):
    rng = np.random.default_rng(sum(shape) + 1)
    state = _rough_state(rng, 2, shape)
    h = (1.0 / shape[1], 0.8 / shape[0])
    inlet = [1.2, 0.1, 0.3, 0.9]
    dt = 0.5 * fv.dt_2d(state, h, 0.4, 1.4, *bcs, inlet)
    for limiter in ("VanLeer", "Albada"):
        want, fx, fy, _ = fv.hydro_2d(state, h[0], h[1], dt, 1.4, limiter, *bcs, inlet)
        got = stepfn.muscl_hancock_step_2d(state, h[0], h[1], dt, 1.4, limiter, *bcs,
                                           return_fluxes=True, inlet_primitive=inlet)
        np.testing.assert_array_equal(got[0], want)
        np.testing.assert_array_equal(got[1], fx)
        np.testing.assert_array_equal(got[2], fy)


def explosion_2d(n, length=2.0, radius=0.4):
    """2D cylindrical explosion on [0, length]^2 (the reference's 2d_explosion
    preset scaled), primitives (rho, u, v, p)."""
    x = (np.arange(n) + 0.5) * length / n
    X, Y = np.meshgrid(x, x)
    inside = np.hypot(X - length / 2, Y - length / 2) <= radius
    z = np.zeros_like(X)
    return np.stack((np.where(inside, 1.0, 0.125), z, z, np.where(inside, 1.0, 0.1)))


def explosion_3d(n):
    c = (np.arange(n) + 0.5) / n
    Z, Y, X = np.meshgrid(c, c, c, indexing="ij")
    inside = (X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2 <= 0.2 ** 2
    p = np.zeros((5, n, n, n))
    p[0] = np.where(inside, 1.0, 0.125)
    p[4] = np.where(inside, 1.0, 0.1)
    return p


def test_session_2d_explosion_cfl08_matches_oracle_bitwise():
    """Cylindrical explosion (VanLeer, Open, CFL 0.8) to t = 0.25 at 64^2."""
    prim = explosion_2d(64)
    kw = dict(t_end=0.25, cfl=0.8, limiter="VanLeer", boundaries=["Open", "Open"],
              strict_cfl=False)
    gpu = torch_gb300.Simulation(prim, [2.0, 2.0], **kw)
    ref = OracleSimulation(prim, [2.0, 2.0], **kw)
    while not ref.completed:
        ref.step()
        gpu.step()
        assert gpu.time == ref.time
    assert gpu.completed and gpu.steps == ref.steps
    np.testing.assert_array_equal(gpu.state, ref.state)
    np.testing.assert_allclose(gpu.boundary_integral, ref.boundary_integral, rtol=1e-11,
                               atol=1e-14)
    assert np.max(np.abs(gpu.balance_residual)) < 1e-12


def test_full_size_2d_explosion_256_cfl08_to_t025_bitwise():
    """The 2D explosion at its full size (256 x 256 on [0, 2]^2, VanLeer,
    Open, CFL 0.8, to t = 0.25: 169 steps): every step's time and the final
    state bit for bit against the oracle."""
    prim = explosion_2d(256)
    kw = dict(t_end=0.25, cfl=0.8, limiter="VanLeer", boundaries=["Open", "Open"],
              strict_cfl=False)
    gpu = torch_gb300.Simulation(prim, [2.0, 2.0], **kw)
    ref = OracleSimulation(prim, [2.0, 2.0], **kw)
    while not ref.completed:
        ref.step()
        gpu.step()
        assert gpu.time == ref.time
    assert gpu.steps == ref.steps == 169
    np.testing.assert_array_equal(gpu.state, ref.state)
    assert np.max(np.abs(gpu.balance_residual)) < 1e-12


def test_session_3d_explosion_superbee_reflective_matches_oracle():
    prim = explosion_3d(24)
    kw = dict(t_end=1.0, cfl=0.6, limiter="Superbee", boundaries=["Reflective"] * 3,
              strict_cfl=False)
    gpu = torch_gb300.Simulation(prim, [1, 1, 1], **kw)
    ref = OracleSimulation(prim, [1, 1, 1], **kw)
    for _ in range(15):
        ref.step()
        gpu.step()
    assert gpu.time == ref.time
    np.testing.assert_array_equal(gpu.state, ref.state)
    assert np.max(np.abs(gpu.balance_residual)) < 1e-12
    # reflective walls: no mass or energy crosses the boundary
    np.testing.assert_allclose(gpu.boundary_integral[[0, 4]], 0, atol=1e-13)


def test_session_3d_explosion_100_steps_fp64_matches_oracle():
    """The headline scheme (3D explosion, Superbee, reflective, CFL 0.6) in
    double precision for 100 steps at 40^3 against the oracle session.  Stated
    criterion: relative L1 difference (sum |gpu - oracle| / sum |oracle|) per
    conserved variable <= 1e-10, and the conservation residual at roundoff; the
    kernels keep the reference's operation order, so the states are expected
    to be bit-identical as well."""
    prim = explosion_3d(40)
    kw = dict(t_end=1.0, cfl=0.6, limiter="Superbee", boundaries=["Reflective"] * 3,
              strict_cfl=False)
    gpu = torch_gb300.Simulation(prim, [1, 1, 1], **kw)
    ref = OracleSimulation(prim, [1, 1, 1], **kw)
    for _ in range(100):
        ref.step()
    gpu.run(step_limit=100)
    assert gpu.steps == ref.steps == 100
    assert gpu.time == ref.time
    got, want = gpu.state, ref.state
    for k in range(5):
        rel = np.sum(np.abs(got[k] - want[k])) / np.sum(np.abs(want[k]))
        assert rel <= 1e-10, (k, rel)
    np.testing.assert_array_equal(got, want)
    assert np.max(np.abs(gpu.balance_residual) / np.abs(gpu.initial_integral).max()) < 1e-12


def pressure(u, gamma=1.4):
    return (gamma - 1.0) * (u[-1] - 0.5 * np.sum(u[1:-1] ** 2, axis=0) / u[0])


def test_fp32_bulk_200_steps_rho_and_p_against_fp64():
    """The headline workload's scheme at 128^3 for its full 200 steps: FP32
    bulk against plain FP64 from the same initial state.  Stated tolerances:
    L1 (mean absolute) error of density and of pressure <= 1e-5 each; the FP32
    session's conservation residual relative to the initial integrals < 1e-6
    (its sums and clock are FP64)."""
    prim = explosion_3d(128)
    kw = dict(t_end=1.0, cfl=0.6, limiter="Superbee", boundaries=["Reflective"] * 3,
              strict_cfl=False, max_steps=10 ** 6)
    s64 = torch_gb300.Simulation(prim, [1, 1, 1], graph_steps=10, **kw)
    s32 = torch_gb300.Simulation(prim, [1, 1, 1], precision="fp32", graph_steps=10, **kw)
    s64.run(step_limit=200)
    s32.run(step_limit=200)
    assert s64.steps == s32.steps == 200
    u64, u32 = s64.state, s32.state
    l1_rho = np.mean(np.abs(u32[0] - u64[0]))
    l1_p = np.mean(np.abs(pressure(u32) - pressure(u64)))
    assert l1_rho <= 1e-5, l1_rho
    assert l1_p <= 1e-5, l1_p
    assert np.all(np.isfinite(u32))
    assert abs(s32.time - s64.time) <= 1e-5 * s64.time
    assert np.max(np.abs(s32.balance_residual) / np.abs(s32.initial_integral).max()) < 1e-6
    assert np.max(np.abs(s64.balance_residual) / np.abs(s64.initial_integral).max()) < 1e-12


def test_sessions_match_reference_trajectories():
    g = load("sessions.npz")
    cases = {
        "s2d_explosion": dict(lengths=[1, 1], t_end=0.05, limiter="VanLeer"),
        "s3d_explosion": dict(lengths=[1, 1, 1], t_end=0.05, limiter="Superbee",
                              boundaries=["Reflective"] * 3),
        "s3d_open_albada": dict(lengths=[1.0, 0.9, 0.8], t_end=0.02, limiter="Albada",
                                boundaries=["Open", "Periodic", "Reflective"]),
    }
    for name, kw in cases.items():
        kw = dict(kw)
        lengths = kw.pop("lengths")
        state0 = g[f"{name}_state0"]
        dim = state0.ndim - 1
        prim = state0.copy()
        prim[1:-1] /= state0[0]
        prim[-1] = 0.4 * (state0[-1] - 0.5 * np.sum(state0[1:-1] ** 2, axis=0) / state0[0])
        gpu = torch_gb300.Simulation(prim, lengths, **kw)
        gpu.state = state0  # start from the reference's exact conservative state
        steps = int(g[f"{name}_scalars"][1])
        for _ in range(steps):
            gpu.step()
        np.testing.assert_array_equal(gpu.state, g[f"{name}_state"], err_msg=name)
        assert gpu.time == g[f"{name}_scalars"][0]
        np.testing.assert_allclose(gpu.boundary_integral, g[f"{name}_boundary"], rtol=1e-10,
                                   atol=1e-14)
        assert gpu.steps == steps and dim in (2, 3)


def test_fallback_step_in_a_session():
    """A rough state whose second-order step is nonphysical: the GPU session
    takes the same first-order fallback as the reference."""
    rng = np.random.default_rng(1)
    shape = (4, 4, 6)
    p = np.empty((5,) + shape)
    p[0] = 10 ** rng.uniform(-3, 1, shape)
    p[1:4] = rng.uniform(-3, 3, (3,) + shape)
    p[4] = 10 ** rng.uniform(-4, 1, shape)
    kw = dict(t_end=10.0, cfl=0.4, limiter="Superbee",
              boundaries=["Open", "Periodic", "Reflective"])
    ref = OracleSimulation(p, [1, 1, 1], **kw)
    gpu = torch_gb300.Simulation(p, [1, 1, 1], **kw)
    ref.step()
    gpu.step()
    assert ref.fallback_steps == 1 and gpu.fallback_steps == 1
    np.testing.assert_array_equal(gpu.state, ref.state)


def test_fp32_bulk_l1_error_against_fp64():
    """FP32 bulk step vs the FP64 path: 3D explosion 48^3, Superbee,
    reflective, CFL 0.6, 40 steps.  Stated tolerance: L1 density error
    (mean |rho32 - rho64|) <= 1e-5."""
    prim = explosion_3d(48)
    kw = dict(t_end=1.0, cfl=0.6, limiter="Superbee", boundaries=["Reflective"] * 3,
              strict_cfl=False)
    s64 = torch_gb300.Simulation(prim, [1, 1, 1], **kw)
    s32 = torch_gb300.Simulation(prim, [1, 1, 1], precision="fp32", **kw)
    s64.run(step_limit=40)
    s32.run(step_limit=40)
    assert s64.steps == s32.steps == 40
    r64, r32 = s64.state[0], s32.state[0]
    l1 = np.mean(np.abs(r32 - r64))
    assert l1 <= 1e-5, l1
    assert abs(s32.time - s64.time) <= 1e-6 * s64.time
    # FP64 conservation sums keep the FP32 session's balance at FP32 roundoff
    assert np.max(np.abs(s32.balance_residual) / np.abs(s32.initial_integral).max()) < 1e-6
