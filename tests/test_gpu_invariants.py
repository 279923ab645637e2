"""Physical invariants the reference's own 3D tests assert
(python/tests/testSolver3D.py:88-336), checked on the GPU session: uniform
states stay uniform, Sod tubes along x, y and z agree with each other and
with the exact solution, an extruded 2D step equals the 3D step, smooth
entropy waves converge, the spherical explosion keeps its symmetry with every
limiter, boundary balances close, species and induction fractions are
transported conservatively, and strong shocks and expansions stay physical.
FP64 uses the reference's tolerances; the FP32 symmetry check states its
own."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import torch_gb300  # noqa: E402
from oracle import exact_riemann  # noqa: E402

LIMITERS = ("VanLeer", "Albada", "MINBEE", "Superbee", "Unos")


def uniform(shape=(4, 4, 4), velocity=(0.3, -0.2, 0.1), pressure=1.0):
    p = np.ones((5, *shape))
    for m, v in enumerate(velocity, 1):
        p[m] = v
    p[4] = pressure
    return p


def physical(state):
    rho = state[0]
    kinetic = 0.5 * np.sum(state[1:-1] ** 2, axis=0) / rho
    return bool(np.all(np.isfinite(state)) and np.all(rho > 1e-12)
                and np.all(state[-1] - kinetic > 1e-12))


def preset(name, nx, ny, nz):
    """Preset initial primitives (python/cfdSolver/torchSolver3D.py:259-286)."""
    z, y, x = np.meshgrid((np.arange(nz) + 0.5) / nz, (np.arange(ny) + 0.5) / ny,
                          (np.arange(nx) + 0.5) / nx, indexing="ij")
    p = np.zeros((5, nz, ny, nx))
    if name.startswith("3d_sod_"):
        c = {"x": x, "y": y, "z": z}[name[-1]]
        p[0] = np.where(c <= 0.5, 1, 0.125)
        p[4] = np.where(c <= 0.5, 1, 0.1)
    else:  # 3d_explosion
        inside = (x - 0.5) ** 2 + (y - 0.5) ** 2 + (z - 0.5) ** 2 <= 0.2 ** 2
        p[0] = np.where(inside, 1, 0.125)
        p[4] = np.where(inside, 1, 0.1)
    return p


def solve(p, t_end, precision="fp64", **kw):
    sim = torch_gb300.Simulation(p, [1.0, 1.0, 1.0], t_end=t_end, precision=precision, **kw)
    sim.run()
    return sim


def test_uniform_state_and_full_periodic_balance():
    p = uniform()
    s = solve(p, 0.05, boundaries=["Periodic"] * 3)
    np.testing.assert_allclose(s.primitive, p, atol=1e-14)
    np.testing.assert_allclose(s.balance_residual, 0, atol=1e-14)
    assert s.time == 0.05


def test_sod_along_each_axis_matches_exact_solution_and_rotation():
    profiles = []
    for axis in ("x", "y", "z"):
        grid = dict(nx=4, ny=4, nz=4)
        grid["n" + axis] = 32
        s = solve(preset("3d_sod_" + axis, **grid), 0.08)
        dimension = ("z", "y", "x").index(axis)
        rho = np.moveaxis(s.primitive[0], dimension, -1)[0, 0]
        centres = (np.arange(32) + 0.5) / 32
        exact = exact_riemann.sod(centres, 0.08)[0]
        assert np.mean(np.abs(rho - exact)) < 0.04
        assert physical(s.state)
        np.testing.assert_allclose(s.balance_residual, 0, atol=1e-13)
        profiles.append(rho)
    for rho in profiles[1:]:
        np.testing.assert_allclose(rho, profiles[0], atol=1e-13)


def test_extruded_2d_step_matches_3d():
    ny, nx, nz = 8, 10, 3
    y, x = np.meshgrid((np.arange(ny) + 0.5) / ny, (np.arange(nx) + 0.5) / nx, indexing="ij")
    p = np.stack((1 + 0.1 * np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y), 0.2 + 0 * x,
                  -0.1 + 0 * x, 1 + 0 * x))
    state2 = p.copy()
    state2[1:-1] *= p[0]
    state2[-1] = p[-1] / 0.4 + 0.5 * p[0] * np.sum(p[1:-1] ** 2, axis=0)
    state3 = np.repeat(np.stack((state2[0], state2[1], state2[2], np.zeros_like(x),
                                 state2[3]))[:, None], nz, axis=1)
    out2 = torch_gb300.muscl_hancock_step_2d(state2, 1 / nx, 1 / ny, 0.002, bc_x="Periodic",
                                             bc_y="Periodic")
    out3 = torch_gb300.muscl_hancock_step_3d(state3, 1 / nx, 1 / ny, 1 / nz, 0.002,
                                             bc_x="Periodic", bc_y="Periodic", bc_z="Periodic")
    np.testing.assert_allclose(np.asarray(out3)[[0, 1, 2, 4], 0], out2, rtol=1e-13, atol=1e-14)


def test_smooth_entropy_wave_mesh_convergence():
    errors = []
    for n in (16, 32, 64):
        p = uniform((4, 4, n), velocity=(1, 0, 0))
        x = (np.arange(n) + 0.5) / n
        p[0] = 1 + 0.2 * np.sin(2 * np.pi * x)
        s = solve(p, 0.1, boundaries=["Periodic"] * 3)
        errors.append(np.mean(np.abs(s.primitive[0] - (1 + 0.2 * np.sin(2 * np.pi * (x - 0.1))))))
    assert errors[0] / errors[1] > 3
    assert errors[1] / errors[2] > 3


@pytest.mark.parametrize("precision,atol", [("fp64", 1e-13), ("fp32", 1e-5)])
def test_spherical_explosion_symmetry_and_all_limiters(precision, atol):
    for limiter in LIMITERS:
        s = solve(preset("3d_explosion", 8, 8, 8), 0.02, precision=precision, limiter=limiter)
        rho = s.primitive[0]
        np.testing.assert_allclose(rho, rho.transpose(2, 1, 0), atol=atol)
        np.testing.assert_allclose(rho, rho[::-1], atol=atol)
        assert physical(s.state)
        assert np.max(np.abs(s.balance_residual)) < (1e-12 if precision == "fp64" else 1e-5)


def test_reflective_wall_mass_energy_and_open_boundary_balance():
    p = uniform(velocity=(1, 0.5, -0.3))
    for bc in ("Reflective", "Open"):
        s = solve(p, 0.04, boundaries=[bc] * 3)
        np.testing.assert_allclose(s.balance_residual, 0, atol=1e-13)
        if bc == "Reflective":
            np.testing.assert_allclose(s.boundary_integral[[0, 4]], 0, atol=1e-13)


def test_periodic_species_and_induction_transport_in_three_directions():
    n = 8
    p = uniform((n, n, n), velocity=(1, 0.5, 0.3), pressure=100)
    lam = np.zeros((n, n, n))
    lam[2:4, 2:4, 2:4] = 1
    s = solve(p, 0.02, boundaries=["Periodic"] * 3, reactive=True, kinetic_model="znd",
              lambda_init=lam, beta_init=1 - lam)
    rho = s.state[0]
    species = rho * s.lam
    assert abs(species.sum() - lam.sum()) < 5e-11
    assert abs((rho * s.beta).sum() - (1 - lam).sum()) < 5e-11
    z, y, x = np.meshgrid(*([(np.arange(n) + 0.5) / n] * 3), indexing="ij")
    for coord in (x, y, z):
        assert (species * coord).sum() > (lam * coord).sum()


def test_strong_shock_and_expansion_remain_physical():
    for limiter in LIMITERS:
        for case in ("shock", "expansion"):
            p = uniform((4, 4, 24), velocity=(0, 0, 0))
            end = 0.002 if case == "shock" else 0.02
            if case == "shock":
                p[4, :, :, :12] = 1000
                p[4, :, :, 12:] = 0.01
            else:
                p[4] = 0.4
                p[1, :, :, :12] = -2
                p[1, :, :, 12:] = 2
            s = solve(p, end, cfl=0.5, limiter=limiter)
            assert physical(s.state)
            assert s.time == end
            np.testing.assert_allclose(s.balance_residual, 0, atol=1e-11)
