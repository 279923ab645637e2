"""Adaptive (AMR) sessions advanced with GPU leaf-face fluxes.

TORCH's adaptive solver keeps its leaf mesh on the host and hands the Rusanov
flux of every leaf face to ``torchAdaptive.rusanov`` in 8,192-face batches
(python/cfdSolver/torchAdaptive.py:115-153).  Here the reference's own
AdaptiveSimulation (installed into baseline/_ref by
baseline/install_reference.py) runs with that call routed to the GPU by
torch_gb300.adaptive.gpu_leaf_fluxes.  On the same host it must follow the
session stepped with the reference's CPU fluxes bit for bit (every step's
time, leaf keys, boundary integral and state), and it must follow the
trajectory the reference recorded on another machine
(tests/golden/adaptive.npz, made by tests/golden/make_golden.py) within the
last bits of the host-side NumPy reductions.  Single-precision fluxes follow
the same trajectory within 1e-5 relative L1 of density."""

import importlib
import importlib.util
import sys
import types
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

ROOT = Path(__file__).resolve().parent.parent
REF = ROOT / "baseline" / "_ref" / "cfdSolver"
if not (REF / "torchAdaptive.py").is_file():
    pytest.skip("the reference is not installed in baseline/_ref "
                "(python baseline/install_reference.py)", allow_module_level=True)

from torch_gb300 import adaptive as gpu_adaptive  # noqa: E402

G = np.load(ROOT / "tests" / "golden" / "adaptive.npz")


def reference():
    """The installed reference package, through a bare namespace module (its
    __init__ imports matplotlib, which the solver does not need)."""
    if "cfdSolver" not in sys.modules or not hasattr(sys.modules["cfdSolver"], "__path__"):
        pkg = types.ModuleType("cfdSolver")
        pkg.__path__ = [str(REF)]
        sys.modules["cfdSolver"] = pkg
    return (importlib.import_module("cfdSolver.torchSession"),
            importlib.import_module("cfdSolver.torchAdaptive"))


def sessions(session_module):
    spec = importlib.util.spec_from_file_location("make_golden",
                                                  ROOT / "tests" / "golden" / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.adaptive_sessions(session_module.Simulation)


@pytest.mark.parametrize("name", ["explosion2d", "cylindrical_blast"])
def test_adaptive_session_with_gpu_fluxes_equals_cpu_fluxes_bitwise(name):
    """The same adaptive session stepped with the reference's CPU Rusanov
    batches and with the GPU ones, side by side on this host: every step's
    time, dt, leaf keys, boundary integral and state bit for bit."""
    S, A = reference()
    cpu, steps = sessions(S)[name]
    gpu, _ = sessions(S)[name]
    for _ in range(steps):
        cpu.step()
        with gpu_adaptive.gpu_leaf_fluxes(A):
            gpu.step()
        assert gpu.time == cpu.time
        np.testing.assert_array_equal(gpu.mesh.keys, cpu.mesh.keys)
        np.testing.assert_array_equal(gpu.boundary_integral, cpu.boundary_integral)
        np.testing.assert_array_equal(gpu.state, cpu.state)
    # the reference's own flux is back in place after the block
    assert A.rusanov.__module__ == "cfdSolver.torchFlux"


@pytest.mark.parametrize("name", ["explosion2d", "cylindrical_blast"])
def test_adaptive_session_with_gpu_fluxes_follows_recorded_trajectory(name):
    """Against the trajectory the reference recorded with its CPU fluxes on
    another machine: leaf counts and keys exactly, time at rtol 1e-12,
    boundary integral and state at rtol 1e-10 (the host-side NumPy reductions
    of the adaptive solver, np.add.at and einsum, may round differently on
    another CPU architecture; the fluxes themselves are bitwise)."""
    S, A = reference()
    a, steps = sessions(S)[name]
    with gpu_adaptive.gpu_leaf_fluxes(A):
        for k in range(steps):
            a.step()
            np.testing.assert_allclose(a.time, G[f"{name}|time"][k], rtol=1e-12)
            assert len(a.mesh.keys) == G[f"{name}|leaves"][k]
            np.testing.assert_allclose(a.boundary_integral, G[f"{name}|boundary"][k],
                                       rtol=1e-10, atol=1e-15)
    assert a.steps == int(G[f"{name}|steps"][0])
    np.testing.assert_array_equal(np.array(a.mesh.keys), G[f"{name}|keys"])
    np.testing.assert_allclose(a.state, G[f"{name}|state"], rtol=1e-10, atol=1e-15)


def test_adaptive_session_with_fp32_fluxes_tracks_reference():
    S, A = reference()
    a, steps = sessions(S)["explosion2d"]
    with gpu_adaptive.gpu_leaf_fluxes(A, precision="fp32"):
        for _ in range(steps):
            a.step()
    want = G["explosion2d|state"]
    if a.state.shape == want.shape:
        rel = np.sum(np.abs(a.state[0] - want[0])) / np.sum(np.abs(want[0]))
        assert rel <= 1e-5, rel
    assert abs(a.time - G["explosion2d|time"][-1]) <= 1e-5 * G["explosion2d|time"][-1]


def test_leaf_fluxes_match_the_reference_batches():
    """The batch function itself on the recorded adaptive batches."""
    R = np.load(ROOT / "tests" / "golden" / "rusanov.npz")
    for key in sorted({k.split("|")[0] for k in R.files if k.startswith("amr")}):
        got = gpu_adaptive.leaf_fluxes(R[f"{key}|left"], R[f"{key}|right"], R[f"{key}|gl"],
                                       R[f"{key}|gr"], int(R[f"{key}|dir"][0]))
        np.testing.assert_array_equal(got, R[f"{key}|flux"])
