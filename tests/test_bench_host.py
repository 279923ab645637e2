"""Host-side pieces of bench.py (no GPU): the error and drift arithmetic of
the precision comparisons, the NUMA helpers of the end-to-end leg, and the
loader of the reference's own CPU step."""

import os
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_pressure_of_a_conserved_state():
    rho, u, v, w, p = 1.3, 0.4, -0.2, 0.1, 2.5
    E = p / 0.4 + 0.5 * rho * (u * u + v * v + w * w)
    state = torch.tensor([rho, rho * u, rho * v, rho * w, E], dtype=torch.float64)
    assert abs(float(bench.pressure(state, 1.4)) - p) < 1e-12
    state2d = torch.tensor([rho, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v)],
                           dtype=torch.float64)
    assert abs(float(bench.pressure(state2d, 1.4)) - p) < 1e-12


def test_state_errors_and_summary():
    a = torch.ones((5, 2, 3, 4), dtype=torch.float64)
    a[1:4] = 0.0  # at rest
    a[4] = 2.5 / 0.4
    b = a.clone()
    b[0, 0, 0, 0] += 1e-3  # density only: the pressure changes by 0 (no momentum)
    e = bench.state_errors(a, b)
    assert e["linf_rho"] == pytest.approx(1e-3)
    assert e["l1_rho"] == pytest.approx(1e-3 / 24)
    assert e["linf_p"] == pytest.approx(0.0, abs=1e-15)
    s = bench.error_summary([e, dict(e, l1_rho=2.0)])
    assert s["l1_rho_max"] == 2.0 and s["l1_rho_median"] == pytest.approx((2.0 + e["l1_rho"]) / 2)


def test_node_cpus_parses_sysfs_lists(tmp_path, monkeypatch):
    cpus = bench.node_cpus(0)
    if os.path.exists("/sys/devices/system/node/node0/cpulist"):
        assert cpus and all(isinstance(c, int) for c in cpus)
    assert bench.node_cpus(10 ** 6) == set()


def test_pages_by_node_finds_the_mapping_of_an_allocation():
    x = np.ones(1 << 20)
    counts = bench.pages_by_node(x.ctypes.data)
    if os.path.exists("/proc/self/numa_maps"):
        assert sum(counts.values()) > 0


def test_near_gpu_memory_restores_the_affinity():
    before = os.sched_getaffinity(0)
    block = bench.near_gpu_memory(0)
    with block:
        pass
    assert os.sched_getaffinity(0) == before


def test_reference_modules_load_the_installed_reference():
    R = bench.reference_modules()
    if R is None:
        pytest.skip("the reference is not installed in baseline/_ref")
    assert hasattr(R.session, "Simulation") and hasattr(R.adaptive, "rusanov")
