"""Checkpoint interchange on the GPU session: reference checkpoints (written
by the reference's own write_checkpoint after 4 steps, tests/golden/
checkpoint.npz) resume on the GPU and continue onto the reference's own
trajectory; a GPU session's checkpoint holds the same datasets and passes
the reference reader's checks; and a restart from a checkpoint is exact in
every dimension and chemistry model (python/tests/testSession.py:81-126).
Inert FP64 results are compared bitwise; reactive ones at the relative
tolerance 1e-10 of the reactive parity tests (CUDA's and NumPy's exp differ
in the last bit).  The metric sessions among them (a cylindrical grid with a
wall at the origin, a Cartesian grid with per-face boundaries, a reactive
spherical shell) resume on the metric engine."""

import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import torch_gb300  # noqa: E402
from torch_gb300 import checkpoint  # noqa: E402
from oracle.session import OracleSimulation  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ("s3d_explosion", "s3d_open_albada", "s2d_explosion", "s1d_sod", "s3d_ignition_znd",
         "s3d_ignition_arr", "s2d_reactive", "s1d_reactive_znd", "m2d_cylindrical_origin",
         "m3d_cartesian_faces", "m2d_spherical_reactive")


def golden(name):
    g = np.load(GOLDEN / "checkpoint.npz")
    saved = {k.split("|", 1)[1]: g[k] for k in g.files
             if k.startswith(name + "|") and "|final/" not in k}
    final = {k.split("|final/", 1)[1]: g[k] for k in g.files if k.startswith(name + "|final/")}
    return saved, final


def same(a, b, reactive, what):
    if reactive:
        np.testing.assert_allclose(a, b, rtol=1e-10, atol=1e-14 * np.abs(b).max(), err_msg=what)
    else:
        np.testing.assert_array_equal(a, b, err_msg=what)


@pytest.mark.parametrize("name", CASES)
def test_reference_checkpoint_resumes_onto_reference_trajectory(name):
    saved, final = golden(name)
    snap = checkpoint.parse(saved)
    sim = torch_gb300.Simulation.from_session(snap)
    reactive = snap.config["reactive"]
    # the GPU session's own checkpoint: same datasets, metadata the reference reader accepts
    ours = checkpoint.contents(sim)
    assert set(ours) == set(saved)
    for key in saved:
        if key != "metadata":
            np.testing.assert_array_equal(ours[key], saved[key], err_msg=key)
    mine, theirs = (json.loads(bytes(d["metadata"]).decode()) for d in (ours, saved))
    np.testing.assert_allclose(mine.pop("current_integral"), theirs.pop("current_integral"),
                               rtol=1e-12, atol=1e-12)
    assert mine == theirs
    checkpoint.parse(ours)
    # 4 more steps reach the reference's state after 8
    for _ in range(4):
        sim.step()
    assert sim.steps == int(final["scalars"][1]) == 8
    assert sim.time == pytest.approx(final["scalars"][0], rel=0 if not reactive else 1e-12)
    same(sim.state, final["state"], reactive, "state")
    for key in ("lam", "beta"):
        if key in final:
            same(getattr(sim, key), final[key], True, key)
    np.testing.assert_array_equal(sim.initial_integral, final["initial"])
    np.testing.assert_allclose(sim.boundary_integral, final["boundary"], rtol=1e-10,
                               atol=1e-13 * np.abs(final["initial"]).max())
    np.testing.assert_allclose(sim.source_integral, final["source"], rtol=1e-8, atol=1e-6)


def example(dim, reactive=False, model="arrhenius", **kw):
    """The restart test's sessions (python/tests/testSession.py:37-52)."""
    counts = [24] if dim == 1 else ([8, 6] if dim == 2 else [6, 4, 4])
    p = np.ones((dim + 2, *counts[::-1]))
    p[1:-1] = 0.2
    x = (np.arange(counts[0]) + 0.5) / counts[0]
    p[0] = 1 + 0.1 * np.sin(2 * np.pi * x)
    p[-1] = np.where(x < 0.5, 1e6, 101325) if reactive else 1
    return torch_gb300.Simulation(p, [1.0] * dim, t_end=1e-4 if reactive else 0.08,
                                  boundaries=["Periodic"] * dim, reactive=reactive,
                                  kinetic_model=model, **kw)


@pytest.mark.parametrize("dim", (1, 2, 3))
@pytest.mark.parametrize("model", ("inert", "arrhenius", "znd"))
def test_restart_is_exact_in_all_dimensions_and_models(dim, model, fake_h5py, tmp_path):
    make = lambda: example(dim, model != "inert", "arrhenius" if model == "inert" else model)
    continuous = make().run()
    a = make()
    path = tmp_path / "checkpoint.h5"
    a.run(step_limit=2, checkpoint=path)
    assert not a.completed and a.steps == 2
    restarted = torch_gb300.Simulation.load(path).run()
    np.testing.assert_array_equal(restarted.state, continuous.state)
    for key in ("lam", "beta", "boundary_integral", "source_integral", "initial_integral"):
        if getattr(continuous, key) is not None:
            np.testing.assert_array_equal(getattr(restarted, key), getattr(continuous, key))
    assert (restarted.steps, restarted.time) == (continuous.steps, continuous.time)
    assert restarted.run_id == a.run_id


def test_run_writes_checkpoints_on_schedule(fake_h5py, tmp_path, monkeypatch):
    written = []
    original = torch_gb300.Simulation.save

    def save(self, path):
        written.append(self.steps)
        return original(self, path)

    monkeypatch.setattr(torch_gb300.Simulation, "save", save)
    p = np.ones((3, 64))
    p[:, 32:] = np.array([0.125, 0.0, 0.1])[:, None]
    p[1, :32] = 0.0
    s = torch_gb300.Simulation(p, [1.0], t_end=0.1)
    s.run(checkpoint=tmp_path / "c.h5", checkpoint_every=3, chunk=8)
    assert s.completed and s.steps > 6
    assert written == [k for k in range(3, s.steps + 1, 3)] + [s.steps]
    back = checkpoint.read(tmp_path / "c.h5")
    assert back.steps == s.steps and back.time == s.time
    np.testing.assert_array_equal(back.state, s.state)
    with pytest.raises(ValueError):
        s.run(checkpoint_every=2)


def test_load_with_later_end_time_and_fp32(fake_h5py, tmp_path):
    s = example(3)
    s.run(step_limit=2, checkpoint=tmp_path / "c.h5")
    assert not s.completed
    with pytest.raises(ValueError):
        torch_gb300.Simulation.load(tmp_path / "c.h5", t_end=s.time / 2)
    longer = torch_gb300.Simulation.load(tmp_path / "c.h5", t_end=0.12).run()
    assert longer.time == 0.12 and longer.config["t_end"] == 0.12
    fp64 = torch_gb300.Simulation.load(tmp_path / "c.h5").run()
    fp32 = torch_gb300.Simulation.load(tmp_path / "c.h5", precision="fp32").run()
    assert fp32.time == fp64.time
    assert np.mean(np.abs(fp32.state - fp64.state)) < 1e-5


def test_oracle_session_continues_on_the_gpu():
    """A session advanced on the host oracle hands over mid-run: the GPU
    continues onto the oracle's own trajectory, bit for bit."""
    rng = np.random.default_rng(7)
    p = np.ones((5, 6, 7, 8))
    p[0] = 1 + 0.3 * rng.random((6, 7, 8))
    p[1:4] = 0.3 * rng.standard_normal((3, 6, 7, 8))
    p[4] = 1 + rng.random((6, 7, 8))
    kw = dict(t_end=0.05, limiter="Unos", boundaries=["Open", "Periodic", "Reflective"])
    host = OracleSimulation(p, [1.0, 0.9, 0.8], **kw)
    for _ in range(3):
        host.step()
    gpu = torch_gb300.Simulation.from_session(host)
    assert gpu.steps == 3 and gpu.time == host.time
    for _ in range(4):
        host.step()
        gpu.step()
    np.testing.assert_array_equal(gpu.state, host.state)
    assert gpu.time == host.time
    np.testing.assert_allclose(gpu.boundary_integral, host.boundary_integral, rtol=1e-10,
                               atol=1e-14)
