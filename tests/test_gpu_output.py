"""Field output of GPU sessions: run(output_prefix=...) copies frames off
the GPU asynchronously and writes the same series the reference wrote for
the same runs (tests/golden/output.npz): VTK files, collections and the
manifest byte for byte, HDF5 datasets value for value, the metadata's
integrals (GPU sums, in another order than NumPy's) at 1e-12."""

import json
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU containers
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import torch_gb300  # noqa: E402
from torch_gb300 import output  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden"
G = np.load(GOLDEN / "output.npz")


def session(case):
    key = f"{case}/frame0"
    config = json.loads(bytes(G[f"{key}|config"]).decode())
    ints = G[f"{key}|integrals"]
    snap = SimpleNamespace(config=config, state=G[f"{key}|state"],
                           lam=G[f"{key}|lam"] if f"{key}|lam" in G.files else None,
                           beta=G[f"{key}|beta"] if f"{key}|beta" in G.files else None,
                           time=0.0, steps=0, initial_integral=ints[0], boundary_integral=ints[1],
                           source_integral=ints[2], run_id=bytes(G[f"{key}|run_id"]).decode())
    return torch_gb300.Simulation.from_session(snap)


@pytest.mark.parametrize("case", ["vtr2d", "vtr1d", "vts3d_annular"])
def test_gpu_series_matches_reference(case, fake_h5py, tmp_path):
    sim = session(case)
    sim.run(step_limit=3, output_prefix=tmp_path / "series", output_every=2)
    want = {}
    for k in G.files:
        prefix = f"{case}/series|file/"
        if k.startswith(prefix):
            want[k[len(prefix):]] = G[k]
    names = {p.name for p in tmp_path.iterdir()}
    assert names == {k.split(".h5/")[0] + ".h5" if ".h5/" in k else k for k in want}
    for name, value in want.items():
        if ".h5/" in name:
            file, dataset = name.split(".h5/", 1)
            with np.load(tmp_path / (file + ".h5")) as z:
                got = z[dataset.replace("/", "|")]
            if dataset == "metadata":
                mine, ref = json.loads(bytes(got).decode()), json.loads(bytes(value).decode())
                for key in ("current_integral", "boundary_integral", "source_integral"):
                    np.testing.assert_allclose(mine.pop(key), ref.pop(key), rtol=1e-12,
                                               atol=1e-15)  # GPU sums: another order
                assert mine == ref
            else:
                np.testing.assert_array_equal(got, value, err_msg=name)
        else:
            assert (tmp_path / name).read_bytes() == bytes(value), name


def test_async_frames_do_not_hold_the_gpu_and_match_a_synchronous_write(fake_h5py, tmp_path):
    p = np.ones((5, 16, 16, 16))
    p[4, :, :, :8] = 4.0
    sim = torch_gb300.Simulation(p, [1, 1, 1], t_end=1.0, precision="fp32")
    sim.run(step_limit=6, output_prefix=tmp_path / "a", output_every=3, formats=("vtk",))
    frame = output.Frame.capture(sim).wait()
    output.write_vtk(tmp_path / "check.vtr", frame)
    last = sorted(tmp_path.glob("a_*.vtr"))[-1]
    assert last.name == "a_00000006.vtr"
    assert last.read_bytes() == (tmp_path / "check.vtr").read_bytes()
    manifest = json.loads((tmp_path / "a.series.json").read_text())
    assert [f["step"] for f in manifest["frames"]] == [0, 3, 6]
