"""Field output in TORCH's formats (python/cfdSolver/torchIO.py:122-733): the
writers reproduce, byte for byte, the files the reference's own write_vtk,
write_xdmf and TemporalWriter produced for the same session states
(tests/golden/output.npz, recorded by tests/golden/make_golden.py for
Cartesian 1D / 2D, a reactive spherical 2D and an annular 3D session; HDF5
files are compared dataset by dataset through the npz-backed h5py stand-in)."""

import json
from pathlib import Path

import numpy as np
import pytest

from torch_gb300 import output

GOLDEN = Path(__file__).resolve().parent / "golden"
G = np.load(GOLDEN / "output.npz")
CASES = ("vtr2d", "vts2d_znd", "vtr1d", "vts3d_annular")


def frame(key):
    config = json.loads(bytes(G[f"{key}|config"]).decode())
    time, steps = G[f"{key}|scalars"]
    lam = G[f"{key}|lam"] if f"{key}|lam" in G.files else None
    beta = G[f"{key}|beta"] if f"{key}|beta" in G.files else None
    return output.Frame.from_arrays(config, G[f"{key}|state"], lam, beta, float(time), int(steps),
                                    bytes(G[f"{key}|run_id"]).decode(), G[f"{key}|integrals"])


def reference_files(prefix):
    """{file name: bytes or {dataset: array}} recorded under prefix."""
    out = {}
    for k in G.files:
        if not k.startswith(prefix + "|file/"):
            continue
        rest = k[len(prefix) + len("|file/"):]
        if ".h5/" in rest:
            name, dataset = rest.split(".h5/", 1)
            out.setdefault(name + ".h5", {})[dataset] = G[k]
        else:
            out[rest] = bytes(G[k])
    return out


def compare(folder, expected):
    produced = {p.name for p in Path(folder).iterdir()}
    assert produced == set(expected), sorted(produced ^ set(expected))
    for name, want in expected.items():
        path = Path(folder) / name
        if isinstance(want, dict):
            with np.load(path) as z:
                got = {k.replace("|", "/"): z[k] for k in z.files}
            assert set(got) == set(want), name
            for dataset, value in want.items():
                np.testing.assert_array_equal(got[dataset], value, err_msg=f"{name}:{dataset}")
        else:
            assert path.read_bytes() == want, name


@pytest.mark.parametrize("case", CASES)
def test_series_matches_reference_files(case, fake_h5py, tmp_path):
    frames = [frame(f"{case}/frame{i}") for i in range(int(G[f"{case}|frames"][0]))]
    formats = ("vtk",) if case.startswith("vts2d") else ("vtk", "xdmf")
    writer = output.TemporalWriter(tmp_path / "series", frames[0], formats)
    for f in frames:
        writer.append(f)
    compare(tmp_path, reference_files(f"{case}/series"))


@pytest.mark.parametrize("case", CASES)
def test_snapshots_match_reference_files(case, fake_h5py, tmp_path):
    f = frame(f"{case}/single")
    output.write_vtk(tmp_path / ("snap" + (".vts" if "vts" in case else ".vtr")), f)
    output.write_xdmf(tmp_path / "snap.xdmf", f)
    compare(tmp_path, reference_files(f"{case}/single"))


def test_series_restart_guards(fake_h5py, tmp_path):
    frames = [frame(f"vtr2d/frame{i}") for i in range(3)]
    writer = output.TemporalWriter(tmp_path / "s", frames[0])
    writer.append(frames[0])
    writer.append(frames[1])
    again = output.TemporalWriter(tmp_path / "s", frames[1])  # a restart continues the series
    again.append(frames[2])
    assert [f["step"] for f in again.data["frames"]] == [0, 2, 3]
    with pytest.raises(ValueError, match="ahead"):
        output.TemporalWriter(tmp_path / "s", frames[0])
    other = frame("vtr2d/frame1")
    other.run_id = "another"
    with pytest.raises(ValueError, match="another run"):
        output.TemporalWriter(tmp_path / "s", other)
    with pytest.raises(ValueError):
        output.TemporalWriter(tmp_path / "t", frames[0], formats=("png",))
    with pytest.raises(ValueError):
        output.write_vtk(tmp_path / "x.vts", frames[0])
