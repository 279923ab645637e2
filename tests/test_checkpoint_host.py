"""Checkpoint interchange on the host: the reference's own checkpoints
(written by python/cfdSolver/torchIO.py write_checkpoint after 4 steps of
seeded Cartesian and metric sessions, tests/golden/make_golden.py) parse into snapshots that
re-encode byte for byte, corrupt files are rejected like the reference's
reader rejects them (python/tests/testSession.py:55-79, 192-261), and files
are replaced atomically.  h5py is not installed, so an npz-backed stand-in
(conftest.fake_h5py) carries the datasets."""

import json
from pathlib import Path

import numpy as np
import pytest

from torch_gb300 import checkpoint

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ("s3d_explosion", "s3d_open_albada", "s2d_explosion", "s1d_sod", "s3d_ignition_znd",
         "s3d_ignition_arr", "s2d_reactive", "s1d_reactive_znd", "m2d_cylindrical_origin",
         "m3d_cartesian_faces", "m2d_spherical_reactive")


def reference_checkpoint(name):
    g = np.load(GOLDEN / "checkpoint.npz")
    return {k.split("|", 1)[1]: g[k] for k in g.files
            if k.startswith(name + "|") and "|final/" not in k}


def meta_of(datasets):
    return json.loads(bytes(datasets["metadata"]).decode())


def with_meta(datasets, meta):
    out = dict(datasets)
    out["metadata"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    return out


@pytest.mark.parametrize("name", CASES)
def test_reference_checkpoint_parses_and_reencodes_byte_identical(name):
    ref = reference_checkpoint(name)
    snap = checkpoint.parse(ref)
    meta = meta_of(ref)
    assert snap.steps == meta["steps"] == 4 and snap.time == meta["time"]
    assert snap.run_id == meta["run_id"]
    assert (snap.lam is not None) == snap.config["reactive"]
    ours = checkpoint.contents(snap)
    assert set(ours) == set(ref)
    assert bytes(ours["metadata"]) == bytes(ref["metadata"])
    for key, value in ref.items():
        assert ours[key].dtype == np.dtype("<f8") or key == "metadata"
        np.testing.assert_array_equal(ours[key], value)


def test_solver_family_12_is_read_and_upgraded_on_write():
    ref = reference_checkpoint("s1d_sod")
    meta = meta_of(ref)
    meta["solver_version"] = "1.2"
    snap = checkpoint.parse(with_meta(ref, meta))
    assert meta_of(checkpoint.contents(snap))["solver_version"] == "1.4"


MUTATIONS = {
    "version": lambda d, m: m.update(schema_version=999),
    "solver": lambda d, m: m.update(solver_version="0.9"),
    "format": lambda d, m: m.update(format="other"),
    "time": lambda d, m: m.update(time=-1),
    "time_after_end": lambda d, m: m.update(time=m["config"]["t_end"] * 2),
    "invalid_time": lambda d, m: m.update(time="invalid"),
    "bool_steps": lambda d, m: m.update(steps=True),
    "steps_over_max": lambda d, m: m.update(steps=m["config"]["max_steps"] + 1),
    "geometry": lambda d, m: m.update(geometry="spherical"),
    "missing_metadata": lambda d, m: m.pop("time"),
    "integral": lambda d, m: m["current_integral"].__setitem__(0, m["current_integral"][0] + 1),
    "integral_shape": lambda d, m: m["boundary_integral"].append(0.0),
    "run_id": lambda d, m: m.update(run_id=""),
    "limiter": lambda d, m: m["config"].update(limiter="Minmod"),
    "boundary": lambda d, m: m["config"].update(boundaries_xyz=["Inflow"] * 3),
    "nan": lambda d, m: d["state/rho"].__setitem__(0, np.nan),
    "negative_density": lambda d, m: d["state/rho"].__setitem__(0, -1.0),
    "precision": lambda d, m: d.__setitem__("state/rho", d["state/rho"].astype(np.float32)),
    "missing": lambda d, m: d.pop("state/energy"),
    "extra": lambda d, m: d.__setitem__("state/lambda", np.zeros_like(d["state/rho"])),
    "shape": lambda d, m: d.__setitem__("state/rho", d["state/rho"][:-1]),
}


@pytest.mark.parametrize("mutation", sorted(MUTATIONS))
def test_corrupt_checkpoints_are_rejected(mutation):
    ref = {k: np.array(v) for k, v in reference_checkpoint("s3d_explosion").items()}
    meta = meta_of(ref)
    MUTATIONS[mutation](ref, meta)
    with pytest.raises(ValueError):
        checkpoint.parse(with_meta(ref, meta))


def test_reactive_composition_is_validated():
    ref = {k: np.array(v) for k, v in reference_checkpoint("s3d_ignition_znd").items()}
    ref["state/beta"][3] = 1.5
    with pytest.raises(ValueError):
        checkpoint.parse(ref)
    ref = {k: np.array(v) for k, v in reference_checkpoint("s3d_ignition_znd").items()}
    del ref["state/beta"]
    with pytest.raises(ValueError):
        checkpoint.parse(ref)


def test_write_read_round_trip_and_atomic_replace(fake_h5py, tmp_path, monkeypatch):
    snap = checkpoint.parse(reference_checkpoint("s3d_ignition_znd"))
    target = tmp_path / "run" / "c.h5"
    assert checkpoint.write(target, snap) == str(target)
    back = checkpoint.read(target)
    for key in ("state", "lam", "beta", "initial_integral", "boundary_integral",
                "source_integral"):
        np.testing.assert_array_equal(getattr(back, key), getattr(snap, key))
    assert (back.time, back.steps, back.run_id) == (snap.time, snap.steps, snap.run_id)
    original = target.read_bytes()
    # a failing write leaves the previous checkpoint and no temporary file
    def fail(*a, **k):
        raise RuntimeError("write failed")
    create = fake_h5py.File.create_dataset
    monkeypatch.setattr(fake_h5py.File, "create_dataset", fail)
    with pytest.raises(RuntimeError):
        checkpoint.write(target, snap)
    assert target.read_bytes() == original
    assert [p.name for p in target.parent.iterdir()] == ["c.h5"]
    # an invalid session is refused before the file system is touched
    monkeypatch.setattr(fake_h5py.File, "create_dataset", create)
    snap.time = -1.0
    with pytest.raises(ValueError):
        checkpoint.write(tmp_path / "other.h5", snap)
    assert not (tmp_path / "other.h5").exists()


def test_missing_h5py_is_a_clear_error(monkeypatch, tmp_path):
    import sys
    monkeypatch.setitem(sys.modules, "h5py", None)
    snap = checkpoint.parse(reference_checkpoint("s1d_sod"))
    with pytest.raises(RuntimeError, match="h5py"):
        checkpoint.write(tmp_path / "c.h5", snap)
    with pytest.raises(RuntimeError, match="h5py"):
        checkpoint.read(tmp_path / "c.h5")
