"""TORCH checkpoint interchange for GPU sessions.

A checkpoint (python/cfdSolver/torchIO.py:1-10, 66-119, 192-391) is an HDF5
file with a ``metadata`` dataset (UTF-8 JSON bytes: format, schema 2, solver
version, the session's config, run_id, time, steps and the four integrals)
and one flat float64 dataset per conservative component under ``state/``
(``rho``, ``momentum_x`` ..., ``energy``, x fastest), plus ``state/lambda``
and ``state/beta`` for reactive sessions.  This module builds exactly those
contents from any session object with the reference's attributes (the GPU
``Simulation`` included), parses and validates them back into a
``Snapshot`` that ``Simulation.from_session`` resumes, and reads / writes the
file through h5py when h5py is installed.  A GPU session saved here is read
by the reference's ``read_checkpoint`` and a reference checkpoint resumes on
the GPU.
"""

import json
import os
import tempfile
from pathlib import Path

import numpy as np

SCHEMA_VERSION = 2
SOLVER_VERSION = "1.4"
# schema / solver families the reference reads (torchIO.py:278-280)
READABLE_VERSIONS = ((1, "1.1"), (2, "1.2"), (2, "1.4"))


def coordinates(config):
    """Names of the logical coordinates (torchGeometry.py:12-27)."""
    dim = config["dimension"]
    g = config.get("geometry", "cartesian")
    if g == "cartesian":
        return list("xyz"[:dim])
    if g == "spherical":
        return ["r", "theta", "phi"][:dim]
    if g == "cylindrical" and dim == 2:
        return ["r", "z"]
    return ["r", "theta", "z"][:dim]


def component_names(config):
    """Dataset names of the conservative components (torchGeometry.py:30-31)."""
    return ["rho"] + ["momentum_" + a for a in coordinates(config)] + ["energy"]


def physical_state(state):
    """Finite, positive density and internal energy (torchSolver.py:1038-1046)."""
    return bool(np.isfinite(state).all() and np.all(state[0] > 1e-12) and np.all(
        state[-1] - 0.5 * np.sum(state[1:-1] ** 2, axis=0) / state[0] > 1e-12))


def _plain(value):
    if isinstance(value, np.ndarray):
        return value.tolist()
    if isinstance(value, np.generic):
        return value.item()
    raise TypeError(f"Cannot serialize {type(value).__name__}")


def encode(meta):
    """Compact JSON, NaN rejected: the byte form the reference writes."""
    return json.dumps(meta, default=_plain, allow_nan=False, separators=(",", ":")).encode("utf-8")


def _fraction_ok(values, shape):
    values = np.asarray(values, dtype=float)
    return values.shape == shape and np.isfinite(values).all() and \
        not np.any((values < 0) | (values > 1))


def metadata(session):
    """The metadata dictionary of a checkpoint of `session`, validated the
    way the reference validates before writing (torchIO.py:66-119)."""
    c = session.config
    dim = c["dimension"]
    state = np.asarray(session.state)
    shape = tuple(c["counts_xyz"][::-1])
    if state.shape != (dim + 2, *shape) or not physical_state(state):
        raise ValueError("Cannot save a nonphysical or mismatched state")
    time, steps = session.time, session.steps
    if (not np.isfinite(time) or not 0 <= time <= c["t_end"] or not isinstance(steps, int)
            or not 0 <= steps <= c["max_steps"]):
        raise ValueError("Cannot save invalid integration counters")
    if c["reactive"]:
        lam, beta = session.lam, session.beta
        if lam is None or (c["kinetic_model"] == "znd" and beta is None):
            raise ValueError("Missing reactive composition")
        if not _fraction_ok(lam, shape) or (c["kinetic_model"] == "znd"
                                            and not _fraction_ok(beta, shape)):
            raise ValueError("lambda / beta must have the spatial shape and values in [0,1]")
    integrals = [np.asarray(v, dtype=float) for v in (
        session.initial_integral, session.boundary_integral, session.source_integral)]
    for value in integrals:
        if value.shape != (dim + 2,) or not np.isfinite(value).all():
            raise ValueError("Cannot save invalid conservation balances")
    return dict(format="TORCH checkpoint", schema_version=SCHEMA_VERSION,
                solver_version=SOLVER_VERSION, geometry=c.get("geometry", "cartesian"),
                units="SI", layout="x-fastest", config=c, run_id=session.run_id, time=time,
                steps=steps, initial_integral=integrals[0], boundary_integral=integrals[1],
                source_integral=integrals[2], current_integral=np.asarray(session.integral))


def contents(session, visualization=False):
    """{dataset name: array} of a checkpoint: ``metadata`` as uint8 bytes and
    the flat little-endian float64 state datasets; with ``visualization``
    also the mesh points and cells and the derived fields that an XDMF file
    points at (torchIO.py:192-218)."""
    out = {"metadata": np.frombuffer(encode(metadata(session)), dtype=np.uint8)}
    state = np.asarray(session.state)
    for name, row in zip(component_names(session.config), state):
        out["state/" + name] = row.ravel().astype("<f8")
    for name, value in (("lambda", session.lam), ("beta", session.beta)):
        if value is not None:
            out["state/" + name] = np.asarray(value).ravel().astype("<f8")
    if visualization:
        from . import output
        _, points, cells = output.mesh(session)
        out["mesh/points"] = points.astype("<f8")
        out["mesh/cells"] = cells
        for name, value in output.fields(session).items():
            out["fields/" + name] = value.astype("<f8")
    return out


def atomic(path, write):
    """Replace `path` atomically: write a temporary file in the same
    directory, fsync it and rename it over the target (torchIO.py:49-63)."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    fd, temp = tempfile.mkstemp(prefix="." + path.name + ".", suffix=".tmp", dir=path.parent)
    os.close(fd)
    try:
        write(Path(temp))
        with open(temp, "rb") as handle:
            os.fsync(handle.fileno())
        os.replace(temp, path)
    finally:
        if os.path.exists(temp):
            os.unlink(temp)


class Snapshot:
    """A validated checkpoint: the session attributes the reference's
    read_checkpoint restores (config, state, lam, beta, time, steps, run_id,
    the three integrals), ready for ``Simulation.from_session``."""

    @property
    def integral(self):
        """Cell sums times the cell volume, or the sum of each cell times its
        own volume on metric grids (torchSession.py:284-294)."""
        c = self.config
        dim = c["dimension"]
        if c.get("geometry", "cartesian") != "cartesian":
            from .metric import factors
            volumes = np.ones(tuple(c["counts_xyz"][::-1]))
            for d, f in enumerate(factors(c)[0]):
                shape = [1] * dim
                shape[dim - 1 - d] = len(f)
                volumes *= np.asarray(f).reshape(shape)
            return (self.state * volumes[None]).reshape(dim + 2, -1).sum(axis=1)
        spacing = np.array(c["lengths_xyz"]) / c["counts_xyz"]
        return self.state.reshape(dim + 2, -1).sum(axis=1) * np.prod(spacing)

    @property
    def completed(self):
        return self.time == self.config["t_end"]


def parse(datasets):
    """Validate checkpoint contents the way the reference's reader does
    (torchIO.py:233-391, schemas 1 and 2) and return a Snapshot.  `datasets`
    maps names (``metadata``, ``state/<name>``) to arrays; every failure is a
    ValueError."""
    from .session import validate_config
    try:
        raw = np.asarray(datasets["metadata"])
        if raw.ndim != 1 or raw.dtype != np.dtype("uint8") or raw.size > 1_000_000:
            raise ValueError("Invalid checkpoint metadata encoding")
        meta = json.loads(raw.tobytes().decode("utf-8"))
        required = {"config", "time", "steps", "run_id", "initial_integral",
                    "boundary_integral", "source_integral", "current_integral"}
        if not isinstance(meta, dict) or not required.issubset(meta):
            raise ValueError("Incomplete checkpoint metadata")
        expected = dict(format="TORCH checkpoint", units="SI", layout="x-fastest")
        if any(meta.get(k) != v for k, v in expected.items()):
            raise ValueError("Unsupported checkpoint schema, solver version, geometry or units")
        version = (meta.get("schema_version"), meta.get("solver_version"))
        if version not in READABLE_VERSIONS:
            raise ValueError("Unsupported checkpoint schema/solver family")
        config = meta["config"]
        if version[0] == 1 and (meta.get("geometry") != "cartesian" or any(
                k in config for k in ("geometry", "origins_xyz", "face_boundaries"))):
            raise ValueError("Schema 1 only supports legacy Cartesian configurations")
        if version[0] == 2 and meta.get("geometry") != config.get("geometry", "cartesian"):
            raise ValueError("Checkpoint geometry/configuration mismatch")
        for key in ("counts_xyz", "lengths_xyz", "boundaries_xyz", "origins_xyz"):
            if key in config:
                config[key] = list(np.atleast_1d(config[key]))
        validate_config(config, strict_cfl=True)
        dim = config["dimension"]
        shape = tuple(config["counts_xyz"][::-1])
        size = int(np.prod(shape))

        def array(name):
            data = np.asarray(datasets["state/" + name])
            if data.shape != (size,) or data.dtype.kind != "f" or data.dtype.itemsize != 8:
                raise ValueError("Checkpoint dataset has incompatible shape or precision")
            return np.asarray(data, dtype=float).reshape(shape)

        snap = Snapshot()
        snap.config = config
        snap.state = np.stack([array(name) for name in component_names(config)])
        snap.lam = array("lambda") if config["reactive"] else None
        snap.beta = array("beta") if config["reactive"] and \
            config["kinetic_model"] == "znd" else None
        present = {k[len("state/"):] for k in datasets if k.startswith("state/")}
        wanted = set(component_names(config)) | ({"lambda"} if snap.lam is not None else set()) \
            | ({"beta"} if snap.beta is not None else set())
        if present != wanted:
            raise ValueError("Unexpected or missing composition datasets")
    except (OSError, KeyError, TypeError, UnicodeError, json.JSONDecodeError) as exc:
        raise ValueError(f"Invalid or incomplete TORCH checkpoint: {exc}") from exc
    snap.time, snap.steps, snap.run_id = meta["time"], meta["steps"], meta["run_id"]
    if (not isinstance(snap.run_id, str) or not snap.run_id
            or not isinstance(snap.time, (int, float)) or isinstance(snap.time, bool)
            or not np.isfinite(snap.time) or not 0 <= snap.time <= config["t_end"]):
        raise ValueError("Invalid checkpoint run identity or time")
    if (not isinstance(snap.steps, int) or isinstance(snap.steps, bool) or snap.steps < 0
            or snap.steps > config["max_steps"]):
        raise ValueError("Invalid checkpoint step counter")
    for name in ("initial_integral", "boundary_integral", "source_integral", "current_integral"):
        value = np.asarray(meta[name], dtype=float)
        if value.shape != (dim + 2,) or not np.isfinite(value).all():
            raise ValueError("Invalid integrated diagnostics")
        if name != "current_integral":
            setattr(snap, name, value)
        elif not np.allclose(value, snap.integral, rtol=1e-12, atol=1e-12):
            raise ValueError("Checkpoint state/integral mismatch")
    if not physical_state(snap.state) or snap.initial_integral[0] <= 0:
        raise ValueError("Nonphysical checkpoint state")
    for name, value in (("lambda", snap.lam), ("beta", snap.beta)):
        if value is not None and not _fraction_ok(value, shape):
            raise ValueError(f"{name} must have the spatial shape and values in [0,1]")
    return snap


def _h5py():
    try:
        import h5py
    except ImportError as exc:
        raise RuntimeError("TORCH checkpoint files are HDF5 and need h5py") from exc
    return h5py


def write(path, session, visualization=False):
    """Write a checkpoint atomically (temporary file in the same directory,
    fsync, rename), with Fletcher-32 checksums on the state datasets
    (torchIO.py:49-63, 192-230).  Returns the path as a string."""
    data = contents(session, visualization)  # validate before touching the file system
    h5py = _h5py()

    def dump(temp):
        with h5py.File(temp, "w") as handle:
            for name, value in data.items():
                if name.startswith("state/"):
                    handle.create_dataset(name, data=value, fletcher32=True)
                else:
                    handle.create_dataset(name, data=value)
            handle.flush()

    atomic(path, dump)
    return str(path)


def read(path):
    """Read and validate a checkpoint file into a Snapshot."""
    h5py = _h5py()
    try:
        with h5py.File(path, "r") as handle:
            datasets = {"metadata": np.asarray(handle["metadata"])}
            for name in handle["state"]:
                datasets["state/" + name] = np.asarray(handle["state/" + name])
    except (OSError, KeyError, TypeError) as exc:
        raise ValueError(f"Invalid or incomplete TORCH checkpoint: {exc}") from exc
    return parse(datasets)
