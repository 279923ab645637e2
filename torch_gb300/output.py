"""Field output of GPU sessions: VTK and XDMF snapshots and temporal series
in TORCH's file formats (python/cfdSolver/torchIO.py:122-733).

* ``write_vtk``: cell-centred VTK XML, RectilinearGrid (``.vtr``) for
  Cartesian grids, StructuredGrid (``.vts``) with mapped points for curved
  ones, every value written with 17 significant digits;
* ``write_xdmf``: an XDMF 3 file whose heavy data is a checkpoint with the
  mesh and derived fields added (HDF5, needs h5py);
* ``TemporalWriter``: immutable frames, a ``.pvd`` collection, a temporal
  ``.xdmf`` collection and a JSON manifest that guards restarts.

Writers take any object with the session's attributes.  For a GPU session,
``Frame.capture`` copies the state (and fractions) to pinned host memory
with a device-to-host copy enqueued on the session's stream, so the GPU keeps
stepping while a background thread formats the frame (``AsyncWriter``).
"""

import json
import queue
import threading
from pathlib import Path
from xml.etree import ElementTree as ET

import numpy as np

from .checkpoint import atomic, component_names, coordinates, encode
from .checkpoint import write as write_checkpoint
from .metric import axes as grid_axes

SERIES_SCHEMA = 1


# -- geometry of the output mesh (torchGeometry.py:205-251, torchIO.py:122-161) --
def map_points(c, points):
    """Logical coordinates to Cartesian positions."""
    g, dim = c.get("geometry", "cartesian"), c["dimension"]
    out = points.copy()
    if g == "cartesian" or dim == 1:
        return out
    r, theta = points[:, 0], points[:, 1]
    if g == "spherical":
        phi = points[:, 2] if dim == 3 else np.zeros(len(points))
        out[:, 0] = r * np.sin(theta) * np.cos(phi)
        out[:, 1] = r * np.sin(theta) * np.sin(phi)
        out[:, 2] = r * np.cos(theta)
    elif g == "cylindrical" and dim == 2:
        out[:, 0], out[:, 1], out[:, 2] = r, 0.0, theta
    else:
        out[:, 0], out[:, 1] = r * np.cos(theta), r * np.sin(theta)
    return out


def cartesian_velocity(c, primitive):
    dim, g = c["dimension"], c.get("geometry", "cartesian")
    local = [primitive[k + 1] for k in range(dim)] + [np.zeros_like(primitive[0])] * (3 - dim)
    if g == "cartesian" or dim == 1:
        return local
    centers = [(a[:-1] + a[1:]) / 2 for a in grid_axes(c)]
    grids = np.meshgrid(*centers[::-1], indexing="ij")[::-1]
    if g == "cylindrical" and dim == 2:
        return [local[0], np.zeros_like(local[0]), local[1]]
    theta = grids[1]
    if g == "spherical":
        phi = grids[2] if dim == 3 else 0.0
        vr, vt, vp = local
        return [(vr * np.sin(theta) + vt * np.cos(theta)) * np.cos(phi) - vp * np.sin(phi),
                (vr * np.sin(theta) + vt * np.cos(theta)) * np.sin(phi) + vp * np.cos(phi),
                vr * np.cos(theta) - vt * np.sin(theta)]
    vr, vt, vz = local
    return [vr * np.cos(theta) - vt * np.sin(theta), vr * np.sin(theta) + vt * np.cos(theta), vz]


def mesh(session):
    """(axes, points, cells) of the cell-centred output mesh."""
    c = session.config
    dim = c["dimension"]
    counts = c["counts_xyz"]
    axes = grid_axes(c) + [np.array([0.0])] * (3 - dim)
    zz, yy, xx = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    points = np.column_stack((xx.ravel(), yy.ravel(), zz.ravel()))
    nx = counts[0]
    ny = counts[1] if dim >= 2 else 1
    nz = counts[2] if dim == 3 else 1
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    base = (i + (nx + 1) * (j + (counts[1] + 1 if dim >= 2 else 1) * k)).ravel()
    if dim == 1:
        offsets = [0, 1]
    elif dim == 2:
        offsets = [0, 1, nx + 2, nx + 1]
    else:
        plane = (nx + 1) * (ny + 1)
        offsets = [0, 1, nx + 2, nx + 1, plane, plane + 1, plane + nx + 2, plane + nx + 1]
    cells = base[:, None] + offsets
    return axes, map_points(c, points), cells.astype(np.int64)


def fields(session):
    """Conservative components, pressure, velocities (and Cartesian
    velocities on curved grids), fractions; flat, x fastest."""
    c = session.config
    dim = c["dimension"]
    prim = session.primitive
    out = {name: row.ravel() for name, row in zip(component_names(c), session.state)}
    out["pressure"] = prim[-1].ravel()
    names = coordinates(c)
    for d in range(dim):
        out["velocity_" + names[d]] = prim[d + 1].ravel()
    if c.get("geometry", "cartesian") != "cartesian":
        for name, value in zip("xyz", cartesian_velocity(c, prim)):
            out["velocity_cartesian_" + name] = value.ravel()
    if session.lam is not None:
        out["lambda"] = session.lam.ravel()
    if session.beta is not None:
        out["beta"] = session.beta.ravel()
    return out


# -- XML writers (torchIO.py:394-579) ------------------------------------------
def _text(values):
    return " ".join(format(v, ".17g") for v in values)


def _xml(path, root):
    ET.indent(root)
    atomic(path, lambda temp: ET.ElementTree(root).write(temp, encoding="utf-8",
                                                         xml_declaration=True))


def _time_field(parent, time):
    ET.SubElement(parent, "DataArray", type="Float64", Name="TimeValue", NumberOfTuples="1",
                  format="ascii").text = format(time, ".17g")


def _cell_data(piece, session):
    cell = ET.SubElement(piece, "CellData", Scalars="rho")
    for name, value in fields(session).items():
        ET.SubElement(cell, "DataArray", type="Float64", Name=name,
                      format="ascii").text = _text(value)


def write_vtk(path, session):
    """Cell-centred VTK XML snapshot: .vtr (Cartesian) or .vts (curved)."""
    c = session.config
    dim = c["dimension"]
    extent = " ".join(f"0 {n}" for n in c["counts_xyz"]) + " 0 0" * (3 - dim)
    if c.get("geometry", "cartesian") != "cartesian":
        if Path(path).suffix.lower() != ".vts":
            raise ValueError("Curved grids require .vts structured VTK output")
        root = ET.Element("VTKFile", type="StructuredGrid", version="1.0",
                          byte_order="LittleEndian")
        grid = ET.SubElement(root, "StructuredGrid", WholeExtent=extent)
        _time_field(ET.SubElement(grid, "FieldData"), session.time)
        piece = ET.SubElement(grid, "Piece", Extent=extent)
        _cell_data(piece, session)
        points = ET.SubElement(piece, "Points")
        ET.SubElement(points, "DataArray", type="Float64", NumberOfComponents="3",
                      format="ascii").text = _text(mesh(session)[1].ravel())
        _xml(path, root)
        return str(path)
    if Path(path).suffix.lower() != ".vtr":
        raise ValueError("VTK rectilinear output requires a .vtr path")
    axes = grid_axes(c) + [np.array([0.0])] * (3 - dim)
    root = ET.Element("VTKFile", type="RectilinearGrid", version="1.0",
                      byte_order="LittleEndian")
    grid = ET.SubElement(root, "RectilinearGrid", WholeExtent=extent)
    piece = ET.SubElement(grid, "Piece", Extent=extent)
    _cell_data(piece, session)
    data = ET.Element("FieldData")
    grid.insert(0, data)
    _time_field(data, session.time)
    coords = ET.SubElement(piece, "Coordinates")
    for axis, value in zip("xyz", axes):
        ET.SubElement(coords, "DataArray", type="Float64", Name=axis,
                      format="ascii").text = _text(value)
    _xml(path, root)
    return str(path)


def _xdmf_grid(parent, filename, time, dimension, counts, names):
    n = int(np.prod(counts))
    points = int(np.prod(np.array(counts) + 1))
    nodes = {1: 2, 2: 4, 3: 8}[dimension]
    grid = ET.SubElement(parent, "Grid", Name=Path(filename).stem, GridType="Uniform")
    ET.SubElement(grid, "Time", Value=format(time, ".17g"))
    topology = ET.SubElement(grid, "Topology",
                             TopologyType={1: "Polyline", 2: "Quadrilateral",
                                           3: "Hexahedron"}[dimension],
                             NumberOfElements=str(n), NodesPerElement=str(nodes))
    ET.SubElement(topology, "DataItem", Dimensions=f"{n} {nodes}", NumberType="Int",
                  Precision="8", Format="HDF").text = filename + ":/mesh/cells"
    geometry = ET.SubElement(grid, "Geometry", GeometryType="XYZ")
    ET.SubElement(geometry, "DataItem", Dimensions=f"{points} 3", NumberType="Float",
                  Precision="8", Format="HDF").text = filename + ":/mesh/points"
    for name in names:
        attribute = ET.SubElement(grid, "Attribute", Name=name, AttributeType="Scalar",
                                  Center="Cell")
        ET.SubElement(attribute, "DataItem", Dimensions=str(n), NumberType="Float",
                      Precision="8", Format="HDF").text = filename + ":/fields/" + name
    return grid


def write_xdmf(path, session):
    """XDMF snapshot; its HDF5 heavy data doubles as a checkpoint."""
    path = Path(path)
    if path.suffix.lower() not in (".xdmf", ".xmf"):
        raise ValueError("XDMF output requires .xdmf or .xmf")
    hdf = path.with_suffix(".h5")
    write_checkpoint(hdf, session, visualization=True)
    root = ET.Element("Xdmf", Version="3.0")
    domain = ET.SubElement(root, "Domain")
    grid = _xdmf_grid(domain, hdf.name, session.time, session.config["dimension"],
                      session.config["counts_xyz"], fields(session))
    grid.remove(grid.find("Time"))  # static readers: the time is in the HDF5 metadata
    _xml(path, root)
    return str(path), str(hdf)


class TemporalWriter:
    """Frames of one run: ``<prefix>_<step>.vtr|vts`` and ``.h5``, the
    ``.pvd`` and ``.xdmf`` collections and the ``.series.json`` manifest
    (torchIO.py:581-733).  Reopening a prefix continues its series after a
    restart and refuses another run's series."""

    def __init__(self, prefix, session, formats=("vtk", "xdmf")):
        curved = session.config.get("geometry", "cartesian") != "cartesian"
        self.vtk_extension = ".vts" if curved else ".vtr"
        self.prefix = Path(prefix)
        self.manifest = Path(str(prefix) + ".series.json")
        self.formats = tuple(formats)
        if not self.formats or set(self.formats) - {"vtk", "xdmf"}:
            raise ValueError("Formats must be vtk and/or xdmf")
        if self.manifest.exists():
            self.data = json.loads(self.manifest.read_text())
            if self.data["run_id"] != session.run_id or self.data["formats"] != list(self.formats):
                raise ValueError("Output prefix belongs to another run or format selection")
            if self.data.get("schema_version") != SERIES_SCHEMA:
                raise ValueError("Unsupported output manifest version")
            for key in ("counts_xyz", "lengths_xyz", "boundaries_xyz", "origins_xyz"):
                if key in self.data["config"]:
                    self.data["config"][key] = list(np.atleast_1d(self.data["config"][key]))
            previous_time, previous_step = -1.0, -1
            for frame in self.data["frames"]:
                if frame["time"] <= previous_time or frame["step"] <= previous_step:
                    raise ValueError("Output series has nonmonotone frames")
                previous_time, previous_step = frame["time"], frame["step"]
                for fmt in self.formats:
                    suffix = self.vtk_extension if fmt == "vtk" else ".h5"
                    if not (self.prefix.parent / (frame["stem"] + suffix)).is_file():
                        raise ValueError("Output series references a missing frame")
            for key in session.config:
                if key not in ("t_end", "max_steps") and \
                        self.data["config"][key] != json.loads(encode(session.config[key])):
                    raise ValueError("Output series configuration mismatch")
            if self.data["frames"] and self.data["frames"][-1]["time"] > session.time:
                raise ValueError("Series is ahead of checkpoint; choose a new output prefix")
        else:
            self.data = dict(schema_version=SERIES_SCHEMA, run_id=session.run_id,
                             formats=list(self.formats),
                             config=json.loads(encode(session.config)), frames=[])

    def append(self, session):
        frames = self.data["frames"]
        if frames and frames[-1]["time"] == session.time:
            if frames[-1]["step"] != session.steps:
                raise ValueError("Duplicate series time at a different step")
            return
        stem = self.prefix.name + f"_{session.steps:08d}"
        parent = self.prefix.parent
        parent.mkdir(parents=True, exist_ok=True)
        if "vtk" in self.formats:
            write_vtk(parent / (stem + self.vtk_extension), session)
        if "xdmf" in self.formats:
            write_checkpoint(parent / (stem + ".h5"), session, visualization=True)
        frames.append(dict(time=session.time, step=session.steps, stem=stem,
                           fields=list(fields(session))))
        if "vtk" in self.formats:
            root = ET.Element("VTKFile", type="Collection", version="1.0",
                              byte_order="LittleEndian")
            collection = ET.SubElement(root, "Collection")
            for frame in frames:
                ET.SubElement(collection, "DataSet", timestep=format(frame["time"], ".17g"),
                              group="", part="0", file=frame["stem"] + self.vtk_extension)
            _xml(str(self.prefix) + ".pvd", root)
        if "xdmf" in self.formats:
            root = ET.Element("Xdmf", Version="3.0")
            domain = ET.SubElement(root, "Domain")
            collection = ET.SubElement(domain, "Grid", Name="TORCH", GridType="Collection",
                                       CollectionType="Temporal")
            for frame in frames:
                _xdmf_grid(collection, frame["stem"] + ".h5", frame["time"],
                           session.config["dimension"], session.config["counts_xyz"],
                           frame["fields"])
            _xml(str(self.prefix) + ".xdmf", root)
        atomic(self.manifest, lambda temp: temp.write_bytes(encode(self.data)))


# -- asynchronous frames of GPU sessions ---------------------------------------
class Frame:
    """A host snapshot of a session at one step: the session's attributes
    with the state and fractions in pinned host memory, filled by copies
    enqueued on the session's stream (``capture``); ``wait`` blocks until they
    have landed."""

    def __init__(self):
        self._event = None

    @classmethod
    def capture(cls, sim):
        import torch
        f = cls()
        eng = sim._engine
        eng.refresh()
        f.config = json.loads(encode(sim.config))
        f.run_id = sim.run_id
        f.time, f.steps = sim.time, sim.steps
        f.initial_integral = sim.initial_integral
        f.boundary_integral = sim.boundary_integral
        f.source_integral = sim.source_integral
        f.integral = sim.integral
        f._gamma = sim.config["gamma"]
        f._reactive = sim.config["reactive"] and getattr(sim, "_closure", "si") == "si"
        with torch.cuda.stream(eng.stream):
            def host(t):
                if t is None:
                    return None
                h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
                h.copy_(t, non_blocking=True)
                return h
            f._state = host(eng.current())
            f._lam = host(eng.current_lam())
            f._beta = host(eng.current_beta())
            f._event = torch.cuda.Event()
            f._event.record(eng.stream)
        return f

    @classmethod
    def from_arrays(cls, config, state, lam, beta, time, steps, run_id, integrals):
        """A frame of host arrays (integral as the reference computes it)."""
        from .checkpoint import Snapshot
        snap = Snapshot()
        snap.config, snap.state = config, np.asarray(state, dtype=float)
        f = cls()
        f.config, f.run_id, f.time, f.steps = config, run_id, float(time), int(steps)
        f.state = snap.state
        f.lam = None if lam is None else np.asarray(lam, dtype=float)
        f.beta = None if beta is None else np.asarray(beta, dtype=float)
        f.initial_integral, f.boundary_integral, f.source_integral = (
            np.asarray(v, dtype=float) for v in integrals)
        f.integral = snap.integral
        f._gamma = config["gamma"]
        f._reactive = bool(config["reactive"])
        return f

    def wait(self):
        if self._event is not None:
            self._event.synchronize()
            self.state = self._state.numpy().astype(np.float64)
            self.lam = None if self._lam is None else self._lam.numpy().astype(np.float64)
            self.beta = None if self._beta is None else self._beta.numpy().astype(np.float64)
            self._event = None
        return self

    @property
    def gamma(self):
        return (4.5 - self.lam) / (3.5 - self.lam) if self._reactive else self._gamma

    @property
    def primitive(self):
        p = self.state.copy()
        p[1:-1] /= self.state[0]
        p[-1] = (self.gamma - 1) * (self.state[-1]
                                    - 0.5 * np.sum(self.state[1:-1] ** 2, axis=0) / self.state[0])
        return p


class AsyncWriter:
    """A TemporalWriter fed by a background thread: ``append`` captures a
    frame (device-to-host copies on the session's stream) and returns; the
    thread waits for the copies and writes the files in order.  ``close``
    drains the queue and re-raises the first writer error."""

    def __init__(self, prefix, sim, formats=("vtk", "xdmf")):
        first = Frame.capture(sim).wait()
        self.writer = TemporalWriter(prefix, first, formats)
        self._queue = queue.Queue()
        self._error = None
        self._thread = threading.Thread(target=self._work, daemon=True)
        self._thread.start()
        self._queue.put(first)

    def _work(self):
        while True:
            frame = self._queue.get()
            if frame is None:
                return
            if self._error is None:
                try:
                    self.writer.append(frame.wait())
                except Exception as exc:  # reported by close()
                    self._error = exc

    def append(self, sim):
        if self._error is not None:
            raise self._error
        self._queue.put(Frame.capture(sim))

    def close(self):
        self._queue.put(None)
        self._thread.join()
        if self._error is not None:
            raise self._error
