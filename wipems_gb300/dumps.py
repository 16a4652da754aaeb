"""Time-domain field dumps (the reference's ProcessFieldsTD,
Common/processfields_td.cpp:49-91, with ProcessFields::CalcMeshPos and
CalcField, Common/processfields.cpp:213-330).

The field values come from the device (`Engine.dump_field`, the reference's
interpolation of Engine_Interface_FDTD); this module picks the dump lines,
their coordinates (GetDiscLine on the main mesh, or the dual mesh for cell
interpolation, scaled to metres) and writes them as legacy-VTK rectilinear
grids.  The reference writes VTK through the VTK library or HDF5 through
libhdf5; neither library is available here, and the legacy VTK format is
read by the same viewers.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np


def disc_line(lines, pos: int, dual: bool) -> float:
    """Operator::GetDiscLine: the mesh line, or the dual line (the midpoint
    to the next line; past the last line, half a cell beyond it)."""
    n = len(lines)
    if not dual:
        return float(lines[pos])
    if pos < n - 1:
        return 0.5 * (lines[pos] + lines[pos + 1])
    return lines[pos] + 0.5 * (lines[pos] - lines[pos - 1])


def snap(lines, coord: float, dual: bool) -> int:
    """Nearest main (or dual) line index to a coordinate in drawing units."""
    cand = [disc_line(lines, i, dual) for i in range(len(lines))]
    return int(np.argmin(np.abs(np.asarray(cand) - coord)))


def dump_coordinates(lines, unit: float, start, stop, step, dual: bool):
    """Coordinates (m) of the dump lines start, start + step, ..., <= stop per
    axis (ProcessFields::CalcMeshPos with sub-sampling)."""
    out = []
    for a in range(3):
        lo, hi = sorted((int(start[a]), int(stop[a])))
        idx = range(lo, hi + 1, max(1, int(step[a])))
        out.append(np.array([disc_line(lines[a], i, dual) * unit for i in idx]))
    return out


def write_vtk(path, coords, name: str, field, header: str = "openEMS TD Field Dump") -> Path:
    """Legacy VTK RECTILINEAR_GRID with one point-data vector field
    (field [3][nx][ny][nz]; VTK orders points x fastest)."""
    path = Path(path)
    x, y, z = (np.asarray(c, np.float64) for c in coords)
    f = np.asarray(field, np.float32)
    if f.shape != (3, len(x), len(y), len(z)):
        raise ValueError(f"field shape {f.shape} does not match the coordinates")
    be = lambda a, t: np.asarray(a, t).astype(t.newbyteorder(">")).tobytes()  # legacy VTK binary is big-endian
    with open(path, "wb") as fh:
        fh.write(b"# vtk DataFile Version 3.0\n")
        fh.write(header.encode()[:255] + b"\n")
        fh.write(b"BINARY\nDATASET RECTILINEAR_GRID\n")
        fh.write(f"DIMENSIONS {len(x)} {len(y)} {len(z)}\n".encode())
        for tag, c in (("X", x), ("Y", y), ("Z", z)):
            fh.write(f"{tag}_COORDINATES {len(c)} double\n".encode())
            fh.write(be(c, np.dtype(np.float64)) + b"\n")
        fh.write(f"POINT_DATA {len(x) * len(y) * len(z)}\n".encode())
        fh.write(f"VECTORS {name} float\n".encode())
        # points x fastest: array [z][y][x][3]
        v = np.transpose(f, (3, 2, 1, 0))
        fh.write(be(v, np.dtype(np.float32)) + b"\n")
    return path


def read_vtk(path):
    """Reads back what write_vtk wrote: (coords, name, field[3][nx][ny][nz])."""
    data = Path(path).read_bytes()
    pos = 0

    def line():
        nonlocal pos
        e = data.index(b"\n", pos)
        s = data[pos:e].decode()
        pos = e + 1
        return s

    line(); line(); line(); line()
    dims = [int(t) for t in line().split()[1:4]]
    coords = []
    for n in dims:
        line()
        coords.append(np.frombuffer(data[pos:pos + 8 * n], ">f8").astype(np.float64))
        pos += 8 * n + 1
    line()
    name = line().split()[1]
    cnt = dims[0] * dims[1] * dims[2] * 3
    v = np.frombuffer(data[pos:pos + 4 * cnt], ">f4").astype(np.float32).reshape(dims[2], dims[1], dims[0], 3)
    return coords, name, np.ascontiguousarray(np.transpose(v, (3, 2, 1, 0)))


class FieldDump:
    """A DumpBox: field "E" or "H", interpolation, a box in drawing units
    (snapped to the main mesh, or the dual mesh for cell interpolation, as
    ProcessFields::SetDumpMode selects), sub-sampling.  dump(engine, folder)
    writes <name>_<timestep>.vtk at the engine's current timestep."""

    def __init__(self, op, name: str, field: str = "E", interp: str = "node", start=None, stop=None,
                 step=(1, 1, 1)):
        self.op, self.name, self.field, self.interp = op, name, field, interp
        self.dual = interp == "cell"
        lines = [np.ctypeslib.as_array(op.desc.lines[a], shape=(op.num_lines[a],)).copy() for a in range(3)]
        unit = float(op.desc.unit)
        self.lines, self.unit = lines, unit
        if start is None:
            start = [l[0] for l in lines]
        if stop is None:
            stop = [l[-1] for l in lines]
        self.start = [snap(lines[a], start[a], self.dual) for a in range(3)]
        self.stop = [snap(lines[a], stop[a], self.dual) for a in range(3)]
        self.step = [max(1, int(s)) for s in step]
        self.coords = dump_coordinates(lines, unit, self.start, self.stop, self.step, self.dual)

    @classmethod
    def from_spec(cls, op, spec: dict) -> "FieldDump":
        """A dump from Scene.dumps() (an XML <DumpBox>)."""
        return cls(op, spec["name"], spec["field"], spec["interp"], spec["start"], spec["stop"], spec["step"])

    def values(self, engine):
        return engine.dump_field(self.field, self.interp, self.start, self.stop, self.step)

    def dump(self, engine, folder) -> Path:
        folder = Path(folder)
        folder.mkdir(parents=True, exist_ok=True)
        f = self.values(engine)
        label = {"E": "E-Field", "H": "H-Field"}[self.field]
        head = f"openEMS TD Field Dump -- Interpolation: {self.interp} -- timestep {engine.num_timesteps}"
        return write_vtk(folder / f"{self.name}_{engine.num_timesteps:08d}.vtk", self.coords, label, f, head)


if __name__ == "__main__":  # python -m wipems_gb300.dumps file.vtk: print a dump's shape
    c, n, f = read_vtk(sys.argv[1])
    print(n, f.shape, [len(x) for x in c])
