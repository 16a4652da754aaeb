"""Field dumps (ProcessFieldsTD / ProcessFields::CalcField): the legacy-VTK
writer round-trips, the dump lines and coordinates follow CalcMeshPos and
GetDiscLine, and the reference interpolation restated in numpy
(tests/helpers.py) behaves as the reference documents it."""
import numpy as np
import pytest

from wipems_gb300 import Operator, scenes
from wipems_gb300.dumps import FieldDump, disc_line, dump_coordinates, read_vtk, write_vtk

from helpers import dump_reference, edge_lengths

pytestmark = pytest.mark.usefixtures("libs")


def test_vtk_roundtrip(tmp_path):
    rng = np.random.default_rng(1)
    coords = [np.linspace(0, 1e-3, 4), np.array([0.0, 2e-4, 5e-4]), np.linspace(-1e-3, 1e-3, 5)]
    f = rng.standard_normal((3, 4, 3, 5)).astype(np.float32)
    p = write_vtk(tmp_path / "e.vtk", coords, "E-Field", f)
    c, name, g = read_vtk(p)
    assert name == "E-Field"
    assert all(np.array_equal(a, b) for a, b in zip(c, coords))
    assert np.array_equal(g, f)


def test_dump_lines_and_coordinates():
    lines = [np.array([0, 1, 3, 6, 10.0])] * 3
    c = dump_coordinates(lines, 1e-3, [4, 0, 1], [0, 4, 1], [2, 3, 1], dual=False)
    assert np.allclose(c[0], [0, 3e-3, 10e-3]) and np.allclose(c[1], [0, 6e-3]) and np.allclose(c[2], [1e-3])
    assert disc_line(lines[0], 1, True) == 2.0 and disc_line(lines[0], 4, True) == 12.0
    op = Operator(scenes.mini("graded", nr_ts=50))
    d = FieldDump(op, "et", "E", "cell", step=(3, 2, 5))
    assert d.dual and d.start == [0, 0, 0] and all(len(x) > 1 for x in d.coords)


def test_reference_interpolation_rules():
    """Node interpolation of E weights the two edges at a node by their
    lengths; cell interpolation of E averages four edges; H is zero on the
    boundary lines the reference zeroes."""
    lines = [np.array([0, 1, 3, 6.0])] * 3
    V = np.zeros((3, 4, 4, 4), np.float32)
    I = np.zeros((3, 4, 4, 4), np.float32)
    V[0, 0, 1, 1], V[0, 1, 1, 1] = 1e-3, 4e-3  # E_x = 1 V/m on [0,1], 2 V/m on [1,3]
    e = dump_reference(V, I, lines, 1e-3, "E", "node", [1, 1, 1], [1, 1, 1], [1, 1, 1])
    # node x=1: delta (up) = 2, delta down = 1 -> rel = 2/3: 2*(1/3) + 1*(2/3)
    assert abs(e[0, 0, 0, 0] - (2.0 / 3 + 2.0 / 3)) < 1e-6
    I[2, 2, 2, 1] = 1.0
    h = dump_reference(V, I, lines, 1e-3, "H", "node", [0, 0, 0], [3, 3, 3], [1, 1, 1])
    assert np.all(h[:, 3, :, :] == 0) and np.all(h[2, :, 0, :] == 0)
    assert np.array_equal(edge_lengths(lines[0], 1.0, True), [1.0, 1.5, 2.5, 3.0])  # dual lines 0.5, 2, 4.5, 7.5


def test_xml_dumpbox_becomes_a_field_dump():
    from pathlib import Path
    from wipems_gb300 import Scene
    sc = Scene.from_xml(str(Path(__file__).parent / "golden" / "port_box.xml"))
    op = Operator(sc)
    (spec,) = sc.dumps()
    d = FieldDump.from_spec(op, spec)
    # the z = 3 plane of the 0.5 mm z mesh, every x and y line
    assert d.start[2] == d.stop[2] == 6 and d.start[:2] == [0, 0] and d.stop[:2] == [24, 25]
    assert [len(c) for c in d.coords] == [25, 26, 1]
    assert abs(d.coords[2][0] - 3e-3) < 1e-15
