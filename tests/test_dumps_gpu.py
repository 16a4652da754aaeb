"""Field dumps from the device: fdtd_engine_dump_field equals the
reference interpolation (engine_interface_fdtd.cpp:60-200, restated in
tests/helpers.py) applied to the engine's own fields, bit for bit, for E
and H with no, node and cell interpolation, on uniform and graded meshes,
sub-sampled boxes, and the fused kernel's alternating field buffers."""
import numpy as np
import pytest

from wipems_gb300 import Engine, Operator, scenes
from wipems_gb300.dumps import FieldDump, read_vtk

from helpers import dump_reference

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("libs")]


def _lines(op):
    return [np.ctypeslib.as_array(op.desc.lines[a], shape=(op.num_lines[a],)).copy() for a in range(3)]


@pytest.mark.parametrize("kind,kw,steps", [("upml", {}, 120), ("graded", {}, 90), ("pec", dict(kernel="fused"), 77)])
def test_device_dump_equals_reference_interpolation(kind, kw, steps):
    op = Operator(scenes.mini(kind, nr_ts=steps))
    eng = Engine(op, **kw)
    eng.iterate(steps)
    V, I = eng.fields()
    lines, unit = _lines(op), float(op.desc.unit)
    N = op.num_lines
    boxes = [((0, 0, 0), tuple(n - 1 for n in N), (3, 2, 3)),
             ((N[0] - 1, 2, 5), (3, N[1] - 1, N[2] - 1), (2, 3, 4)),
             (tuple(n - 3 for n in N), tuple(n - 1 for n in N), (1, 1, 1)),   # the upper boundary lines
             ((0, 0, 0), (2, 2, 2), (1, 1, 1))]                                # the lower ones
    for field in ("E", "H"):
        for interp in ("none", "node", "cell"):
            for start, stop, step in boxes:
                got = eng.dump_field(field, interp, start, stop, step)
                ref = dump_reference(V, I, lines, unit, field, interp, start, stop, step)
                assert got.shape == ref.shape
                assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (field, interp, start)
    assert np.abs(eng.dump_field("E", "node")).max() > 0


def test_field_dump_file(tmp_path):
    op = Operator(scenes.mini("upml", nr_ts=60))
    eng = Engine(op)
    eng.iterate(60)
    d = FieldDump(op, "et", "E", "node", step=(2, 2, 2))
    p = d.dump(eng, tmp_path)
    assert p.name == "et_00000060.vtk"
    coords, name, f = read_vtk(p)
    assert name == "E-Field" and f.shape == (3,) + tuple(len(c) for c in coords)
    assert np.array_equal(f, d.values(eng))
