"""The oracle itself, pinned without a GPU:
  * its two engine restatements (basic Engine and the multithreaded
    SSE-compressed engine) agree bitwise, the property the reference's
    TESTSUITE/enginetests/cavity.m:144-167 demands of its own engines;
  * the PEC cavity of TESTSUITE/combinedtests/cavity.m resonates at the
    analytic TE/TM frequencies within the test's own limits;
  * golden fixtures committed under tests/golden (generated by
    tests/golden/make_golden.py) are reproduced.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from wipems_gb300 import Operator, scenes

from helpers import cavity_check, oracle_inputs

pytestmark = pytest.mark.usefixtures("libs")
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("kind", ["pec", "upml", "drude", "lorentz", "mixed", "mur", "rlc", "rlc_mur"])
def test_basic_and_sse_compressed_engines_agree_bitwise(kind):
    op = Operator(scenes.mini(kind, nr_ts=200))
    a = oracle.run(*oracle_inputs(op), 150, op.probe_interval, engine=oracle.BASIC)
    b = oracle.run(*oracle_inputs(op), 150, op.probe_interval, engine=oracle.SSE_COMPRESSED_MT, threads=3)
    assert np.array_equal(a["volt"].view(np.uint32), b["volt"].view(np.uint32))
    assert np.array_equal(a["curr"].view(np.uint32), b["curr"].view(np.uint32))
    assert np.array_equal(a["values"], b["values"])
    assert np.abs(a["volt"]).max() > 0


def test_cavity_resonances_within_reference_limits():
    sc = scenes.cavity(nr_ts=20000)
    op = Operator(sc)
    r = oracle.run(*oracle_inputs(op), 20000, 1, engine=oracle.SSE_COMPRESSED_MT, threads=8, energy=False,
                   fields=False)
    t = r["ts"] * op.dT
    res = cavity_check([t] * 3, [r["values"][:, k] for k in range(3)], sc.meta)
    assert all(res.values()), res


@pytest.mark.parametrize("name", ["p64_200", "mini_upml_150", "mini_mixed_120"])
def test_golden_fixtures(name):
    meta = json.loads((GOLDEN / f"{name}.json").read_text())
    data = np.load(GOLDEN / f"{name}.npz")
    kind, nsteps = meta["scene"], meta["steps"]
    sc = scenes.p64(nr_ts=meta["nr_ts"]) if kind == "p64" else scenes.mini(kind, nr_ts=meta["nr_ts"])
    op = Operator(sc)
    r = oracle.run(*oracle_inputs(op), nsteps, op.probe_interval, engine=oracle.BASIC)
    assert np.array_equal(r["values"], data["values"])
    assert np.array_equal(r["energy"], data["energy"])
    crc = int(np.bitwise_xor.reduce(r["volt"].view(np.uint32).ravel()))
    assert crc == meta["volt_xor"]


def test_mur_boundaries_absorb():
    """Mur faces (engine_ext_mur_abc.cpp) let the port's pulse leave: the
    energy falls far below what remains in the same box closed by PEC walls
    (where only the port's 50 ohm load takes energy out)."""
    from wipems_gb300 import Operator, scenes
    from wipems_gb300.fdtd import BC_PEC
    op = Operator(scenes.mini("mur", nr_ts=900))
    assert op.desc.num_mur == 5
    m = op.desc.mur[0]
    # vacuum at the face, uniform 0.5 mm mesh: c = (c0 dT - d) / (c0 dT + d)
    c0t = 299792458.0 * op.dT
    assert abs(m.coef_p[0] - (c0t - 0.5e-3) / (c0t + 0.5e-3)) < 1e-7
    r = oracle.run(*oracle_inputs(op), 900, op.probe_interval, engine=oracle.BASIC, fields=False)
    e = r["energy"]
    assert e[-1] < 1e-3 * e.max()
    sc = scenes.mini("mur", nr_ts=900)
    sc.set_boundary([BC_PEC] * 6, [0] * 6)
    op2 = Operator(sc)
    r2 = oracle.run(*oracle_inputs(op2), 900, op2.probe_interval, engine=oracle.BASIC, fields=False)
    assert e[-1] / e.max() < 0.01 * r2["energy"][-1] / r2["energy"].max()


def test_oracle_field_probes_are_field_over_edge_length():
    """ProcessFieldProbe through GetRawField / GetRawDualField: the sample is
    the field value over the (main or dual) edge length at the snapped
    point, weighted."""
    from helpers import edge_lengths
    s = scenes.mini("upml", nr_ts=200)
    s.add_probe([5.0, 6.0, 9.0], [5.0, 6.0, 9.0], 2)
    s.add_probe([7.25, 4.25, 12.25], [7.25, 4.25, 12.25], 3, weight=3.0)
    op = Operator(s)
    pe, ph = op.probes[-2], op.probes[-1]
    assert pe.enabled and ph.enabled and list(pe.start) == [10, 12, 18] and list(ph.start) == [14, 8, 24]
    n = 4 * op.probe_interval
    r = oracle.run(*oracle_inputs(op), n, op.probe_interval, engine=oracle.BASIC)
    assert r["values"].shape[1] == len(op.probes) - 2 + 6
    lines = [np.ctypeslib.as_array(op.desc.lines[a], shape=(op.num_lines[a],)) for a in range(3)]
    for c in range(3):
        lm = edge_lengths(lines[c], op.desc.unit, False)[pe.start[c]]
        ld = edge_lengths(lines[c], op.desc.unit, True)[ph.start[c]]
        assert r["values"][-1, -6 + c] == float(r["volt"][c][tuple(pe.start)]) / lm
        assert r["values"][-1, -3 + c] == float(r["curr"][c][tuple(ph.start)]) / ld * 3.0
