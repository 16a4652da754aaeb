"""Lumped RLC elements (Operator_Ext_LumpedRLC / Engine_Ext_LumpedRLC,
operator_ext_lumpedRLC.cpp:112-486, engine_ext_lumpedRLC.cpp:83-145), pinned
without a GPU:
  * known answer: one RLC edge in a UPML-bounded vacuum box, driven from a
    nearby soft source; the ratio of the voltage along the edge to the loop
    current around it is the element's impedance in parallel with the edge
    capacitance (series: the parasitic capacitance by the reference's
    20x-impedance rule; parallel: C replaces the edge capacitance).  The
    signals are differenced before the transform, which removes the charge
    a series capacitor keeps after the pulse and leaves V/I unchanged;
  * the operator build (counts, caps, the type rules of IsLElumpedRLC and
    IsLEparRC) and the compression's refusals.
"""
import math

import numpy as np
import pytest

import oracle
from wipems_gb300 import CompressedOperator, Operator, Scene, scenes
from wipems_gb300._abi import FdtdError
from wipems_gb300.fdtd import BC_PEC
from wipems_gb300.ports import dft_time2freq

from helpers import oracle_inputs

pytestmark = pytest.mark.usefixtures("libs")

EPS0 = 8.85418781762e-12


def _impedance(series, R, L, Cap, f0, fc, steps=8000):
    op = Operator(scenes.rlc_probe(series, R, L, Cap, nr_ts=steps, f0=f0, fc=fc))
    assert op.desc.rlc and op.desc.rlc.contents.count == 1
    r = oracle.run(*oracle_inputs(op), steps, 1, engine=oracle.SSE_COMPRESSED_MT, threads=8, fields=False)
    t = r["ts"] * op.dT
    dv = np.diff(r["values"][:, 0])
    di = np.diff(r["values"][:, 1])
    f = np.linspace(max(f0 - fc, 0.5e9), f0 + 0.75 * fc, 9)
    # voltage differences sit at t + dT/2, current differences (dual time) at t + dT
    Z = dft_time2freq(t[:-1] + 0.5 * op.dT, dv, f) / dft_time2freq(t[:-1] + op.dT, di, f)
    return f, Z


@pytest.mark.parametrize("R,L,Cap", [(20.0, 10e-9, 1e-12), (300.0, 10e-9, 1e-12)])
def test_series_rlc_impedance_known_answer(R, L, Cap):
    f0, fc = 2e9, 2e9
    f, Z = _impedance(True, R, L, Cap, f0, fc)
    w = 2 * np.pi * f
    fmax = f0 + fc
    Cd = EPS0 * 1e-3 * 1e-3 / 1e-3  # vacuum edge: eps0 * dual area / length (1 mm cells)
    zmin = math.sqrt(R ** 2 + (2 * math.pi * fmax * L - 1 / (Cap * 2 * math.pi * fmax)) ** 2)
    raised = 1 / (2 * math.pi * fmax * Cd) < 20 * zmin
    if raised:
        Cd = 1 / (2 * math.pi * fmax * zmin * 20)
    assert raised == (R == 300.0)  # the second case exercises the parasitic-capacitance rule
    Ze = 1 / (1 / (R + 1j * w * L + 1 / (1j * w * Cap)) + 1j * w * Cd)
    assert np.max(np.abs(Z - Ze) / np.abs(Ze)) < 2e-3


def test_parallel_rlc_impedance_known_answer():
    R, L, Cap = 100.0, 5e-9, 1e-12
    f, Z = _impedance(False, R, L, Cap, 2e9, 1e9)
    w = 2 * np.pi * f
    Ze = 1 / (1 / R + 1 / (1j * w * L) + 1j * w * Cap)
    assert np.max(np.abs(Z - Ze) / np.abs(Ze)) < 1e-3


@pytest.mark.parametrize("kind", ["rlc", "rlc_mur"])
def test_rlc_scenes_build(kind):
    op = Operator(scenes.mini(kind, nr_ts=200))
    d = op.desc.rlc.contents
    # series: 3 edges along z; parallel: 2 cells along x times 2 lines across
    n = 3 + 4 + (2 if kind == "rlc_mur" else 0)
    assert d.count == n
    dirs = [d.dir[k] for k in range(n)]
    assert dirs[:3] == [2, 2, 2] and dirs[3:7] == [0] * 4
    # series rows carry the series coefficients, parallel rows the inductor terms
    assert all(d.ilv[k] == 0 and d.vvd[k] < 1 for k in range(3))
    assert all(d.ilv[k] > 0 and d.vvd[k] == 1 and d.vj1[k] == 0 for k in range(3, 7))


def _one_element(le_type, L):
    lines = [np.arange(11, dtype=float)] * 3
    s = Scene(*lines, 1e-3)
    s.set_boundary([BC_PEC] * 6)
    s.set_gauss_excite(2e9, 2e9, 100)
    s.add_excitation([2, 5, 5], [2, 5, 6], [0, 0, 1])
    s.add_lumped_rlc([5, 5, 4], [5, 5, 6], 2, R=50.0, L=L, Cap=1e-12, le_type=le_type)
    return Operator(s)


def test_type_rules():
    # IsLElumpedRLC: parallel with L > 0, or series; IsLEparRC: parallel without L
    assert _one_element(0, 1e-9).desc.rlc.contents.count == 2
    assert not _one_element(0, -1).desc.rlc           # plain parallel R/C: main operator
    assert _one_element(1, -1).desc.rlc.contents.count == 2
    assert not _one_element(-1, 1e-9).desc.rlc         # invalid type: ignored by both


def test_compression_refuses_excitation_on_an_rlc_edge():
    lines = [np.arange(11, dtype=float)] * 3
    s = Scene(*lines, 1e-3)
    s.set_boundary([BC_PEC] * 6)
    s.set_gauss_excite(2e9, 2e9, 100)
    s.add_excitation([5, 5, 4], [5, 5, 5], [0, 0, 1])
    s.add_lumped_rlc([5, 5, 4], [5, 5, 6], 2, R=50.0, L=1e-9, Cap=1e-12, series=True)
    op = Operator(s)
    with pytest.raises(FdtdError, match="excitation on a lumped RLC edge"):
        CompressedOperator(op)
