"""Field probes (ProbeBox Type 2 / 3, ProcessFieldProbe): E and H at a
point, three columns each, sampled on the device -- bit-identical to the
oracle, equal to the field dump at the same point (the check of the
reference's TESTSUITE/probes/fieldprobes.m), the same inside a batch, and
accumulated in the frequency domain at their own (dual) times."""
import ctypes

import numpy as np
import pytest

import oracle
from wipems_gb300 import Batch, CompressedOperator, Engine, Operator, scenes

from helpers import oracle_inputs
from test_parity_gpu import compare

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("libs")]


def _scene(nr_ts=400, kind="upml"):
    s = scenes.mini(kind, nr_ts=nr_ts)
    s.add_probe([5.0, 6.0, 9.0], [5.0, 6.0, 9.0], 2, name="E")       # on lines (0.5 mm mesh)
    s.add_probe([7.25, 4.25, 12.25], [7.25, 4.25, 12.25], 3, name="H")  # on dual lines
    s.add_probe([8.0, 8.0, 10.0], [8.0, 8.0, 10.0], 2, weight=-2.0, name="E2")
    return s


@pytest.mark.parametrize("kind,kernel", [("upml", "tma"), ("upml", "direct"), ("graded", "tma"),
                                         ("pec", "fused")])
def test_field_probes_match_oracle(kind, kernel):
    """Bit for bit; on the graded mesh against the oracle run on the
    coefficients the factorized kernels apply (a point value is more
    sensitive to their few-ulp re-rounding than the integral probes)."""
    op = Operator(_scene(kind=kind))
    assert [p.type for p in op.probes][-3:] == [2, 3, 2]
    cop = CompressedOperator(op)
    d = op.desc
    if cop.factorized:
        vv, vi, ii, iv = [np.ascontiguousarray(a) for a in cop.expand()[:4]]
        d = type(op.desc).from_buffer_copy(op.desc)
        PF = ctypes.POINTER(ctypes.c_float)
        d.vv, d.vi, d.ii, d.iv = (a.ctypes.data_as(PF) for a in (vv, vi, ii, iv))
    ref = oracle.run(d, op.probes, 400, op.probe_interval, engine=oracle.BASIC)
    eng = Engine(cop, kernel=kernel)
    eng.iterate(400)
    compare(op, eng, ref)
    s = eng.samples()
    assert s.values.shape[1] == len(op.probes) - 3 + 9
    assert np.abs(s.values[:, -9:]).max() > 0


def test_field_probe_equals_field_dump_and_batch():
    op = Operator(_scene())
    n = 6 * op.probe_interval  # ends on a sample step
    eng = Engine(op)
    eng.iterate(n)
    s = eng.samples()
    k = len(op.probes) - 3
    pe, ph = op.probes[k], op.probes[k + 1]
    e = eng.dump_field("E", "none", tuple(pe.start), tuple(pe.start))[:, 0, 0, 0]
    h = eng.dump_field("H", "none", tuple(ph.start), tuple(ph.start))[:, 0, 0, 0]
    assert s.ts[-1] == n
    assert np.array_equal(s.values[-1, k:k + 3].astype(np.float32), e)
    assert np.array_equal(s.values[-1, k + 3:k + 6].astype(np.float32), h)
    # the batched sampler records the same columns
    other = Engine(Operator(scenes.mini("pec", nr_ts=400)), kernel="tma")
    job = Engine(op, kernel="tma")
    Batch([job, other]).iterate(n)
    assert np.array_equal(job.samples().values, s.values)


def test_field_probe_frequency_domain():
    op = Operator(_scene(nr_ts=700))
    eng = Engine(op)
    freqs = eng.set_frequencies(np.linspace(2e9, 9e9, 5))
    fdint = eng.fd_interval
    eng.iterate(600)
    got, count = eng.fd_results()
    ref = oracle.run(*oracle_inputs(op), 600, fdint, engine=oracle.BASIC)
    assert count == len(ref["ts"])
    dual = np.array([0.5 if t in (1, 3) else 0.0 for t in eng.probe_types])
    t = (ref["ts"][:, None] + dual[None, :]) * op.dT
    phase = np.exp(-2j * np.pi * freqs[None, None, :] * t[:, :, None])
    want = np.einsum("sp,spf->pf", ref["values"], phase) * 2 * op.dT * fdint
    assert np.max(np.abs(got - want)) <= 1e-12 * np.abs(want).max()
