"""Checkpoint / resume: an engine restored from a checkpoint steps on to
the same fields, probe samples and frequency-domain sums, bit for bit, as
the engine that was checkpointed (the energy column is a double-atomic sum
over blocks, equal to rounding)."""
import numpy as np
import pytest

from wipems_gb300 import Engine, Operator, scenes
from wipems_gb300._abi import FdtdError

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("libs")]


def _engine(op, **kw):
    e = Engine(op, **kw)
    e.set_frequencies(np.linspace(2e9, 9e9, 4))
    return e


@pytest.mark.parametrize("kind,kw", [("upml", {}), ("drude", {}), ("mur", {}), ("rlc_mur", {}),
                                     ("pec", dict(kernel="fused")),
                                     ("lorentz", dict(use_graphs=False, kernel="direct"))])
def test_resume_is_bit_identical(kind, kw):
    op = Operator(scenes.mini(kind, seed=2, nr_ts=800))
    a = _engine(op, **kw)
    a.iterate(251)
    blob = a.checkpoint()
    a.iterate(173)
    b = _engine(op, **kw)
    b.restore(blob)
    assert b.num_timesteps == 251
    b.iterate(173)
    Va, Ia = a.fields()
    Vb, Ib = b.fields()
    assert np.array_equal(Va.view(np.uint32), Vb.view(np.uint32))
    assert np.array_equal(Ia.view(np.uint32), Ib.view(np.uint32))
    sa, sb = a.samples(), b.samples()
    assert np.array_equal(sa.ts, sb.ts) and np.array_equal(sa.values, sb.values)
    # energies are sums over blocks in double atomics: equal to rounding
    np.testing.assert_allclose(sb.energy, sa.energy, rtol=1e-12, atol=0)
    fa, na = a.fd_results()
    fb, nb = b.fd_results()
    assert na == nb and np.array_equal(fa, fb)


def test_restore_checks_the_engine_and_keeps_a_stopped_job_stopped():
    op = Operator(scenes.mini("upml", seed=3, nr_ts=800))
    a = Engine(op, end_crit=1e-3)
    a.iterate(800)
    assert a.done
    blob = a.checkpoint()
    b = Engine(op, end_crit=1e-3)
    b.restore(blob)
    assert b.done and b.num_timesteps == a.num_timesteps
    b.iterate(100)
    assert b.num_timesteps == a.num_timesteps
    other = Engine(Operator(scenes.mini("pec", nr_ts=800)))
    with pytest.raises(FdtdError) as ei:
        other.restore(blob)
    assert ei.value.code == -1
