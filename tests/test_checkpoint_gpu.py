"""Checkpoint / resume: an engine restored from a checkpoint steps on to
the same fields, probe samples, energies and frequency-domain sums, bit for
bit, as the engine that was checkpointed."""
import numpy as np
import pytest

from wipems_gb300 import Engine, Operator, scenes
from wipems_gb300._abi import FdtdError

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("libs")]


def _engine(op, **kw):
    e = Engine(op, **kw)
    e.set_frequencies(np.linspace(2e9, 9e9, 4))
    return e


@pytest.mark.parametrize("kind,kw", [("upml", {}), ("drude", {}), ("mur", {}), ("rlc_mur", {}), ("multipole", {}),
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
    assert np.array_equal(sb.energy, sa.energy)  # fixed-order energy: the same bits
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


def _same_run(x, y):
    Vx, Ix = x.fields()
    Vy, Iy = y.fields()
    assert np.array_equal(Vx.view(np.uint32), Vy.view(np.uint32))
    assert np.array_equal(Ix.view(np.uint32), Iy.view(np.uint32))
    sx, sy = x.samples(), y.samples()
    assert np.array_equal(sx.ts, sy.ts) and np.array_equal(sx.values, sy.values)
    assert sx.ts[0] == 0  # the ts = 0 sample of RunFDTD's first PA->Process()


def test_rejected_restore_leaves_a_fresh_engine_untouched():
    """A blob rejected for any reason -- another configuration, truncated,
    trailing bytes, a corrupted part size -- changes nothing: the fresh
    engine afterwards steps exactly like a clean one, ts = 0 sample and
    frequency-domain sums included."""
    op = Operator(scenes.mini("upml", seed=3, nr_ts=800))
    a = _engine(op)
    a.iterate(120)
    blob = a.checkpoint()
    pec = Operator(scenes.mini("pec", nr_ts=800))
    import struct
    bad_size = bytearray(blob)
    # the blob header is 8 magic bytes and 14 uint32 words; the first part
    # (the four int control words, 16 bytes) follows it: claim 4 bytes more
    first_count_at = struct.calcsize("<8s14I")
    assert struct.unpack_from("<Q", blob, first_count_at)[0] == 16
    struct.pack_into("<Q", bad_size, first_count_at, 20)
    for eng_op, payload in ((pec, blob), (op, blob[:-8]), (op, blob + b"\0" * 8), (op, bytes(bad_size))):
        x = _engine(eng_op)
        with pytest.raises(FdtdError) as ei:
            x.restore(payload)
        assert ei.value.code == -1
        x.iterate(100)
        clean = _engine(eng_op)
        clean.iterate(100)
        _same_run(x, clean)
        fx, nx = x.fd_results()
        fc, nc = clean.fd_results()
        assert nx == nc and np.array_equal(fx, fc)
