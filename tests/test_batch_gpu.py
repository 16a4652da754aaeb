"""Batched mode: jobs of different sizes and kernel variants advanced by the
persistent batched kernels must produce exactly what each job produces when
run alone: fields and probe values bit for bit (same per-node arithmetic).
The energy is a float-Kahan-per-thread, double-across-threads sum whose
grouping follows the tile shape, so it agrees to 1e-6 relative (it only
feeds the -40 dB end criterion).
"""
import numpy as np
import pytest

from wipems_gb300 import Batch, CompressedOperator, Engine, Operator, scenes

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("libs")]

KINDS = ["pec", "upml", "drude", "lorentz", "mixed", "graded"]


def _ops(nr_ts):
    ops = [Operator(scenes.mini(k, seed=3, nr_ts=nr_ts)) for k in KINDS]
    ops.append(Operator(scenes.b96_job(1, nr_ts=nr_ts)))
    ops.append(Operator(scenes.b96_job(2, nr_ts=nr_ts)))
    return ops


def _check_same(solo, batched):
    Vs, Is = solo.fields()
    Vb, Ib = batched.fields()
    assert np.array_equal(Vs.view(np.uint32), Vb.view(np.uint32))
    assert np.array_equal(Is.view(np.uint32), Ib.view(np.uint32))
    ss, sb = solo.samples(), batched.samples()
    assert np.array_equal(ss.ts, sb.ts)
    assert np.array_equal(ss.values, sb.values)
    ok = ss.energy > 0
    assert np.allclose(sb.energy[ok], ss.energy[ok], rtol=1e-6, atol=0)


@pytest.mark.parametrize("graph_steps", [8, 1])
def test_batch_equals_solo_runs(graph_steps):
    nsteps = 130
    ops = _ops(400)
    cops = [CompressedOperator(op) for op in ops]
    solo = [Engine(c) for c in cops]
    for e in solo:
        e.iterate(nsteps)
    jobs = [Engine(c) for c in cops]
    b = Batch(jobs, graph_steps=graph_steps)
    st = b.stats()
    assert st["num_jobs"] == len(jobs) and st["num_groups"] >= 3
    b.iterate(nsteps - 37)
    b.iterate(37)
    for s, j in zip(solo, jobs):
        assert j.num_timesteps == nsteps
        _check_same(s, j)


def test_batch_jobs_at_different_timesteps():
    ops = _ops(300)[:4]
    cops = [CompressedOperator(op) for op in ops]
    solo = [Engine(c) for c in cops]
    jobs = [Engine(c) for c in cops]
    jobs[1].iterate(17)          # job 1 runs ahead on its own first
    solo[1].iterate(17 + 60)
    for k in (0, 2, 3):
        solo[k].iterate(60)
    b = Batch(jobs, x_chunk=4, stages=4)
    b.iterate(60)
    for s, j in zip(solo, jobs):
        _check_same(s, j)
