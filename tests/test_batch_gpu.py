"""Batched mode: jobs of different sizes and kernel variants advanced by the
persistent batched kernels must produce exactly what each job produces when
run alone: fields, probe values and energies bit for bit (same per-node
arithmetic; the energy is summed in an order fixed by each job's grid).
"""
import numpy as np
import pytest

from wipems_gb300 import Batch, CompressedOperator, Engine, Operator, run_fdtd, scenes

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
    assert np.array_equal(ss.energy, sb.energy)  # fixed-order energy: the same bits


@pytest.mark.parametrize("graph_steps,bin_mib,bps,chains,ty", [(8, 0, 0, 0, 0), (1, 0, 0, 0, 0), (8, 1, 0, 0, 0),
                                                               (8, 0, -1, 0, 0), (8, 0, -1, 3, 0), (1, 0, -1, 2, 4),
                                                               (8, 1, -1, 2, 4), (8, 0, 0, 0, 4)])
def test_batch_equals_solo_runs(graph_steps, bin_mib, bps, chains, ty):
    """Persistent and one-block-per-item kernels, 8- and 4-row tiles, one
    chain per kernel variant or several job-range chains on their own
    streams (graphs and single steps, with and without L2 bins): every job
    bit-identical to its solo run."""
    nsteps = 130
    ops = _ops(400)
    cops = [CompressedOperator(op) for op in ops]
    solo = [Engine(c) for c in cops]
    for e in solo:
        e.iterate(nsteps)
    jobs = [Engine(c, kernel="tma") for c in cops]
    b = Batch(jobs, graph_steps=graph_steps, bin_mib=bin_mib, blocks_per_sm=bps, chains=chains, tile_y=ty)
    st = b.stats()
    assert st["num_jobs"] == len(jobs) and st["num_groups"] >= 3
    assert (st["num_bins"] > 1) == (bin_mib > 0)
    b.iterate(nsteps - 37)
    b.iterate(37)
    for s, j in zip(solo, jobs):
        assert j.num_timesteps == nsteps
        _check_same(s, j)


def test_batch_jobs_at_different_timesteps():
    ops = _ops(300)[:4]
    cops = [CompressedOperator(op) for op in ops]
    solo = [Engine(c) for c in cops]
    jobs = [Engine(c, kernel="tma") for c in cops]
    jobs[1].iterate(17)          # job 1 runs ahead on its own first
    solo[1].iterate(17 + 60)
    for k in (0, 2, 3):
        solo[k].iterate(60)
    b = Batch(jobs, x_chunk=4, stages=4)
    b.iterate(60)
    for s, j in zip(solo, jobs):
        _check_same(s, j)


@pytest.mark.parametrize("stages", [3, 5, 7])
def test_batch_ring_runs_on_across_work_items(stages):
    """One persistent block per SM walks many work items, so each block's
    mbarrier ring count runs on from item to item and wraps mid-tile for
    stage counts that do not divide the planes of an item: every job stays
    bit-identical to its solo run."""
    nsteps = 40
    ops = _ops(200)
    cops = [CompressedOperator(op) for op in ops]
    solo = [Engine(c) for c in cops]
    for e in solo:
        e.iterate(nsteps)
    jobs = [Engine(c, kernel="tma") for c in cops]
    b = Batch(jobs, x_chunk=3, stages=stages, blocks_per_sm=1, graph_steps=8)
    b.iterate(nsteps)
    for s, j in zip(solo, jobs):
        _check_same(s, j)


END_KINDS = ["upml", "drude", "graded", "lorentz"]   # the last one never decays to 1e-3 in 800 steps


def test_device_end_criterion_matches_host_loop():
    """The on-device end criterion stops a job at the same timestep as
    RunFDTD's host loop (run_fdtd), with identical samples and fields; later
    iterate calls leave a stopped job untouched."""
    nr_ts, crit = 800, 1e-3
    stops = []
    for k in END_KINDS:
        op = Operator(scenes.mini(k, seed=3, nr_ts=nr_ts))
        host = Engine(op)
        r = run_fdtd(host, nr_ts, crit)
        dev = Engine(op, end_crit=crit)
        for n in (100, 300, 400):
            dev.iterate(n)
        assert dev.num_timesteps == r["timesteps"]
        assert dev.done
        _check_same(host, dev)
        V0, _ = dev.fields()
        dev.iterate(50)
        assert dev.num_timesteps == r["timesteps"]
        assert np.array_equal(dev.fields()[0], V0)
        stops.append(r["timesteps"])
    assert min(stops) < nr_ts and max(stops) == nr_ts


def test_batch_end_criterion_same_as_alone():
    """Jobs that stop on their own end criterion inside a batch (L2 bins,
    graphs) stop at the same step with the same results as alone."""
    nr_ts, crit = 800, 1e-3
    cops = [CompressedOperator(Operator(scenes.mini(k, seed=3, nr_ts=nr_ts))) for k in END_KINDS]
    solo = [Engine(c, end_crit=crit) for c in cops]
    for e in solo:
        e.iterate(nr_ts)
    jobs = [Engine(c, end_crit=crit, kernel="tma") for c in cops]
    b = Batch(jobs, graph_steps=16, bin_mib=1)
    b.iterate(nr_ts + 64)
    for s, j in zip(solo, jobs):
        assert j.num_timesteps == s.num_timesteps and j.done == s.done
        _check_same(s, j)


@pytest.mark.parametrize("kind,what", [("mur", "Mur"), ("rlc", "lumped RLC")])
def test_batch_refuses_unbatched_extensions(kind, what):
    from wipems_gb300._abi import FdtdError
    plain = Engine(Operator(scenes.mini("upml", seed=3, nr_ts=100)))
    other = Engine(Operator(scenes.mini(kind, seed=3, nr_ts=100)))
    with pytest.raises(FdtdError, match=what):
        Batch([plain, other])
