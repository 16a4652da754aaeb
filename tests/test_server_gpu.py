"""Continuous-batching server: every job's result (stopping timestep,
probe samples, final fields) is the same as when the job runs alone on the
plain engine with the same end criterion, whatever else shares the GPU."""
import numpy as np
import pytest

from wipems_gb300 import Engine, Operator, Server, scenes

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("libs")]

KINDS = ["upml", "drude", "lorentz", "graded", "mixed", "pec"]
NR_TS, CRIT = 700, 1e-3


def _alone(kind, seed):
    op = Operator(scenes.mini(kind, seed=seed, nr_ts=NR_TS))
    e = Engine(op, end_crit=CRIT)
    e.iterate(NR_TS)
    return e


def _same(e, srv, jid):
    st = srv.status(jid)
    assert st["state"] == "done", st
    assert st["timesteps"] == e.num_timesteps
    a, b = e.samples(), srv.samples(jid)
    assert np.array_equal(a.ts, b.ts)
    assert np.array_equal(a.values, b.values)
    assert np.array_equal(a.energy, b.energy)  # fixed-order energy: the same bits
    Va, Ia = e.fields()
    Vb, Ib = srv.fields(jid)
    assert np.array_equal(Va.view(np.uint32), Vb.view(np.uint32))
    assert np.array_equal(Ia.view(np.uint32), Ib.view(np.uint32))


@pytest.mark.parametrize("round_steps,bin_mib,batch_min,tile_share",
                         [(64, 0, 0, 0), (37, 1, 1, 0), (50, 0, 3, 0), (29, 0, 0, 16)])
def test_server_results_same_as_alone(round_steps, bin_mib, batch_min, tile_share):
    """Concurrent engines (the default, each job tiled for a share of the
    SMs), persistent-batch rounds with L2 bins, and a mix of both modes all
    give each job its solo result."""
    srv = Server(round_steps=round_steps, bin_mib=bin_mib, build_workers=2, batch_min_jobs=batch_min,
                 tile_share=tile_share)
    ids = {}
    for seed in (3, 4):
        for k in KINDS:
            ids[(k, seed)] = srv.submit(scenes.mini(k, seed=seed, nr_ts=NR_TS), end_crit=CRIT, keep_fields=True)
    srv.wait(0, timeout=600)
    st = srv.stats()
    assert st["jobs_done"] == len(ids) and st["jobs_failed"] == 0
    for (k, seed), jid in ids.items():
        _same(_alone(k, seed), srv, jid)
    srv.close()


def test_server_admission_by_footprint():
    """A budget that holds about two jobs at a time: every job still runs,
    the resident footprint never exceeds the budget, and results match."""
    probe = Server(max_active=1)
    j = probe.submit(scenes.mini("upml", seed=3, nr_ts=NR_TS), end_crit=CRIT)
    probe.wait(j, timeout=300)
    foot = probe.status(j)["footprint"]
    probe.close()
    budget = int(2.5 * foot)
    srv = Server(hbm_budget=budget, round_steps=50, batch_min_jobs=1)  # resident jobs run as a batch
    ids = [srv.submit(scenes.mini("upml", seed=s, nr_ts=NR_TS), end_crit=CRIT, keep_fields=True) for s in range(3, 9)]
    srv.wait(0, timeout=600)
    st = srv.stats()
    assert st["jobs_done"] == len(ids)
    assert st["peak_bytes"] <= budget
    assert st["rebuilds"] >= 3            # jobs entered as earlier ones retired
    t_admit = sorted(srv.status(i)["t_admit"] for i in ids)
    t_done = sorted(srv.status(i)["t_done"] for i in ids)
    assert t_admit[-1] >= t_done[0]       # the last admissions waited for retirements
    for s, jid in zip(range(3, 9), ids):
        _same(_alone("upml", s), srv, jid)
    srv.close()


def test_server_rejects_oversized_job_and_keeps_serving():
    """A job whose footprint exceeds the whole budget fails cleanly; the
    server keeps serving jobs that fit."""
    srv = Server(hbm_budget=8 << 20)
    big = srv.submit(scenes.mini("upml", seed=3, nr_ts=NR_TS), end_crit=CRIT)
    srv.wait(big, timeout=300)
    st = srv.status(big)
    assert st["state"] == "failed" and "budget" in st["message"]
    srv.close()
    srv = Server(hbm_budget=1 << 30)
    ok = srv.submit(scenes.mini("pec", seed=3, nr_ts=200), end_crit=CRIT)
    srv.wait(ok, timeout=300)
    assert srv.status(ok)["state"] == "done"
    srv.close()


def test_batch_mode_runs_unbatchable_jobs_beside_the_batch():
    """With batch rounds on, jobs the persistent batch cannot take (Mur
    faces, lumped RLC edges, dispersion of order > 1) run as concurrent
    engines next to it, and magnetic Lorentz/Drude jobs join the batch;
    every job still gets its solo result."""
    srv = Server(round_steps=40, build_workers=2, batch_min_jobs=2)
    kinds = [("upml", 3), ("mur", 3), ("pec", 4), ("rlc", 3), ("drude", 4), ("rlc_mur", 5), ("multipole", 3),
             ("magnetic", 4)]
    ids = {(k, s): srv.submit(scenes.mini(k, seed=s, nr_ts=NR_TS), end_crit=CRIT, keep_fields=True)
           for k, s in kinds}
    srv.wait(0, timeout=600)
    st = srv.stats()
    assert st["jobs_done"] == len(ids) and st["jobs_failed"] == 0, st
    assert st["rebuilds"] >= 1
    for (k, s), jid in ids.items():
        _same(_alone(k, s), srv, jid)
    srv.close()


def test_server_job_with_field_probes():
    """Field probes add three sample columns; the server's samples match the
    job run alone."""
    s = scenes.mini("upml", seed=3, nr_ts=NR_TS)
    s.add_probe([5.0, 6.0, 9.0], [5.0, 6.0, 9.0], 2)
    s.add_probe([7.25, 4.25, 12.25], [7.25, 4.25, 12.25], 3)
    srv = Server(round_steps=64)
    jid = srv.submit(s, end_crit=CRIT, keep_fields=True)
    srv.wait(0, timeout=300)
    st = srv.status(jid)
    assert st["state"] == "done" and st["num_probes"] == 2 + 6
    s2 = scenes.mini("upml", seed=3, nr_ts=NR_TS)
    s2.add_probe([5.0, 6.0, 9.0], [5.0, 6.0, 9.0], 2)
    s2.add_probe([7.25, 4.25, 12.25], [7.25, 4.25, 12.25], 3)
    e = Engine(Operator(s2), end_crit=CRIT)
    e.iterate(NR_TS)
    _same(e, srv, jid)
    assert srv.samples(jid).times(4)[1] - srv.samples(jid).times(4)[0] > 0
    assert srv.samples(jid).probe_types == e.samples().probe_types == [0, 1, 2, 2, 2, 3, 3, 3]
    srv.close()


def test_server_serves_an_xml_scene():
    """A scene read from an openEMS XML document (no Python-side probe
    list) through the server: sample columns and their types come from the
    server, and the result equals the document run alone."""
    import os
    from wipems_gb300 import Scene
    path = os.path.join(os.path.dirname(__file__), "golden", "lorentz_mur.xml")
    srv = Server(round_steps=64)
    jid = srv.submit(Scene.from_xml(path), end_crit=CRIT, keep_fields=True)
    srv.wait(0, timeout=300)
    e = Engine(Operator(Scene.from_xml(path)), end_crit=CRIT)
    e.iterate(Scene.from_xml(path).nr_ts)
    _same(e, srv, jid)
    assert srv.samples(jid).probe_types == e.samples().probe_types
    srv.close()


def test_server_job_without_end_criterion_runs_its_timesteps():
    """A job submitted without an energy criterion runs exactly its scene's
    NumberOfTimesteps (or max_timesteps), whatever the round length, in
    batch mode too (such jobs run beside the batch), and equals the plain
    engine run for that many timesteps."""
    srv = Server(round_steps=37, batch_min_jobs=2)
    ids = {}
    for seed in (3, 4):
        for k in ("upml", "drude"):
            ids[(k, seed, 0)] = srv.submit(scenes.mini(k, seed=seed, nr_ts=250), keep_fields=True)
            ids[(k, seed, 1)] = srv.submit(scenes.mini(k, seed=seed, nr_ts=250), max_timesteps=111,
                                           keep_fields=True)
    srv.wait(0, timeout=600)
    st = srv.stats()
    assert st["jobs_done"] == len(ids) and st["jobs_failed"] == 0
    for (k, seed, capped), jid in ids.items():
        n = 111 if capped else 250
        e = Engine(Operator(scenes.mini(k, seed=seed, nr_ts=250)), max_timesteps=n)
        e.iterate(n)
        _same(e, srv, jid)
    srv.close()
