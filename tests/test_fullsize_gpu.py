"""Full-length parity on the headline configurations: the CUDA engine against
the oracle (its own operator build, checked bitwise against the product's,
and its SSE-compressed multithreaded stepping) over the whole run.

Bar: probe series within 1e-5 relative L2 and final fields within 1e-4
relative max-norm; bit-identical where the engine keeps the reference's
coefficients exactly (uniform meshes, and the exact-table engine on graded
ones).
"""
import os

import numpy as np
import pytest

import oracle
from wipems_gb300 import Batch, CompressedOperator, Engine, Operator, Scene, Server, scenes

from helpers import oracle_inputs, rel_l2, rel_max
from test_parity_gpu import FIELD_TOL, PROBE_TOL, compare

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("libs")]

THREADS = os.cpu_count() or 1


def _oracle(op, n, interval=None):
    desc, probes = oracle_inputs(op)
    return oracle.run(desc, probes, n, op.probe_interval if interval is None else interval,
                      engine=oracle.SSE_COMPRESSED_MT, threads=THREADS)


def test_l256_full_1000_timesteps_bitwise():
    """L256 (257^3 nodes, UPML-8, 40 bricks, 50 ohm port), all 1000
    timesteps: the pulse crosses the bricks and reaches the UPML."""
    op = Operator(scenes.l256(nr_ts=1000))
    ref = _oracle(op, 1000)
    eng = Engine(op)
    eng.iterate(1000)
    compare(op, eng, ref)


def test_d192_full_3000_timesteps():
    """D192 (193^3 graded nodes, UPML-8, Drude and Lorentz bricks), all
    3000 timesteps: the exact-table engine bit-identical, the default
    factorized-geometry engine within the tolerance."""
    op = Operator(scenes.d192(nr_ts=3000))
    ref = _oracle(op, 3000)
    exact = Engine(CompressedOperator(op, mode="exact"))
    exact.iterate(3000)
    compare(op, exact, ref)
    exact.close()
    cop = CompressedOperator(op)
    assert cop.factorized
    eng = Engine(cop)
    eng.iterate(3000)
    compare(op, eng, ref, bitwise=False)


def test_drude_metamaterial_plane_wave_full_6000_timesteps_bitwise():
    """The double-negative Drude slab plane wave (E and H ADE both on,
    PMC / PEC / Mur walls, a whole-plane soft E excitation), 6000
    timesteps: the pulse crosses the slab and leaves through the Mur face;
    bit-identical, on both kernel families."""
    op = Operator(scenes.drude_metamaterial(nr_ts=6000))
    ref = _oracle(op, 6000)
    for kernel in ("tma", "direct"):
        eng = Engine(op, kernel=kernel)
        eng.iterate(6000)
        compare(op, eng, ref)
        eng.close()


def test_b96_jobs_full_1500_timesteps_in_one_batch():
    """Four B96 jobs (two PEC, two UPML-8, uneven non-cubic grids) advanced
    together by the persistent batched kernels for the full 1500 timesteps:
    each job bit-identical to the oracle."""
    ops = [Operator(scenes.b96_job(s, nr_ts=1500)) for s in range(4)]
    jobs = [Engine(CompressedOperator(op), kernel="tma") for op in ops]
    b = Batch(jobs, graph_steps=16)
    b.iterate(1500)
    for op, e in zip(ops, jobs):
        assert e.num_timesteps == 1500
        compare(op, e, _oracle(op, 1500))


# serving jobs of each kind: dielectric + UPML, Lorentz, Drude
SERVE_SEEDS = {0: "dielectric", 4: "lorentz", 21: "drude", 33: "drude"}


def test_serve_jobs_full_length_match_oracle():
    """Serving-stream jobs run through the server to their own end
    criterion (-40 dB energy decay, or the 20000-timestep cap) while they
    share the GPU: each job's probe series and final fields equal the
    oracle's run of the same number of timesteps, and the oracle's energy
    record stops the job at the same sample."""
    crit = 1e-4
    srv = Server(round_steps=128, build_workers=2)
    ids = {}
    for seed, kind in SERVE_SEEDS.items():
        sc = scenes.serve_job(seed)
        assert sc.meta["kind"] == kind
        ids[seed] = srv.submit(sc, end_crit=crit, keep_fields=True)
    srv.wait(0, timeout=900)
    for seed, jid in ids.items():
        st = srv.status(jid)
        assert st["state"] == "done", st
        n = st["timesteps"]
        op = Operator(scenes.serve_job(seed))
        ref = _oracle(op, n, interval=st["probe_interval"])
        s = srv.samples(jid)
        assert np.array_equal(s.ts, ref["ts"])
        for p in range(s.values.shape[1]):
            assert rel_l2(s.values[:, p], ref["values"][:, p]) <= PROBE_TOL, (seed, p)
        assert np.array_equal(s.values, ref["values"]), seed
        V, I = srv.fields(jid)
        assert rel_max(V, ref["volt"]) <= FIELD_TOL and rel_max(I, ref["curr"]) <= FIELD_TOL
        assert np.array_equal(V.view(np.uint32), ref["volt"].view(np.uint32)), seed
        assert np.array_equal(I.view(np.uint32), ref["curr"].view(np.uint32)), seed
        # RunFDTD's rule (openems.cpp:1285-1314), checked at every sample, on
        # the oracle's own energies: stop at the first sample whose energy
        # over the largest so far is <= crit.  The two energies are sums in
        # different orders, so a crossing within 1e-6 of crit may fall on
        # either side.
        e = ref["energy"]
        emax = np.maximum.accumulate(e)
        ratio = np.where(emax > 0, e / np.where(emax > 0, emax, 1), 1.0)
        hit = np.nonzero(ratio <= crit)[0]
        first = int(ref["ts"][hit[0]]) if len(hit) else None
        if first != (n if n < 20000 else None):
            k = int(np.nonzero(ref["ts"] == n)[0][0])
            assert abs(ratio[k] / crit - 1) < 1e-6 or (first is not None and abs(ratio[hit[0]] / crit - 1) < 1e-6), \
                (seed, n, first)
    srv.close()


@pytest.mark.parametrize("name", ["port_box.xml", "lorentz_mur.xml", "drude_mtm.xml"])
def test_xml_scene_full_length_matches_oracle(name):
    """openEMS XML input: the engine library's reader + operator on the GPU
    against the oracle's own XML reader + operator + stepping, over the
    document's NumberOfTimesteps."""
    from oracle.xml_spec import xml_spec
    from helpers import assert_same_operator
    path = os.path.join(os.path.dirname(__file__), "golden", name)
    sc = Scene.from_xml(path)
    op = Operator(sc)
    ref_op = oracle.Operator(xml_spec(path), threads=THREADS)
    assert_same_operator(op, ref_op)
    n = sc.nr_ts
    ref = oracle.run(ref_op.desc, ref_op.probes, n, ref_op.probe_interval, engine=oracle.BASIC)
    cop = CompressedOperator(op)  # factorized geometry on a graded mesh: within the tolerance
    eng = Engine(cop)
    eng.iterate(n)
    assert np.isfinite(ref["volt"]).all()
    compare(op, eng, ref, bitwise=not cop.factorized)
