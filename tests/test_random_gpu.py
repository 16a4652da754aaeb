"""Seeded random scenes against the oracle, bit for bit.

Each seed draws a grid (6 to 60 cells per axis, odd sizes far from the
32 x 4 / 32 x 8 tiles), boundaries per axis (PEC / PMC faces, UPML on
both faces or an 8-layer UPML on one), dielectric, magnetic and metal bricks, Lorentz / Drude bricks of
the electric and the magnetic family, a 50 ohm lumped port along a random
axis and field probes; the engine draws its kernel family, tile height,
x-chunk, ring stages, CUDA-graph use and the way the run is split into
iterate calls.  Fields and samples must equal the oracle's (its own
operator build and the reference's stepping order) exactly.  The same
scenes advanced together in one batch must give the same bits again.
"""
import math

import numpy as np
import pytest

import oracle
from wipems_gb300 import Batch, CompressedOperator, Engine, Operator, Scene
from wipems_gb300.fdtd import BC_PEC, BC_PMC, BC_PML
from wipems_gb300.scenes import graded_lines, uniform_lines

from helpers import oracle_inputs
from test_parity_gpu import compare

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("libs")]

NR_TS = 180
SEEDS = list(range(16))
GRADED_SEEDS = [100, 101, 102, 103]


def _box(rng, lines, lo, hi, emax):
    start, stop = [], []
    for a in range(3):
        e = int(rng.integers(1, max(2, min(emax, hi[a] - lo[a]) + 1)))
        s0 = int(rng.integers(lo[a], max(lo[a] + 1, hi[a] - e + 1)))
        start.append(float(lines[a][s0]))
        stop.append(float(lines[a][min(s0 + e, hi[a])]))
    return start, stop


def random_scene(seed: int, graded: bool = False) -> Scene:
    rng = np.random.default_rng(seed)
    cells = [int(rng.integers(6, 61)) for _ in range(3)]
    if graded:
        lines = [graded_lines(c, rng) for c in cells]
    else:
        delta = float(rng.choice([0.25, 0.5, 1.0]))
        lines = [uniform_lines(c, delta) for c in cells]
    s = Scene(*lines, 1e-3)
    # per axis: PEC / PMC faces, a UPML of 2 to 6 layers on both faces, or
    # an 8-layer UPML on one face.  openEMS grades an upper UPML with the
    # lower face's size (8 when that face is not PML), so a one-sided UPML
    # of other than 8 layers gets a profile squeezed from 8 layers, which
    # makes the fields grow; such scenes are left out here.
    bc, pml = [], []
    for a in range(3):
        r = rng.random()
        walls = [int(rng.choice([BC_PEC, BC_PMC])) for _ in range(2)]
        if r < 0.4 and cells[a] >= 18:
            k = int(rng.integers(2, min(6, (cells[a] - 14) // 2) + 1))
            bc += [BC_PML, BC_PML]
            pml += [k, k]
        elif r < 0.6 and cells[a] >= 20:
            side = int(rng.integers(0, 2))
            walls[side] = BC_PML
            bc += walls
            pml += [8 if side == 0 else 0, 8 if side == 1 else 0]
        else:
            bc += walls
            pml += [0, 0]
    s.set_boundary(bc, pml)
    f0 = float(rng.uniform(2e9, 20e9))
    s.set_gauss_excite(f0, f0, NR_TS)
    # everything but the port stays one line clear of the UPML slabs
    lo = [pml[2 * a] + 1 for a in range(3)]
    hi = [cells[a] - pml[2 * a + 1] - 1 for a in range(3)]
    prio = 10
    for _ in range(int(rng.integers(0, 6))):
        start, stop = _box(rng, lines, lo, hi, 12)
        kind = rng.random()
        if kind < 0.15:
            s.add_metal(start, stop, priority=prio)
        else:
            s.add_material(start, stop, eps_r=float(rng.uniform(1, 10)),
                           kappa=float(math.exp(rng.uniform(math.log(1e-4), 0.0))) if rng.random() < 0.6 else 0.0,
                           mue_r=float(rng.uniform(1, 3)) if rng.random() < 0.3 else 1.0,
                           sigma=float(rng.uniform(0, 50)) if rng.random() < 0.2 else 0.0, priority=prio)
        prio += 1
    for _ in range(int(rng.integers(0, 3))):
        start, stop = _box(rng, lines, lo, hi, 10)
        fp = float(rng.uniform(3e9, 9e9))
        tau = 1.0 / float(rng.uniform(1e8, 1e9))
        r = rng.random()
        if r < 0.35:  # electric Drude
            s.add_lorentz(start, stop, plasma_f=[fp], relax_t=[tau], priority=prio)
        elif r < 0.7:  # electric Lorentz
            fL = float(rng.uniform(4e9, 15e9))
            s.add_lorentz(start, stop, eps_r=float(rng.uniform(2, 4)), plasma_f=[fL * math.sqrt(rng.uniform(1, 4))],
                          relax_t=[1e-9], pole_f=[fL], priority=prio)
        else:  # magnetic Drude, with or without an electric one
            kw = dict(plasma_f=[fp], relax_t=[tau]) if rng.random() < 0.5 else {}
            s.add_lorentz(start, stop, mue_plasma_f=[fp], mue_relax_t=[tau], priority=prio, **kw)
        prio += 1
    # the port: one cell across, four cells along its axis, inside the slabs
    d = int(rng.integers(0, 3))
    c = [int(rng.integers(lo[a] + 2, max(lo[a] + 3, hi[a] - 2))) for a in range(3)]
    start = [float(lines[a][c[a]]) for a in range(3)]
    stop = [float(lines[a][min(c[a] + 1, len(lines[a]) - 1)]) for a in range(3)]
    start[d] = float(lines[d][max(c[d] - 2, 0)])
    stop[d] = float(lines[d][min(c[d] + 2, len(lines[d]) - 1)])
    s.add_lumped_port(start, stop, d, 50.0, excite=1.0, priority=1000)
    for ptype in (2, 3):
        p = [float(lines[a][int(rng.integers(0, len(lines[a])))]) for a in range(3)]
        s.add_probe(p, p, ptype, name=f"f{ptype}")
    return s


def _engine_options(rng):
    if rng.random() < 0.3:
        return dict(kernel="direct", tile_y=int(rng.choice([1, 2, 4, 8])), x_chunk=int(rng.integers(1, 21)),
                    use_graphs=bool(rng.random() < 0.5))
    return dict(kernel="tma", tile_y=int(rng.choice([4, 8])), x_chunk=int(rng.integers(1, 21)),
                stages=int(rng.integers(3, 7)), use_graphs=bool(rng.random() < 0.7))


def _splits(rng, total):
    cuts = sorted(set(int(x) for x in rng.integers(1, total, size=int(rng.integers(0, 4)))))
    parts, prev = [], 0
    for k in cuts + [total]:
        parts.append(k - prev)
        prev = k
    return parts


_REF = {}


def _reference(op, key):
    if key not in _REF:
        _REF[key] = oracle.run(*oracle_inputs(op), NR_TS, op.probe_interval, engine=oracle.BASIC)
    return _REF[key]


@pytest.mark.parametrize("seed", SEEDS + GRADED_SEEDS)
def test_random_scene_matches_oracle(seed):
    graded = seed in GRADED_SEEDS
    op = Operator(random_scene(seed, graded=graded))
    ref = _reference(op, seed)
    cop = CompressedOperator(op)
    rng = np.random.default_rng(1000 + seed)
    kw = _engine_options(rng)
    eng = Engine(cop, **kw)
    for n in _splits(rng, NR_TS):
        eng.iterate(n)
    assert eng.num_timesteps == NR_TS
    compare(op, eng, ref, bitwise=not cop.factorized)


def test_random_scenes_in_one_batch_match_oracle():
    ops = [Operator(random_scene(seed)) for seed in SEEDS]
    refs = [_reference(op, seed) for op, seed in zip(ops, SEEDS)]
    jobs = [Engine(CompressedOperator(op), kernel="tma") for op in ops]
    b = Batch(jobs, graph_steps=8, chains=2)
    b.iterate(NR_TS - 41)
    b.iterate(41)
    for op, eng, ref in zip(ops, jobs, refs):
        assert eng.num_timesteps == NR_TS
        compare(op, eng, ref)
