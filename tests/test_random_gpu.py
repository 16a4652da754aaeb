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


@pytest.mark.parametrize("cfg", [dict(graph_steps=8, chains=2),
                                 dict(graph_steps=1, tile_y=4, blocks_per_sm=2, x_chunk=5, stages=4),
                                 dict(graph_steps=16, tile_y=8, blocks_per_sm=-1, chains=3, x_chunk=32),
                                 dict(graph_steps=5, tile_y=4, blocks_per_sm=-1, x_chunk=2, stages=6)])
def test_random_scenes_in_one_batch_match_oracle(cfg):
    """The uniform random scenes as one batch, under persistent and
    one-block-per-item schedules, both tile heights, job-range chains and
    several x-chunks, stage counts and graph lengths."""
    ops = [Operator(random_scene(seed)) for seed in SEEDS]
    refs = [_reference(op, seed) for op, seed in zip(ops, SEEDS)]
    jobs = [Engine(CompressedOperator(op), kernel="tma") for op in ops]
    b = Batch(jobs, **cfg)
    b.iterate(NR_TS - 41)
    b.iterate(41)
    for op, eng, ref in zip(ops, jobs, refs):
        assert eng.num_timesteps == NR_TS
        compare(op, eng, ref)


# ------------------------------------------------------------------ the wider sweep
EXT_SEEDS = list(range(200, 212))


def random_scene_ext(seed: int) -> Scene:
    """The extensions around the hot path, drawn at random: Mur faces, one
    signal of the reference's five (Gaussian, sinusoid, Dirac, step, custom
    function of t), soft excitations with random vectors, lumped RLC
    elements (series or parallel), Lorentz / Drude of dispersion order 2,
    voltage lines and current loops.  Placements keep to what the engine
    provides: no Lorentz / Drude or excitation within a line of a Mur face,
    no RLC element on an excited edge or inside a Lorentz / Drude brick."""
    from wipems_gb300.fdtd import BC_MUR
    rng = np.random.default_rng(seed)
    cells = [int(rng.integers(14, 45)) for _ in range(3)]
    delta = float(rng.choice([0.5, 1.0]))
    lines = [uniform_lines(c, delta) for c in cells]
    s = Scene(*lines, 1e-3)
    bc, pml = [], []
    for a in range(3):
        r = rng.random()
        if r < 0.3 and cells[a] >= 18:
            k = int(rng.integers(2, min(6, (cells[a] - 14) // 2) + 1))
            bc += [BC_PML, BC_PML]
            pml += [k, k]
        else:
            bc += [int(rng.choice([BC_PEC, BC_PMC, BC_MUR, BC_MUR])) for _ in range(2)]
            pml += [0, 0]
    s.set_boundary(bc, pml)
    nts = NR_TS
    f0 = float(rng.uniform(3e9, 15e9))
    kind = int(rng.integers(0, 5))
    if kind == 0:
        s.set_gauss_excite(f0, f0, nts)
    elif kind == 1:
        s.set_sinus_excite(f0, nts)
    elif kind == 2:
        s.set_dirac_excite(f0, nts)
    elif kind == 3:
        s.set_step_excite(f0, nts)
    else:
        s.set_custom_excite(f"sin(2*pi*{f0:.6g}*t)*exp(-((t-2e-10)/8e-11)^2)", f0, nts)
    # margins: 3 lines from a Mur face or the UPML for everything placed inside
    lo = [(pml[2 * a] + 1) if bc[2 * a] == BC_PML else 3 for a in range(3)]
    hi = [(cells[a] - pml[2 * a + 1] - 1) if bc[2 * a + 1] == BC_PML else cells[a] - 3 for a in range(3)]
    prio = 10
    for _ in range(int(rng.integers(0, 4))):
        start, stop = _box(rng, lines, lo, hi, 8)
        s.add_material(start, stop, eps_r=float(rng.uniform(1, 8)),
                       kappa=float(math.exp(rng.uniform(math.log(1e-4), 0.0))) if rng.random() < 0.5 else 0.0,
                       priority=prio)
        prio += 1
    disp_boxes = []
    if rng.random() < 0.5:
        start, stop = _box(rng, lines, lo, hi, 6)
        fL = float(rng.uniform(4e9, 12e9))
        s.add_lorentz(start, stop, eps_r=2.0, plasma_f=[fL, float(rng.uniform(3e9, 8e9))], relax_t=[1e-9, 2e-9],
                      pole_f=[fL * 0.8, 0.0], priority=prio)
        disp_boxes.append((start, stop))
        prio += 1

    def inside(p, box):
        return all(box[0][a] <= p[a] <= box[1][a] for a in range(3))

    def pick_edge():
        """A z/y/x edge at least two lines inside the margins and clear of
        the Lorentz / Drude bricks."""
        for _ in range(100):
            d = int(rng.integers(0, 3))
            c = [int(rng.integers(lo[a] + 2, max(lo[a] + 3, hi[a] - 2))) for a in range(3)]
            p0 = [float(lines[a][c[a]]) for a in range(3)]
            p1 = list(p0)
            p1[d] = float(lines[d][c[d] + 1])
            if not any(inside(p0, b) or inside(p1, b) for b in disp_boxes):
                return d, c, p0, p1
        raise RuntimeError("no free edge")

    used = set()
    d, c, p0, p1 = pick_edge()  # a soft excitation on one edge, random vector
    vec = [0.0, 0.0, 0.0]
    vec[d] = float(rng.choice([-1.0, 1.0])) * float(rng.uniform(0.5, 2.0))
    s.add_excitation(p0, p1, vec, priority=500)
    used.add(tuple(c))
    s.add_probe(p0, p1, 0, name="v_exc")
    for k in range(int(rng.integers(0, 3))):
        d, c, p0, p1 = pick_edge()
        if tuple(c) in used:
            continue
        used.add(tuple(c))
        series = bool(rng.random() < 0.5)
        # a series element whose impedance at the signal's maximum frequency
        # is far above the edge's own capacitance gets that capacitance cut
        # to 1/20 of its impedance (operator_ext_lumpedRLC.cpp:357-364) after
        # the timestep is fixed, and grows; series elements stay low-ohmic
        R = float(rng.uniform(5, 40)) if series else float(rng.uniform(10, 200))
        s.add_lumped_rlc(p0, p1, d, R=R, L=float(rng.uniform(0.1e-9, 1e-9)) if series else float(rng.uniform(0.5e-9, 5e-9)),
                         Cap=float(rng.uniform(1e-12, 5e-12)) if series else float(rng.uniform(0.1e-12, 2e-12)),
                         series=series, caps=False, priority=900 + k)
        s.add_probe(p0, p1, 0, name=f"v_rlc{k}")
    # a current loop around a random edge and the field at a random node
    d, c, p0, p1 = pick_edge()
    half = [0.5 * (lines[a][c[a]] + lines[a][c[a] + 1]) for a in range(3)]
    a_lo = [float(lines[a][c[a]]) - 0.5 * delta for a in range(3)]
    a_hi = [float(lines[a][c[a]]) + 0.5 * delta for a in range(3)]
    a_lo[d] = a_hi[d] = half[d]
    s.add_probe(a_lo, a_hi, 1, norm_dir=d, name="i_loop")
    q = [float(lines[a][int(rng.integers(0, len(lines[a])))]) for a in range(3)]
    s.add_probe(q, q, int(rng.choice([2, 3])), name="field")
    return s


@pytest.mark.parametrize("seed", EXT_SEEDS)
def test_random_extension_scene_matches_oracle(seed):
    """The wider sweep, with a checkpoint taken mid-run and restored into a
    fresh engine for half of the seeds: bit-identical to the oracle."""
    op = Operator(random_scene_ext(seed))
    ref = _reference(op, seed)
    cop = CompressedOperator(op)
    rng = np.random.default_rng(1000 + seed)
    kw = _engine_options(rng)
    eng = Engine(cop, **kw)
    parts = _splits(rng, NR_TS)
    if rng.random() < 0.5 and len(parts) > 1:
        eng.iterate(parts[0])
        blob = eng.checkpoint()
        eng.close()
        eng = Engine(cop, **kw)
        eng.restore(blob)
        parts = parts[1:]
    for n in parts:
        eng.iterate(n)
    assert eng.num_timesteps == NR_TS
    compare(op, eng, ref)


class _ServedJob:
    """A served job's results with the Engine methods compare() reads."""

    def __init__(self, srv, jid):
        self.srv, self.jid = srv, jid

    def samples(self):
        return self.srv.samples(self.jid)

    def fields(self):
        return self.srv.fields(self.jid)


def test_random_scenes_through_the_server_match_oracle():
    """Both sweeps as one stream through the server, with persistent-batch
    rounds for the jobs a batch takes and plain engines beside them for the
    rest (Mur faces, lumped RLC, dispersion of order 2): every job's samples
    and fields equal the oracle's."""
    from wipems_gb300 import Server
    cases = [(s, lambda s=s: random_scene(s)) for s in SEEDS] + [(s, lambda s=s: random_scene_ext(s)) for s in EXT_SEEDS]
    srv = Server(round_steps=41, build_workers=2, batch_min_jobs=3)
    ids = {seed: srv.submit(make(), keep_fields=True) for seed, make in cases}
    srv.wait(0, timeout=600)
    st = srv.stats()
    assert st["jobs_done"] == len(ids) and st["jobs_failed"] == 0
    for seed, make in cases:
        op = Operator(make())
        assert srv.status(ids[seed])["timesteps"] == NR_TS
        compare(op, _ServedJob(srv, ids[seed]), _reference(op, seed))
    srv.close()


@pytest.mark.parametrize("seed", SEEDS[:4] + EXT_SEEDS[:6])
def test_random_fd_accumulation_matches_oracle_dft(seed):
    """Frequency-domain accumulation on the device (integral and field
    probes) in random scenes and tilings against the DFT over the oracle's
    samples at the FD steps."""
    op = Operator(random_scene_ext(seed) if seed in EXT_SEEDS else random_scene(seed))
    rng = np.random.default_rng(3000 + seed)
    eng = Engine(CompressedOperator(op), **_engine_options(rng))
    freqs = eng.set_frequencies(np.linspace(1e9, float(rng.uniform(5e9, 15e9)), 7))
    fdint = eng.fd_interval
    for n in _splits(rng, NR_TS):
        eng.iterate(n)
    got, count = eng.fd_results()
    ref = oracle.run(*oracle_inputs(op), NR_TS, fdint, engine=oracle.BASIC)
    assert count == len(ref["ts"]) == NR_TS // fdint + 1
    dual = np.array([0.5 if t in (1, 3) else 0.0 for t in eng.probe_types])
    t = (ref["ts"][:, None] + dual[None, :]) * op.dT
    phase = np.exp(-2j * np.pi * freqs[None, None, :] * t[:, :, None])
    want = np.einsum("sp,spf->pf", ref["values"], phase) * 2 * op.dT * fdint
    scale = max(np.abs(want).max(), 1e-300)
    assert np.max(np.abs(got - want)) <= 1e-12 * scale


@pytest.mark.parametrize("seed", SEEDS[:3] + GRADED_SEEDS[:2] + EXT_SEEDS[:3])
def test_random_field_dumps_equal_reference_interpolation(seed):
    """Field dumps of random boxes (corners in either order, sub-sampling
    steps 1 to 4, boxes on the boundary lines) after a random run: E and H
    with no, node and cell interpolation equal the reference interpolation
    (engine_interface_fdtd.cpp:60-200, restated in tests/helpers.py) of the
    engine's own fields, bit for bit."""
    from helpers import dump_reference
    graded = seed in GRADED_SEEDS
    op = Operator(random_scene_ext(seed) if seed in EXT_SEEDS else random_scene(seed, graded=graded))
    rng = np.random.default_rng(4000 + seed)
    eng = Engine(CompressedOperator(op), **_engine_options(rng))
    eng.iterate(int(rng.integers(20, NR_TS)))
    V, I = eng.fields()
    lines = [np.ctypeslib.as_array(op.desc.lines[a], shape=(op.num_lines[a],)).copy() for a in range(3)]
    unit, N = float(op.desc.unit), op.num_lines
    for _ in range(6):
        a = [int(rng.integers(0, n)) for n in N]
        b = [int(rng.integers(0, n)) for n in N]
        step = tuple(int(rng.integers(1, 5)) for _ in range(3))
        for field in ("E", "H"):
            for interp in ("none", "node", "cell"):
                got = eng.dump_field(field, interp, tuple(a), tuple(b), step)
                ref = dump_reference(V, I, lines, unit, field, interp, tuple(a), tuple(b), step)
                assert got.shape == ref.shape, (field, interp, a, b, step)
                assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (field, interp, a, b, step)


@pytest.mark.parametrize("stream_seed", [0, 1])
def test_random_server_stream_equals_solo_runs(stream_seed):
    """A random stream through the server under load: random scenes of both
    sweeps with their own timestep counts, half of them with an energy
    criterion, an HBM budget that holds only part of the stream (admission
    waits for retirements), batch rounds, a random round length and tile
    share.  Every job ends exactly as the plain engine does with the same
    settings alone: stopping timestep, samples, energies and fields."""
    from wipems_gb300 import Server
    from test_server_gpu import _same
    rng = np.random.default_rng(7000 + stream_seed)
    picks = rng.permutation(SEEDS + EXT_SEEDS)[:18]
    jobs = []
    for s in picks:
        s = int(s)
        nts = int(rng.integers(60, 400))
        crit = float(rng.choice([0.0, 1e-2, 1e-3]))
        jobs.append((s, nts, crit))

    def make(s, nts):  # the run length is the job's max_timesteps (nts), on both sides
        return random_scene_ext(s) if s in EXT_SEEDS else random_scene(s)

    probe = Server(max_active=1)
    j0 = probe.submit(make(*jobs[0][:2]), max_timesteps=jobs[0][1])
    probe.wait(j0, timeout=300)
    foot = probe.status(j0)["footprint"]
    probe.close()
    srv = Server(hbm_budget=int(6 * foot), round_steps=int(rng.integers(17, 90)), build_workers=2,
                 batch_min_jobs=3, tile_share=int(rng.choice([2, 4, 8])))
    ids = [srv.submit(make(s, nts), end_crit=crit, max_timesteps=nts, keep_fields=True) for s, nts, crit in jobs]
    srv.wait(0, timeout=900)
    st = srv.stats()
    assert st["jobs_done"] == len(ids) and st["jobs_failed"] == 0
    for (s, nts, crit), jid in zip(jobs, ids):
        e = Engine(Operator(make(s, nts)), end_crit=crit, max_timesteps=nts)
        e.iterate(nts)
        _same(e, srv, jid)
    srv.close()


def test_random_scenes_on_the_fused_kernel_match_oracle():
    """The optional single-pass kernel (kernel="fused": uniform meshes
    without Lorentz / Drude, Mur or lumped RLC) on the random scenes it
    takes, with random x-chunks, stage counts and run splits: bitwise."""
    import copy
    from wipems_gb300 import SceneSpec
    ran = 0
    for seed in SEEDS:
        spec = copy.deepcopy(random_scene(seed).spec)  # the scene without its Lorentz / Drude bricks
        spec["prims"] = [p for p in spec["prims"] if not p.get("disp_order")]
        sp = SceneSpec(*spec["lines"], spec["unit"])
        sp.spec = spec
        op = Operator(Scene.from_spec(sp))
        cop = CompressedOperator(op)
        if cop.factorized or cop.info["num_ade_nodes"]:
            continue
        rng = np.random.default_rng(6000 + seed)
        eng = Engine(cop, kernel="fused", x_chunk=int(rng.integers(1, 17)), stages=int(rng.integers(3, 6)),
                     use_graphs=bool(rng.random() < 0.5))
        for n in _splits(rng, NR_TS):
            eng.iterate(n)
        compare(op, eng, _reference(op, ("no dispersion", seed)))
        ran += 1
    assert ran >= 12
