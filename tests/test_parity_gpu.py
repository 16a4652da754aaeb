"""GPU parity: the CUDA engine (through the C ABI) against the oracle.

Bar: probe series within 1e-5 relative L2, final
fields within 1e-4 relative max-norm.  The kernels keep the reference's
FP32 operation order, so fields are in fact required to be bit-identical;
probe sums differ only by reduction order (device warp sums in double vs the
reference's sequential double / float accumulation), energy likewise.
"""
import os

import numpy as np
import pytest

import oracle
from wipems_gb300 import CompressedOperator, Engine, Operator, scenes

from helpers import cavity_check, oracle_inputs, rel_l2, rel_max, with_signal

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("libs")]

PROBE_TOL = 1e-5
FIELD_TOL = 1e-4


def probe_columns(types):
    """Column groups of the sample rows, one per probe: a voltage or current
    probe is one column, an E or H field probe the three columns of its
    field vector (ProcessFieldProbe records the vector)."""
    groups, c = [], 0
    while c < len(types):
        w = 3 if types[c] in (2, 3) else 1
        groups.append(list(range(c, c + w)))
        c += w
    return groups


def compare(op, eng, ref, bitwise=True):
    """Probe series and fields against an oracle run; bit-identical fields
    unless bitwise is False (factorized geometry on graded meshes).  Each
    probe's series is held to the relative L2 bound as a whole (a field
    probe's three components together)."""
    s = eng.samples()
    assert np.array_equal(s.ts, ref["ts"]), (s.ts[:5], ref["ts"][:5])
    for cols in probe_columns(s.probe_types):
        assert rel_l2(s.values[:, cols], ref["values"][:, cols]) <= PROBE_TOL, cols
    if bitwise:  # the probe sums run in the reference's order and precision
        assert np.array_equal(s.values, ref["values"])
    e_ok = ref["energy"] > 0
    if e_ok.any():
        assert np.max(np.abs(s.energy[e_ok] / ref["energy"][e_ok] - 1)) < 1e-6
    V, I = eng.fields()
    assert rel_max(V, ref["volt"]) <= FIELD_TOL
    assert rel_max(I, ref["curr"]) <= FIELD_TOL
    if bitwise:
        dv = int((V.view(np.uint32) != ref["volt"].view(np.uint32)).sum())
        di = int((I.view(np.uint32) != ref["curr"].view(np.uint32)).sum())
        assert dv == 0 and di == 0, (dv, di, rel_max(V, ref["volt"]), rel_max(I, ref["curr"]))


@pytest.mark.parametrize("kernel", ["tma", "direct"])
@pytest.mark.parametrize("kind", ["pec", "upml", "graded", "drude", "lorentz", "mixed", "mur", "rlc", "rlc_mur",
                                  "magnetic", "magnetic_graded", "multipole", "multipole_graded"])
def test_mini_scenes_match_oracle(kind, kernel):
    """Uniform meshes: bit-identical.  Graded meshes (automatic factorized
    geometry): within the probe / field tolerance of the oracle on the
    operator's own coefficients."""
    op = Operator(scenes.mini(kind, nr_ts=400))
    ref = oracle.run(*oracle_inputs(op), 400, op.probe_interval, engine=oracle.BASIC)
    cop = CompressedOperator(op)
    eng = Engine(cop, kernel=kernel)
    eng.iterate(400)
    compare(op, eng, ref, bitwise=not cop.factorized)


@pytest.mark.parametrize("kind", ["upml", "rlc_mur"])
@pytest.mark.parametrize("etype,f", [(1, 6e9), (2, 2e10), (3, 0.0), (10, 6e9)])
def test_excitation_signals_match_oracle(kind, etype, f):
    """Sinusoid (periodic: the signal index wraps with the period), Dirac
    pulse, step and a custom function of t through the graph-chunked TMA
    engine: bit-identical."""
    fn = "sin(2*pi*6e9*t)*exp(-((t-3e-10)/1e-10)^2)" if etype == 10 else ""
    op = Operator(with_signal(scenes.mini(kind, nr_ts=700), etype, f, fn))
    ref = oracle.run(*oracle_inputs(op), 700, op.probe_interval, engine=oracle.BASIC)
    eng = Engine(CompressedOperator(op), kernel="tma")
    eng.iterate(700)
    compare(op, eng, ref)


def expanded_desc(op, cop):
    """A copy of op's engine description carrying the coefficients the
    compressed operator's kernels apply (fdtd_cop_expand / _ext: the
    factorized vi / iv, and the UPML and ADE terms after the merging of
    rounding variants), with the arrays kept alive on the returned object."""
    import ctypes
    from wipems_gb300 import _abi
    PF = ctypes.POINTER(ctypes.c_float)
    keep = [np.ascontiguousarray(a) for a in cop.expand()[:4]]
    d = type(op.desc).from_buffer_copy(op.desc)
    d.vv, d.vi, d.ii, d.iv = (a.ctypes.data_as(PF) for a in keep)
    N = op.num_lines
    ext = [cop.expand_ext(h) for h in (0, 1)]
    slabs = (_abi.FdtdUpmlDesc * max(1, op.desc.num_upml))()
    for s in range(op.desc.num_upml):
        u = op.desc.upml[s]
        slabs[s] = u
        st, nl = list(u.start), list(u.num_lines)
        sl = tuple(slice(st[a], st[a] + nl[a]) for a in range(3))
        for h, names in ((0, ("vv", "vvfo", "vvfn")), (1, ("ii", "iifo", "iifn"))):
            for k, name in enumerate(names):
                arr = np.ascontiguousarray(ext[h][1][3 * k:3 * k + 3][(slice(None),) + sl])
                keep.append(arr)
                setattr(slabs[s], name, arr.ctypes.data_as(PF))
    d.upml = ctypes.cast(slabs, ctypes.POINTER(_abi.FdtdUpmlDesc))
    ades = (_abi.FdtdAdeDesc * max(1, op.desc.num_ade_orders))()
    for o in range(op.desc.num_ade_orders):
        a = op.desc.ade[o]
        ades[o] = a
        c = a.count
        pos = [np.ctypeslib.as_array(a.pos[k], shape=(c,)) for k in range(3)] if c else [np.zeros(0, int)] * 3
        for h, names in ((0, ("v_int", "v_ext", "v_lor")), (1, ("i_int", "i_ext", "i_lor"))):
            terms = ext[h][0] if o == 0 else cop.expand_ade(h, o)
            for k, name in enumerate(names):
                if not getattr(a, name):
                    continue
                arr = np.ascontiguousarray(terms[3 * k:3 * k + 3][:, pos[0], pos[1], pos[2]].astype(np.float32))
                keep.append(arr)
                setattr(ades[o], name, arr.ctypes.data_as(PF))
    d.ade = ctypes.cast(ades, ctypes.POINTER(_abi.FdtdAdeDesc))
    keep += [slabs, ades]
    return d, keep


@pytest.mark.parametrize("kind", ["graded", "mixed", "magnetic_graded", "multipole_graded"])
def test_factorized_kernels_bitwise_against_expanded_operator(kind):
    """The factorized kernels apply exactly the coefficients fdtd_cop_expand
    and fdtd_cop_expand_ext report: run the oracle on those and require
    bit-identical fields."""
    op = Operator(scenes.mini(kind, nr_ts=300))
    cop = CompressedOperator(op)
    assert cop.factorized
    d, keep = expanded_desc(op, cop)
    ref = oracle.run(d, op.probes, 300, op.probe_interval, engine=oracle.BASIC)
    eng = Engine(cop)
    eng.iterate(300)
    compare(op, eng, ref, bitwise=True)


def test_multipole_dispersion_reset_and_tilings():
    """Dispersion of order 2 and 3: the states of the further orders are
    reset with the fields, and tile heights, x-chunks and graph chunking
    leave the result bit-identical; the batch refuses such jobs (they run
    as plain engines)."""
    from wipems_gb300 import Batch
    from wipems_gb300._abi import FdtdError
    op = Operator(scenes.mini("multipole", nr_ts=300))
    ref = oracle.run(*oracle_inputs(op), 300, op.probe_interval, engine=oracle.BASIC)
    for kw in (dict(tile_y=4, x_chunk=3), dict(tile_y=8, x_chunk=16, use_graphs=False)):
        eng = Engine(op, **kw)
        eng.iterate(120)
        eng.reset()
        eng.iterate(300)
        compare(op, eng, ref)
        eng.close()
    eng = Engine(op, kernel="tma")
    with pytest.raises(FdtdError) as ei:
        Batch([eng])
    assert "order > 1" in str(ei.value)


def test_exact_mode_on_graded_mesh_is_bitwise():
    op = Operator(scenes.mini("mixed", nr_ts=200))
    cop = CompressedOperator(op, mode="exact")
    ref = oracle.run(*oracle_inputs(op), 200, op.probe_interval, engine=oracle.BASIC)
    eng = Engine(cop)
    eng.iterate(200)
    compare(op, eng, ref, bitwise=True)


def test_p64_full_2000_steps():
    op = Operator(scenes.p64(nr_ts=2000))
    ref = oracle.run(*oracle_inputs(op), 2000, op.probe_interval, engine=oracle.SSE_COMPRESSED_MT,
                     threads=os.cpu_count())
    eng = Engine(op)
    eng.iterate(2000)
    compare(op, eng, ref)


def test_chunking_graphs_and_tiles_are_invisible():
    op = Operator(scenes.mini("upml", nr_ts=300))
    base = Engine(op, use_graphs=False)
    base.iterate(300)
    V0, I0 = base.fields()
    s0 = base.samples()
    for kw, chunks in [(dict(use_graphs=True), [300]), (dict(use_graphs=True), [7, 1, 50, 242]),
                       (dict(tile_y=4, x_chunk=5, kernel="direct"), [300]),
                       (dict(tile_y=1, x_chunk=64, kernel="direct"), [100, 200]),
                       (dict(x_chunk=3), [300]), (dict(x_chunk=64), [300]),
                       (dict(tile_y=8, x_chunk=3), [300]), (dict(tile_y=8, stages=4, x_chunk=16), [150, 150]),
                       (dict(kernel="direct", use_graphs=True), [300])]:
        e = Engine(op, **kw)
        for c in chunks:
            e.iterate(c)
        V, I = e.fields()
        assert np.array_equal(V.view(np.uint32), V0.view(np.uint32)), kw
        assert np.array_equal(I.view(np.uint32), I0.view(np.uint32)), kw
        s = e.samples()
        assert np.array_equal(s.ts, s0.ts)
        assert np.array_equal(s.values, s0.values), kw
        assert np.array_equal(s.energy, s0.energy), kw  # energy summed in an order fixed by the grid


def test_tma_tile_heights():
    """The two-pass TMA kernels run 4- or 8-row tiles (the autotuner picks);
    other heights are refused; 8-row tiles are bit-identical to the oracle
    on a graded exact-table grid with Lorentz/Drude nodes and UPML."""
    from wipems_gb300._abi import FdtdError
    op = Operator(scenes.mini("mixed", nr_ts=300))
    with pytest.raises(FdtdError):
        Engine(op, tile_y=2)
    cop = CompressedOperator(op, mode="exact")
    ref = oracle.run(*oracle_inputs(op), 300, op.probe_interval, engine=oracle.BASIC)
    eng = Engine(cop, tile_y=8)
    assert eng.stats()["tile_y"] == 8
    eng.iterate(300)
    compare(op, eng, ref)


def test_reset_and_compressed_upload_reproduce():
    op = Operator(scenes.mini("lorentz", nr_ts=200))
    cop = CompressedOperator(op)
    e1 = Engine(cop)
    e1.iterate(200)
    V1, I1 = e1.fields()
    s1 = e1.samples()
    e1.reset()
    assert e1.num_timesteps == 0
    e1.iterate(200)
    V2, I2 = e1.fields()
    assert np.array_equal(V1, V2) and np.array_equal(I1, I2)
    assert np.array_equal(e1.samples().values, s1.values)
    e2 = Engine(op)
    e2.iterate(200)
    assert np.array_equal(e2.fields()[0], V1)


def test_l256_full_size_first_steps_bitwise():
    op = Operator(scenes.l256(nr_ts=1000))
    n = 18
    ref = oracle.run(*oracle_inputs(op), n, op.probe_interval, engine=oracle.SSE_COMPRESSED_MT,
                     threads=os.cpu_count())
    eng = Engine(op)
    st = eng.stats()
    assert st["index_bytes"] == 2
    eng.iterate(n)
    compare(op, eng, ref)


def test_d192_full_size_first_steps():
    """D192 (graded mesh, UPML, Drude + Lorentz bricks) at full size: the
    default (factorized-geometry) engine within the probe / field tolerance,
    the exact-table engine (uint32 index) bit-identical to the oracle."""
    op = Operator(scenes.d192(nr_ts=3000))
    n = 40
    ref = oracle.run(*oracle_inputs(op), n, op.probe_interval, engine=oracle.SSE_COMPRESSED_MT,
                     threads=os.cpu_count())
    cop = CompressedOperator(op)
    assert cop.info["geometry_factored"] == 1 and cop.info["num_ade_nodes"] > 0
    eng = Engine(cop)
    eng.iterate(n)
    compare(op, eng, ref, bitwise=False)
    eng.close()
    exact = CompressedOperator(op, mode="exact")
    assert exact.info["index_bytes_e"] == 4
    eng = Engine(exact)
    eng.iterate(n)
    compare(op, eng, ref)


def test_cavity_resonances_on_gpu():
    sc = scenes.cavity(nr_ts=20000)
    op = Operator(sc)
    eng = Engine(op, probe_interval=1, max_timesteps=20000)
    eng.iterate(20000)
    s = eng.samples()
    t = s.ts * op.dT
    res = cavity_check([t] * 3, [s.values[:, k] for k in range(3)], sc.meta)
    assert all(res.values()), res


def test_energy_on_demand_equals_the_sample_energy():
    """fdtd_engine_energy sums the same per-node terms in the same fixed
    order as the sample steps: right after a sample step it returns the
    recorded energy bit for bit, for every kernel family."""
    op = Operator(scenes.mini("mixed", nr_ts=400))
    for kw in (dict(), dict(kernel="direct", tile_y=2, x_chunk=3), dict(x_chunk=1, stages=4)):
        eng = Engine(op, **kw)
        eng.iterate(5 * op.probe_interval)
        s = eng.samples()
        assert s.ts[-1] == eng.num_timesteps and s.energy[-1] > 0
        assert eng.energy() == s.energy[-1], kw
    op = Operator(scenes.mini("upml", nr_ts=400))
    eng = Engine(op, kernel="fused")
    eng.iterate(4 * op.probe_interval)
    assert eng.energy() == eng.samples().energy[-1]


def test_field_access_and_energy():
    op = Operator(scenes.mini("pec", nr_ts=100))
    eng = Engine(op)
    eng.iterate(60)
    V, I = eng.fields()
    assert eng.get_volt(2, 10, 8, 18) == V[2, 10, 8, 18]
    assert eng.get_curr(1, 5, 6, 7) == I[1, 5, 6, 7]
    ref = oracle.run(oracle_inputs(op)[0], [], 60, 0, engine=oracle.BASIC)
    eps0, mue0 = 8.85418781762e-12, 1.256637062e-6
    Vr, Ir = ref["volt"][:, :-1, :-1, :-1].astype(np.float64), ref["curr"][:, :-1, :-1, :-1].astype(np.float64)
    e_ref = eps0 * np.sum(Vr * Vr) + mue0 * np.sum(Ir * Ir)
    assert abs(eng.energy() / e_ref - 1) < 1e-6


# ---------------------------------------------------------------- fused kernel
@pytest.mark.parametrize("kind", ["pec", "upml"])
def test_fused_kernel_matches_oracle(kind):
    """The single-pass kernel (double-buffered fields, redundant halo E) is
    bit-identical to the reference stepping, across odd tile edges."""
    op = Operator(scenes.mini(kind, nr_ts=400))
    n = 301
    ref = oracle.run(*oracle_inputs(op), n, op.probe_interval, engine=oracle.BASIC)
    eng = Engine(op, kernel="fused")
    assert eng.stats()["kernel"] == 2
    eng.iterate(137)
    eng.iterate(n - 137)
    compare(op, eng, ref)


def test_fused_kernel_tilings_and_graphs_invisible():
    op = Operator(scenes.mini("upml", seed=2, nr_ts=400))
    ref = oracle.run(*oracle_inputs(op), 120, op.probe_interval, engine=oracle.BASIC)
    two_pass = Engine(op)
    two_pass.iterate(120)
    e0 = two_pass.samples().energy
    for kw in (dict(x_chunk=1), dict(x_chunk=3, stages=4), dict(x_chunk=16, use_graphs=False), dict(stages=5)):
        eng = Engine(op, kernel="fused", **kw)
        eng.iterate(57)
        eng.iterate(63)
        compare(op, eng, ref)
        assert np.array_equal(eng.samples().energy, e0), kw
        eng.close()


def test_fused_kernel_graded_exact_and_p64():
    """32-bit indices (graded mesh, exact table) and a grid whose last lines
    fall on tile edges (P64: 64 cells, the last y row and z column are
    owned by the tiles below them)."""
    op = Operator(scenes.mini("graded", nr_ts=400))
    cop = CompressedOperator(op, mode="exact")
    ref = oracle.run(*oracle_inputs(op), 200, op.probe_interval, engine=oracle.BASIC)
    eng = Engine(cop, kernel="fused")
    eng.iterate(200)
    compare(op, eng, ref)
    op = Operator(scenes.p64(nr_ts=2000))
    ref = oracle.run(*oracle_inputs(op), 700, op.probe_interval, engine=oracle.SSE_COMPRESSED_MT,
                     threads=os.cpu_count())
    eng = Engine(op, kernel="fused")
    eng.iterate(700)
    compare(op, eng, ref)
    V, I = eng.fields()
    assert eng.get_volt(2, 32, 31, 30) == V[2, 32, 31, 30]
    assert eng.get_curr(0, 63, 63, 63) == I[0, 63, 63, 63]


def test_fused_kernel_l256_first_steps_bitwise():
    op = Operator(scenes.l256(nr_ts=1000))
    n = 18
    ref = oracle.run(*oracle_inputs(op), n, op.probe_interval, engine=oracle.SSE_COMPRESSED_MT,
                     threads=os.cpu_count())
    eng = Engine(op, kernel="fused")
    eng.iterate(n)
    compare(op, eng, ref)


def test_fused_kernel_refuses_ade():
    from wipems_gb300._abi import FdtdError
    op = Operator(scenes.mini("drude", nr_ts=100))
    with pytest.raises(FdtdError) as ei:
        Engine(op, kernel="fused")
    assert ei.value.code == -5


def test_mur_chunking_graphs_and_excitation_on_the_face():
    """Mur faces through graph chunks and single steps, and a face that
    carries an excitation (active only after the pulse, start_ts), match
    the reference stepping bit for bit."""
    op = Operator(scenes.mini("mur", seed=1, nr_ts=700))
    ref = oracle.run(*oracle_inputs(op), 333, op.probe_interval, engine=oracle.BASIC)
    for kw in (dict(), dict(use_graphs=False, x_chunk=3)):
        eng = Engine(op, **kw)
        eng.iterate(100)
        eng.iterate(233)
        compare(op, eng, ref)
    from wipems_gb300 import Scene
    from wipems_gb300.fdtd import BC_MUR, BC_PEC
    from wipems_gb300.scenes import uniform_lines
    L = [uniform_lines(c, 0.5) for c in (24, 20, 30)]
    s = Scene(*L, 1e-3)
    s.set_boundary([BC_MUR, BC_MUR, BC_MUR, BC_MUR, BC_PEC, BC_MUR], [0] * 6)
    s.set_gauss_excite(10e9, 10e9, 600)
    # a soft Ez source on the xmin face (x = 0): that face starts after the pulse
    s.add_excitation([L[0][0], L[1][8], L[2][12]], [L[0][0], L[1][12], L[2][18]], [0, 0, 1], priority=5)
    s.add_probe([L[0][6], L[1][10], L[2][10]], [L[0][6], L[1][10], L[2][20]], 0)
    op = Operator(s)
    assert op.desc.mur[0].start_ts > 0
    n = op.desc.mur[0].start_ts + 60
    ref = oracle.run(*oracle_inputs(op), n, op.probe_interval, engine=oracle.BASIC)
    eng = Engine(op)
    eng.iterate(n)
    compare(op, eng, ref)


def test_rlc_through_graph_chunks_and_single_steps():
    """The lumped RLC pass keeps its Vd / J history in a ring indexed by the
    timestep, so CUDA-graph chunks, single steps and the direct kernels all
    reproduce the reference's pointer rotation bit for bit; the fused
    single-pass kernel refuses RLC elements."""
    op = Operator(scenes.mini("rlc_mur", seed=1, nr_ts=700))
    ref = oracle.run(*oracle_inputs(op), 333, op.probe_interval, engine=oracle.BASIC)
    for kw, chunks in ((dict(), [100, 233]), (dict(use_graphs=False, x_chunk=3), [1, 2, 330]),
                       (dict(kernel="direct"), [333])):
        eng = Engine(op, **kw)
        for c in chunks:
            eng.iterate(c)
        compare(op, eng, ref)
    from wipems_gb300._abi import FdtdError
    with pytest.raises(FdtdError, match="lumped RLC"):
        Engine(Operator(scenes.mini("rlc", nr_ts=100)), kernel="fused")


def test_probe_now_and_field_writes():
    """fdtd_engine_probe_now evaluates a voltage / current integral on the
    current fields in the sampler's order and precision (the engine
    interface of an openEMS processing that samples on its own schedule):
    times the probe's weight it equals the sample recorded at that
    timestep, bit for bit.  SetVolt / SetCurr write one value."""
    op = Operator(scenes.mini("upml", nr_ts=300))
    eng = Engine(op)
    eng.iterate(4 * op.probe_interval)
    s = eng.samples()
    assert s.ts[-1] == eng.num_timesteps
    for k, p in enumerate(op.probes):
        assert eng.probe_now(p) * p.weight == s.values[-1, k], k
    v = eng.get_volt(2, 5, 6, 7)
    eng.set_volt(2, 5, 6, 7, v + 1.5)
    assert eng.get_volt(2, 5, 6, 7) == np.float32(v + 1.5)
    eng.set_curr(0, 3, 4, 5, -2.25)
    assert eng.get_curr(0, 3, 4, 5) == -2.25


@pytest.mark.parametrize("kind", ["upml", "mur", "rlc_mur", "magnetic", "multipole", "graded"])
def test_axis_rotations_are_invisible(kind):
    """The device axes are a cyclic relabelling of the operator's
    (fdtd_compress_rot): every rotation gives the oracle's fields and
    probe samples bit for bit (the factorized graded case against the
    expanded coefficients, which do not depend on the rotation), and the
    API speaks in the operator's axes: field arrays, single values, E / H
    dumps with node and cell interpolation, and probe_now agree across
    rotations; a checkpoint restores only into an engine of the same
    rotation."""
    from wipems_gb300._abi import FdtdError
    op = Operator(scenes.mini(kind, nr_ts=300))
    base = CompressedOperator(op, rotation=0)
    if base.factorized:
        d, keep = expanded_desc(op, base)
        ref = oracle.run(d, op.probes, 300, op.probe_interval, engine=oracle.BASIC)
    else:
        ref = oracle.run(*oracle_inputs(op), 300, op.probe_interval, engine=oracle.BASIC)
    dumps, blobs = [], []
    for r in (0, 1, 2):
        cop = CompressedOperator(op, rotation=r)
        assert cop.rotation == r
        n = op.num_lines
        assert cop.info["device_lines"] == [n[r % 3], n[(1 + r) % 3], n[(2 + r) % 3]]
        eng = Engine(cop)
        eng.iterate(300)
        compare(op, eng, ref)
        dumps.append([eng.dump_field(f, i, start=(1, 2, 3), stop=(n[0] - 1, n[1] - 2, n[2] - 1), step=(2, 1, 3))
                      for f in ("E", "H") for i in ("node", "cell")]
                     + [np.float32(eng.get_volt(1, 4, 5, 6)), np.float32(eng.get_curr(2, 6, 5, 4))]
                     + [eng.probe_now(p) for p in op.probes if p.type in (0, 1)])
        blobs.append(eng.checkpoint())
        eng.close()
    for r in (1, 2):
        for k, (a, b) in enumerate(zip(dumps[0], dumps[r])):
            assert np.asarray(a).tobytes() == np.asarray(b).tobytes(), (r, k)
    other = Engine(CompressedOperator(op, rotation=1))
    with pytest.raises(FdtdError):
        other.restore(blobs[0])
    other.restore(blobs[1])
    assert other.num_timesteps == 300


@pytest.mark.parametrize("dims,bc", [((2, 2, 2), 0), ((3, 2, 4), 1), ((5, 2, 33), 0), ((33, 3, 2), 1),
                                     ((5, 40, 5), 2), ((2, 37, 65), 1), ((66, 5, 5), 2)])
def test_degenerate_grids_match_oracle(dims, bc):
    """Grids of two or three lines on an axis, extents just past a tile
    width, PEC / PMC / Mur walls (Mur on five or more lines: an excitation
    on the line next to a Mur face is refused): a soft E excitation and a
    voltage probe on an edge along the longest axis; both kernel families
    bit-identical to the oracle (the update ranges, trimmed last lines,
    partial tiles and the axis relabelling meet their smallest cases)."""
    from wipems_gb300 import Scene
    lines = [np.arange(n, dtype=np.float64) for n in dims]
    s = Scene(*lines, 1e-3)
    s.set_boundary([bc] * 6, [0] * 6)
    s.set_gauss_excite(5e9, 5e9, 120)
    a = [(n - 1) // 2 for n in dims]
    b = [k + 1 for k in a]
    n = int(np.argmax(dims))  # an edge along the longest axis
    start = [float(lines[k][a[k]]) for k in range(3)]
    stop = list(start)
    stop[n] = float(lines[n][b[n]])
    vec = [0.0, 0.0, 0.0]
    vec[n] = 1.0
    s.add_excitation(start, stop, vec, priority=1)
    s.add_probe(start, stop, 0, name="u")
    op = Operator(s)
    ref = oracle.run(*oracle_inputs(op), 120, op.probe_interval, engine=oracle.BASIC)
    for kernel in ("tma", "direct"):
        eng = Engine(op, kernel=kernel)
        eng.iterate(120)
        compare(op, eng, ref)
        eng.close()
