"""Host operator build (restated Operator::CalcECOperator and extension
builds): closed-form known answers.  CPU only."""
import math

import numpy as np
import pytest

from wipems_gb300 import EPS0, MUE0, C0, CompressedOperator, Operator, Scene, scenes

pytestmark = pytest.mark.usefixtures("libs")


def f32(x):
    return np.float32(x)


def test_var3_timestep_is_courant_on_uniform_cube():
    op = Operator(scenes.p64(nr_ts=100))
    courant = 1e-3 / (C0 * math.sqrt(3))
    assert abs(op.dT / courant - 1) < 1e-6


def test_vacuum_coefficients_closed_form():
    op = Operator(scenes.p64(nr_ts=100))
    vv, vi, ii, iv = op.coefficients()
    dT, d = op.dT, 1e-3
    # interior edge: C = eps0*A/delta with A = delta^2 (float-rounded EC store)
    C = float(np.float32(EPS0 * d * d / d))
    L = float(np.float32(MUE0 * d * d / d))
    assert vv[0, 10, 10, 10] == f32(1.0)
    assert vi[0, 10, 10, 10] == f32((dT / C) / (1.0 + dT * 0.0 / 2.0 / C))
    assert ii[2, 10, 10, 10] == f32(1.0)
    assert iv[2, 10, 10, 10] == f32((dT / L) / 1.0)


def test_pec_faces_and_last_current_lines():
    op = Operator(scenes.p64(nr_ts=100))
    vv, vi, ii, iv = op.coefficients()
    # x = 0 face: tangential y/z voltages are PEC (operator.cpp:1086-1129)
    assert not vi[1, 0].any() and not vi[2, 0].any()
    assert vi[0, 0, 5, 5] != 0
    # last lines: currents outside the domain are zero (operator.cpp:1160-1171)
    assert not iv[:, -1].any() and not iv[:, :, -1].any() and not iv[:, :, :, -1].any()


def test_gauss_signal_and_nyquist():
    op = Operator(scenes.p64(nr_ts=2000))
    sv, sc = op.signals()
    dT, f0, fc = op.dT, 5e9, 5e9
    n = np.arange(len(sv))
    t = n * dT
    ref = np.cos(2 * np.pi * f0 * (t - 9 / (2 * np.pi * fc))) * np.exp(-((2 * np.pi * fc * t / 3 - 3) ** 2))
    assert np.array_equal(sv, ref.astype(np.float32))
    t2 = t + 0.5 * dT
    ref2 = np.cos(2 * np.pi * f0 * (t2 - 9 / (2 * np.pi * fc))) * np.exp(-((2 * np.pi * fc * t2 / 3 - 3) ** 2))
    assert np.array_equal(sc, ref2.astype(np.float32))
    assert len(sv) == math.ceil(2 * 9 / (2 * np.pi * fc) / dT)
    assert op.nyquist == math.floor(1 / (f0 + fc) / 2 / dT)
    assert op.probe_interval == op.nyquist // 4


def test_p64_excitation_and_probe_snapping():
    op = Operator(scenes.p64(nr_ts=100))
    ex = op.excitation()
    assert ex["index"].T.tolist() == [[32, 32, 32]] and ex["dir"].tolist() == [2]
    assert ex["amp"][0] == np.float32(1e-3)
    pv, pc = op.probes
    assert list(pv.start) == [42, 32, 22] and list(pv.stop) == [42, 32, 42]
    assert list(pc.start) == [31, 31, 32] and list(pc.stop) == [32, 32, 32] and pc.norm_dir == 2


def test_lumped_port_conductance():
    """Parallel R lumped element: G = (1/R/unitGC) * A/delta on the port edges
    (operator.cpp:1535-1712), vv/vi recomputed from it; caps set PEC."""
    L = scenes.uniform_lines(20, 1.0)
    s = Scene(L, L, L, 1e-3)
    s.set_boundary([0] * 6)
    s.set_gauss_excite(5e9, 5e9, 100)
    s.add_lumped_port([10, 10, 8], [11, 11, 12], 2, 50.0)
    op = Operator(s)
    vv, vi, _, _ = op.coefficients()
    d = 1e-3
    # 2x2 parallel edges per plane, 4 planes in series
    plane = 4 * (d * d / d)
    unitGC = 1 / (4 * (1 / plane))
    kappa = 1 / 50.0 / unitGC
    G = float(np.float32(kappa * d * d / d))
    C = float(np.float32(EPS0 * d * d / d))
    dT = op.dT
    assert vv[2, 10, 10, 9] == f32((1.0 - dT * G / 2.0 / C) / (1.0 + dT * G / 2.0 / C))
    assert vi[2, 10, 10, 9] == f32((dT / C) / (1.0 + dT * G / 2.0 / C))
    # caps: x/y edges on the end planes are PEC
    assert vi[0, 10, 10, 8] == 0 and vi[1, 10, 10, 12] == 0


def test_upml_grading_closed_form():
    """Operator_Ext_UPML with the default grading function
    (operator_ext_upml.cpp:31, 289-466) at the outermost E-edge of the
    x-lower slab."""
    L = scenes.uniform_lines(30, 1.0)
    s = Scene(L, L, L, 1e-3)
    s.set_boundary([3] * 6, [8] * 6)
    s.set_gauss_excite(5e9, 5e9, 100)
    op = Operator(s)
    assert op.info.num_upml == 6
    vv, vi, _, _ = op.coefficients()
    dT = op.dT
    W = 8e-3
    dl = W / 8
    grad = lambda D: -math.log(1e-6) * math.log(2.5) / (2 * dl * 376.730313461 * (2.5 ** (W / dl) - 1)) * 2.5 ** (D / dl)
    # y-edge at x=1 (in the x slab only, y/z interior): kappa_v[x] for an edge
    # normal to x at depth W - 1mm  (n != ny -> no half-cell shift)
    kx = grad(W - 1e-3)
    # nP of y is z (no grading), so main vv = 1 and vi = 2eps0 dT/(2eps0) * d/A
    assert vv[1, 1, 15, 15] == f32((2 * EPS0 - 0 * dT) / (2 * EPS0 + 0 * dT))
    assert vi[1, 1, 15, 15] == f32((2 * EPS0 * dT) / (2 * EPS0) * 1e-3 / 1e-6)
    # z-edge: nP = x -> graded main vv
    assert vv[2, 1, 15, 15] == f32((2 * EPS0 - kx * dT) / (2 * EPS0 + kx * dT))


def test_drude_coefficients_closed_form():
    """Operator_Ext_LorentzMaterial for a Drude brick interior edge
    (operator_ext_lorentzmaterial.cpp:231-351)."""
    L = scenes.uniform_lines(20, 1.0)
    s = Scene(L, L, L, 1e-3)
    s.set_boundary([0] * 6)
    s.set_gauss_excite(5e9, 5e9, 100)
    fp, tau = 2e9, 1e-8
    s.add_lorentz([5, 5, 5], [15, 15, 15], plasma_f=[fp], relax_t=[tau], pole_f=[0.0])
    op = Operator(s)
    d = op.desc
    assert d.num_ade_orders == 1
    a = d.ade[0]
    cnt = a.count
    pos = np.stack([np.ctypeslib.as_array(a.pos[k], shape=(cnt,)) for k in range(3)], 1)
    i = int(np.where((pos == [10, 10, 10]).all(1))[0][0])
    v_int = np.ctypeslib.as_array(a.v_int, shape=(3 * cnt,)).reshape(3, cnt)
    v_ext = np.ctypeslib.as_array(a.v_ext, shape=(3 * cnt,)).reshape(3, cnt)
    _, vi, _, _ = op.coefficients()
    dT = op.dT
    C = float(np.float32(EPS0 * 1e-3))
    wp = fp * 2 * math.pi
    LD = 1 / (wp * wp * C)
    RD = LD / tau
    assert v_int[0, i] == f32((2.0 * LD - dT * RD) / (2.0 * LD + dT * RD))
    assert v_ext[0, i] == f32(dT / (LD + dT * RD / 2.0) * float(vi[0, 10, 10, 10]))
    assert not a.volt_lor_on


@pytest.mark.parametrize("kind", ["pec", "upml", "graded", "drude", "lorentz", "mixed"])
def test_compression_round_trip_exact(kind):
    """Exact mode: index + tables expand back to the operator bit for bit."""
    op = Operator(scenes.mini(kind))
    cop = CompressedOperator(op, mode="exact")
    assert not cop.factorized
    ex = cop.expand()
    for a, b in zip(ex[:4], op.coefficients()):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), kind
    fe = ex[4]
    assert (cop.info["num_upml_nodes"] > 0) == (kind != "pec")
    assert int(((fe & 1) != 0).sum()) == cop.info["num_upml_nodes"]
    if kind in ("drude", "lorentz", "mixed"):
        assert int(((fe & 2) != 0).sum()) == cop.info["num_ade_nodes"] > 0


@pytest.mark.parametrize("kind", ["graded", "mixed"])
def test_factorized_geometry_on_graded_meshes(kind):
    """Graded meshes compress with vi = VI * delta/A rebuilt per node (and
    last-bit variants merged): few tuples, vv / ii exact, vi / iv within
    4 float steps of the operator's."""
    op = Operator(scenes.mini(kind))
    auto = CompressedOperator(op)
    exact = CompressedOperator(op, mode="exact")
    assert auto.factorized
    assert auto.info["num_tuples_e"] < exact.info["num_tuples_e"] / 4
    vv, vi, ii, iv = op.coefficients()
    evv, evi, eii, eiv = auto.expand()[:4]
    assert np.array_equal(evv, vv) and np.array_equal(eii, ii)
    for a, b in ((evi, vi), (eiv, iv)):
        nz = b != 0
        assert np.array_equal(a[~nz], b[~nz])
        ulps = np.abs(a[nz].view(np.int32).astype(np.int64) - b[nz].view(np.int32).astype(np.int64))
        assert ulps.max() <= 4, ulps.max()


def test_uniform_mesh_is_exact_and_fits_uint16_index():
    op = Operator(scenes.l256(cells=96, n_bricks=40))
    cop = CompressedOperator(op)
    assert not cop.factorized
    assert cop.info["index_bytes_e"] == 2 and cop.info["index_bytes_h"] == 2
    assert cop.info["trim_e"] == [1, 1, 1]


def _operator_bytes(op):
    """The coefficient arrays, UPML slabs, dispersion coefficients and dT
    of a built operator as one byte string."""
    d = op.desc

    def arr(p, n):
        return np.ctypeslib.as_array(p, shape=(n,)).tobytes() if n else b""

    parts = [np.float64(d.dT).tobytes()]
    nn = 3 * d.num_lines[0] * d.num_lines[1] * d.num_lines[2]
    parts += [arr(getattr(d, f), nn) for f in ("vv", "vi", "ii", "iv")]
    for i in range(d.num_upml):
        u = d.upml[i]
        n = 3 * u.num_lines[0] * u.num_lines[1] * u.num_lines[2]
        parts += [arr(getattr(u, f), n) for f in ("vv", "vvfo", "vvfn", "ii", "iifo", "iifn")]
    for i in range(d.num_ade_orders):
        a = d.ade[i]
        for f, on in (("v_int", a.volt_on), ("v_ext", a.volt_on), ("v_lor", a.volt_lor_on),
                      ("i_int", a.curr_on), ("i_ext", a.curr_on), ("i_lor", a.curr_lor_on)):
            if on:
                parts.append(arr(getattr(a, f), 3 * a.count))
    return b"".join(parts)


@pytest.mark.parametrize("make", [lambda: scenes.mini("upml", seed=2), lambda: scenes.mini("mixed", seed=1),
                                  lambda: scenes.mini("graded", seed=5), lambda: scenes.serve_job(1)],
                         ids=["upml", "mixed", "graded", "serve_lorentz"])
def test_operator_independent_of_build_threads(make):
    """The parallel build loops (EC pass, Var3 timestep search with its
    vectorized interior lines, UPML slabs handed out in chunks of lines,
    dispersion) give the same bytes for any thread count."""
    ref = _operator_bytes(Operator(make(), threads=1))
    for th in (3, 8):
        assert _operator_bytes(Operator(make(), threads=th)) == ref


def test_device_axes_rotation_choice_and_expansion():
    """fdtd_compress_rot: the automatic rotation puts the axis that pads
    least to 32-lane z tiles on z (a cube stays as it is; a 36-line z
    extent next to a 208-line x extent moves), and the tables expanded back
    to the operator's axes are the same arrays whatever the rotation."""
    from wipems_gb300 import CompressedOperator, Scene
    def grid(nx, ny, nz):
        s = Scene(*[np.arange(n, dtype=np.float64) for n in (nx, ny, nz)], 1e-3)
        s.set_boundary([0] * 6, [0] * 6)
        s.set_gauss_excite(5e9, 5e9, 50)
        return Operator(s)
    assert CompressedOperator(grid(40, 40, 40)).rotation == 0
    c = CompressedOperator(grid(208, 148, 36))
    assert c.rotation == 1 and c.info["device_lines"] == [148, 36, 208]
    assert CompressedOperator(grid(21, 4, 1001)).rotation == 0
    op = Operator(scenes.mini("rlc_mur"))
    ref = CompressedOperator(op, rotation=0)
    e0, x0 = ref.expand(), [ref.expand_ext(h) for h in (0, 1)]
    for r in (1, 2):
        c = CompressedOperator(op, rotation=r)
        n = op.num_lines
        assert c.info["device_lines"] == [n[r % 3], n[(1 + r) % 3], n[(2 + r) % 3]]
        assert all(np.array_equal(a, b) for a, b in zip(e0, c.expand()))
        assert all(np.array_equal(x0[h][k], c.expand_ext(h)[k]) for h in (0, 1) for k in (0, 1))
        assert c.info["num_tuples_e"] == ref.info["num_tuples_e"]


def test_overlapping_upml_slabs_are_refused():
    """openEMS ends its y and z UPML slabs size[0]+1 lines before the x-max
    face (operator_ext_upml.cpp:163), size[0] being 8 when x-min is not PML
    (openems.cpp:101), so an x-max UPML thicker than that makes them reach
    into the x-max slab, where two UPML extensions would update the same
    nodes.  The operator build keeps openEMS's ranges; the compressor refuses
    the overlap with an error that says why."""
    from wipems_gb300._abi import FdtdError
    from wipems_gb300.fdtd import BC_PEC, BC_PML
    lines = [scenes.uniform_lines(n, 1.0) for n in (40, 24, 12)]

    def op(bc, size):
        s = Scene(*lines, 1e-3)
        s.set_boundary(bc, size)
        s.set_gauss_excite(10e9, 10e9, 50)
        return Operator(s)

    y_pml = [BC_PML, BC_PEC, BC_PEC, BC_PEC]
    for xbc, size in (([BC_PEC, BC_PML], [0, 10]), ([BC_PML, BC_PML], [3, 5])):
        o = op(xbc + y_pml, size + [3, 0, 0, 0])
        sl = [(list(o.desc.upml[k].start), list(o.desc.upml[k].num_lines)) for k in range(o.desc.num_upml)]
        ymin = sl[-1]
        x_min_size = size[0] if xbc[0] == BC_PML else 8
        assert ymin[0][0] + ymin[1][0] - 1 == len(lines[0]) - 1 - (x_min_size + 1)  # the y slab's last x line
        with pytest.raises(FdtdError, match="UPML slabs overlap"):
            CompressedOperator(o)
    # an x-max UPML no thicker than the x-min size (8 for PEC) leaves them disjoint
    for xbc, size in (([BC_PEC, BC_PML], [0, 8]), ([BC_PML, BC_PML], [5, 5]), ([BC_PML, BC_PML], [6, 3])):
        CompressedOperator(op(xbc + y_pml, size + [3, 0, 0, 0]))


def test_pml_on_one_face_of_an_axis_grades_with_the_default_size():
    """zmin PEC, zmax PML_8 (the reference's Coax test sets this): openEMS
    grades the upper layer with dl = width / size[zmin], and size[zmin] is
    its default 8 (operator_ext_upml.cpp:337, openems.cpp:101), so every
    coefficient is finite -- in the product's build and in the oracle's."""
    import oracle
    from wipems_gb300.fdtd import BC_PEC, BC_PML
    lines = [scenes.uniform_lines(n, 1.0) for n in (14, 12, 30)]
    s = Scene(*lines, 1e-3)
    s.set_boundary([BC_PEC] * 5 + [BC_PML], [0, 0, 0, 0, 0, 8])
    s.set_gauss_excite(10e9, 10e9, 50)
    o = Operator(s)
    arrs = oracle.desc_arrays(o.desc)
    assert all(np.isfinite(v).all() for v in arrs.values() if v.dtype.kind == "f")
    ref = oracle.Operator(s.spec)
    b = oracle.desc_arrays(ref.desc)
    assert sorted(arrs) == sorted(b) and all(arrs[k].tobytes() == b[k].tobytes() for k in arrs)
    CompressedOperator(o)
