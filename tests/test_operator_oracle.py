"""The product's operator build (wipems_gb300/csrc/operator.cpp: per-line EC
pass, grid-sampled box lookups, vectorized timestep search) against the
oracle's independent restatement of the reference's build
(oracle/operator_oracle.cpp: edge-by-edge Calc_ECPos / AverageMatQuarterCell
with coordinate lookups, CalcTimestep_Var3 with the AdrOp shift state,
Calc_LumpedElements, the excitation, Mur, UPML, Lorentz/Drude and lumped RLC
BuildExtension in openEMS's extension order, probe snapping).  Bar: bitwise
on every array, on the mini scenes of every feature, P64, the cavity, L256,
D192, B96 jobs (PEC and UPML) and serving jobs of each kind (dielectric,
Drude, Lorentz), and the magnetic (mue) family of the Lorentz material on
its own and beside the electric one."""
import numpy as np
import pytest

import oracle
from wipems_gb300 import Operator, scenes

from helpers import assert_same_operator, with_signal

pytestmark = pytest.mark.usefixtures("libs")


def both(scene):
    return Operator(scene), oracle.Operator(scene.spec)


@pytest.mark.parametrize("kind", ["pec", "upml", "graded", "drude", "lorentz", "mixed", "mur", "rlc", "rlc_mur",
                                  "magnetic", "magnetic_graded", "multipole", "multipole_graded"])
def test_mini_scene_operators_identical(kind):
    assert_same_operator(*both(scenes.mini(kind)))


@pytest.mark.parametrize("name", ["p64", "cavity", "rlc_series", "rlc_parallel", "drude_metamaterial"])
def test_small_scene_operators_identical(name):
    s = {"p64": lambda: scenes.p64(),
         "drude_metamaterial": lambda: scenes.drude_metamaterial(),
         "cavity": lambda: scenes.cavity(),
         "rlc_series": lambda: scenes.rlc_probe(True, R=50.0, L=1e-9, Cap=1e-12),
         "rlc_parallel": lambda: scenes.rlc_probe(False, R=50.0, L=1e-9, Cap=1e-12)}[name]()
    assert_same_operator(*both(s))


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_b96_job_operators_identical(seed):
    """Even seeds are PEC jobs, odd seeds UPML-8 jobs."""
    assert_same_operator(*both(scenes.b96_job(seed)))


@pytest.mark.parametrize("seed", [0, 1, 18, 21])
def test_serve_job_operators_identical(seed):
    """Seeds 0: dielectric + UPML, 1: Lorentz, 18 and 21: Drude."""
    s = scenes.serve_job(seed)
    assert s.meta["kind"] == {0: "dielectric", 1: "lorentz", 18: "drude", 21: "drude"}[seed]
    assert_same_operator(*both(s))


@pytest.mark.parametrize("name", ["l256", "d192"])
def test_headline_operators_identical(name):
    """Full-size L256 (257^3 nodes, UPML-8, 40 bricks, 50 ohm port) and D192
    (193^3 graded nodes, UPML-8, Drude and Lorentz bricks)."""
    s = scenes.l256() if name == "l256" else scenes.d192()
    P, O = both(s)
    assert_same_operator(P, O)
    if name == "d192":
        assert O.desc.num_ade_orders == 1 and O.desc.ade[0].count > 100_000
    else:
        assert O.desc.num_upml == 6


def test_magnetic_dispersion_builds_the_current_side_terms():
    """The mue family drives the H-side ADE: the double-negative Drude
    plane-wave scene turns both halves on (Drude: no Lorentz pole terms), the
    magnetic Lorentz pole of the mini scene turns on the H-side pole term,
    and the reference's coefficients come out: i_int = (2 C_D - dT G_D) /
    (2 C_D + dT G_D) with C_D = 1 / (w_p^2 EC_L) and G_D = C_D / tau
    (operator_ext_lorentzmaterial.cpp:248-276, 300-330), so i_int depends
    only on w_p, tau and dT."""
    s = scenes.drude_metamaterial()
    O = oracle.Operator(s.spec)
    a = O.desc.ade[0]
    assert a.volt_on and a.curr_on and not a.volt_lor_on and not a.curr_lor_on
    c = a.count
    i_int = np.ctypeslib.as_array(a.i_int, shape=(3 * c,))
    i_ext = np.ctypeslib.as_array(a.i_ext, shape=(3 * c,))
    on = i_ext != 0
    assert on.sum() > c  # the two H components across the channel, in the slab
    dT, tau = O.dT, s.meta["relax_t"]
    # C_D cancels: (2 - dT/tau) / (2 + dT/tau), rounded once to float
    want = np.float32((2.0 - dT / tau) / (2.0 + dT / tau))
    assert np.max(np.abs(i_int[on] - want)) <= 2 * np.spacing(want)
    m = oracle.Operator(scenes.mini("magnetic").spec)
    assert m.desc.ade[0].curr_lor_on and m.desc.ade[0].volt_lor_on


@pytest.mark.parametrize("kind", ["upml", "rlc_mur"])
@pytest.mark.parametrize("etype,f", [(1, 6e9), (1, 13.7e9), (2, 2e10), (3, 0.0)])
def test_excitation_signal_operators_identical(kind, etype, f):
    """Sinusoid, Dirac pulse and step (excitation.cpp:179-218, 273-295) in
    place of the Gaussian: identical operators, including the sinusoid's
    shortened timestep (operator.cpp:1001-1007), its two-period signal and
    the engine's period (engine_ext_excitation.cpp:45-46), the RLC elements
    built with fMax = f0 and the Mur faces' start timestep."""
    s = with_signal(scenes.mini(kind, nr_ts=400), etype, f)
    P, O = both(s)
    assert_same_operator(P, O)
    d = O.desc
    sig = np.ctypeslib.as_array(d.signal_volt, shape=(d.signal_length,))
    gauss = oracle.Operator(scenes.mini(kind, nr_ts=400).spec)
    if etype == 1:
        T = 1 / f
        assert O.dT <= gauss.dT and O.dT > gauss.dT * 0.9
        ts = round(T / O.dT)
        assert abs(T / O.dT - ts) < 1e-9 and d.signal_period_ts in (ts - 1, ts)
        assert d.signal_length == round(2 * T / O.dT) and sig[0] == 0
        assert np.max(np.abs(sig)) > 0.99
        assert O.nyquist == int(np.floor(T / 2 / O.dT))
    else:
        assert O.dT == gauss.dT and d.signal_period_ts == 0
        assert sig.tolist() == ([0.0, 1.0] if etype == 2 else [1.0, 1.0])
        assert O.nyquist == 1 and O.probe_interval == 1


CUSTOM = ["sin(2*pi*6e9*t)*exp(-((t-3e-10)/1e-10)^2)", "-t^2*1e18 + 2^-3",
          "sin(2*pi*5e9*t)^3 - cos(atan2(t, 1e-10))", "max(0, 1 - t/5e-10) * (1 - exp(-t/1e-11))",
          "pow(2, 3^2)*1e-3 + log10(1+t*1e9) % 0.7", "-(-t)*-1e9*-2"]


@pytest.mark.parametrize("fn", CUSTOM)
def test_custom_signal_matches_oracle_and_numpy(fn):
    """Excitation::CalcCustomExcitation (excitation.cpp:233-271): the
    product's expression compiler (recursive descent), the oracle's
    (shunting yard) and numpy evaluating the same formula give the same
    float samples at t = n dT; the Nyquist number follows f0."""
    s = with_signal(scenes.mini("rlc", nr_ts=400), 10, 6e9, fn)
    P, O = both(s)
    assert_same_operator(P, O)
    d = P.desc
    assert d.signal_length == 400 and P.nyquist == int(np.floor(1 / 6e9 / 2 / P.dT))
    sig = np.ctypeslib.as_array(d.signal_volt, shape=(400,))
    t = np.arange(400) * P.dT
    env = {"t": t, "pi": np.pi, "e": np.e, "sin": np.sin, "cos": np.cos, "exp": np.exp, "atan2": np.arctan2,
           "max": np.maximum, "pow": np.power, "log10": np.log10}
    ref = np.asarray(eval(fn.replace("^", "**"), {"__builtins__": {}}, env) * np.ones_like(t), np.float32)
    assert np.array_equal(sig, ref)


def test_custom_signal_refuses_what_it_does_not_cover():
    from wipems_gb300 import Scene
    from wipems_gb300._abi import FdtdError
    s = Scene(*[np.arange(5, dtype=np.float64)] * 3, 1e-3)
    for bad in ("t < 1e-9", "if(t, 1, 0)", "sin(t", "foo(t)", "x + 1", "2 ** t"):
        with pytest.raises(FdtdError):
            s.set_custom_excite(bad, 1e9, 100)


def test_voltage_probes_need_a_line():
    """A voltage probe box that is a point or spans more than one axis is
    skipped, with no sample column (openems.cpp:481-486); current and field
    probes on a point are kept (disabled where the reference disables them).
    Product and oracle agree, and the scene's probe names follow the kept
    probes."""
    from wipems_gb300 import Scene
    lines = [np.arange(4, dtype=np.float64)] * 3
    s = Scene(*lines, 1e-3)
    s.set_boundary([0] * 6, [0] * 6)
    s.set_gauss_excite(5e9, 5e9, 100)
    s.add_probe([1, 1, 1], [1, 1, 1], 0, name="point")
    s.add_probe([1, 1, 1], [1, 1, 1], 1, name="i_point")
    s.add_probe([0, 0, 0], [2, 2, 0], 0, name="diagonal")
    s.add_probe([0, 1, 1], [3, 1, 1], 0, name="line")
    s.add_probe([1, 2, 1], [1, 2, 1], 2, name="e_point")
    P, O = both(s)
    assert oracle.probe_tuples(P.probes) == oracle.probe_tuples(O.probes)
    assert [p.type for p in P.probes] == [1, 0, 2]
    assert [p["name"] for p in s.probes] == ["i_point", "line", "e_point"]


def test_comparison_sees_a_planted_mistake():
    """The comparison is not vacuous: the oracle built from a scene whose one
    brick has eps_r raised by 1e-6 (a few float ulps), or whose UPML is one line thinner on one
    face, or whose port resistance is changed, differs from the product in
    exactly the arrays that depend on it.  (The mistake is planted in the
    oracle's input, on the CPU.)"""
    s = scenes.mini("upml")
    P = Operator(s)
    a = oracle.desc_arrays(P.desc)

    def diff(spec):
        O = oracle.Operator(spec)  # keeps the arrays the description points into alive
        b = oracle.desc_arrays(O.desc)
        return {k for k in a if k in b and (a[k].shape != b[k].shape or not np.array_equal(a[k], b[k]))}

    import copy
    spec = copy.deepcopy(s.spec)
    brick = next(p for p in spec["prims"] if p["kind"] == "material")
    brick["eps"] *= 1 + 1e-6
    d = diff(spec)
    assert "vi" in d and "ii" not in d, d

    spec = copy.deepcopy(s.spec)
    spec["pml_size"][5] -= 1
    d = diff(spec)
    assert any(k.startswith("upml") for k in d), d

    spec = copy.deepcopy(s.spec)
    port = next(p for p in spec["prims"] if p["kind"] == "lumped")
    port["R"] = 51.0
    d = diff(spec)
    assert d & {"vv", "vi"}, d
