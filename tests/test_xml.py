"""openEMS XML input: a document in the front ends' format builds the same
operator as the same scene made through the scene API, and content outside
the covered subset is refused by name."""
from pathlib import Path

import numpy as np
import pytest

from wipems_gb300 import BC_PEC, BC_PMC, BC_PML, CompressedOperator, Operator, Scene
from wipems_gb300.fdtd import BC_MUR
from wipems_gb300._abi import FdtdError

GOLDEN = Path(__file__).parent / "golden"


def _lines():
    x = np.arange(0, 12.01, 0.5)
    y = np.array([0, 1, 2, 3] + list(np.arange(3.5, 11.6, 0.5)) + [12, 13, 14, 15, 16], float)
    z = np.arange(0, 8.01, 0.5)
    return x, y, z


def _api_scene():
    s = Scene(*_lines(), 1e-3)
    s.set_boundary([BC_PML, BC_PML, BC_PML, BC_PML, BC_PEC, BC_PMC], [8, 8, 8, 6, 0, 0])
    s.set_gauss_excite(10e9, 5e9, 600)
    s.set_oversampling(4)
    s.add_material([2, 3.5, 1], [9.5, 12, 6], eps_r=3.66, kappa=0.01, priority=10)
    s.add_metal([3, 4, 6], [8, 11, 6], priority=20)
    s.add_lumped([6, 7.5, 1], [6.5, 8, 6], 2, R=50.0, caps=True, priority=5)
    s.add_excitation([6, 7.5, 1], [6.5, 8, 6], [0, 0, -1], exc_type=0, priority=5)
    s.add_probe([6.25, 7.75, 1], [6.25, 7.75, 6], 0, weight=-1.0)
    s.add_probe([6, 7.5, 3.5], [6.5, 8, 3.5], 1, weight=1.0, norm_dir=2)
    return s


def _same_operator(a: Operator, b: Operator):
    assert a.num_lines == b.num_lines
    assert a.dT == b.dT and a.probe_interval == b.probe_interval
    for x, y in zip(a.coefficients(), b.coefficients()):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    assert len(a.probes) == len(b.probes)
    for p, q in zip(a.probes, b.probes):
        assert bytes(p) == bytes(q)
    ea, eb = a.excitation(), b.excitation()
    for k in ea:
        assert np.array_equal(np.asarray(ea[k]), np.asarray(eb[k])), k
    for x, y in zip(a.signals(), b.signals()):
        assert np.array_equal(x, y)
    ca, cb = CompressedOperator(a, mode="exact"), CompressedOperator(b, mode="exact")
    assert ca.info["num_tuples_e"] == cb.info["num_tuples_e"] and ca.info["num_upml_nodes"] == cb.info["num_upml_nodes"]
    for x, y in zip(ca.expand(), cb.expand()):  # applied coefficients and per-node UPML / ADE / excitation flags
        assert np.array_equal(x, y)


def test_xml_document_builds_the_api_operator():
    sx = Scene.from_xml(str(GOLDEN / "port_box.xml"))
    info = sx.xml_info
    assert info["nr_ts"] == 600 and info["end_crit"] == 1e-5 and info["excite_type"] == 0
    assert info["num_probes"] == 2 and info["skipped"] == 0
    # the E-field dump (DumpType 0, node interpolation) is recorded for the caller
    d = sx.dumps()
    assert d == [dict(name="Et", field="E", interp="node", file_type=0, start=[0.0, 0.0, 3.0],
                      stop=[12.0, 16.0, 3.0], step=[1, 1, 1])]
    _same_operator(Operator(sx), Operator(_api_scene()))


def test_xml_text_and_lorentz_material():
    text = (GOLDEN / "port_box.xml").read_text()
    text = text.replace(
        '<Metal ID="1" Name="plate">',
        '<LorentzMaterial ID="7" Name="drude" Order="1"><Primitives><Box Priority="15">'
        '<P1 X="4" Y="5" Z="2"/><P2 X="7" Y="9" Z="4"/></Box></Primitives>'
        '<Property Epsilon="2" EpsilonPlasmaFrequency="5e9" EpsilonRelaxTime="1e-9" '
        'EpsilonLorPoleFrequency="0"/></LorentzMaterial>\n      <Metal ID="1" Name="plate">')
    sx = Scene.from_xml(text)
    s = _api_scene()
    s.add_lorentz([4, 5, 2], [7, 9, 4], eps_r=2.0, plasma_f=[5e9], relax_t=[1e-9], pole_f=[0.0], priority=15)
    _same_operator(Operator(sx), Operator(s))


def test_xml_magnetic_lorentz_material():
    """MuePlasmaFrequency / MueRelaxTime / MueLorPoleFrequency read into
    the magnetic family of the API's Lorentz material."""
    text = (GOLDEN / "port_box.xml").read_text()
    text = text.replace(
        '<Metal ID="1" Name="plate">',
        '<LorentzMaterial ID="7" Name="dng" Order="1"><Primitives><Box Priority="15">'
        '<P1 X="4" Y="5" Z="2"/><P2 X="7" Y="9" Z="4"/></Box></Primitives>'
        '<Property Epsilon="2" Mue="1.5" EpsilonPlasmaFrequency="5e9" EpsilonRelaxTime="1e-9" '
        'MuePlasmaFrequency="6e9" MueRelaxTime="2e-9" MueLorPoleFrequency="3e9"/></LorentzMaterial>\n'
        '      <Metal ID="1" Name="plate">')
    sx = Scene.from_xml(text)
    s = _api_scene()
    s.add_lorentz([4, 5, 2], [7, 9, 4], eps_r=2.0, mue_r=1.5, plasma_f=[5e9], relax_t=[1e-9], priority=15,
                  mue_plasma_f=[6e9], mue_relax_t=[2e-9], mue_pole_f=[3e9])
    _same_operator(Operator(sx), Operator(s))
    assert Operator(sx).desc.ade[0].curr_lor_on


@pytest.mark.parametrize("edit,needle", [
    (('<Box Priority="20">', '<Cylinder Priority="20" Radius="1">'), "Cylinder"),
    (('<Excitation Type="0" f0="1e+10"', '<Excitation Type="11" f0="1e+10"'), "excitation Type 11"),
    (('Epsilon="3.66"', 'Epsilon="3.66,3.66,4"'), "anisotropic"),
    (('<Weight Epsilon="1"', '<Weight Epsilon="2*x"'), "weighting"),
    (('<Metal ID="1" Name="plate">', '<ConductingSheet ID="1" Name="plate">'), "ConductingSheet"),
])
def test_xml_refuses_uncovered_content(edit, needle):
    text = (GOLDEN / "port_box.xml").read_text().replace(*edit)
    if needle == "Cylinder":
        text = text.replace('</Box>\n        </Primitives>\n      </Metal>', '</Cylinder>\n        </Primitives>\n      </Metal>')
    if needle == "ConductingSheet":
        text = text.replace("</Metal>", "</ConductingSheet>")
    with pytest.raises(FdtdError) as ei:
        Scene.from_xml(text)
    assert ei.value.code == -5, str(ei.value)
    assert needle.lower() in str(ei.value).lower()


def test_xml_malformed_documents():
    for text in ("<openEMS><FDTD></openEMS>", "<notopenEMS/>", "<openEMS><FDTD/></openEMS>",
                 "<openEMS><FDTD a=1/></openEMS>"):
        with pytest.raises(FdtdError) as ei:
            Scene.from_xml(text)
        assert ei.value.code == -1


def test_xml_mur_boundaries():
    text = (GOLDEN / "port_box.xml").read_text().replace(
        'zmax="PMC"', 'zmax="MUR" MUR_PhaseVelocity="2.5e8" MUR_PhaseVelocity_zmax="2e8"')
    sx = Scene.from_xml(text)
    s = _api_scene()
    s.set_boundary([BC_PML, BC_PML, BC_PML, BC_PML, BC_PEC, BC_MUR], [8, 8, 8, 6, 0, 0])
    s.set_mur_velocity([2.5e8] * 5 + [2e8])
    a, b = Operator(sx), Operator(s)
    _same_operator(a, b)
    assert a.desc.num_mur == b.desc.num_mur == 1
    m = a.desc.mur[0]
    n = m.n_p * m.n_pp
    ca = np.ctypeslib.as_array(m.coef_p, shape=(n,))
    cb = np.ctypeslib.as_array(b.desc.mur[0].coef_p, shape=(n,))
    assert np.array_equal(ca, cb)
    c0t = 2e8 * a.dT  # phase velocity given: c = (v dT - d) / (v dT + d), d = 0.5 mm
    assert np.allclose(ca, np.float32((c0t - 0.5e-3) / (c0t + 0.5e-3)))


@pytest.mark.parametrize("letype,extra,n_rlc", [("1", 'L="2e-9" C="1e-12"', 4), ("0", 'L="2e-9"', 4),
                                                ("-1", 'L="2e-9"', 0)])
def test_xml_lumped_rlc(letype, extra, n_rlc):
    """<LumpedElement LEtype> with an inductance or the series type goes to
    the lumped RLC extension; an invalid type is ignored, as the reference
    ignores it (neither Calc_LumpedElements nor the RLC extension takes it)."""
    text = (GOLDEN / "port_box.xml").read_text().replace(
        "</Properties>",
        f'<LumpedElement ID="9" Name="rlc" Direction="0" Caps="0" R="25" {extra} LEtype="{letype}">'
        '<Primitives><Box Priority="7"><P1 X="3" Y="2" Z="3"/><P2 X="4" Y="3" Z="3"/></Box></Primitives>'
        "</LumpedElement></Properties>", 1)
    a = Operator(Scene.from_xml(text))
    s = _api_scene()
    L = 2e-9
    C = 1e-12 if letype == "1" else -1.0
    s.add_lumped_rlc([3, 2, 3], [4, 3, 3], 0, R=25.0, L=L, Cap=C, caps=False, priority=7, le_type=int(letype))
    b = Operator(s)
    _same_operator(a, b)
    na = a.desc.rlc.contents.count if a.desc.rlc else 0
    nb = b.desc.rlc.contents.count if b.desc.rlc else 0
    assert na == nb == n_rlc


def test_xml_field_probes():
    text = (GOLDEN / "port_box.xml").read_text().replace(
        "</Properties>",
        '<ProbeBox ID="7" Name="et" Type="2"><Primitives><Box Priority="0"><P1 X="4" Y="5" Z="2"/>'
        '<P2 X="4" Y="5" Z="2"/></Box></Primitives></ProbeBox>'
        '<ProbeBox ID="8" Name="ht" Type="3" Weight="2"><Primitives><Box Priority="0"><P1 X="4.25" Y="5.25" Z="2.25"/>'
        '<P2 X="4.25" Y="5.25" Z="2.25"/></Box></Primitives></ProbeBox>'
        '<ProbeBox ID="9" Name="mm" Type="10"><Primitives><Box Priority="0"><P1 X="4" Y="5" Z="2"/>'
        '<P2 X="4" Y="5" Z="2"/></Box></Primitives></ProbeBox></Properties>', 1)
    sx = Scene.from_xml(text)
    assert sx.xml_info["num_probes"] == 4 and sx.xml_info["skipped"] == 1  # the mode-match probe
    op = Operator(sx)
    types = [p.type for p in op.probes]
    assert types[-2:] == [2, 3] and op.probes[-1].weight == 2.0


@pytest.mark.parametrize("etype", [1, 2, 3, 10])
def test_xml_excitation_signals(etype):
    """<Excitation Type="1" f0> (sinusoid), Type 2 / 3 (Dirac / step, with
    <FDTD f_max>): the engine library's reader equals the API scene and the
    oracle's reader + operator."""
    import oracle
    from oracle.xml_spec import xml_spec
    from helpers import assert_same_operator
    fn = ' Function="sin(2*pi*7e9*t)*(1-exp(-t/2e-10))"' if etype == 10 else ""
    text = (GOLDEN / "port_box.xml").read_text().replace(
        '<Excitation Type="0" f0="1e+10" fc="5e+09"/>', f'<Excitation Type="{etype}" f0="7e+09" fc="5e+09"{fn}/>')
    sx = Scene.from_xml(text)
    assert sx.xml_info["excite_type"] == etype
    s = _api_scene()
    if etype == 1:
        s.set_sinus_excite(7e9, 600)
    elif etype == 10:
        s.set_custom_excite("sin(2*pi*7e9*t)*(1-exp(-t/2e-10))", 7e9, 600, 1.5e10)
    else:
        (s.set_dirac_excite if etype == 2 else s.set_step_excite)(1.5e10, 600)
    _same_operator(Operator(sx), Operator(s))
    assert_same_operator(Operator(sx), oracle.Operator(xml_spec(text)))


@pytest.mark.parametrize("name", ["port_box.xml", "lorentz_mur.xml", "drude_mtm.xml"])
def test_xml_operator_matches_oracle_reader(name):
    """The engine library's XML reader + operator build against the
    oracle's own reader (oracle/xml_spec.py, Python's XML parser) + its
    operator build: bit-identical operators and probes."""
    import oracle
    from oracle.xml_spec import xml_spec
    from helpers import assert_same_operator
    path = str(Path(__file__).parent / "golden" / name)
    assert_same_operator(Operator(Scene.from_xml(path)), oracle.Operator(xml_spec(path)))
