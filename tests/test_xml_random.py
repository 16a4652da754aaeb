"""Random scenes written as openEMS XML documents, the way the front ends
write them, with the spellings the reference accepts drawn at random
(boundary names or codes, PML_n or a bare 3 for eight layers, grid lines
unsorted and repeated, isotropic values given once or per axis, unset
lumped values as nan).  The engine library's reader and the oracle's own
reader (Python's XML parser, oracle/xml_spec.py) must build operators
bit-identical to the one the scene API builds from the same scene.
CPU only."""
import math

import numpy as np
import pytest

import oracle
from oracle.xml_spec import xml_spec
from wipems_gb300 import Operator, Scene, SceneSpec

from helpers import assert_same_operator
from test_random_gpu import SEEDS, EXT_SEEDS, random_scene, random_scene_ext
from test_xml import _same_operator

pytestmark = pytest.mark.usefixtures("libs")

_BC_NAMES = {0: "PEC", 1: "PMC", 2: "MUR"}
_FACES = ["xmin", "xmax", "ymin", "ymax", "zmin", "zmax"]


def _num(v: float) -> str:
    return repr(float(v))


def _iso(v: float, rng) -> str:
    return ",".join([_num(v)] * 3) if rng.random() < 0.3 else _num(v)


def _box(p, rng) -> str:
    a, b = p["start"], p["stop"]
    pts = (f'<P1 X="{_num(a[0])}" Y="{_num(a[1])}" Z="{_num(a[2])}"/>'
           f'<P2 X="{_num(b[0])}" Y="{_num(b[1])}" Z="{_num(b[2])}"/>')
    return f'<Primitives><Box Priority="{p["priority"]}">{pts}</Box></Primitives>'


def spec_xml(spec: dict, rng) -> str:
    """The openEMS document of a recorded scene (dispersion order 1)."""
    et = spec.get("excite_type", 0)
    fd = [f'NumberOfTimesteps="{spec["nr_ts"]}"', 'endCriteria="1e-06"', f'OverSampling="{spec["oversampling"]}"']
    ex = [f'Type="{et}"']
    if et in (0, 1, 10):
        ex.append(f'f0="{_num(spec["f0"])}"')
    if et == 0:
        ex.append(f'fc="{_num(spec["fc"])}"')
    if et in (2, 3, 10):
        fd.append(f'f_max="{_num(spec.get("f_max", 0.0))}"')
    if et == 10:
        ex.append(f'Function="{spec["function"]}"')
    bcs = []
    for k, name in enumerate(_FACES):
        b = spec["bc"][k]
        if b == 3:
            n = spec["pml_size"][k]
            v = "3" if n == 8 and rng.random() < 0.5 else f"PML_{n}"
        else:
            v = _BC_NAMES[b] if rng.random() < 0.6 else str(b)
        bcs.append(f'{name}="{v}"')
    if any(spec["mur_vph"]):
        bcs += [f'MUR_PhaseVelocity_{f}="{_num(v)}"' for f, v in zip(_FACES, spec["mur_vph"]) if v]
    grid = []
    for tag, ln in zip(("XLines", "YLines", "ZLines"), spec["lines"]):
        ln = list(np.asarray(ln, float))
        extra = [ln[int(rng.integers(0, len(ln)))]] if rng.random() < 0.5 else []
        order = rng.permutation(len(ln) + len(extra))
        vals = (ln + extra)
        grid.append(f'<{tag}>{",".join(_num(vals[i]) for i in order)}</{tag}>')
    props = []
    for i, p in enumerate(spec["prims"]):
        k, box = p["kind"], _box(p, rng)
        if k == "material" and p.get("disp_order"):
            assert p["disp_order"] == 1
            a = [f'Epsilon="{_iso(p["eps"], rng)}"', f'Mue="{_iso(p["mue"], rng)}"', f'Kappa="{_iso(p["kappa"], rng)}"',
                 f'Sigma="{_iso(p["sigma"], rng)}"']
            for key, attr in (("eps_plasma_f", "EpsilonPlasmaFrequency"), ("eps_relax_t", "EpsilonRelaxTime"),
                              ("eps_pole_f", "EpsilonLorPoleFrequency"), ("mue_plasma_f", "MuePlasmaFrequency"),
                              ("mue_relax_t", "MueRelaxTime"), ("mue_pole_f", "MueLorPoleFrequency")):
                if p[key][0] or rng.random() < 0.5:
                    a.append(f'{attr}="{_iso(p[key][0], rng)}"')
            props.append(f'<LorentzMaterial ID="{i}" Name="lor{i}" Order="1">{box}<Property {" ".join(a)}/>'
                         f'</LorentzMaterial>')
        elif k == "material":
            a = f'Epsilon="{_iso(p["eps"], rng)}" Mue="{_iso(p["mue"], rng)}" Kappa="{_iso(p["kappa"], rng)}" ' \
                f'Sigma="{_iso(p["sigma"], rng)}"'
            props.append(f'<Material ID="{i}" Name="mat{i}" Isotropy="1">{box}<Property {a}/></Material>')
        elif k == "metal":
            props.append(f'<Metal ID="{i}" Name="metal{i}">{box}</Metal>')
        elif k == "lumped":
            vals = []
            for key, attr in (("R", "R"), ("C", "C"), ("L", "L")):
                v = p[key]
                if v < 0:
                    if rng.random() < 0.5:
                        vals.append(f'{attr}="nan"')
                else:
                    vals.append(f'{attr}="{_num(v)}"')
            props.append(f'<LumpedElement ID="{i}" Name="le{i}" Direction="{p["ny"]}" Caps="{p["caps"]}" '
                         f'LEtype="{p["le_type"]}" {" ".join(vals)}>{box}</LumpedElement>')
        elif k == "excitation":
            vec = ",".join(_num(v) for v in p["exc_vec"])
            props.append(f'<Excitation ID="{i}" Name="exc{i}" Number="0" Enabled="1" Frequency="0" '
                         f'Delay="{_num(p["delay"])}" Type="{p["exc_type"]}" Excite="{vec}">{box}</Excitation>')
        elif k == "probe":
            props.append(f'<ProbeBox ID="{i}" Name="probe{i}" Number="0" NormDir="{p["norm_dir"]}" '
                         f'Type="{p["probe_type"]}" Weight="{_num(p["weight"])}">{box}</ProbeBox>')
        else:
            raise ValueError(k)
    return ('<?xml version="1.0" encoding="UTF-8" standalone="yes" ?>\n<openEMS>'
            f'<FDTD {" ".join(fd)}><Excitation {" ".join(ex)}/><BoundaryCond {" ".join(bcs)}/></FDTD>'
            '<ContinuousStructure CoordSystem="0"><Properties>' + "".join(props) + '</Properties>'
            f'<RectilinearGrid DeltaUnit="{_num(spec["unit"])}" CoordSystem="0">' + "".join(grid) +
            '</RectilinearGrid></ContinuousStructure></openEMS>\n')


def _order1(spec: dict) -> dict:
    """The scene with every Lorentz / Drude material cut to its first pole
    (the XML reader takes dispersion order 1)."""
    import copy
    spec = copy.deepcopy(spec)
    for p in spec["prims"]:
        if p.get("disp_order", 0) > 1:
            p["disp_order"] = 1
            for key in ("eps_plasma_f", "eps_relax_t", "eps_pole_f", "mue_plasma_f", "mue_relax_t", "mue_pole_f"):
                p[key] = p[key][:1]
    return spec


@pytest.mark.parametrize("seed", SEEDS[:10] + EXT_SEEDS)
def test_random_xml_documents_build_the_api_operator(seed):
    scene = random_scene_ext(seed) if seed in EXT_SEEDS else random_scene(seed)
    spec = _order1(scene.spec)
    rng = np.random.default_rng(5000 + seed)
    text = spec_xml(spec, rng)
    sp = SceneSpec(*spec["lines"], spec["unit"])
    sp.spec = spec
    api = Operator(Scene.from_spec(sp))
    from_xml = Operator(Scene.from_xml(text))
    _same_operator(from_xml, api)
    assert_same_operator(from_xml, oracle.Operator(xml_spec(text)))
