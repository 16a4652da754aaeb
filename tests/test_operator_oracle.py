"""The product's operator build (wipems_gb300/csrc/operator.cpp: per-line EC
pass, grid-sampled box lookups, vectorized timestep search) against the
oracle's independent restatement of the reference's build
(oracle/operator_oracle.cpp: edge-by-edge Calc_ECPos / AverageMatQuarterCell
with coordinate lookups, CalcTimestep_Var3 with the AdrOp shift state,
Calc_LumpedElements, the excitation, Mur, UPML, Lorentz/Drude and lumped RLC
BuildExtension in openEMS's extension order, probe snapping).  Bar: bitwise
on every array, on the mini scenes of every feature, P64, the cavity, L256,
D192, B96 jobs (PEC and UPML) and serving jobs of each kind (dielectric,
Drude, Lorentz)."""
import numpy as np
import pytest

import oracle
from wipems_gb300 import Operator, scenes

from helpers import assert_same_operator

pytestmark = pytest.mark.usefixtures("libs")


def both(scene):
    return Operator(scene), oracle.Operator(scene.spec)


@pytest.mark.parametrize("kind", ["pec", "upml", "graded", "drude", "lorentz", "mixed", "mur", "rlc", "rlc_mur"])
def test_mini_scene_operators_identical(kind):
    assert_same_operator(*both(scenes.mini(kind)))


@pytest.mark.parametrize("name", ["p64", "cavity", "rlc_series", "rlc_parallel"])
def test_small_scene_operators_identical(name):
    s = {"p64": lambda: scenes.p64(),
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
