"""Edge cases of the grid and of the run, GPU against the oracle bit for
bit: thin and ragged grids (an axis of two or three lines, sizes far from
the 32 x 8 tile), PMC walls, excitation and probes at the domain edge, a
zero-step iterate, and a run with nothing excited (the end criterion must
not fire on 0 / 0, as RunFDTD's `if (maxE)` guard keeps it from doing)."""
import numpy as np
import pytest

import oracle
from wipems_gb300 import Engine, Operator, Scene
from wipems_gb300.fdtd import BC_PEC, BC_PMC

from helpers import oracle_inputs
from test_parity_gpu import compare

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("libs")]


def _thin(n, pmc_faces=(), steps=200):
    lines = [np.arange(k, dtype=float) for k in n]
    s = Scene(*lines, 1e-3)
    bc = [BC_PEC] * 6
    for f in pmc_faces:
        bc[f] = BC_PMC
    s.set_boundary(bc)
    s.set_gauss_excite(20e9, 20e9, steps)
    # a soft source along the longest axis at the middle of the other two
    a = int(np.argmax(n))
    c = [k // 2 for k in n]
    st, sp = list(c), list(c)
    st[a], sp[a] = 0, n[a] - 1
    vec = [0.0, 0.0, 0.0]
    vec[a] = 1.0
    s.add_excitation(st, sp, vec)
    s.add_probe(st, sp, 0)  # the excited line itself, edge to edge
    lo = [max(c[k] - 1, 0) + 0.5 if n[k] > 2 else 0.5 for k in range(3)]
    hi = list(lo)
    lo[a] = hi[a] = 0.5 * (n[a] - 1)
    s.add_probe(lo, hi, 1, norm_dir=a)
    return s


@pytest.mark.parametrize("n,pmc", [((3, 3, 3), ()), ((2, 9, 40), (0, 1)), ((41, 2, 6), (2, 3)),
                                   ((6, 35, 2), (4, 5)), ((4, 4, 70), ()), ((33, 9, 65), (1, 4))])
@pytest.mark.parametrize("kernel", ["tma", "direct"])
def test_thin_and_ragged_grids_match_oracle(n, pmc, kernel):
    op = Operator(_thin(n, pmc))
    ref = oracle.run(*oracle_inputs(op), 200, op.probe_interval, engine=oracle.BASIC)
    eng = Engine(op, kernel=kernel)
    eng.iterate(200)
    compare(op, eng, ref)


def test_zero_step_iterate_and_nothing_excited():
    op = Operator(_thin((9, 10, 11)))
    eng = Engine(op)
    eng.iterate(0)
    assert eng.num_timesteps == 0
    eng.iterate(37)
    V0, I0 = eng.fields()
    eng.iterate(0)
    V1, I1 = eng.fields()
    assert eng.num_timesteps == 37 and np.array_equal(V0, V1) and np.array_equal(I0, I1)
    # no excitation: the energy stays 0 and the job runs to its cap
    lines = [np.arange(12, dtype=float)] * 3
    s = Scene(*lines, 1e-3)
    s.set_boundary([BC_PEC] * 6)
    s.set_gauss_excite(10e9, 10e9, 300)
    s.add_probe([5, 5, 2], [5, 5, 9], 0)
    op = Operator(s)
    eng = Engine(op, end_crit=1e-3, max_timesteps=300)
    eng.iterate(300)
    assert eng.num_timesteps == 300 and eng.done
    smp = eng.samples()
    assert np.all(smp.energy == 0) and np.all(smp.values == 0)
