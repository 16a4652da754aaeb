"""Frequency-domain probe accumulation on the device against the same DFT
sum over the oracle's samples at the FD steps, and the lumped-port result
from it against the one from the time-domain samples."""
import os

import numpy as np
import pytest

import oracle
from wipems_gb300 import Engine, Operator, scenes
from wipems_gb300.ports import lumped_port_fd, lumped_port_td

from helpers import oracle_inputs

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("libs")]


@pytest.mark.parametrize("kind,graphs", [("p64", True), ("upml", True), ("upml", False)])
def test_fd_accumulation_matches_oracle_dft(kind, graphs):
    sc = scenes.p64(nr_ts=2000) if kind == "p64" else scenes.mini("upml", nr_ts=700)
    op = Operator(sc)
    n = 600
    eng = Engine(op, use_graphs=graphs)
    freqs = eng.set_frequencies(np.linspace(1e9, 9e9, 9))
    fdint = eng.fd_interval
    assert fdint > 0 and (kind != "p64" or fdint != eng.interval)  # FD steps off the sample grid
    eng.iterate(250)
    eng.iterate(n - 250)
    got, count = eng.fd_results()
    ref = oracle.run(*oracle_inputs(op), n, fdint, engine=oracle.SSE_COMPRESSED_MT, threads=os.cpu_count())
    assert count == len(ref["ts"]) == n // fdint + 1
    dual = np.array([0.5 if p.type == 1 else 0.0 for p in op.probes])
    t = (ref["ts"][:, None] + dual[None, :]) * op.dT                  # [sample][probe]
    phase = np.exp(-2j * np.pi * freqs[None, None, :] * t[:, :, None])  # [sample][probe][freq]
    want = np.einsum("sp,spf->pf", ref["values"], phase) * 2 * op.dT * fdint
    scale = np.abs(want).max()
    assert np.max(np.abs(got - want)) <= 1e-12 * scale


def test_lumped_port_from_device_fd_and_from_samples():
    sc = scenes.port_scene([30, 30, 40], 0.5, 8, 3, 7, 10e9, 5e9, 3000, edge_range=(3, 8))
    op = Operator(sc)
    names = [p["name"] for p in sc.probes]
    eng = Engine(op)
    f = eng.set_frequencies(np.linspace(4e9, 10e9, 4))
    eng.iterate(3000)
    fd, _ = eng.fd_results()
    a = lumped_port_fd(fd, f, names, 50.0)
    b = lumped_port_td(eng.samples(), names, f, 50.0)
    assert np.all(np.isfinite(a.s11)) and np.all(a.P_inc > 0)
    # two quadratures of the same spectrum: the FD steps come at the Nyquist
    # rate of the 15 GHz band edge, the samples four times as often, so they
    # agree well below the band edge
    assert np.max(np.abs(a.s11 - b.s11)) < 1e-3
