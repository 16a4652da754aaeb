"""fdtd_field_energy_static: the energy reduction for callers that may not
allocate device memory.  It reads device fields the caller owns and keeps
its partial sums in a static device array; its result must equal
fdtd_engine_energy's on the same fields, on consecutive calls.

Collected last on purpose (file name), so that a stop-at-first-failure run
has already run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_static_energy_matches_engine_energy(libs):
    import torch
    from wipems_gb300 import Engine, Operator, _abi, scenes

    op = Operator(scenes.mini("upml", nr_ts=200))
    eng = Engine(op)
    L = _abi.lib()
    nl = (ctypes.c_uint32 * 3)(*op.num_lines)
    out = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    states = []
    for steps in (90, 60):  # two field states, the second 60 steps after the first
        eng.iterate(steps)
        ref = eng.energy()
        assert ref > 0
        V, I = eng.fields()
        states.append((ref, torch.from_numpy(np.ascontiguousarray(V)).to("cuda:0"),
                       torch.from_numpy(np.ascontiguousarray(I)).to("cuda:0")))

    def call(Vd, Id):
        out.fill_(-1.0)
        rc = L.fdtd_field_energy_static(ctypes.c_void_p(Vd.data_ptr()), ctypes.c_void_p(Id.data_ptr()), nl,
                                        op.num_lines[2], stream, ctypes.c_void_p(out.data_ptr()))
        assert rc == 0, _abi.last_error()
        torch.cuda.synchronize()
        return out.item()

    call(*states[0][1:])  # the first call on the device does the set-up
    free0, _ = torch.cuda.mem_get_info(0)
    for ref, Vd, Id in states:  # two calls in a row
        got = call(Vd, Id)
        assert abs(got / ref - 1) < 1e-6, (got, ref)
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, (free0, free1)  # the calls allocated no device memory


def test_static_energy_rejects_oversized_grid(libs):
    from wipems_gb300 import _abi
    L = _abi.lib()
    nl = (ctypes.c_uint32 * 3)(5000, 4, 4)
    rc = L.fdtd_field_energy_static(ctypes.c_void_p(16), ctypes.c_void_p(16), nl, 4, None, ctypes.c_void_p(16))
    assert rc == -1 and "exceeds the static scratch capacity" in _abi.last_error()
