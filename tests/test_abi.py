"""The C-ABI library loads and exports every entry point include/*.h declares
(no compute call: runs without a GPU)."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"^\s*(?:int|size_t|void)\s+(fdtd_\w+)\s*\(", text, flags=re.M))
    return names


def test_library_exports_every_declared_symbol(libs):
    from wipems_gb300 import _abi
    L = ctypes.CDLL(str(_abi.LIB_PATH))
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_header(libs):
    from wipems_gb300 import _abi
    bound = {n for n, _, _ in _abi.SIGNATURES}
    assert declared_functions() <= bound


def test_errors_are_reported_not_trapped(libs):
    import pytest
    import numpy as np
    from wipems_gb300 import Scene, _abi
    with pytest.raises(_abi.FdtdError) as ei:
        Scene(np.array([0.0, 0.0]), np.arange(3.0), np.arange(3.0), 1e-3)
    assert "strictly increasing" in str(ei.value)
    s = Scene(np.arange(5.0), np.arange(5.0), np.arange(5.0), 1e-3)
    with pytest.raises(_abi.FdtdError) as ei:
        s.set_boundary([7] * 6)
    assert ei.value.code == -1


def test_null_arguments_are_refused_not_dereferenced(libs):
    """Every declared entry point called with null / zero arguments returns
    a status instead of crashing (run in a child process, so a crash would
    fail the test instead of the suite).  Without a GPU, calls that get as
    far as the device report FDTD_ERR_CUDA."""
    import subprocess
    import sys
    code = r'''
import ctypes, sys
from wipems_gb300 import _abi
L = ctypes.CDLL(str(_abi.LIB_PATH))
bad = []
for name, res, args in _abi.SIGNATURES:
    f = getattr(L, name)
    f.restype = res
    f.argtypes = args
    vals = []
    for a in args:
        if a in (ctypes.c_double, ctypes.c_float):
            vals.append(0.0)
        elif a in (ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_size_t, ctypes.c_long, ctypes.c_int64):
            vals.append(0)
        else:
            vals.append(None)
    try:
        r = f(*vals)
    except ctypes.ArgumentError as e:
        bad.append((name, "args", str(e)))
        continue
    if res is ctypes.c_int and r > 0:
        bad.append((name, r))
print("BAD", bad)
sys.exit(1 if bad else 0)
'''
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300,
                       cwd=str(ROOT))
    assert p.returncode == 0, (p.returncode, p.stdout[-2000:], p.stderr[-2000:])
