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
