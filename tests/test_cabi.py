"""The C ABI library builds, loads without a GPU and exports every entry
point that include/dbsrg.h declares (no compute calls here)."""
import ctypes
import os
import re

from dbsr_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "dbsrg.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(dbsrg_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    names = declared_symbols()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    bound = {s[0] for s in _lib.SIGNATURES}
    assert set(names) <= bound, set(names) - bound


def test_create_fails_cleanly_without_gpu_or_with_bad_args():
    L = _lib.load()
    h = ctypes.c_void_p()
    # invalid descriptor: ns < ks
    import numpy as np

    t = np.zeros(10)
    d = _lib.GridDesc(3, 9, 8, 9, ctypes.c_void_p(t.ctypes.data), 0)
    assert L.dbsrg_create(ctypes.byref(h), ctypes.byref(d)) == -1
    assert L.dbsrg_create(ctypes.byref(h), None) == -1
