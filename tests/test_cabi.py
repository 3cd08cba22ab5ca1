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


def test_host_memory_and_graph_entry_points_check_their_arguments():
    """dbsrg_host_alloc / dbsrg_host_free and the captured-assembly and
    streamed-host entry points refuse bad arguments without touching a GPU;
    without one, dbsrg_host_alloc reports that the registration failed."""
    L = _lib.load()
    p = ctypes.c_void_p()
    assert L.dbsrg_host_alloc(ctypes.c_size_t(0), ctypes.byref(p)) == -1
    assert L.dbsrg_host_alloc(ctypes.c_size_t(1 << 20), None) == -1
    assert L.dbsrg_host_free(None) == 0
    import numpy as np

    x = np.zeros(8)
    assert L.dbsrg_host_free(ctypes.c_void_p(x.ctypes.data)) == -1  # not from dbsrg_host_alloc
    rc = L.dbsrg_host_alloc(ctypes.c_size_t(1 << 20), ctypes.byref(p))
    assert rc in (0, -3)
    if rc == 0:
        assert L.dbsrg_host_free(p) == 0
    else:
        assert not p.value
    assert L.dbsrg_graph_capture(None, 0, None) == -1
    assert L.dbsrg_graph_launch(None, None) == -1
    assert L.dbsrg_graph_release(None) == -1
    assert L.dbsrg_assemble_streamed_host(None, 0, None, 0, None, None, None, None) == -1
