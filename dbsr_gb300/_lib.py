"""ctypes binding of libdbsrgpu.so (the C ABI declared in include/dbsrg.h).

There is no CPU fallback: if the shared library is missing or no usable
sm_103a GPU is present, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdbsrgpu.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p

STATUS = {0: "OK", -1: "EINVAL", -2: "ECUDA", -3: "ENOMEM", -4: "ERANGE", -5: "ESTATE",
          -6: "ETIMEOUT", -7: "EIO"}

# (name, restype, argtypes) for every entry point of include/dbsrg.h
# void fn(void *user, int ictx, int blo, int nblocks, const double *window)
WindowFn = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p)


class ListDesc(C.Structure):
    """dbsrg_list of include/dbsrg.h"""

    _fields_ = [("icase", C.c_int), ("itype", C.c_int), ("kpol", C.c_int), ("ncdata", C.c_int),
                ("ipt", C.c_void_p), ("k1", C.c_void_p), ("k2", C.c_void_p),
                ("k3", C.c_void_p), ("k4", C.c_void_p), ("cdata", C.c_void_p)]


SIGNATURES = [
    ("dbsrg_create", C.c_int, [C.POINTER(_vp), _vp]),
    ("dbsrg_destroy", C.c_int, [_vp]),
    ("dbsrg_last_error", C.c_char_p, [_vp]),
    ("dbsrg_set_orbitals", C.c_int, [_vp, C.c_int, _vp, _vp]),
    ("dbsrg_alloc_matrix", C.c_int, [_vp, C.c_int, _vp, C.c_int, C.c_int]),
    ("dbsrg_zero_matrix", C.c_int, [_vp]),
    ("dbsrg_set_precision", C.c_int, [_vp, C.c_int]),
    ("dbsrg_gen_matrix", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp,
                                   _vp, _vp]),
    ("dbsrg_update_hx", C.c_int, [_vp, C.c_int, C.c_int, _vp, C.c_double]),
    ("dbsrg_get_block", C.c_int, [_vp, C.c_int, C.c_int, _vp]),
    ("dbsrg_get_matrix", C.c_int, [_vp, _vp]),
    ("dbsrg_get_acf", C.c_int, [_vp, _vp]),
    ("dbsrg_matrix_device_ptr", C.c_int, [_vp, C.POINTER(_vp)]),
    ("dbsrg_get_table", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _vp]),
    ("dbsrg_get_moments", C.c_int, [_vp, C.c_int, C.c_int, _vp]),
    ("dbsrg_get_diag_cells", C.c_int, [_vp, C.c_int, C.c_int, _vp]),
    ("dbsrg_get_grid_array", C.c_int, [_vp, C.c_char_p, _vp]),
    ("dbsrg_kernel_launches", C.c_longlong, [_vp]),
    ("dbsrg_sync", C.c_int, [_vp]),
    ("dbsrg_set_async", C.c_int, [_vp, C.c_int]),
    ("dbsrg_set_tuning", C.c_int, [_vp, C.c_char_p, C.c_int]),
    ("dbsrg_set_wait_limit", C.c_int, [_vp, C.c_longlong]),
    ("dbsrg_inject_wait_timeout", C.c_int, [_vp, C.c_int]),
    ("dbsrg_diag_channels", C.c_int,
     [_vp, _vp, _vp, C.c_double, C.c_double, C.c_double, _vp, _vp, _vp]),
    ("dbsrg_channel_basis", C.c_int, [_vp, _vp, _vp, _vp]),
    ("dbsrg_record_header", C.c_int, [_vp, C.c_char_p, C.c_int, C.c_int, _vp, _vp, _vp]),
    ("dbsrg_record_matrix", C.c_int, [_vp, _vp, _vp, C.c_int, C.c_char_p, _vp]),
    ("dbsrg_record_acf", C.c_int, [_vp, C.c_char_p, _vp]),
    ("dbsrg_orth_channels", C.c_int, [_vp, _vp]),
    ("dbsrg_hf_matrix", C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp, C.c_double, _vp, _vp]),
    ("dbsrg_mchf_matrix", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, C.c_int, _vp,
                                    _vp, _vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_double,
                                    _vp, _vp, _vp, _vp, _vp]),
    ("dbsrg_mchf_core", C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp, _vp, _vp, C.c_int, _vp, _vp]),
    ("dbsrg_lists_create", C.c_int, [C.POINTER(_vp), C.c_int, C.c_int, _vp, _vp, _vp, C.c_int,
                                     C.c_double, C.c_int]),
    ("dbsrg_lists_destroy", C.c_int, [_vp]),
    ("dbsrg_lists_decode", C.c_int, [C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("dbsrg_lists_add", C.c_int, [_vp, C.c_int] + [_vp] * 10),
    ("dbsrg_lists_count", C.c_int, [_vp, C.c_int, C.c_int]),
    ("dbsrg_lists_get", C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp]),
    ("dbsrg_lists_gen_matrix", C.c_int, [_vp, _vp]),
    ("dbsrg_get_tuning", C.c_int, [_vp, C.c_char_p, _ip]),
    ("dbsrg_alloc_matrix_window", C.c_int, [_vp, C.c_int, _vp, C.c_int, C.c_int, C.c_int]),
    ("dbsrg_set_window", C.c_int, [_vp, C.c_int]),
    ("dbsrg_window_blocks", C.c_int, [_vp]),
    ("dbsrg_release_tables", C.c_int, [_vp]),
    ("dbsrg_invalidate_tables", C.c_int, [_vp]),
    ("dbsrg_timing", C.c_int, [_vp, C.c_int]),
    ("dbsrg_timing_report", C.c_int, [_vp, C.c_char_p, C.c_size_t]),
    ("dbsrg_gen_batch", C.c_int, [C.c_int, _vp, _vp, _vp]),
    ("dbsrg_gen_batch_streamed", C.c_int, [C.c_int, _vp, _vp, _vp, _vp, _vp]),
    ("dbsrg_assemble_to_host", C.c_int, [_vp, C.c_int, _vp, C.c_int, _vp, _vp]),
    ("dbsrg_assemble_streamed_host", C.c_int, [_vp, C.c_int, _vp, C.c_int, _vp, _vp, _vp, _vp]),
    ("dbsrg_host_alloc", C.c_int, [C.c_size_t, _vp]),
    ("dbsrg_graph_capture", C.c_int, [_vp, C.c_int, _vp]),
    ("dbsrg_graph_launch", C.c_int, [_vp, _vp]),
    ("dbsrg_graph_release", C.c_int, [_vp]),
    ("dbsrg_host_free", C.c_int, [_vp]),
    ("dbsrg_backward", C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("dbsrg_alloc_perturbers", C.c_int, [_vp, C.c_int, _vp, C.c_int, _vp, C.c_int]),
    ("dbsrg_get_perturbers", C.c_int, [_vp, _vp, _vp]),
    ("dbsrg_set_targets", C.c_int, [_vp, C.c_int, _vp, C.c_int, C.c_int]),
    ("dbsrg_get_targets", C.c_int, [_vp, _vp, _vp]),
    ("dbsrg_set_dhl", C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    ("dbsrg_set_eps_c", C.c_int, [_vp, C.c_double]),
    ("dbsrg_update_hw", C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp, C.c_double]),
    ("dbsrg_update_hv", C.c_int, [_vp, C.c_int, C.c_int, _vp, C.c_double]),
    ("dbsrg_update_hb", C.c_int, [_vp, C.c_int, C.c_int, C.c_double]),
    ("dbsrg_scale_matrix", C.c_int, [_vp, C.c_double]),
    ("dbsrg_hf_breit_list", C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, _vp]),
    ("dbsrg_exchange_segment_noalloc", C.c_int,
     [C.c_int, C.c_int, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp]),
]


class GridDesc(C.Structure):
    _fields_ = [("ns", C.c_int), ("ks", C.c_int), ("ksp", C.c_int), ("ksq", C.c_int),
                ("t", _vp), ("device", C.c_int)]


_lib = None


def load(path: str | None = None):
    """Load the library (building it first when the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        from . import build as _b

        _b.build()
    L = C.CDLL(p)
    for name, res, args in SIGNATURES:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


class DbsrgError(RuntimeError):
    pass


def check(ctx, rc: int, what: str):
    if rc != 0:
        msg = ""
        if ctx:
            try:
                msg = load().dbsrg_last_error(ctx).decode()
            except Exception:
                pass
        raise DbsrgError(f"{what}: {STATUS.get(rc, rc)} {msg}")
