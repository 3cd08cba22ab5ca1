"""Host-side mirror of the reference's Gen_matrix interface.

``Assembler`` owns one library context: the B-spline grid of one partial
wave, the orbitals (module DBS_orbitals_pq), the channel-pair matrix
(hch/icc/acf of module dbsr_mat) and the cached R^k/S^k tables.  Its
methods carry the reference's names and argument meaning:

* ``gen_matrix(icase, itype, kpol, k1, k2, k3, k4, cdata, ipt=None)`` --
  Gen_matrix (DBSR_MAT3/gen_matrix.f90:2-17) for a list laid out as
  Add_matrix leaves it (MOD_c_data.f90:318-368);
* ``update_hx(ich, jch, d, c)`` -- UPDATE_HX (updates.f90:79-106);
* ``get_block(ich, jch)`` -- block icc(ich,jch) of hch(ms,ms,:).

Arrays may be numpy arrays (host; the library copies them) or torch CUDA
tensors (device; used in place).  Errors raise ``DbsrgError`` where the
reference would stop.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import check, load

PLAIN_FP64 = 0   # the reference's loop structure over assembled tables
SPLIT_BF16 = 1   # cell-factored contraction, far field on the tensor cores
FACTOR_FP64 = 2  # cell-factored contraction, all FP64
RK = 0
SK = 1


def _ptr(a, dtype):
    """(pointer, keepalive) for a numpy array or a torch tensor."""
    if a is None:
        return None, None
    if hasattr(a, "data_ptr") and hasattr(a, "is_cuda"):
        if not a.is_contiguous():
            raise ValueError("torch tensor arguments must be contiguous")
        want = {np.float64: "float64", np.int32: "int32"}[dtype]
        if str(a.dtype).split(".")[-1] != want:
            raise TypeError(f"expected torch.{want}, got {a.dtype}")
        return C.c_void_p(a.data_ptr()), a
    arr = np.asarray(a)
    if arr.dtype != dtype or not (arr.flags.c_contiguous or arr.flags.f_contiguous):
        arr = np.array(arr, dtype=dtype, order="F")
    return C.c_void_p(arr.ctypes.data), arr


class Assembler:
    def __init__(self, t, ks: int = 9, ksp: int = 8, ksq: int = 9, device: int = 0,
                 tuning: str | dict | None = "auto"):
        """tuning: "auto" applies the autotuned parameters recorded for this
        GPU and grid size (dbsr_gb300/tuning.json, written by autotune.py), a
        dict sets them explicitly, None keeps the library defaults."""
        L = load()
        t = np.ascontiguousarray(t, dtype=np.float64)
        self.ks, self.ksp, self.ksq = ks, ksp, ksq
        self.ns = t.size - ks
        self.nv = self.ns - ks + 1
        self.ms = 2 * self.ns
        d = _lib.GridDesc(self.ns, ks, ksp, ksq, C.c_void_p(t.ctypes.data), device)
        h = C.c_void_p()
        rc = L.dbsrg_create(C.byref(h), C.byref(d))
        check(None, rc, "dbsrg_create")
        self._h = h
        self._L = L
        self.nch = 0
        self.iicc = 0
        self.mk = -1
        self.nbf = 0
        self.npert = 0
        if tuning == "auto":
            from . import autotune

            tuning = autotune.lookup(self.ns, device)
        for name, value in (tuning or {}).items():
            self.set_tuning(name, int(value))

    def close(self):
        if getattr(self, "_h", None):
            self._L.dbsrg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state ------------------------------------------------------------
    def set_orbitals(self, pq, ipbs):
        """pq(ns,2,nbf) in Fortran order; ipbs(nbf) channel of each orbital."""
        if not hasattr(pq, "data_ptr"):
            pq = np.asfortranarray(pq, dtype=np.float64)
        nbf = int(pq.shape[-1]) if pq.ndim == 3 else int(pq.size // (2 * self.ns))
        p, k1 = _ptr(pq, np.float64)
        q, k2 = _ptr(np.ascontiguousarray(ipbs, dtype=np.int32), np.int32)
        check(self._h, self._L.dbsrg_set_orbitals(self._h, nbf, p, q), "set_orbitals")
        self.nbf = nbf

    def alloc_matrix(self, nch: int, icc, iicc: int, mk: int, window: int | None = None):
        """hch(ms,ms,iicc) on the device, or a window of `window` consecutive
        blocks of it (streamed assembly: set_window, stream)."""
        icc = np.asfortranarray(icc, dtype=np.int32)
        p, keep = _ptr(icc, np.int32)
        if window is None:
            rc = self._L.dbsrg_alloc_matrix(self._h, nch, p, iicc, mk)
        else:
            rc = self._L.dbsrg_alloc_matrix_window(self._h, nch, p, iicc, mk, int(window))
        check(self._h, rc, "alloc_matrix")
        self.nch, self.iicc, self.mk = nch, iicc, mk
        self.wcap = iicc if window is None else int(window)
        self.icc = icc

    def assemble_to_host(self, lists, out=None, acf=None, nwin: int = 0):
        """dbsrg_assemble_to_host: every list (icase, itype, kpol, k1, k2, k3, k4,
        cdata[, ipt]) into `out` (ms, ms, iicc), window by window, with the copy
        of each window overlapped with the next one's assembly.  `out` may be
        host (pinned for the overlap) or device memory; returns (out, acf)."""
        if out is None:
            out = np.zeros((self.ms, self.ms, self.iicc), order="F")
        if acf is None:
            acf = np.zeros((self.iicc, self.mk + 1), order="F")
        arr, keep, counts = _list_descs([lists])
        po, k1 = _ptr(out, np.float64)
        pa, k2 = _ptr(acf, np.float64)
        rc = self._L.dbsrg_assemble_to_host(self._h, counts[0], arr, int(nwin), po, pa)
        check(self._h, rc, "assemble_to_host")
        return out, acf

    def assemble_streamed(self, lists, stage, consumer, acf=None, nwin: int = 0):
        """dbsrg_assemble_streamed_host: every list, window by window of at most
        `nwin` blocks, each window copied into one half of `stage` (room for
        2*nwin blocks of ms x ms; numpy or torch, host -- pinned for the
        overlap -- or device) while the next window is assembled.
        consumer(blo, nblocks, view) runs on this thread for every window, in
        block order, once its copy is complete; `view` is the window's part of
        `stage` as (ms, ms, nblocks), valid until the consumer returns.  An
        exception in the consumer is raised when the call returns.  Returns
        acf (iicc, 0:mk)."""
        if acf is None:
            acf = np.zeros((self.iicc, self.mk + 1), order="F")
        arr, keep, counts = _list_descs([lists])
        ps, hold = _ptr(stage, np.float64)
        pa, k2 = _ptr(acf, np.float64)
        if hasattr(hold, "data_ptr"):
            flat, base = hold.view(-1), int(hold.data_ptr())
        else:
            flat, base = hold.ravel(order="K"), int(hold.ctypes.data)
        ms = self.ms
        errors = []

        def fn(user, ictx, blo, nblocks, ptr):
            if errors:
                return
            try:
                off = (int(ptr) - base) // 8
                n = int(nblocks) * ms * ms
                view = flat[off:off + n]
                view = view.reshape(int(nblocks), ms, ms).permute(2, 1, 0) if hasattr(
                    view, "permute") else view.reshape((ms, ms, int(nblocks)), order="F")
                consumer(int(blo), int(nblocks), view)
            except BaseException as e:  # surfaces after the call
                errors.append(e)

        cb = _lib.WindowFn(fn)
        rc = self._L.dbsrg_assemble_streamed_host(self._h, counts[0], arr, int(nwin), ps,
                                                  C.cast(cb, C.c_void_p), None, pa)
        if errors:
            raise errors[0]
        check(self._h, rc, "assemble_streamed")
        return acf

    def graph_capture(self, lists):
        """dbsrg_graph_capture: every list (icase, itype, kpol, k1, k2, k3, k4,
        cdata[, ipt]) planned, the whole assembly (table builds included)
        captured as one CUDA graph and run once."""
        arr, keep, counts = _list_descs([lists])
        check(self._h, self._L.dbsrg_graph_capture(self._h, counts[0], arr), "graph_capture")

    def graph_launch(self, pq=None):
        """dbsrg_graph_launch: the captured assembly again, from new orbitals
        pq(ns,2,nbf) (same count and channels) or the orbitals held."""
        p, keep = (None, None) if pq is None else _ptr(
            pq if hasattr(pq, "data_ptr") else np.asfortranarray(pq, dtype=np.float64), np.float64)
        check(self._h, self._L.dbsrg_graph_launch(self._h, p), "graph_launch")

    def graph_release(self):
        check(self._h, self._L.dbsrg_graph_release(self._h), "graph_release")

    def set_window(self, blo: int):
        """Hold (and zero) blocks blo .. blo + window - 1."""
        check(self._h, self._L.dbsrg_set_window(self._h, int(blo)), "set_window")

    @property
    def window_blocks(self) -> int:
        return int(self._L.dbsrg_window_blocks(self._h))

    def stream(self, lists):
        """Assemble the matrix window by window: every list (icase, itype, kpol,
        k1, k2, k3, k4, cdata) once per window.  Yields (first block, number of
        blocks) with the window assembled on the device; read it (get_matrix,
        matrix_device_ptr) before the generator advances."""
        for blo in range(1, self.iicc + 1, self.wcap):
            self.set_window(blo)
            for item in lists:
                self.gen_matrix(*item[:8])
            self.sync()
            yield blo, self.window_blocks

    def zero_matrix(self):
        check(self._h, self._L.dbsrg_zero_matrix(self._h), "zero_matrix")

    def set_precision(self, mode: int):
        check(self._h, self._L.dbsrg_set_precision(self._h, mode), "set_precision")

    # -- the drop-in ----------------------------------------------------------
    def gen_matrix(self, icase, itype, kpol, k1, k2, k3, k4, cdata, ipt=None):
        n = int(len(k1))
        ptrs, keep = [], []
        for a, dt in ((ipt, np.int32), (k1, np.int32), (k2, np.int32), (k3, np.int32),
                      (k4, np.int32), (cdata, np.float64)):
            p, kk = _ptr(a, dt)
            ptrs.append(p)
            keep.append(kk)
        rc = self._L.dbsrg_gen_matrix(self._h, icase, itype, kpol, n, *ptrs)
        check(self._h, rc, f"gen_matrix(icase={icase},itype={itype},kpol={kpol})")

    def update_hx(self, ich, jch, d, c):
        p, keep = _ptr(np.asfortranarray(d, dtype=np.float64) if not hasattr(d, "data_ptr") else d,
                       np.float64)
        check(self._h, self._L.dbsrg_update_hx(self._h, ich, jch, p, float(c)), "update_hx")

    # -- matrix parts beside hch: perturbers, targets, one-electron data --
    def alloc_perturbers(self, npert: int, icb, ibb):
        """hcp(ms,iicb) and hp(iibb) with icb(nch,npert) and ibb(npert,npert)
        (the perturber part of Alloc_dbsr_matrix, updates.f90:47-72)."""
        icb = np.asfortranarray(icb, dtype=np.int32)
        ibb = np.asfortranarray(ibb, dtype=np.int32)
        self.iicb, self.iibb = int(icb.max(initial=0)), int(ibb.max(initial=0))
        self.npert = int(npert)
        check(self._h, self._L.dbsrg_alloc_perturbers(self._h, int(npert), C.c_void_p(icb.ctypes.data),
                                                      self.iicb, C.c_void_p(ibb.ctypes.data),
                                                      self.iibb), "alloc_perturbers")

    def get_perturbers(self):
        """(hcp(ms,iicb), hp(iibb))"""
        hcp = np.zeros((self.ms, max(self.iicb, 1)), order="F")
        hp = np.zeros(max(self.iibb, 1))
        check(self._h, self._L.dbsrg_get_perturbers(self._h, C.c_void_p(hcp.ctypes.data),
                                                    C.c_void_p(hp.ctypes.data)), "get_perturbers")
        return hcp, hp

    def set_targets(self, ntarg: int, iptar, iitar: int = 0, check_target: int = 1):
        """Target_h's matrices htarg/otarg (target_subs.f90:2-31) over ntarg
        targets, iptar(nch) the target of each channel."""
        iptar = np.ascontiguousarray(iptar, dtype=np.int32)
        self.ntarg = int(ntarg)
        check(self._h, self._L.dbsrg_set_targets(self._h, int(ntarg), C.c_void_p(iptar.ctypes.data),
                                                 int(iitar), int(check_target)), "set_targets")

    def get_targets(self):
        n = max(self.ntarg * (self.ntarg + 1) // 2, 1)
        ht, ot = np.zeros(n), np.zeros(n)
        check(self._h, self._L.dbsrg_get_targets(self._h, C.c_void_p(ht.ctypes.data),
                                                 C.c_void_p(ot.ctypes.data)), "get_targets")
        return ht, ot

    def set_dhl(self, kap_list, hd, kbs):
        """One-electron Dirac matrices hd(ms,ms,nkap) of the kappas kap_list
        and the kappa of every orbital kbs(nbf), read by L_data."""
        kap = np.ascontiguousarray(kap_list, dtype=np.int32)
        hd = np.asfortranarray(hd, dtype=np.float64)
        kbs = np.ascontiguousarray(kbs, dtype=np.int32)
        check(self._h, self._L.dbsrg_set_dhl(self._h, kap.size, C.c_void_p(kap.ctypes.data),
                                             C.c_void_p(hd.ctypes.data), C.c_void_p(kbs.ctypes.data)),
              "set_dhl")

    def scale_matrix(self, s: float):
        """hch, hcp and hp times s (SUB1's core-energy shifts, sub1.f90:96,222)."""
        check(self._h, self._L.dbsrg_scale_matrix(self._h, float(s)), "scale_matrix")

    def set_eps_c(self, eps_c: float):
        check(self._h, self._L.dbsrg_set_eps_c(self._h, float(eps_c)), "set_eps_c")

    def update_hw(self, ich, jch, v, w, c):
        """UPDATE_HW (updates.f90:183-216): c v w^T into block (ich,jch)."""
        p, kv = _ptr(v, np.float64)
        q, kw = _ptr(w, np.float64)
        check(self._h, self._L.dbsrg_update_hw(self._h, ich, jch, p, q, float(c)), "update_hw")

    def update_hv(self, ich, ip, v, c):
        """UPDATE_HV (updates.f90:220-242): c v into hcp(:, icb(ich,ip))."""
        p, kv = _ptr(v, np.float64)
        check(self._h, self._L.dbsrg_update_hv(self._h, ich, ip, p, float(c)), "update_hv")

    def update_hb(self, ic, jc, c):
        """UPDATE_HB (updates.f90:245-264): c into hp(ibb(ic,jc))."""
        check(self._h, self._L.dbsrg_update_hb(self._h, ic, jc, float(c)), "update_hb")

    # -- energy functional and its gradient ------------------------------------
    def backward(self, k, i1, i2, i3, i4, coef, grad: bool = True):
        """(E, dE/dpq) of E = sum_e coef[e] R^k[e](i1,i2;i3,i4) over the orbitals
        set by set_orbitals (1-based, bound); dE/dpq has the shape (ns, 2, nbf)
        in Fortran order, or is None when grad is False."""
        n = int(len(coef))
        ptrs, keep = [], []
        for a, dt in ((k, np.int32), (i1, np.int32), (i2, np.int32), (i3, np.int32),
                      (i4, np.int32), (coef, np.float64)):
            p, kk = _ptr(a, dt)
            ptrs.append(p)
            keep.append(kk)
        e = C.c_double(0.0)
        g = np.zeros((self.ns, 2, self.nbf), order="F") if grad else None
        rc = self._L.dbsrg_backward(self._h, n, *ptrs, C.byref(e),
                                    C.c_void_p(g.ctypes.data) if grad else None)
        check(self._h, rc, "backward")
        return e.value, g

    # -- results --------------------------------------------------------------
    def get_block(self, ich, jch):
        out = np.zeros((self.ms, self.ms), order="F")
        check(self._h, self._L.dbsrg_get_block(self._h, ich, jch, C.c_void_p(out.ctypes.data)),
              "get_block")
        return out

    def get_matrix(self, out=None):
        """The blocks held: all of hch, or the current window's blocks."""
        if out is None:
            out = np.zeros((self.ms, self.ms, self.window_blocks), order="F")
        p, keep = _ptr(out, np.float64)
        check(self._h, self._L.dbsrg_get_matrix(self._h, p), "get_matrix")
        return out

    def get_acf(self):
        out = np.zeros((self.iicc, self.mk + 1), order="F")
        check(self._h, self._L.dbsrg_get_acf(self._h, C.c_void_p(out.ctypes.data)), "get_acf")
        return out

    def matrix_device_ptr(self) -> int:
        p = C.c_void_p()
        check(self._h, self._L.dbsrg_matrix_device_ptr(self._h, C.byref(p)), "matrix_device_ptr")
        return int(p.value)

    def get_table(self, family: int, typ: int, k: int):
        kb = self.ks if family == RK else 2 * self.ks - 1
        out = np.zeros((self.ns, self.ns, kb, kb), order="F")
        rc = self._L.dbsrg_get_table(self._h, family, typ, k, C.c_void_p(out.ctypes.data))
        check(self._h, rc, "get_table")
        return out

    def get_moments(self, which: int, k: int):
        kk = self.ks * self.ks
        out = np.zeros((kk, self.nv), order="F")
        check(self._h, self._L.dbsrg_get_moments(self._h, which, k, C.c_void_p(out.ctypes.data)),
              "get_moments")
        return out

    def get_diag_cells(self, typ: int, k: int):
        kk = self.ks * self.ks
        out = np.zeros((kk, kk, self.nv), order="F")
        rc = self._L.dbsrg_get_diag_cells(self._h, typ, k, C.c_void_p(out.ctypes.data))
        check(self._h, rc, "get_diag_cells")
        return out

    def grid_array(self, name: str):
        nv, ks, ns, ms = self.nv, self.ks, self.ns, self.ms
        shapes = {"gr": (nv, ks), "grw": (nv, ks), "grm": (nv, ks), "gx": (ks,), "gw": (ks,),
                  "pbsp": (nv + 1, ks, self.ksp), "qbsp": (nv + 1, ks, self.ksq),
                  "fpbs": (ns, ns), "fqbs": (ns, ns), "fppqq": (ms, ms)}
        out = np.zeros(shapes[name], order="F")
        rc = self._L.dbsrg_get_grid_array(self._h, name.encode(), C.c_void_p(out.ctypes.data))
        check(self._h, rc, "grid_array")
        return out

    def release_tables(self):
        """Free the cached tables and everything derived from them."""
        check(self._h, self._L.dbsrg_release_tables(self._h), "release_tables")

    def invalidate_tables(self):
        """Mark the cached tables stale; they are rebuilt in their memory."""
        check(self._h, self._L.dbsrg_invalidate_tables(self._h), "invalidate_tables")

    def timing(self, enable: bool = True):
        check(self._h, self._L.dbsrg_timing(self._h, int(enable)), "timing")

    def timing_report(self) -> dict:
        """{kernel: (launches, total ms, algorithmic bytes, algorithmic FLOPs)} of
        the launches since timing(True); bytes/FLOPs are 0 where a launch
        states none."""
        import json

        buf = C.create_string_buffer(1 << 16)
        check(self._h, self._L.dbsrg_timing_report(self._h, buf, len(buf)), "timing_report")
        return {k: (int(v[0]), float(v[1]), float(v[2]), float(v[3]))
                for k, v in json.loads(buf.value.decode()).items()}

    @property
    def launches(self) -> int:
        return int(self._L.dbsrg_kernel_launches(self._h))

    def sync(self):
        """Wait for the queued kernels; raises on a failure of any of them."""
        check(self._h, self._L.dbsrg_sync(self._h), "sync")

    def diag_channels(self, bdiag, iprm, emin=-1.0e30, emax=1.0e30, egap=0.0):
        """dbsrg_diag_channels: (sol(ms,ms,nch), eval(ms,nch), nsol(nch)) of the
        generalized channel problems H c = E B c, B = bdiag(:,:,ich) (host or
        device), on the B-splines with iprm(:,ich) != 0."""
        sol = np.zeros((self.ms, self.ms, self.nch), order="F")
        ev = np.zeros((self.ms, self.nch), order="F")
        ns = np.zeros(self.nch, dtype=np.int32)
        pb, k1 = _ptr(bdiag, np.float64)
        pi, k2 = _ptr(np.asfortranarray(iprm, dtype=np.int32), np.int32)
        rc = self._L.dbsrg_diag_channels(self._h, pb, pi, float(emin), float(emax), float(egap),
                                         C.c_void_p(sol.ctypes.data), C.c_void_p(ev.ctypes.data),
                                         C.c_void_p(ns.ctypes.data))
        check(self._h, rc, "diag_channels")
        return sol, ev, ns

    def channel_basis(self, sol, nsol, out=None):
        """dbsrg_channel_basis: every off-diagonal block to D_i^T H D_j in place;
        returns the transformed matrix when `out` is given or True."""
        ps, k1 = _ptr(sol, np.float64)
        pn, k2 = _ptr(np.ascontiguousarray(nsol, dtype=np.int32), np.int32)
        if out is True:
            out = np.zeros((self.ms, self.ms, self.iicc), order="F")
        po, k3 = _ptr(out, np.float64) if out is not None else (None, None)
        check(self._h, self._L.dbsrg_channel_basis(self._h, ps, pn, po), "channel_basis")
        return out

    def record_header(self, path, sol, ev, nsol, nsp=None, nsq=None):
        """dbsrg_record_header: SUB1's records after Diag_channels
        (sub1.f90:164-168) to a new file at `path`."""
        ps, k1 = _ptr(sol, np.float64)
        e = np.asfortranarray(ev, dtype=np.float64)
        n = np.ascontiguousarray(nsol, dtype=np.int32)
        nsp = self.ns if nsp is None else nsp
        nsq = self.ns if nsq is None else nsq
        rc = self._L.dbsrg_record_header(self._h, os.fsencode(path), int(nsp), int(nsq), ps,
                                         C.c_void_p(e.ctypes.data), C.c_void_p(n.ctypes.data))
        check(self._h, rc, "record_header")

    def record_matrix(self, path, sol, nsol, icase=2, overlaps=None):
        """dbsrg_record_matrix: Record_matrix (record_matrix.f90:2-60)
        appended to `path`; with icase 0 fills and returns `overlaps`
        ((nch+npert)^2, created zero when None).  hch is left transformed."""
        ps, k1 = _ptr(sol, np.float64)
        n = np.ascontiguousarray(nsol, dtype=np.int32)
        if icase == 0 and overlaps is None:
            no = self.nch + self.npert
            overlaps = np.zeros((no, no), order="F")
        po = C.c_void_p(overlaps.ctypes.data) if overlaps is not None else None
        rc = self._L.dbsrg_record_matrix(self._h, ps, C.c_void_p(n.ctypes.data), int(icase),
                                         os.fsencode(path), po)
        check(self._h, rc, "record_matrix")
        return overlaps

    def record_acf(self, path, bcf):
        """dbsrg_record_acf: the records (mk) and (bcf(nch,nch,0:mk))."""
        b = np.asfortranarray(bcf, dtype=np.float64)
        if b.shape != (self.nch, self.nch, self.mk + 1):
            raise ValueError("bcf must be (nch, nch, mk+1)")
        rc = self._L.dbsrg_record_acf(self._h, os.fsencode(path), C.c_void_p(b.ctypes.data))
        check(self._h, rc, "record_acf")

    def orth_channels(self, iort):
        """dbsrg_orth_channels (DBS_ORTH, dbs_orth.f90:2-84): iort(nbf, nch)
        nonzero where channel ich is made orthogonal to bound orbital j; the
        whole matrix is transformed in place."""
        io = np.asfortranarray(iort, dtype=np.int32)
        if io.shape != (self.nbf, self.nch):
            raise ValueError(f"iort must be (nbf, nch) = ({self.nbf}, {self.nch})")
        pi, k = _ptr(io, np.int32)
        check(self._h, self._L.dbsrg_orth_channels(self._h, pi), "orth_channels")

    def hf_breit_list(self, kr1, kr2, kr3, kr4, crk):
        """rk4 entries of the Breit energy for the Breit part of hf_matrix
        (hf_matrix_breit, DBSR_HF/hf_matrix.f90:91-163)."""
        arrs = [np.ascontiguousarray(x, dtype=np.int32) for x in (kr1, kr2, kr3, kr4)]
        c = np.ascontiguousarray(crk, dtype=np.float64)
        check(self._h, self._L.dbsrg_hf_breit_list(self._h, int(c.size),
                                                   *[C.c_void_p(x.ctypes.data) for x in arrs],
                                                   C.c_void_p(c.ctypes.data)), "hf_breit_list")

    def hf_matrix(self, iorb: int, a, b, qsum: float, dhl=None, out=None):
        """dbsrg_hf_matrix (hf_matrix.f90:2-70, Coulomb part): the potential
        matrix (ms, ms) of orbital iorb (1-based); a, b: (nbf, kmax+1) values
        of a(iorb,j,k), b(iorb,j,k).  Needs a one-channel matrix
        (alloc_matrix(1, [[1]], 1, mk))."""
        A = np.asfortranarray(a, dtype=np.float64)
        B = np.asfortranarray(b, dtype=np.float64)
        if A.shape != B.shape or A.shape[0] != self.nbf:
            raise ValueError("a and b must be (nbf, kmax+1)")
        if out is None:
            out = np.zeros((self.ms, self.ms), order="F")
        po, k1 = _ptr(out, np.float64)
        pd, k2 = _ptr(dhl, np.float64) if dhl is not None else (None, None)
        rc = self._L.dbsrg_hf_matrix(self._h, int(iorb), A.shape[1] - 1, A.ctypes.data,
                                     B.ctypes.data, float(qsum), pd, po)
        check(self._h, rc, "hf_matrix")
        return out

    def mchf_matrix(self, iorb: int, kmax: int, lint, rint, dhl, irhs=1, newton=0, eps_c=1e-10):
        """dbsrg_mchf_matrix (DBSR_MCHF/mchf_matrix.f90:2-251) of orbital iorb
        outside the core: lint = (i1, i2, c), rint = (k, i1, i2, i3, i4, c)
        with the expansion weights applied; dhl (ms, ms).  Needs a
        one-channel matrix.  Returns (hfm, rhs, hx, e, qsum)."""
        li = [np.ascontiguousarray(x, dtype=np.int32) for x in lint[:2]]
        lc = np.ascontiguousarray(lint[2], dtype=np.float64)
        ri = [np.ascontiguousarray(x, dtype=np.int32) for x in rint[:5]]
        rc = np.ascontiguousarray(rint[5], dtype=np.float64)
        D = np.asfortranarray(dhl, dtype=np.float64)
        ms = self.ms
        hfm = np.zeros((ms, ms), order="F")
        hx = np.zeros((ms, ms), order="F")
        rhs = np.zeros(ms)
        e = np.zeros(1)
        q = np.zeros(1)
        ptr = lambda a: C.c_void_p(a.ctypes.data)  # noqa: E731
        rcode = self._L.dbsrg_mchf_matrix(
            self._h, int(iorb), int(kmax), lc.size, ptr(li[0]), ptr(li[1]), ptr(lc), rc.size,
            *[ptr(x) for x in ri], ptr(rc), ptr(D), int(irhs), int(newton), float(eps_c),
            ptr(hfm), ptr(rhs), ptr(hx), ptr(e), ptr(q))
        check(self._h, rcode, "mchf_matrix")
        return hfm, rhs, hx, float(e[0]), float(q[0])

    def mchf_core(self, iorb: int, a, b, qsum, hd, newton=0):
        """dbsrg_mchf_core (core_matrix, mchf_matrix.f90:255-346): a, b
        (nbf, kmax+1), qsum (nbf), hd (ms, ms).  Returns (hfm, hx)."""
        A = np.asfortranarray(a, dtype=np.float64)
        B = np.asfortranarray(b, dtype=np.float64)
        if A.shape != B.shape or A.shape[0] != self.nbf:
            raise ValueError("a and b must be (nbf, kmax+1)")
        Q = np.ascontiguousarray(qsum, dtype=np.float64)
        H = np.asfortranarray(hd, dtype=np.float64)
        ms = self.ms
        hfm = np.zeros((ms, ms), order="F")
        hx = np.zeros((ms, ms), order="F")
        ptr = lambda x: C.c_void_p(x.ctypes.data)  # noqa: E731
        rc = self._L.dbsrg_mchf_core(self._h, int(iorb), A.shape[1] - 1, ptr(A), ptr(B), ptr(Q),
                                     ptr(H), int(newton), ptr(hfm), ptr(hx))
        check(self._h, rc, "mchf_core")
        return hfm, hx

    def set_wait_limit(self, ns: int):
        """Limit of the tensor-core kernel's pipeline waits (ns)."""
        check(self._h, self._L.dbsrg_set_wait_limit(self._h, int(ns)), "set_wait_limit")

    def inject_wait_timeout(self, enable: bool = True):
        """Test switch: the tensor-core kernel's epilogue waits on a barrier
        nothing completes, so the call must end in DBSRG_ETIMEOUT."""
        check(self._h, self._L.dbsrg_inject_wait_timeout(self._h, int(enable)),
              "inject_wait_timeout")

    def set_tuning(self, name: str, value: int):
        """dbsrg_set_tuning: "xchunk", "dchunk" or "windows"."""
        check(self._h, self._L.dbsrg_set_tuning(self._h, name.encode(), int(value)),
              f"set_tuning({name})")

    def get_tuning(self, name: str) -> int:
        v = C.c_int(0)
        check(self._h, self._L.dbsrg_get_tuning(self._h, name.encode(), C.byref(v)),
              f"get_tuning({name})")
        return int(v.value)

    def set_async(self, enable: bool = True):
        """Asynchronous mode: gen() returns once the list's kernels are
        queued, so the set-up of the next list overlaps them; failures surface
        at the next sync() or read-out."""
        check(self._h, self._L.dbsrg_set_async(self._h, int(enable)), "set_async")


def _list_descs(lists_per_assembler):
    descs, keep, counts = [], [], []
    for lists in lists_per_assembler:
        counts.append(len(lists))
        for item in lists:
            icase, itype, kpol, k1, k2, k3, k4, cd = item[:8]
            ipt = item[8] if len(item) > 8 else None
            ptrs = []
            for a, dt in ((ipt, np.int32), (k1, np.int32), (k2, np.int32), (k3, np.int32),
                          (k4, np.int32), (cd, np.float64)):
                p, kk = _ptr(a, dt)
                ptrs.append(p.value if p is not None else None)
                keep.append(kk)
            descs.append(_lib.ListDesc(icase, itype, kpol, int(len(k1)), *ptrs))
    arr = (_lib.ListDesc * max(1, len(descs)))(*descs)
    return arr, keep, counts


def _raise_batch(L, assemblers, rc, what):
    for a in assemblers:
        msg = L.dbsrg_last_error(a._h).decode()
        if msg:
            check(a._h, rc, what)
    check(None, rc, what)


def gen_batch(assemblers, lists_per_assembler):
    """dbsrg_gen_batch: every assembler's lists (icase, itype, kpol, k1, k2, k3,
    k4, cdata[, ipt]) through Gen_matrix, the assemblers concurrently."""
    L = load()
    arr, keep, counts = _list_descs(lists_per_assembler)
    n = len(assemblers)
    ctxs = (C.c_void_p * max(1, n))(*[a._h.value for a in assemblers])
    cnt = (C.c_int * max(1, n))(*counts)
    rc = L.dbsrg_gen_batch(n, ctxs, cnt, arr)
    if rc != 0:
        for a in assemblers:
            msg = L.dbsrg_last_error(a._h).decode()
            if msg:
                check(a._h, rc, "gen_batch")
        check(None, rc, "gen_batch")


class HostMatrix:
    """dbsrg_host_alloc: n float64 values of page-locked host memory in huge
    pages, zeroed, for a matrix the device writes (the `out` of
    Assembler.assemble_to_host, the `stage` of assemble_streamed).  `array`
    is the numpy view; the memory is returned by close() or when the object
    is collected, so keep the object while the array is in use."""

    def __init__(self, n: int):
        self._L = load()
        self.nbytes = int(n) * 8
        p = C.c_void_p()
        check(None, self._L.dbsrg_host_alloc(C.c_size_t(self.nbytes), C.byref(p)), "host_alloc")
        self._p = p
        buf = (C.c_char * self.nbytes).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=np.float64, count=int(n))

    def close(self):
        if self._p is not None:
            self.array = None
            self._L.dbsrg_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gen_batch_streamed(assemblers, lists_per_assembler, consumer):
    """dbsrg_gen_batch_streamed: the assemblers (each allocated with a block
    window) run their lists once per window, concurrently; after every window
    consumer(i, blo, nblocks, device_ptr) is called for assembler i (from the
    assembler's host thread, one call at a time) and may read the window, e.g.
    with assemblers[i].get_matrix(out=...).  An exception in the consumer is
    raised once the batch returns."""
    L = load()
    arr, keep, counts = _list_descs(lists_per_assembler)
    n = len(assemblers)
    ctxs = (C.c_void_p * max(1, n))(*[a._h.value for a in assemblers])
    cnt = (C.c_int * max(1, n))(*counts)
    errors = []

    def fn(user, ictx, blo, nblocks, ptr):
        if errors:
            return
        try:
            consumer(int(ictx), int(blo), int(nblocks), int(ptr or 0))
        except BaseException as e:  # surfaces after the batch
            errors.append(e)

    cb = _lib.WindowFn(fn)
    rc = L.dbsrg_gen_batch_streamed(n, ctxs, cnt, arr, C.cast(cb, C.c_void_p), None)
    if errors:
        raise errors[0]
    if rc != 0:
        _raise_batch(L, assemblers, rc, "gen_batch_streamed")


class Lists:
    """The list producer between the decoded angular bank and Gen_matrix
    (dbsrg_lists_*): Add_integral, the Idef_* classification and the sorted,
    merged (kpol, itype) lists of Add_coef/Add_cdata (add_integral.f90,
    idef_type.f90, MOD_c_data.f90).  Host code; `gen_matrix(assembler)`
    hands every list the library assembles to the assembler."""

    def __init__(self, icase: int, ipbs, lbs=None, kbs=None, mk: int = 0, eps_c: float = 1e-10,
                 check_target: int = 1):
        self._L = load()
        self.icase = icase
        self._keep = [np.ascontiguousarray(x, dtype=np.int32) if x is not None else None
                      for x in (ipbs, lbs, kbs)]
        ptrs = [x.ctypes.data if x is not None else None for x in self._keep]
        h = C.c_void_p()
        rc = self._L.dbsrg_lists_create(C.byref(h), int(icase), int(self._keep[0].size), *ptrs,
                                        int(mk), float(eps_c), int(check_target))
        check(None, rc, "lists_create")
        self._h = h

    def add(self, kpol, i1, i2, i3, i4, c, ic=None, jc=None, io=None, jo=None):
        """Add_integral for arrays of decoded coefficients."""
        n = int(np.asarray(c).size)
        z = np.zeros(n, dtype=np.int32)
        arrs = [np.ascontiguousarray(x, dtype=np.int32) for x in (kpol, i1, i2, i3, i4)]
        cc = np.ascontiguousarray(c, dtype=np.float64)
        rest = [np.ascontiguousarray(x if x is not None else z, dtype=np.int32)
                for x in (ic, jc, io, jo)]
        ptrs = [a.ctypes.data for a in arrs] + [cc.ctypes.data] + [a.ctypes.data for a in rest]
        check(None, self._L.dbsrg_lists_add(self._h, n, *ptrs), "lists_add")

    def get(self, kpol: int, itype: int):
        """(k1, k2, k3, k4, cdata) of the merged list, in (K1,K2,K3,K4) order."""
        n = self._L.dbsrg_lists_count(self._h, int(kpol), int(itype))
        check(None, min(n, 0), "lists_count")
        out = [np.zeros(n, dtype=np.int32) for _ in range(4)] + [np.zeros(n)]
        check(None, self._L.dbsrg_lists_get(self._h, int(kpol), int(itype),
                                            *[o.ctypes.data for o in out]), "lists_get")
        return tuple(out)

    def gen_matrix(self, assembler: "Assembler"):
        check(assembler._h, self._L.dbsrg_lists_gen_matrix(self._h, assembler._h),
              "lists_gen_matrix")

    @staticmethod
    def decode(code):
        """(jcase, kpol, i1, i2, i3, i4) of bank integral codes."""
        code = np.ascontiguousarray(code, dtype=np.int32)
        out = [np.zeros(code.size, dtype=np.int32) for _ in range(6)]
        check(None, load().dbsrg_lists_decode(code.size, code.ctypes.data,
                                               *[o.ctypes.data for o in out]), "lists_decode")
        return tuple(out)

    def close(self):
        if getattr(self, "_h", None):
            self._L.dbsrg_lists_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
