"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle is a C restatement of the reference's DBSR_MAT3 assembly path
(dbsr_oracle.c).  Only tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module; the product library
never does.  ``build()`` compiles the C file into ``oracle/_build``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
IBO = 32768

_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class _Grid(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("ns", "ks", "ksp", "ksq", "nv", "nsp", "nsq", "ms")] + [
        (n, _dp)
        for n in (
            "t", "tp", "tq", "gx", "gw", "gr", "grw", "grm", "pbsp", "pbsd", "qbsp", "qbsd",
            "fpbs", "fqbs", "fpqbs", "fqpbs", "fpqbsd", "fqpbsd", "fppqq",
        )
    ]


def build(force: bool = False) -> str:
    """Compile the oracle shared library (make in oracle/)."""
    src = os.path.join(HERE, "dbsr_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_grid_new.restype = C.POINTER(_Grid)
        L.orc_grid_new.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp]
        L.orc_grid_free.argtypes = [C.POINTER(_Grid)]
        L.orc_gauleg.argtypes = [C.c_double, C.c_double, _dp, _dp, C.c_int]
        L.orc_mkgrid_01.restype = C.c_int
        L.orc_mkgrid_01.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                    C.c_double, C.c_double, _dp, C.c_int]
        L.orc_moments.argtypes = [C.POINTER(_Grid), C.c_int, C.c_int, _dp]
        L.orc_triang.argtypes = [C.POINTER(_Grid), C.c_int, C.c_int, _dp]
        L.orc_mrk.argtypes = [C.POINTER(_Grid), C.c_int, C.c_int, _dp]
        L.orc_msk.argtypes = [C.POINTER(_Grid), C.c_int, C.c_int, _dp]
        L.orc_density.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, C.c_char]
        L.orc_dbs_orth.argtypes = [C.c_void_p, _ip]
        L.orc_hf_matrix.argtypes = [C.POINTER(_Grid), C.c_int, _dp, C.c_int, C.c_int, _dp, _dp,
                                    C.c_double, _dp, _dp]
        L.orc_hf_matrix_breit.argtypes = [C.POINTER(_Grid), C.c_int, _dp, C.c_int, C.c_int,
                                          C.c_int, _ip, _ip, _ip, _ip, _dp, _dp]
        L.orc_convol.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, C.c_int, C.c_char, C.c_char]
        L.orc_sum_amb.restype = C.c_double
        L.orc_sum_amb.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_char]
        L.orc_quadr.restype = C.c_double
        L.orc_quadr.argtypes = [C.POINTER(_Grid), _dp, _dp, C.c_int]
        L.orc_rk.restype = C.c_double
        L.orc_rk.argtypes = [C.POINTER(_Grid), _dp, _dp, _dp, _dp, C.c_int]
        L.orc_rk_energy_grad.restype = C.c_double
        L.orc_rk_energy_grad.argtypes = [C.POINTER(_Grid), C.c_int, _ip, _ip, _ip, _ip, _ip, _dp,
                                         _dp, C.c_int, _dp]
        L.orc_mat_new.restype = C.c_void_p
        L.orc_mat_new.argtypes = [C.POINTER(_Grid), C.c_int, _dp, _ip, C.c_int, _ip, C.c_int,
                                  _dp, C.c_int, _dp]
        L.orc_mat_free.argtypes = [C.c_void_p]
        L.orc_gen_matrix.restype = C.c_int
        L.orc_gen_matrix.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                     _ip, _ip, _ip, _ip, _ip, _dp]
        L.orc_v_ch.argtypes = [C.POINTER(_Grid), _dp, _dp]
        L.orc_mat_set_perturbers.argtypes = [C.c_void_p, C.c_int, _ip, C.c_int, _ip, C.c_int,
                                             _dp, _dp]
        L.orc_mat_set_targets.argtypes = [C.c_void_p, C.c_int, _ip, _dp, _dp, C.c_int, C.c_int]
        L.orc_mat_set_dhl.argtypes = [C.c_void_p, C.c_int, _ip, _dp, _ip]
        L.orc_mat_set_eps_c.argtypes = [C.c_void_p, C.c_double]
        L.orc_bav.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, C.c_char, C.c_char]
        L.orc_update_hw.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, C.c_double]
        L.orc_update_hv.restype = C.c_int
        L.orc_update_hv.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, C.c_double]
        L.orc_update_hb.restype = C.c_int
        L.orc_update_hb.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double]
        L.orc_sort_merge.restype = C.c_int
        L.orc_sort_merge.argtypes = [C.c_int, _ip, _ip, _ip, _ip, _dp, _ip, _ip, _ip, _ip, _dp]
        L.orc_sygv.restype = C.c_int
        L.orc_sygv.argtypes = [C.c_int, _dp, _dp, C.c_int, _dp, _dp]
        L.orc_diag_channels.restype = C.c_int
        L.orc_diag_channels.argtypes = [C.c_void_p, _dp, _ip, C.c_double, C.c_double, C.c_double,
                                        _dp, _dp, _ip]
        L.orc_record_block.argtypes = [C.c_int, _dp, _dp, C.c_int, _dp, C.c_int, _dp]
        L.orc_mchf_matrix.argtypes = [C.POINTER(_Grid), C.c_int, _dp, C.c_int, C.c_int, C.c_int,
                                      _ip, _ip, _dp, C.c_int, _ip, _ip, _ip, _ip, _ip, _dp, _dp,
                                      C.c_int, C.c_int, C.c_double, _dp, _dp, _dp, _dp, _dp]
        L.orc_mchf_core.argtypes = [C.POINTER(_Grid), C.c_int, _dp, C.c_int, C.c_int, _dp, _dp,
                                    _dp, _dp, C.c_int, _dp, _dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def f64(a):
    """Fortran-ordered float64 copy/view (the oracle uses column-major)."""
    return np.asfortranarray(a, dtype=np.float64)


def i32(a):
    return np.asfortranarray(a, dtype=np.int32)


def gauleg(n: int, x1: float = 0.0, x2: float = 1.0):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().orc_gauleg(x1, x2, _d(x), _d(w), n)
    return x, w


def mkgrid_01(ks: int, ml: int, hs: float, he: float, hmax: float, rmax: float):
    """Knots of the semi-exponential grid (mkgrid_01); returns (ns, t)."""
    buf = np.zeros(100000)
    ns = lib().orc_mkgrid_01(ks, ml, hs, 0.0, he, hmax, rmax, _d(buf), buf.size)
    if ns < 0:
        raise ValueError("grid too large")
    return ns, buf[: ns + ks].copy()


class Grid:
    """B-spline grid (alloc_DBS_gauss + Def_pbsp/qbsp + Def_pq_arrays)."""

    def __init__(self, t, ks: int = 9, ksp: int = 8, ksq: int = 9):
        t = f64(t)
        self.ks = ks
        self.ns = t.size - ks
        self._t = t
        self._p = lib().orc_grid_new(self.ns, ks, ksp, ksq, _d(t))
        g = self._p.contents
        self.ksp, self.ksq, self.nv, self.nsp, self.nsq, self.ms = g.ksp, g.ksq, g.nv, g.nsp, g.nsq, g.ms

    def __del__(self):
        try:
            if getattr(self, "_p", None) is not None:
                lib().orc_grid_free(self._p)
                self._p = None
        except Exception:
            pass

    def array(self, name: str) -> np.ndarray:
        """Copy of a grid array in Fortran order with its reference shape."""
        g = self._p.contents
        ns, ks, nv, ms = self.ns, self.ks, self.nv, self.ms
        shapes = {
            "t": (ns + ks,), "tp": (self.nsp + self.ksp,), "tq": (self.nsq + self.ksq,),
            "gx": (ks,), "gw": (ks,), "gr": (nv, ks), "grw": (nv, ks), "grm": (nv, ks),
            "pbsp": (nv + 1, ks, self.ksp), "pbsd": (nv + 1, ks, self.ksp),
            "qbsp": (nv + 1, ks, self.ksq), "qbsd": (nv + 1, ks, self.ksq),
            "fpbs": (ns, ns), "fqbs": (ns, ns), "fpqbs": (ns, ns), "fqpbs": (ns, ns),
            "fpqbsd": (ns, ns), "fqpbsd": (ns, ns), "fppqq": (ms, ms),
        }
        shp = shapes[name]
        n = int(np.prod(shp))
        flat = np.ctypeslib.as_array(getattr(g, name), shape=(n,)).copy()
        return flat.reshape(shp, order="F")

    # ---- level 1
    def moments(self, which: int, k: int) -> np.ndarray:
        kk = self.ks * self.ks
        out = np.zeros(kk * self.nv)
        lib().orc_moments(self._p, which, k, _d(out))
        return out.reshape((kk, self.nv), order="F")

    def triang(self, typ: int, k: int) -> np.ndarray:
        kk = self.ks * self.ks
        out = np.zeros(kk * kk * self.nv)
        lib().orc_triang(self._p, typ, k, _d(out))
        return out.reshape((kk, kk, self.nv), order="F")

    def mrk(self, typ: int, k: int) -> np.ndarray:
        out = np.zeros(self.ns * self.ns * self.ks * self.ks)
        lib().orc_mrk(self._p, typ, k, _d(out))
        return out.reshape((self.ns, self.ns, self.ks, self.ks), order="F")

    def msk(self, typ: int, k: int) -> np.ndarray:
        kb = 2 * self.ks - 1
        out = np.zeros(self.ns * self.ns * kb * kb)
        lib().orc_msk(self._p, typ, k, _d(out))
        return out.reshape((self.ns, self.ns, kb, kb), order="F")

    def quadr(self, fi, fj, m: int) -> float:
        return lib().orc_quadr(self._p, _d(f64(fi)), _d(f64(fj)), m)

    def rk(self, f1, f2, f3, f4, k: int) -> float:
        return lib().orc_rk(self._p, _d(f64(f1)), _d(f64(f2)), _d(f64(f3)), _d(f64(f4)), k)

    def rk_energy_grad(self, k, i1, i2, i3, i4, coef, pq, grad: bool = True):
        """(E, dE/dpq) of E = sum_e coef[e] R^k[e](i1,i2;i3,i4) (1-based orbitals)."""
        pq = f64(pq)
        nbf = pq.size // (2 * self.ns)
        ints = [np.ascontiguousarray(x, dtype=np.int32) for x in (k, i1, i2, i3, i4)]
        c = np.ascontiguousarray(coef, dtype=np.float64)
        g = np.zeros((self.ns, 2, nbf), order="F") if grad else None
        E = lib().orc_rk_energy_grad(self._p, len(c), *[x.ctypes.data_as(_ip) for x in ints],
                                     _d(c), _d(pq), nbf, _d(g) if grad else None)
        return E, g

    def hf_matrix(self, pq, iorb: int, a, b, qsum: float, dhl=None) -> np.ndarray:
        """hf_matrix (DBSR_HF/hf_matrix.f90:2-70, Coulomb part) of orbital
        iorb (1-based); a, b: (nbf, kmax+1) coefficient values."""
        pq = f64(pq)
        nbf = pq.size // (2 * self.ns)
        a, b = f64(a), f64(b)
        kmax = a.shape[1] - 1
        out = np.zeros((self.ms, self.ms), order="F")
        lib().orc_hf_matrix(self._p, nbf, _d(pq), iorb, kmax, _d(a), _d(b), float(qsum),
                            _d(f64(dhl)) if dhl is not None else None, _d(out))
        return out

    def mchf_matrix(self, pq, iorb: int, kmax: int, lint, rint, dhl, irhs=1, newton=0,
                    eps_c=1e-10):
        """mchf_matrix (DBSR_MCHF/mchf_matrix.f90:2-251) of orbital iorb outside
        the core.  lint = (i1, i2, c) one-electron entries, rint = (k, i1, i2,
        i3, i4, c) R^k entries, both with the expansion weights applied.
        Returns (hfm, rhs, hx, e, qsum)."""
        pq = f64(pq)
        nbf = pq.size // (2 * self.ns)
        li1, li2 = i32(lint[0]), i32(lint[1])
        lc = f64(lint[2])
        rk, r1, r2, r3, r4 = (i32(x) for x in rint[:5])
        rc = f64(rint[5])
        ms = self.ms
        hfm = np.zeros((ms, ms), order="F")
        hx = np.zeros((ms, ms), order="F")
        rhs = np.zeros(ms)
        e = np.zeros(1)
        q = np.zeros(1)
        lib().orc_mchf_matrix(self._p, nbf, _d(pq), iorb, kmax, li1.size, _i(li1), _i(li2),
                              _d(lc), rk.size, _i(rk), _i(r1), _i(r2), _i(r3), _i(r4), _d(rc),
                              _d(f64(dhl)), int(irhs), int(newton), float(eps_c), _d(hfm),
                              _d(rhs), _d(hx), _d(e), _d(q))
        return hfm, rhs, hx, float(e[0]), float(q[0])

    def mchf_core(self, pq, iorb: int, a, b, qsum, hd, newton=0):
        """core_matrix (DBSR_MCHF/mchf_matrix.f90:255-346); a, b: (nbf,
        kmax+1), qsum(nbf).  Returns (hfm, hx)."""
        pq = f64(pq)
        nbf = pq.size // (2 * self.ns)
        a, b = f64(a), f64(b)
        ms = self.ms
        hfm = np.zeros((ms, ms), order="F")
        hx = np.zeros((ms, ms), order="F")
        lib().orc_mchf_core(self._p, nbf, _d(pq), iorb, a.shape[1] - 1, _d(a), _d(b),
                            _d(f64(qsum)), _d(f64(hd)), int(newton), _d(hfm), _d(hx))
        return hfm, hx

    def hf_matrix_breit(self, pq, iorb: int, kmax: int, kr1, kr2, kr3, kr4, crk,
                        hfm=None) -> np.ndarray:
        """hf_matrix_breit (DBSR_HF/hf_matrix.f90:91-163) of orbital iorb added
        into hfm (a zero matrix when None)."""
        pq = f64(pq)
        nbf = pq.size // (2 * self.ns)
        out = np.zeros((self.ms, self.ms), order="F") if hfm is None else f64(hfm).copy(order="F")
        ints = [i32(x) for x in (kr1, kr2, kr3, kr4)]
        lib().orc_hf_matrix_breit(self._p, nbf, _d(pq), iorb, kmax, len(crk), *[_i(x) for x in ints],
                                  _d(f64(crk)), _d(out))
        return out

    def v_ch(self, pq_b) -> np.ndarray:
        v = np.zeros(self.ms)
        lib().orc_v_ch(self._p, _d(f64(pq_b)), _d(v))
        return v


def density(ns, ks, p1, p2, typ: str) -> np.ndarray:
    ncol = {"s": ks, "u": ks, "l": ks, "n": 2 * ks - 1}.get(typ, ns)
    d = np.zeros(ns * max(ncol, ns))
    lib().orc_density(ns, ks, _d(d), _d(f64(p1)), _d(f64(p2)), typ.encode())
    return d.reshape((ns, max(ncol, ns)), order="F")[:, :ncol].copy(order="F")


def convol(ns, ks, rkb, d, icase: int, sym_i: str, sym_j: str) -> np.ndarray:
    rkb = np.asfortranarray(rkb, dtype=np.float64)
    kb = rkb.shape[2]
    dd = np.zeros((ns, ns), order="F")
    dd[:, : d.shape[1]] = d
    a = np.zeros((ns, ns), order="F")
    lib().orc_convol(ns, ks, kb, rkb.ctypes.data_as(_dp), a.ctypes.data_as(_dp),
                     dd.ctypes.data_as(_dp), icase, sym_i.encode(), sym_j.encode())
    return a


def bav(ns, ks, a, b, sym: str, direction: str) -> np.ndarray:
    """BAV restatement: band matrix a ('s' (ns,ks) or 'n' (ns,2ks-1)) times
    vector b, v = A b ('r') or A^T b ('l')."""
    a = f64(a)
    v = np.zeros(ns)
    lib().orc_bav(ns, ks, _d(a), _d(f64(b)), _d(v), sym.encode(), direction.encode())
    return v


def sort_merge(k1, k2, k3, k4, c):
    """Add_cdata list semantics: sorted unique keys with summed coefficients."""
    k1, k2, k3, k4, c = i32(k1), i32(k2), i32(k3), i32(k4), f64(c)
    n = k1.size
    o = [np.zeros(max(n, 1), np.int32) for _ in range(4)]
    oc = np.zeros(max(n, 1))
    u = lib().orc_sort_merge(n, _i(k1), _i(k2), _i(k3), _i(k4), _d(c), _i(o[0]), _i(o[1]),
                             _i(o[2]), _i(o[3]), _d(oc))
    return o[0][:u].copy(), o[1][:u].copy(), o[2][:u].copy(), o[3][:u].copy(), oc[:u].copy()


class Matrix:
    """hch/acf state plus Gen_matrix dispatch (DBSR_MAT3)."""

    def __init__(self, grid: Grid, pq, ipbs, nch: int, icc, mk: int):
        self.grid = grid
        self.pq = np.asfortranarray(pq, dtype=np.float64)  # (ns,2,nbf)
        self.ipbs = i32(ipbs)
        self.nch = nch
        self.icc = np.asfortranarray(icc, dtype=np.int32)
        self.iicc = int(self.icc.max())
        ms = grid.ms
        self.hch = np.zeros((ms, ms, self.iicc), order="F")
        self.mk = mk
        self.acf = np.zeros((self.iicc, mk + 1), order="F")
        self._m = lib().orc_mat_new(
            grid._p, self.pq.shape[2], self.pq.ctypes.data_as(_dp), _i(self.ipbs), nch,
            self.icc.ctypes.data_as(_ip), self.iicc, self.hch.ctypes.data_as(_dp), mk,
            self.acf.ctypes.data_as(_dp))

    def __del__(self):
        try:
            if getattr(self, "_m", None):
                lib().orc_mat_free(self._m)
                self._m = None
        except Exception:
            pass

    def set_perturbers(self, npert: int, icb, ibb):
        """hcp(ms,iicb) and hp(iibb) with icb(nch,npert), ibb(npert,npert)."""
        self.icb = np.asfortranarray(icb, dtype=np.int32)
        self.ibb = np.asfortranarray(ibb, dtype=np.int32)
        iicb, iibb = int(self.icb.max(initial=0)), int(self.ibb.max(initial=0))
        self.hcp = np.zeros((self.grid.ms, max(iicb, 1)), order="F")
        self.hp = np.zeros(max(iibb, 1))
        lib().orc_mat_set_perturbers(self._m, npert, _i(self.icb), iicb, _i(self.ibb), iibb,
                                     _d(self.hcp), _d(self.hp))

    def set_targets(self, ntarg: int, iptar, iitar: int = 0, check_target: int = 1):
        self.iptar = i32(iptar)
        n = ntarg * (ntarg + 1) // 2
        self.htarg = np.zeros(max(n, 1))
        self.otarg = np.zeros(max(n, 1))
        lib().orc_mat_set_targets(self._m, ntarg, _i(self.iptar), _d(self.htarg),
                                  _d(self.otarg), iitar, check_target)

    def set_dhl(self, kap_list, hd, kbs):
        """hd(ms,ms,nkap) one-electron matrices of the kappas in kap_list;
        kbs(nbf) the kappa of every orbital."""
        self.kap_list = i32(kap_list)
        self.hd = f64(hd)
        self.kbs = i32(kbs)
        lib().orc_mat_set_dhl(self._m, self.kap_list.size, _i(self.kap_list), _d(self.hd),
                              _i(self.kbs))

    def set_eps_c(self, eps_c: float):
        lib().orc_mat_set_eps_c(self._m, float(eps_c))

    def diag_channels(self, bdiag, iprm, emin: float, emax: float, egap: float):
        """Diag_channels (diag.f90:2-81) on the diagonal blocks of hch:
        bdiag(ms, ms, nch) overlap blocks, iprm(ms, nch) kept B-splines.
        Returns sol(ms, ms, nch), eval(ms, nch), nsol(nch)."""
        ms, nch = self.grid.ms, self.nch
        bd, ip = f64(bdiag), np.asfortranarray(iprm, dtype=np.int32)
        sol = np.zeros((ms, ms, nch), order="F")
        ev = np.zeros((ms, nch), order="F")
        ns_ = np.zeros(nch, dtype=np.int32)
        rc = lib().orc_diag_channels(self._m, _d(bd), _i(ip), float(emin), float(emax),
                                     float(egap), _d(sol), _d(ev), _i(ns_))
        if rc != 0:
            raise RuntimeError(f"channel diagonalization failed (channel {-rc})")
        return sol, ev, ns_

    def dbs_orth(self, iort):
        """DBS_ORTH (dbs_orth.f90:28-84) on hch in place; iort(nbf, nch)."""
        io = np.asfortranarray(iort, dtype=np.int32)
        lib().orc_dbs_orth(self._m, io.ctypes.data_as(_ip))

    def gen_matrix(self, icase, itype, kpol, k1, k2, k3, k4, cdata, ipt=None):
        k1, k2, k3, k4, cdata = i32(k1), i32(k2), i32(k3), i32(k4), f64(cdata)
        n = k1.size
        ipt = i32(np.arange(1, n + 1) if ipt is None else ipt)
        rc = lib().orc_gen_matrix(self._m, icase, itype, kpol, n, _i(ipt), _i(k1), _i(k2),
                                  _i(k3), _i(k4), _d(cdata))
        if rc != 0:
            raise RuntimeError(f"orc_gen_matrix failed: {rc}")


def sygv(a, b):
    """A x = E B x from the lower triangles (restated DSYGV itype 1):
    eigenvalues ascending, eigenvectors with x^T B x = 1."""
    a, b = f64(a), f64(b)
    n = a.shape[0]
    w = np.zeros(n)
    x = np.zeros((n, n), order="F")
    if lib().orc_sygv(n, _d(a), _d(b), n, _d(w), _d(x)) != 0:
        raise RuntimeError("overlap matrix not positive definite")
    return w, x


def record_block(h, di, dj):
    """Record_matrix's c = D_i^T H D_j (record_matrix.f90:21-24)."""
    h, di, dj = f64(h), f64(di), f64(dj)
    ms, ni, nj = h.shape[0], di.shape[1], dj.shape[1]
    c = np.zeros((ni, nj), order="F")
    if ni and nj:
        lib().orc_record_block(ms, _d(h), _d(di), ni, _d(dj), nj, _d(c))
    return c
