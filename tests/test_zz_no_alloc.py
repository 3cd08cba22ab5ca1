"""The allocation-free exchange entry point against the regular one.

dbsrg_exchange_segment_noalloc serves callers that cannot allocate device
memory (MPI ranks sharing one GPU under a memory split fixed at start-up,
programs whose device memory is reserved up front by their own pool): its
scratch is a static device array instead of a
cudaMalloc'd buffer.  Here the test (not the entry point) allocates the
inputs and the output, calls the new entry point twice in a row through the
C ABI and compares each result with the block that Gen_matrix
(dbsrg_gen_matrix) adds for the same segment.

For a channel pair with ich > jch, UPDATE_HS adds the exchange result of
PQ type 0 (P-P table, P components) unchanged into quadrant (1,1) and that
of PQ type 1 (Q-Q) into quadrant (2,2); those quadrants are the reference
values.  Tolerance: 1e-12 of the largest element, the plain-FP64 bar of
the other GPU tests.  This file sorts last so a stop-at-first-failure run
has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from dbsr_gb300 import RK, Assembler, _lib, synth

pytestmark = pytest.mark.gpu


def _segment_case():
    for seed in range(11, 60):
        w = synth.small(ns=60, nch=2, mk=3, n_entries=400, breit=False, seed=seed)
        for L in w.lists:
            if L.icase == 2 and L.itype == 4:
                sel = L.k1 == 2 * synth.IBO + 1
                if sel.sum() >= 2:
                    return w, L, sel
    raise RuntimeError("no exchange segment for channel pair (2,1)")


def test_noalloc_exchange_matches_gen_matrix_twice():
    import torch

    w, L, sel = _segment_case()
    k1, k2, k3, k4, c = (np.ascontiguousarray(x[sel]) for x in (L.k1, L.k2, L.k3, L.k4, L.c))
    ns, ks = w.ns, w.ks

    # the existing entry point
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.gen_matrix(2, 4, L.kpol, k1, k2, k3, k4, c)
    blk = a.get_block(2, 1)
    ref = {0: blk[:ns, :ns].copy(), 1: blk[ns:, ns:].copy()}
    tables = {t: a.get_table(RK, t, L.kpol) for t in (0, 1)}
    a.close()

    dev = torch.device("cuda", 0)
    pq = torch.from_numpy(np.asfortranarray(w.pq).ravel(order="F").copy()).to(dev)
    dk2 = torch.from_numpy(k2.astype(np.int32)).to(dev)
    dk3 = torch.from_numpy(k3.astype(np.int32)).to(dev)
    dc = torch.from_numpy(c.astype(np.float64)).to(dev)
    L_ = _lib.load()
    for atype in (0, 1):  # two calls in a row on the shared static scratch
        rkb = torch.from_numpy(tables[atype].ravel(order="F").copy()).to(dev)
        out = torch.full((ns * ns,), float("nan"), dtype=torch.float64, device=dev)
        jp = atype + 1
        rc = L_.dbsrg_exchange_segment_noalloc(
            ns, ks, ctypes.c_void_p(rkb.data_ptr()), ctypes.c_void_p(pq.data_ptr()), w.nbf, jp,
            jp, int(k2.size), ctypes.c_void_p(dk2.data_ptr()), ctypes.c_void_p(dk3.data_ptr()),
            ctypes.c_void_p(dc.data_ptr()), ctypes.c_void_p(out.data_ptr()), None)
        assert rc == 0, rc
        got = out.cpu().numpy().reshape((ns, ns), order="F")
        r = ref[atype]
        assert np.abs(r).max() > 0
        err = np.abs(got - r).max() / np.abs(r).max()
        assert err <= 1e-12, (atype, err)


def _noalloc(ns, ks, rkb, pq, nbf, jp, k2, k3, c):
    """One call of the entry point on device copies of the arguments."""
    import torch

    L_ = _lib.load()
    dev = torch.device("cuda", 0)
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(dev)  # noqa: E731
    drkb = t(np.asarray(rkb).ravel(order="F"), np.float64)
    dpq = t(np.asarray(pq).ravel(order="F"), np.float64)
    dk2, dk3, dc = t(k2, np.int32), t(k3, np.int32), t(c, np.float64)
    out = torch.full((ns * ns,), float("nan"), dtype=torch.float64, device=dev)
    p = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
    rc = L_.dbsrg_exchange_segment_noalloc(ns, ks, p(drkb), p(dpq), nbf, jp, jp, len(k2), p(dk2),
                                           p(dk3), p(dc), p(out), None)
    return rc, out.cpu().numpy().reshape((ns, ns), order="F")


@pytest.mark.parametrize("ns", [60, 512])
def test_noalloc_exchange_matches_oracle_convol_case3(ns):
    """Against the oracle's convol case 3 ('s','s'; dbsr_lib_dbs.f90:2344-
    2356) of the accumulated 'x' density, on a seeded table and orbitals;
    ns = 512 fills the whole static scratch.  1e-12 of the largest element."""
    from oracle import oracle as O

    ks, nbf = 9, 3
    rng = np.random.default_rng(ns)
    rkb = np.asfortranarray(rng.uniform(-1.0, 1.0, (ns, ns, ks, ks)))
    pq = np.asfortranarray(rng.uniform(-1.0, 1.0, (ns, 2, nbf)))
    k2 = np.array([1, 2, 3, 1], np.int32)
    k3 = np.array([2, 2, 1, 3], np.int32)
    c = rng.uniform(-1.0, 1.0, 4)
    for _ in range(2):  # two calls in a row on the shared static scratch
        rc, got = _noalloc(ns, ks, rkb, pq, nbf, 1, k2, k3, c)
        assert rc == 0, rc
        xx = np.zeros((ns, ns), order="F")
        for a, b, ce in zip(k2, k3, c):
            xx += ce * np.outer(pq[:, 0, a - 1], pq[:, 0, b - 1])
        ref = O.convol(ns, ks, rkb, xx, 3, "s", "s")
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_noalloc_orbital_out_of_range_is_erange():
    ns, ks = 20, 9
    rkb = np.zeros((ns, ns, ks, ks), order="F")
    pq = np.zeros((ns, 2, 2), order="F")
    rc, _ = _noalloc(ns, ks, rkb, pq, 2, 1, np.array([1, 3], np.int32),
                     np.array([1, 1], np.int32), np.array([1.0, 1.0]))
    assert rc == -4  # DBSRG_ERANGE
    # the next call with valid indices succeeds (the error word is cleared)
    rc, _ = _noalloc(ns, ks, rkb, pq, 2, 1, np.array([1], np.int32), np.array([2], np.int32),
                     np.array([1.0]))
    assert rc == 0


def test_noalloc_rejects_sizes_beyond_its_scratch():
    L_ = _lib.load()
    one = ctypes.c_void_p(1)
    rc = L_.dbsrg_exchange_segment_noalloc(600, 9, one, one, 1, 1, 1, 0, None, None, None, one,
                                           None)
    assert rc == -4  # DBSRG_ERANGE
