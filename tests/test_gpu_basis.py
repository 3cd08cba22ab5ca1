"""The channel basis of the write-out (dbsrg_diag_channels,
dbsrg_channel_basis) against a numpy/scipy restatement of Diag_channels
(diag.f90:2-81: DSYGV on the B-splines the zero conditions keep, the energy
window, the largest component made positive) and of the block
transformation of Record_matrix (record_matrix.f90:14-26:
c = D_ich^T H D_jch)."""
import numpy as np
import pytest

from dbsr_gb300 import SPLIT_BF16, Assembler, synth

pytestmark = pytest.mark.gpu


def oracle_solutions(Hk, B, keep, emin, emax, egap):
    import scipy.linalg as sl

    idx = np.flatnonzero(keep)
    A = Hk[np.ix_(idx, idx)]
    A = np.tril(A) + np.tril(A, -1).T  # DSYGV 'L': the lower triangle
    Bc = B[np.ix_(idx, idx)]
    Bc = np.tril(Bc) + np.tril(Bc, -1).T
    w, V = sl.eigh(A, Bc)
    sel = [i for i in range(len(w)) if emin <= w[i] <= emax and abs(w[i]) >= egap]
    D = np.zeros((Hk.shape[0], len(sel)))
    for s, i in enumerate(sel):
        v = np.zeros(Hk.shape[0])
        v[idx] = V[:, i]
        if v[np.argmax(np.abs(v))] < 0:
            v = -v
        D[:, s] = v
    return w[sel], D, w


def test_channel_basis_against_scipy():
    pytest.importorskip("scipy")
    w = synth.small(ns=40, nch=4, mk=2, n_entries=500, breit=True, seed=91)
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.set_precision(SPLIT_BF16)
    for L in w.lists:
        a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    ms, ns = a.ms, a.ns
    rng = np.random.default_rng(3)
    for ich in range(1, w.nch + 1):  # a generic symmetric part on every channel
        X = rng.standard_normal((ms, ms))
        a.update_hx(ich, ich, np.asfortranarray(0.5 * (X + X.T)), 1.0)
    H = a.get_matrix()
    B = a.grid_array("fppqq").reshape(ms, ms, order="F")
    bdiag = np.asfortranarray(np.repeat(B[:, :, None], w.nch, axis=2))
    iprm = np.ones((ms, w.nch), dtype=np.int32, order="F")
    for comp in range(2):  # zero conditions: first and last B-spline of P and Q
        iprm[comp * ns, :] = 0
        iprm[comp * ns + ns - 1, :] = 0
    iprm[comp * ns + 1, 1] = 0  # one more on channel 2
    emin, emax, egap = -40.0, 60.0, 0.05
    sol, ev, nsol = a.diag_channels(bdiag, iprm, emin, emax, egap)
    D = []
    for ich in range(1, w.nch + 1):
        k = w.icc[ich - 1, ich - 1]
        e, Dr, wall = oracle_solutions(H[:, :, k - 1], B, iprm[:, ich - 1], emin, emax, egap)
        assert 0 < nsol[ich - 1] == len(e) < len(wall)
        scale = np.abs(wall).max()
        assert np.abs(ev[: len(e), ich - 1] - e).max() <= 1e-10 * scale
        assert not ev[len(e):, ich - 1].any()
        assert np.abs(sol[:, : len(e), ich - 1] - Dr).max() <= 1e-8
        assert not sol[:, len(e):, ich - 1].any()
        D.append(Dr)
    out = a.channel_basis(sol, nsol, out=True)
    for ich in range(1, w.nch + 1):
        for jch in range(1, w.nch + 1):
            k = w.icc[ich - 1, jch - 1]
            if k < 1:
                continue
            if ich == jch:
                assert np.array_equal(out[:, :, k - 1], H[:, :, k - 1])
            elif ich > jch:
                ref = D[ich - 1].T @ H[:, :, k - 1] @ D[jch - 1]
                ni, nj = ref.shape
                got = out[:, :, k - 1]
                assert np.abs(got[:ni, :nj] - ref).max() <= 1e-9 * max(np.abs(ref).max(), 1.0)
                assert not got[ni:, :].any() and not got[:, nj:].any()
    a.close()
