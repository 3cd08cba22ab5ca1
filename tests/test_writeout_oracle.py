"""The oracle's write-out restatements on the CPU: the generalised
eigenproblem (Cholesky + cyclic Jacobi in place of LAPACK DSYGV) against
scipy's LAPACK, Diag_channels' selection, restoration and sign rule, the
record transformation against numpy, and the record layout of the writer."""
import struct

import numpy as np
import pytest

from oracle import oracle as O
from oracle import records as R


def test_sygv_matches_lapack():
    sl = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(7)
    for n in (1, 2, 17, 64):
        X = rng.standard_normal((n, n))
        A = X + X.T
        Y = rng.standard_normal((n, n))
        B = Y @ Y.T + n * np.eye(n)
        w, x = O.sygv(np.tril(A), np.tril(B))  # the lower triangles only
        wr, xr = sl.eigh(A, B)
        assert np.abs(w - wr).max() <= 1e-12 * np.abs(wr).max()
        sg = np.sign((x * xr).sum(0))
        assert np.abs(x - xr * sg).max() <= 1e-10 * np.abs(xr).max()
        assert np.abs(x.T @ B @ x - np.eye(n)).max() <= 1e-12


def test_sygv_rejects_indefinite_overlap():
    with pytest.raises(RuntimeError):
        O.sygv(np.eye(3), np.diag([1.0, -1.0, 1.0]))


def test_diag_channels_selection_and_sign():
    from dbsr_gb300 import synth

    w = synth.small(ns=24, nch=3, mk=1, n_entries=40, breit=False, seed=4)
    g = O.Grid(w.t, w.ks, w.ksp, w.ksq)
    m = O.Matrix(g, w.pq, w.ipbs, w.nch, w.icc, w.mk)
    ms = g.ms
    rng = np.random.default_rng(9)
    B = np.array(g.array("fppqq")).reshape(ms, ms, order="F")
    bdiag = np.asfortranarray(np.repeat(B[:, :, None], w.nch, axis=2))
    for ich in range(1, w.nch + 1):
        X = rng.standard_normal((ms, ms))
        m.hch[:, :, w.icc[ich - 1, ich - 1] - 1] = X + X.T
    ns = g.ns
    iprm = np.ones((ms, w.nch), dtype=np.int32, order="F")
    for comp in range(2):  # zero conditions: first and last B-spline of P and Q
        iprm[comp * ns, :] = 0
        iprm[comp * ns + ns - 1, :] = 0
    iprm[ns + 1, 2] = 0
    # a window inside the spectrum of channel 1 that cuts both ends and
    # some eigenvalues near zero
    keep = np.flatnonzero(iprm[:, 0])
    H1 = m.hch[:, :, w.icc[0, 0] - 1]
    w1, _ = O.sygv(np.tril(H1[np.ix_(keep, keep)]), np.tril(B[np.ix_(keep, keep)]))
    emin, emax = np.quantile(w1, 0.2), np.quantile(w1, 0.8)
    egap = np.sort(np.abs(w1))[3]
    sol, ev, nsol = m.diag_channels(bdiag, iprm, emin, emax, egap)
    for ich in range(w.nch):
        keep = np.flatnonzero(iprm[:, ich])
        H = m.hch[:, :, w.icc[ich, ich] - 1]
        wall, _ = O.sygv(np.tril(H[np.ix_(keep, keep)]), np.tril(B[np.ix_(keep, keep)]))
        sel = wall[(wall >= emin) & (wall <= emax) & (np.abs(wall) >= egap)]
        n = nsol[ich]
        assert n == sel.size and n > 0
        assert np.array_equal(ev[:n, ich], sel)
        for s in range(n):
            v = sol[:, s, ich]
            assert not v[iprm[:, ich] == 0].any()
            assert v[np.argmax(np.abs(v))] > 0
            r = H @ v - ev[s, ich] * (B * np.outer(iprm[:, ich], iprm[:, ich])) @ v
            assert np.abs(r[keep]).max() <= 1e-9 * np.abs(H).max()


def test_record_block_and_layout():
    rng = np.random.default_rng(2)
    h = rng.standard_normal((12, 12))
    di, dj = rng.standard_normal((12, 5)), rng.standard_normal((12, 3))
    c = O.record_block(h, di, dj)
    assert np.abs(c - di.T @ h @ dj).max() <= 1e-13 * np.abs(c).max()
    assert O.record_block(h, di[:, :0], dj).shape == (0, 3)
    icc = np.array([[1, 2], [2, 3]], dtype=np.int32)
    hch = np.asfortranarray(rng.standard_normal((12, 12, 3)))
    sol = np.zeros((12, 12, 2), order="F")
    sol[:, :4, 0] = rng.standard_normal((12, 4))
    sol[:, :2, 1] = rng.standard_normal((12, 2))
    body, ov = R.record_matrix(hch, icc, sol, [4, 2], icase=0)
    recs = R.read_records(body)
    assert [len(r) for r in recs] == [8, 4 * 2 * 8, 8]
    assert struct.unpack("=ii", recs[0]) == (2, 1) and struct.unpack("=ii", recs[2]) == (0, 0)
    # block (2,1): nsol(2) x nsol(1) = 2 x 4
    c21 = np.frombuffer(recs[1]).reshape(2, 4, order="F")
    ref = sol[:, :2, 1].T @ hch[:, :, 1] @ sol[:, :4, 0]
    assert np.abs(c21 - ref).max() <= 1e-12 * np.abs(c21).max()
    assert ov[1, 0] == np.abs(c21).max()
    hdr = R.header(6, 2, 0, 6, 6, sol, np.ones((12, 2)), [4, 2])
    h = R.read_records(hdr)
    assert struct.unpack("=5i", h[0]) == (6, 2, 0, 6, 6) and struct.unpack("=i", h[1]) == (6,)
    assert struct.unpack("=3i", h[2]) == (0, 4, 6) and len(h[4]) == 12 * 6 * 8
    with pytest.raises(ValueError):
        R.read_records(hdr[:-1] + b"\x01")
