"""Orthogonality of the channels to bound orbitals: DBS_ORTH
(DBSR_MAT3/dbs_orth.f90:2-84), H(ich,jch) -> (1 - aa_ich) H (1 - bb_jch).

CPU: the oracle's literal restatement (full ms x ms aa, bb and matmul loops)
against the same projection written with numpy.  GPU: dbsrg_orth_channels
(rank-|O| factors, both channels' updates in one pass per block) against
the oracle on an assembled matrix, per block within 1e-12 of the block's
largest element (the plain-FP64 bar)."""
import numpy as np
import pytest

from oracle import oracle as orc
from dbsr_gb300 import synth


def _iort_same_kappa(w):
    """The reference's selection: bound orbitals of the channel's kappa."""
    io = np.zeros((w.nbf, w.nch), dtype=np.int32, order="F")
    for ich, kc in enumerate(w.kappa_ch):
        for j in range(w.nbound):
            if w.ipbs[j] == 0 and w.kappa_bound[j] == kc:
                io[j, ich] = 1
    return io


def _numpy_orth(hch, icc, nch, pq, fpbs, fqbs, iort):
    ns = pq.shape[0]
    ms = 2 * ns
    aa = []
    for ich in range(nch):
        a = np.zeros((ms, ms))
        for j in np.flatnonzero(iort[:, ich]):
            v = np.concatenate([pq[:, 0, j], pq[:, 1, j]])
            wv = np.concatenate([fpbs @ pq[:, 0, j], fqbs @ pq[:, 1, j]])
            a += np.outer(wv, v)
        aa.append(a)
    out = hch.copy()
    eye = np.eye(ms)
    for ich in range(nch):
        for jch in range(ich + 1):
            b = icc[ich, jch]
            if b == 0:
                continue
            out[:, :, b - 1] = (eye - aa[ich]) @ hch[:, :, b - 1] @ (eye - aa[jch].T)
    return out


def _block_err(a, b):
    return max(np.abs(a[:, :, k] - b[:, :, k]).max() / max(np.abs(b[:, :, k]).max(), 1e-300)
               for k in range(b.shape[2]))


def test_oracle_dbs_orth_matches_projection():
    w = synth.small(ns=30, nch=3, mk=1, n_entries=50, breit=False, seed=17, norb=4)
    g = orc.Grid(w.t, w.ks, w.ksp, w.ksq)
    m = orc.Matrix(g, w.pq, w.ipbs, w.nch, w.icc, w.mk)
    rng = np.random.default_rng(5)
    m.hch[...] = rng.uniform(-1, 1, m.hch.shape)
    h0 = m.hch.copy()
    io = np.zeros((w.nbf, w.nch), dtype=np.int32, order="F")
    io[:w.nbound, :] = 1  # every bound orbital for every channel: both sides active
    io[0, 1] = 0
    m.dbs_orth(io)
    ref = _numpy_orth(h0, w.icc, w.nch, w.pq, g.array("fpbs"), g.array("fqbs"), io)
    assert _block_err(m.hch, ref) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["kappa", "all"])
def test_orth_channels_matches_oracle(mode):
    from dbsr_gb300 import PLAIN_FP64, Assembler

    w = synth.small(ns=48, nch=4, mk=2, n_entries=400, breit=True, seed=23, norb=6)
    io = _iort_same_kappa(w) if mode == "kappa" else np.asfortranarray(
        np.vstack([np.ones((w.nbound, w.nch), np.int32),
                   np.zeros((w.nbf - w.nbound, w.nch), np.int32)]))
    assert io.sum() > 0
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.set_precision(PLAIN_FP64)
    for L in w.lists:
        a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    h0 = a.get_matrix()
    a.orth_channels(io)
    got = a.get_matrix()
    a.close()
    g = orc.Grid(w.t, w.ks, w.ksp, w.ksq)
    m = orc.Matrix(g, w.pq, w.ipbs, w.nch, w.icc, w.mk)
    m.hch[...] = h0
    m.dbs_orth(io)
    err = _block_err(got, m.hch)
    assert err <= 1e-12, err
    assert _block_err(h0, m.hch) > 1e-6  # the projection changed the matrix


@pytest.mark.gpu
def test_orth_channels_refuses_channel_orbitals():
    from dbsr_gb300 import Assembler

    w = synth.small(ns=40, nch=2, mk=1, n_entries=50, breit=False, seed=3)
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    io = np.zeros((w.nbf, w.nch), dtype=np.int32, order="F")
    io[w.nbf - 1, 0] = 1  # a channel orbital (ipbs != 0)
    with pytest.raises(RuntimeError):
        a.orth_channels(io)
    a.close()
