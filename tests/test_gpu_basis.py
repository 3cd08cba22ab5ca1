"""The channel basis and the write-out on the GPU (dbsrg_diag_channels,
dbsrg_channel_basis, dbsrg_record_header/matrix/acf) against the oracle's
restatements: Diag_channels (diag.f90:2-81, the generalised problem by
Cholesky and cyclic Jacobi in place of LAPACK DSYGV), the block
transformation of Record_matrix (record_matrix.f90:14-26) and the records
of Record_matrix and SUB1 (record_matrix.f90:2-60, sub1.f90:164-168,
286-287), byte layout and all.

Tolerances: eigenvalues 1e-10 of the largest modulus; eigenvectors 1e-8
(a vector moves by about eps ||A|| / gap, and the generic test matrices
have gaps near 1e-3 of their scale); transformed blocks and records 1e-12
of each record's largest element when both sides use the same solutions
(1e-10 for the split form's tensor-core products).
"""
import os

import numpy as np
import pytest

from dbsr_gb300 import PLAIN_FP64, SPLIT_BF16, Assembler, synth
from oracle import oracle as O
from oracle import records as R

pytestmark = pytest.mark.gpu


def _assembler(w, precision):
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.set_precision(precision)
    return a


def _generic_diagonal(a, w, seed):
    """a generic symmetric part on every diagonal block (distinct eigenvalues)"""
    rng = np.random.default_rng(seed)
    for ich in range(1, w.nch + 1):
        X = rng.standard_normal((a.ms, a.ms))
        a.update_hx(ich, ich, np.asfortranarray(0.5 * (X + X.T)), 1.0)


def _zero_conditions(ms, ns, nch):
    iprm = np.ones((ms, nch), dtype=np.int32, order="F")
    for comp in range(2):  # first and last B-spline of P and Q
        iprm[comp * ns, :] = 0
        iprm[comp * ns + ns - 1, :] = 0
    iprm[ns + 1, 1 % nch] = 0  # one more on channel 2
    return iprm


def _oracle_matrix(w, H):
    g = O.Grid(w.t, w.ks, w.ksp, w.ksq)
    m = O.Matrix(g, w.pq, w.ipbs, w.nch, w.icc, w.mk)
    m.hch[...] = H
    return g, m


@pytest.mark.parametrize("precision,tol", [(PLAIN_FP64, 1e-12), (SPLIT_BF16, 1e-10)])
def test_channel_basis_against_oracle(precision, tol):
    """The plain form transforms the blocks with cuBLAS DGEMM (1e-12 of each
    block's largest element); the split form with the split-BF16 tcgen05
    products (1e-10)."""
    w = synth.small(ns=40, nch=4, mk=2, n_entries=500, breit=True, seed=91)
    a = _assembler(w, precision)
    for L in w.lists:
        a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    _generic_diagonal(a, w, 3)
    ms, ns = a.ms, a.ns
    H = a.get_matrix()
    B = a.grid_array("fppqq").reshape(ms, ms, order="F")
    bdiag = np.asfortranarray(np.repeat(B[:, :, None], w.nch, axis=2))
    iprm = _zero_conditions(ms, ns, w.nch)
    emin, emax, egap = -40.0, 60.0, 0.05
    sol, ev, nsol = a.diag_channels(bdiag, iprm, emin, emax, egap)
    _, m = _oracle_matrix(w, H)
    rsol, rev, rnsol = m.diag_channels(bdiag, iprm, emin, emax, egap)
    assert np.array_equal(nsol, rnsol)
    for ich in range(w.nch):
        n = int(nsol[ich])
        assert 0 < n < ms - 4
        scale = np.abs(rev[:n, ich]).max()
        assert np.abs(ev[:n, ich] - rev[:n, ich]).max() <= 1e-10 * scale
        assert not ev[n:, ich].any()
        assert np.abs(sol[:, :n, ich] - rsol[:, :n, ich]).max() <= 1e-8
        assert not sol[:, n:, ich].any()
    out = a.channel_basis(rsol, rnsol, out=True)  # the oracle's solutions on both sides
    for ich in range(1, w.nch + 1):
        for jch in range(1, w.nch + 1):
            k = w.icc[ich - 1, jch - 1]
            if k < 1:
                continue
            if ich == jch:
                assert np.array_equal(out[:, :, k - 1], H[:, :, k - 1])
            elif ich > jch:
                ni, nj = rnsol[ich - 1], rnsol[jch - 1]
                ref = O.record_block(H[:, :, k - 1], rsol[:, :ni, ich - 1], rsol[:, :nj, jch - 1])
                got = out[:, :, k - 1]
                assert np.abs(got[:ni, :nj] - ref).max() <= tol * max(np.abs(ref).max(), 1e-300)
                assert not got[ni:, :].any() and not got[:, nj:].any()
    a.close()


def test_write_out_against_oracle(tmp_path):
    """Header, overlap records (icase 0, with perturber rows and elements
    and the overlaps array) and Hamiltonian records plus the acf records of
    the structures workload (3 channels, 3 perturbers), written by the
    library and by the oracle from the same solutions."""
    w = synth.structures_case()
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.alloc_perturbers(w.npert, w.icb, w.ibb)
    a.set_targets(w.ntarg, w.iptar, w.iitar, 1)
    a.set_dhl(w.kap_list, w.hd, w.kbs)
    a.set_precision(PLAIN_FP64)
    for L in w.lists:
        a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    _generic_diagonal(a, w, 5)
    ms, ns = a.ms, a.ns
    H = a.get_matrix()
    hcp, hp = a.get_perturbers()
    assert np.abs(hcp).max() > 0 and np.abs(hp).max() > 0
    B = a.grid_array("fppqq").reshape(ms, ms, order="F")
    bdiag = np.asfortranarray(np.repeat(B[:, :, None], w.nch, axis=2))
    iprm = _zero_conditions(ms, ns, w.nch)
    _, m = _oracle_matrix(w, H)
    sol, ev, nsol = m.diag_channels(bdiag, iprm, -1e30, 1e30, 0.0)
    path = str(tmp_path / "dbsr_mat.001")
    a.record_header(path, sol, ev, nsol, nsp=ns, nsq=ns)
    ov = a.record_matrix(path, sol, nsol, icase=0)
    a.close()
    # the Hamiltonian: the same matrix again (hch was left transformed)
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.alloc_perturbers(w.npert, w.icb, w.ibb)
    a.set_targets(w.ntarg, w.iptar, w.iitar, 1)
    a.set_dhl(w.kap_list, w.hd, w.kbs)
    a.set_precision(PLAIN_FP64)
    for L in w.lists:
        a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    _generic_diagonal(a, w, 5)
    assert np.array_equal(a.get_matrix(), H)
    a.record_matrix(path, sol, nsol, icase=2)
    bcf = np.asfortranarray(np.arange(w.nch * w.nch * (w.mk + 1), dtype=np.float64)
                            .reshape(w.nch, w.nch, w.mk + 1, order="F") / 7.0)
    a.record_acf(path, bcf)
    a.close()
    got = open(path, "rb").read()

    ref = R.header(ns, w.nch, w.npert, ns, ns, sol, ev, nsol)
    body, rov = R.record_matrix(H, w.icc, sol, nsol, 0, w.npert, w.icb, hcp, w.ibb, hp)
    ref += body
    ref += R.record_matrix(H, w.icc, sol, nsol, 2, w.npert, w.icb, hcp, w.ibb, hp)[0]
    ref += R.acf(w.mk, bcf)
    rg, rr = R.read_records(got), R.read_records(ref)
    assert len(rg) == len(rr) and len(rg) > 12
    # header: the integer records and the solutions bit for bit (no arithmetic)
    for i in range(5):
        assert rg[i] == rr[i], i
    # matrix records: integer pairs equal, real records to 1e-12 of their max
    i = 5
    n_blocks = 0
    while i < len(rr) - 2:
        ig = np.frombuffer(rg[i], dtype=np.int32)
        assert np.array_equal(ig, np.frombuffer(rr[i], dtype=np.int32)), i
        if ig[0] == 0 and ig[1] == 0:
            i += 1
            continue
        x, y = np.frombuffer(rg[i + 1]), np.frombuffer(rr[i + 1])
        assert x.size == y.size, i
        if y.size:
            assert np.abs(x - y).max() <= 1e-12 * max(np.abs(y).max(), 1e-300), (ig, i)
        n_blocks += 1
        i += 2
    assert n_blocks >= 6
    assert rg[-2] == rr[-2] and rg[-1] == rr[-1]  # (mk), bcf
    assert np.abs(ov - rov).max() <= 1e-12 * np.abs(rov).max()
    assert rov[w.nch:, :w.nch].any() and rov[w.nch:, w.nch:].any()
    assert os.path.getsize(path) == len(got)


@pytest.mark.parametrize("ns,nch", [(70, 3), (150, 2)])
def test_split_transform_sizes(ns, nch):
    """The split-BF16 transform at sizes with several 128-row tiles and K
    chunks (ms = 140, 300) and uneven solution counts, against the oracle's
    loops, two calls in a row on the same solutions."""
    w = synth.small(ns=ns, nch=nch, mk=1, n_entries=60 * nch, breit=False, seed=ns + nch,
                    rmax=30.0)
    a = _assembler(w, SPLIT_BF16)
    for L in w.lists:
        a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    ms = a.ms
    rng = np.random.default_rng(ns)
    for ich in range(1, nch + 1):
        for jch in range(1, ich + 1):
            X = rng.standard_normal((ms, ms)) * 10.0 ** rng.uniform(-3, 3)
            a.update_hx(ich, jch, np.asfortranarray(X if ich != jch else X + X.T), 1.0)
    H = a.get_matrix()
    sol = np.zeros((ms, ms, nch), order="F")
    nsol = np.array([ms - 5 - 17 * i for i in range(nch)], dtype=np.int32)
    for ich in range(nch):
        sol[:, :nsol[ich], ich] = rng.standard_normal((ms, nsol[ich]))
    for rep in range(2):
        out = a.channel_basis(sol, nsol, out=True)
        for ich in range(2, nch + 1):
            for jch in range(1, ich):
                k = w.icc[ich - 1, jch - 1]
                ni, nj = nsol[ich - 1], nsol[jch - 1]
                src = H if rep == 0 else prev
                ref = O.record_block(src[:, :, k - 1], sol[:, :ni, ich - 1], sol[:, :nj, jch - 1])
                got = out[:, :, k - 1]
                assert np.abs(got[:ni, :nj] - ref).max() <= 1e-10 * np.abs(ref).max(), (rep, ich, jch)
                assert not got[ni:, :].any() and not got[:, nj:].any()
        prev = out.copy()
    a.close()
