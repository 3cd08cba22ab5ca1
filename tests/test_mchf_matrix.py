"""SCF potential matrices of DBSR_MCHF: mchf_matrix (mchf_matrix.f90:2-251)
and core_matrix (:255-346).

CPU: the oracle's restatements against its hf_matrix (hf_matrix.f90:2-70,
itself checked against the energy gradient in test_hf_matrix.py) where the
two coincide -- a single configuration whose R^k entries are the F^k and
G^k integrals of orbital i gives mchf_matrix = hf_matrix with qsum = S;
core_matrix with a(i,j,k) q_i q_j is hf_matrix of rescaled coefficients.
GPU: dbsrg_mchf_matrix and dbsrg_mchf_core against the oracle on a case
with every classification pattern of the R^k entries (direct, exchange,
Newton and right-hand-side entries, one-electron cross terms), plain FP64
within 1e-12 of the largest element, the factored FP64 form within 1e-12,
the split form within 1e-10; e(i) and qsum(i) likewise."""
import numpy as np
import pytest

from dbsr_gb300 import synth
from oracle import oracle as orc

KMAX = 3


def _case(ns=48, norb=6, seed=41):
    w = synth.energy_workload("mchf", seed, ns, 16.0, 10.0, norb, KMAX, 8)
    rng = np.random.default_rng(seed)
    ms = 2 * ns
    X = rng.standard_normal((ms, ms))
    dhl = np.asfortranarray(0.05 * (X + X.T))
    return w, dhl, rng


def _patterned_entries(rng, norb, i, n_each=3):
    """R^k entries (k, i1, i2, i3, i4, c) covering all fifteen patterns of
    the positions of orbital i (1-based), the other orbitals random."""
    others = [j for j in range(1, norb + 1) if j != i]
    ent = []
    for code in range(1, 16):
        for _ in range(n_each):
            idx = [i if code & (8 >> p) else int(rng.choice(others)) for p in range(4)]
            ent.append((int(rng.integers(0, KMAX + 1)), *idx, float(rng.uniform(-1, 1))))
    ent.sort(key=lambda e: e[0])  # k ascending, as the integral lists are ordered
    return ent


def _lint(rng, norb, i, S):
    li1, li2, lc = [i], [i], [S]
    for j in range(1, norb + 1):
        if j != i:
            li1.append(j if j % 2 else i)
            li2.append(i if j % 2 else j)
            lc.append(float(rng.uniform(-0.3, 0.3)))
    return li1, li2, lc


def _cols(ent):
    a = np.array(ent, dtype=object)
    return [a[:, c].astype(np.int32) for c in range(5)] + [a[:, 5].astype(np.float64)]


def test_oracle_mchf_single_configuration_is_hf_matrix():
    w, dhl, rng = _case(ns=40, norb=4)
    g = orc.Grid(w.t, w.ks, w.ksp, w.ksq)
    S = 1.7
    norb = 4
    coef = rng.uniform(-1, 1, (norb, KMAX + 1))
    coefx = rng.uniform(-1, 1, (norb, KMAX + 1))
    for i in range(1, norb + 1):
        ent = []
        for k in range(KMAX + 1):
            for j in range(1, norb + 1):
                # mchf_matrix divides the weighted coefficients by S, as
                # hf_matrix divides its two-electron part by qsum
                if j == i:
                    ent.append((k, i, i, i, i, coef[j - 1, k]))
                else:
                    ent.append((k, i, j, i, j, coef[j - 1, k]))
                    ent.append((k, i, j, j, i, coefx[j - 1, k]))
        hfm, rhs, _, e, q = g.mchf_matrix(w.pq, i, KMAX, ([i], [i], [S]), _cols(ent), dhl,
                                          irhs=1, newton=0, eps_c=0.0)
        a = np.asfortranarray(coef)
        b = np.asfortranarray(coefx)
        b[i - 1] = 0.0
        ref = g.hf_matrix(w.pq, i, a, b, S, dhl)
        assert q == S
        assert not rhs.any()
        assert np.abs(hfm - ref).max() <= 1e-13 * np.abs(ref).max()
        v = np.concatenate([w.pq[:, 0, i - 1], w.pq[:, 1, i - 1]])
        assert abs(e - v @ hfm @ v) <= 1e-13 * abs(e)


def test_oracle_core_matrix_is_rescaled_hf_matrix():
    w, hd, rng = _case(ns=40, norb=4)
    g = orc.Grid(w.t, w.ks, w.ksp, w.ksq)
    norb = 4
    a = rng.uniform(-1, 1, (norb, KMAX + 1))
    b = rng.uniform(-1, 1, (norb, KMAX + 1))
    qs = rng.uniform(1.0, 4.0, norb)
    for i in range(1, norb + 1):
        qi = qs[i - 1]
        hfm, hx = g.mchf_core(w.pq, i, a, b, qs, hd, newton=1)
        a2 = a * (qi * qs)[:, None]
        b2 = b * (qi * qs)[:, None]
        a2[i - 1] = a[i - 1] * qi * (qi - 1) / 2  # hf_matrix doubles j = i
        b2[i - 1] = b[i - 1] * qi * (qi - 1)
        ref = g.hf_matrix(w.pq, i, np.asfortranarray(a2), np.asfortranarray(b2), qi, hd)
        assert np.abs(hfm - ref).max() <= 1e-13 * np.abs(ref).max()
        assert np.abs(hx).max() > 0


def _assembler(w, prec):
    from dbsr_gb300 import Assembler

    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, np.zeros(w.pq.shape[2], np.int32))
    a.alloc_matrix(1, np.ones((1, 1), np.int32, order="F"), 1, KMAX)
    a.set_precision(prec)
    return a


def _rel(x, r):
    return np.abs(x - r).max() / max(np.abs(r).max(), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (2, 1e-12), (1, 1e-10)])
def test_mchf_matrix_matches_oracle(prec, tol):
    norb = 6
    w, dhl, rng = _case(norb=norb)
    g = orc.Grid(w.t, w.ks, w.ksp, w.ksq)
    a = _assembler(w, prec)
    seen_rhs = seen_hx = 0
    for i in (1, 3, 6):
        ent = _patterned_entries(rng, norb, i)
        lint = _lint(rng, norb, i, 1.3 + 0.1 * i)
        for irhs, newton in ((1, 1), (0, 1), (1, 0)):
            ref = g.mchf_matrix(w.pq, i, KMAX, lint, _cols(ent), dhl, irhs, newton, 1e-10)
            got = a.mchf_matrix(i, KMAX, lint, _cols(ent), dhl, irhs, newton, 1e-10)
            assert got[4] == ref[4]  # qsum
            assert _rel(got[0], ref[0]) <= tol, ("hfm", i, irhs, newton)
            if np.abs(ref[1]).max() > 0:
                seen_rhs += 1
                assert _rel(got[1], ref[1]) <= tol, ("rhs", i)
            else:
                assert not got[1].any()
            if newton:
                seen_hx += 1
                assert _rel(got[2], ref[2]) <= tol, ("hx", i)
            assert abs(got[3] - ref[3]) <= tol * max(abs(ref[3]), np.abs(ref[0]).max()), ("e", i)
    assert seen_rhs > 0 and seen_hx > 0
    a.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-10)])
def test_mchf_core_matches_oracle(prec, tol):
    norb = 5
    w, hd, rng = _case(norb=norb, seed=43)
    g = orc.Grid(w.t, w.ks, w.ksp, w.ksq)
    A = rng.uniform(-1, 1, (norb, KMAX + 1))
    B = rng.uniform(-1, 1, (norb, KMAX + 1))
    A[rng.uniform(size=A.shape) < 0.2] = 0.0
    qs = rng.uniform(1.0, 4.0, norb)
    a = _assembler(w, prec)
    for i in (1, 4):
        ref = g.mchf_core(w.pq, i, A, B, qs, hd, newton=1)
        got = a.mchf_core(i, A, B, qs, hd, newton=1)
        assert _rel(got[0], ref[0]) <= tol
        assert _rel(got[1], ref[1]) <= tol
    a.close()
