"""SCF potential matrices: DBSR_HF's hf_matrix (hf_matrix.f90:2-70, Coulomb
part) for every orbital.

CPU: the oracle's restatement of hf_matrix against the oracle's energy
gradient (rk, dbsr_lib_dbs.f90:3981-4022): for E = sum coef(i,j,k) F^k(i,j)
(i >= j) + coef(i,j,k) G^k(i,j) (i < j), with a(i,j,k) = coef(max,min,k)
and b(i,j,k) = coef(min,max,k) (hf_MOD_energy.f90:20-57),
dE/dp_i = 2 qsum hfm_i p_i.
GPU: dbsrg_hf_matrix against the oracle (plain FP64 within 1e-12 of the
largest element, split form within 1e-10), and dbsrg_backward's gradient of
the same energy against 2 qsum hfm_i p_i from dbsrg_hf_matrix."""
import numpy as np
import pytest

from oracle import oracle as orc
from dbsr_gb300 import synth

QSUM = 1.7


def _case(ns=48, norb=5, kmax=3, seed=31):
    w = synth.energy_workload("hf", seed, ns, 16.0, 10.0, norb, kmax, 8)
    rng = np.random.default_rng(seed)
    coef = rng.uniform(-1, 1, (norb, norb, kmax + 1))
    coef[rng.uniform(size=coef.shape) < 0.2] = 0.0
    ent = []
    for i in range(norb):
        for j in range(norb):
            for k in range(kmax + 1):
                if coef[i, j, k] == 0.0:
                    continue
                if i >= j:
                    ent.append((k, i + 1, j + 1, i + 1, j + 1, coef[i, j, k]))
                else:
                    ent.append((k, i + 1, j + 1, j + 1, i + 1, coef[i, j, k]))
    ent = np.array(ent)
    return w, coef, ent


def _ab(coef, i):
    norb, kmax1 = coef.shape[0], coef.shape[2]
    a = np.zeros((norb, kmax1), order="F")
    b = np.zeros((norb, kmax1), order="F")
    for j in range(norb):
        a[j] = coef[max(i, j), min(i, j)]
        if i != j:
            b[j] = coef[min(i, j), max(i, j)]
    return a, b


def _ints(ent):
    return [ent[:, c].astype(np.int32) for c in range(5)] + [ent[:, 5].copy()]


def test_oracle_hf_matrix_is_the_energy_gradient():
    w, coef, ent = _case(ns=40, norb=4, kmax=2)
    g = orc.Grid(w.t, w.ks, w.ksp, w.ksq)
    _, grad = g.rk_energy_grad(*_ints(ent), w.pq)
    for i in range(coef.shape[0]):
        a, b = _ab(coef, i)
        h = g.hf_matrix(w.pq, i + 1, a, b, QSUM)
        p = np.concatenate([w.pq[:, 0, i], w.pq[:, 1, i]])
        gi = np.concatenate([grad[:, 0, i], grad[:, 1, i]])
        assert np.abs(2 * QSUM * h @ p - gi).max() <= 1e-12 * np.abs(gi).max()


def _assembler(w, kmax, prec):
    from dbsr_gb300 import Assembler

    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, np.zeros(w.pq.shape[2], np.int32))
    a.alloc_matrix(1, np.ones((1, 1), np.int32, order="F"), 1, kmax)
    a.set_precision(prec)
    return a


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-10), (2, 1e-12)])
def test_hf_matrix_matches_oracle(prec, tol):
    w, coef, _ = _case()
    kmax = coef.shape[2] - 1
    ms = 2 * w.ns
    rng = np.random.default_rng(4)
    dhl = rng.uniform(-1, 1, (ms, ms))
    dhl = np.asfortranarray(dhl + dhl.T)
    g = orc.Grid(w.t, w.ks, w.ksp, w.ksq)
    a = _assembler(w, kmax, prec)
    for i in range(coef.shape[0]):
        A, B = _ab(coef, i)
        got = a.hf_matrix(i + 1, A, B, QSUM, dhl=dhl if i % 2 else None)
        ref = g.hf_matrix(w.pq, i + 1, A, B, QSUM, dhl=dhl if i % 2 else None)
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err <= tol, (i, err)
    a.close()


@pytest.mark.gpu
def test_backward_gradient_is_twice_the_potential_times_the_orbital():
    w, coef, ent = _case(ns=60, norb=6, kmax=4, seed=8)
    kmax = coef.shape[2] - 1
    a = _assembler(w, kmax, 0)
    _, grad = a.backward(*_ints(ent))
    for i in range(coef.shape[0]):
        A, B = _ab(coef, i)
        h = a.hf_matrix(i + 1, A, B, QSUM)
        p = np.concatenate([w.pq[:, 0, i], w.pq[:, 1, i]])
        gi = np.concatenate([grad[:, 0, i], grad[:, 1, i]])
        assert np.abs(2 * QSUM * h @ p - gi).max() <= 1e-11 * np.abs(gi).max(), i
    a.close()


@pytest.mark.gpu
def test_hf_matrix_needs_a_one_channel_matrix():
    from dbsr_gb300 import Assembler

    w, coef, _ = _case(ns=40, norb=3, kmax=1)
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, np.zeros(w.pq.shape[2], np.int32))
    icc = synth.block_numbering(2)
    a.alloc_matrix(2, icc, 3, 1)
    A, B = _ab(coef, 0)
    with pytest.raises(RuntimeError):
        a.hf_matrix(1, A, B, QSUM)
    a.close()
