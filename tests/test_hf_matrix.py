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


def _breit_entries(norb, kmax, n, seed):
    """rk4 entries of a Breit energy: kr1 = k + 1000 itype, kr2 = int 1..4,
    kr3, kr4 orbitals, crk uniform in [-1, 1]."""
    rng = np.random.default_rng(seed)
    kr1 = (rng.integers(0, kmax + 1, n) + 1000 * rng.integers(0, 2, n)).astype(np.int32)
    kr2 = rng.integers(1, 5, n).astype(np.int32)
    kr3 = rng.integers(1, norb + 1, n).astype(np.int32)
    kr4 = rng.integers(1, norb + 1, n).astype(np.int32)
    return kr1, kr2, kr3, kr4, rng.uniform(-1, 1, n)


def test_oracle_breit_part_equals_s_data_on_one_channel():
    """hf_matrix_breit (hf_matrix.f90:91-163) restated loop for loop equals
    the oracle's S_data itypes 6 and 7 (S_data.f90:240-274) on a one-channel
    block with K2 = K3 = the partner orbital: the equivalence the device
    builds the Breit part on.  Its exchange forms (int 3, 4) add nothing:
    it passes the storage 'x','x' to convol_sk, which has no branch for it
    (dbsr_lib_dbs.f90:2610-2700)."""
    w, coef, _ = _case(ns=44, norb=4, kmax=2, seed=12)
    kmax = 2
    kr1, kr2, kr3, kr4, crk = _breit_entries(4, kmax, 60, 5)
    g = orc.Grid(w.t, w.ks, w.ksp, w.ksq)
    kint = [2, 1, 4, 3]
    for i in range(1, 5):
        ref = g.hf_matrix_breit(w.pq, i, kmax, kr1, kr2, kr3, kr4, crk)
        m = orc.Matrix(g, w.pq, np.zeros(4, np.int32), 1, np.ones((1, 1), np.int32), kmax)
        for itype in (0, 1):
            for k in range(kmax + 1):
                for it in (1, 2):
                    ent = []
                    for e in range(crk.size):
                        if kr1[e] != k + 1000 * itype:
                            continue
                        if kr3[e] == i:
                            jnt, j = kr2[e], kr4[e]
                        elif kr4[e] == i:
                            jnt, j = kint[kr2[e] - 1], kr3[e]
                        else:
                            continue
                        if jnt == it:
                            ent.append((j, crk[e]))
                    if not ent:
                        continue
                    ent.sort(key=lambda t: t[0])
                    jj = np.array([t[0] for t in ent], np.int32)
                    m.gen_matrix(3, 10 * itype + 5 + it, k, np.full(jj.size, 32769, np.int32), jj,
                                 jj, np.zeros(jj.size, np.int32), np.array([t[1] for t in ent]))
        got = m.hch[:, :, 0]
        assert np.abs(ref).max() > 0
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max(), i
        ex = kr2 >= 3  # the exchange forms alone
        zero = g.hf_matrix_breit(w.pq, i, kmax, kr1[ex], kr2[ex], kr3[ex], kr4[ex], crk[ex])
        assert not np.abs(zero).max() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-10), (2, 1e-12)])
def test_hf_matrix_with_breit_matches_oracle(prec, tol):
    w, coef, _ = _case(seed=17)
    kmax = coef.shape[2] - 1
    norb = coef.shape[0]
    kr1, kr2, kr3, kr4, crk = _breit_entries(norb, kmax, 80, 9)
    g = orc.Grid(w.t, w.ks, w.ksp, w.ksq)
    a = _assembler(w, kmax, prec)
    a.hf_breit_list(kr1, kr2, kr3, kr4, crk)
    for i in range(norb):
        A, B = _ab(coef, i)
        got = a.hf_matrix(i + 1, A, B, QSUM)
        ref = g.hf_matrix(w.pq, i + 1, A, B, QSUM)
        ref = ref + g.hf_matrix_breit(w.pq, i + 1, kmax, kr1, kr2, kr3, kr4, crk) / QSUM
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err <= tol, (i, err)
    a.close()
