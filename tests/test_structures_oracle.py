"""The oracle's restatement of the list structures that are not channel-pair
contractions (R_data itypes 1/2, S_data 1-5, L_data, O_data 1/2/4 with
UPDATE_HV/HB/HW/HX and Target_h), checked on the CPU:

* BAV (unvendored; restated as a band matrix times a vector) against the
  same product with the dense matrix (numpy);
* R_data itype 1 with an UPDATE_HB target: the four atypes' SUM_AmB of
  convol case 2 add up to rk(i1,i2;i3,i4) (dbsr_lib_dbs.f90:3981-4022),
  which the configuration-energy tests pin to DBSR_HF's printed energies;
* R_data itype 2 with an UPDATE_HV target: the perturber vector dotted with
  orbital i1 is rk(i1,i2;i3,i4) as well (the potential of the (i2,i4)
  density on the (i1,i3) pair);
* L_data itype 1: hp = c * p_i^T hd p_j;
* every structure of the synthetic workload runs without an error code.
"""
import numpy as np
import pytest

from dbsr_gb300 import synth
from oracle import oracle as O

IBO = synth.IBO


def dense_s(a, ns, ks):
    A = np.zeros((ns, ns))
    for jp in range(1, ks + 1):
        for i in range(1, ns - jp + 2):
            j = i + jp - 1
            A[i - 1, j - 1] = a[i - 1, jp - 1]
            A[j - 1, i - 1] = a[i - 1, jp - 1]
    return A


def dense_n(a, ns, ks):
    A = np.zeros((ns, ns))
    for jp in range(1, 2 * ks):
        for i in range(max(1, 1 + ks - jp), min(ns, ns + ks - jp) + 1):
            A[i - 1, i + jp - ks - 1] = a[i - 1, jp - 1]
    return A


def test_bav_against_dense_products():
    rng = np.random.default_rng(3)
    ns, ks = 30, 9
    b = rng.uniform(-1, 1, ns)
    a = np.asfortranarray(rng.uniform(-1, 1, (ns, ks)))
    A = dense_s(a, ns, ks)
    for d in ("r", "l"):
        assert np.allclose(O.bav(ns, ks, a, b, "s", d), A @ b, rtol=1e-14, atol=1e-14)
    a = np.asfortranarray(rng.uniform(-1, 1, (ns, 2 * ks - 1)))
    A = dense_n(a, ns, ks)
    assert np.allclose(O.bav(ns, ks, a, b, "n", "r"), A @ b, rtol=1e-14, atol=1e-14)
    assert np.allclose(O.bav(ns, ks, a, b, "n", "l"), A.T @ b, rtol=1e-14, atol=1e-14)


@pytest.fixture(scope="module")
def wl():
    return synth.structures_case()


def matrix(w):
    g = O.Grid(w.t, w.ks, w.ksp, w.ksq)
    m = O.Matrix(g, w.pq, w.ipbs, w.nch, w.icc, w.mk)
    m.set_perturbers(w.npert, w.icb, w.ibb)
    m.set_targets(w.ntarg, w.iptar, w.iitar, 1)
    m.set_dhl(w.kap_list, w.hd, w.kbs)
    return g, m


@pytest.mark.parametrize("k", [0, 1, 2])
def test_r_itype1_bound_bound_is_rk(wl, k):
    g, m = matrix(wl)
    i1, i2, i3, i4 = 1, 2, 3, 4
    one = np.array([1], np.int32)
    m.gen_matrix(2, 1, k, one * (i1 * IBO + i3), one * (i2 * IBO + i4), -one, -one,
                 np.array([1.0]))
    p = [wl.pq[:, :, i - 1] for i in (i1, i2, i3, i4)]
    rk = g.rk(*p, k)
    assert abs(rk) > 0
    assert abs(m.hp[wl.ibb[0, 0] - 1] - rk) <= 1e-13 * abs(rk)


@pytest.mark.parametrize("k", [0, 2])
def test_r_itype2_vector_dotted_with_orbital_is_rk(wl, k):
    g, m = matrix(wl)
    i1, i2, i3, i4 = 1, 2, 1, 3  # the potential of (i2,i4) on orbital i3
    one = np.array([1], np.int32)
    m.gen_matrix(2, 2, k, one * (i2 * IBO + i4), one * i3, one * 1, -one, np.array([1.0]))
    col = m.hcp[:, wl.icb[0, 0] - 1]
    v1 = wl.pq[:, :, i1 - 1].ravel(order="F")  # (P; Q) of orbital i1
    rk = g.rk(*(wl.pq[:, :, i - 1] for i in (i1, i2, i3, i4)), k)
    assert abs(rk) > 0
    assert abs(col @ v1 - rk) <= 1e-12 * abs(rk)


def test_l_itype1_bound_bound_value(wl):
    g, m = matrix(wl)
    one = np.array([1], np.int32)
    i, j = 1, 2  # 1s and 2s: one kappa
    assert wl.kbs[0] == wl.kbs[1]
    m.gen_matrix(1, 1, 0, one * i, one * j, one * 2, one * 3, np.array([0.5]))
    slot = list(wl.kap_list).index(wl.kbs[0])
    pi, pj = (wl.pq[:, :, o - 1].ravel(order="F") for o in (i, j))
    want = 0.5 * (pi @ wl.hd[:, :, slot] @ pj)
    assert abs(m.hp[wl.ibb[1, 2] - 1] - want) <= 1e-13 * abs(want)


def test_every_structure_runs(wl):
    g, m = matrix(wl)
    for L in wl.lists:
        m.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    assert np.abs(m.hch).max() > 0
    assert np.abs(m.hcp).max() > 0 and np.abs(m.hp).max() > 0
    assert np.abs(m.htarg).max() > 0 and np.abs(m.otarg).max() > 0


def test_perturber_term_without_perturbers_is_an_error(wl):
    g = O.Grid(wl.t, wl.ks, wl.ksp, wl.ksq)
    m = O.Matrix(g, wl.pq, wl.ipbs, wl.nch, wl.icc, wl.mk)
    L = next(L for L in wl.lists if (L.icase, L.itype) == (0, 1))
    with pytest.raises(RuntimeError, match="-4"):
        m.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
