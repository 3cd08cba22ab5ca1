"""A whole assembly captured as one CUDA graph (dbsrg_graph_capture,
dbsrg_graph_launch): the captured run and every replay equal, bit for bit,
the matrix dbsrg_gen_matrix assembles from the same lists, in every
precision form, for the contractions (R^k, S^k, overlaps) and for the other
structures with perturbers and target matrices; a replay with new orbitals
equals a fresh assembly from those orbitals; the calls that free memory the
graph names drop it."""
import numpy as np
import pytest

from dbsr_gb300 import FACTOR_FP64, PLAIN_FP64, SPLIT_BF16, Assembler, synth
from dbsr_gb300._lib import DbsrgError

pytestmark = pytest.mark.gpu


def items(w):
    return [(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c) for L in w.lists]


def make(w, precision, pq=None, structures=False):
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq if pq is None else pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    if structures:
        a.alloc_perturbers(w.npert, w.icb, w.ibb)
        a.set_targets(w.ntarg, w.iptar, w.iitar, 1)
        a.set_dhl(w.kap_list, w.hd, w.kbs)
    a.set_precision(precision)
    return a


def assembled(w, precision, pq=None, structures=False):
    a = make(w, precision, pq, structures)
    for it in items(w):
        a.gen_matrix(*it)
    out = (a.get_matrix(), a.get_acf()) + (a.get_perturbers() if structures else ())
    a.close()
    return out


def perturbed(pq, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(pq * (1.0 + 1e-3 * rng.standard_normal(pq.shape)))


def same(x, y):
    return all(np.array_equal(p, q) for p, q in zip(x, y))


@pytest.mark.parametrize("precision", [PLAIN_FP64, FACTOR_FP64, SPLIT_BF16])
def test_graph_equals_gen_matrix_and_replays_new_orbitals(precision):
    w = synth.small(ns=60, nch=5, mk=3, n_entries=2000, breit=True, seed=59)
    ref = assembled(w, precision)
    a = make(w, precision)
    a.gen_matrix(*items(w)[0])  # leftovers in the matrix must not matter
    a.graph_capture(items(w))
    assert same((a.get_matrix(), a.get_acf()), ref)
    n0 = a.launches
    a.graph_launch()
    assert a.launches > n0
    assert same((a.get_matrix(), a.get_acf()), ref)
    pq2 = perturbed(w.pq, 7)
    ref2 = assembled(w, precision, pq2)
    assert not np.array_equal(ref2[0], ref[0])
    a.graph_launch(pq2)
    assert same((a.get_matrix(), a.get_acf()), ref2)
    # the normal path after replays sees the tables of the orbitals held
    a.zero_matrix()
    for it in items(w):
        a.gen_matrix(*it)
    assert np.array_equal(a.get_matrix(), ref2[0])
    a.graph_launch(w.pq)
    assert same((a.get_matrix(), a.get_acf()), ref)
    a.close()


def test_graph_with_structures_perturbers_and_targets():
    w = synth.structures_case()
    ref = assembled(w, SPLIT_BF16, structures=True)
    a = make(w, SPLIT_BF16, structures=True)
    a.graph_capture(items(w))
    got = (a.get_matrix(), a.get_acf()) + a.get_perturbers()
    assert same(got, ref)
    assert np.abs(ref[2]).max() > 0  # hcp holds terms
    pq2 = perturbed(w.pq, 8)
    ref2 = assembled(w, SPLIT_BF16, pq2, structures=True)
    a.graph_launch(pq2)
    assert same((a.get_matrix(), a.get_acf()) + a.get_perturbers(), ref2)
    a.close()


def test_graph_dropped_by_calls_that_free_its_memory():
    w = synth.small(ns=50, nch=4, mk=2, n_entries=600, seed=61)
    a = make(w, SPLIT_BF16)
    a.graph_capture(items(w))
    a.graph_launch()
    a.invalidate_tables()
    with pytest.raises(DbsrgError, match="ESTATE"):
        a.graph_launch()
    a.graph_capture(items(w))
    a.set_orbitals(w.pq, w.ipbs)
    with pytest.raises(DbsrgError, match="ESTATE"):
        a.graph_launch()
    a.graph_capture(items(w))
    a.graph_release()
    with pytest.raises(DbsrgError, match="ESTATE"):
        a.graph_launch()
    a.close()


def test_graph_needs_the_whole_matrix():
    w = synth.small(ns=50, nch=4, mk=2, n_entries=300, seed=62)
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk, window=3)
    with pytest.raises(DbsrgError, match="ESTATE"):
        a.graph_capture(items(w))
    a.close()
