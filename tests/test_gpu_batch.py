"""dbsrg_gen_batch: independent symmetry blocks with their own grids,
assembled concurrently, give exactly the matrices of one-by-one assembly;
an error in one block is reported without disturbing the others."""
import numpy as np
import pytest

from dbsr_gb300 import PLAIN_FP64, SPLIT_BF16, Assembler, DbsrgError, synth
from dbsr_gb300.api import gen_batch

pytestmark = pytest.mark.gpu


def blocks():
    return [synth.small(ns=ns, nch=nch, mk=2, n_entries=150, breit=True, seed=s)
            for ns, nch, s in ((50, 2, 41), (64, 3, 42), (58, 2, 43))]


def make(w, precision):
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.set_precision(precision)
    return a


def lists_of(w):
    return [(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c) for L in w.lists]


@pytest.mark.parametrize("precision", [PLAIN_FP64, SPLIT_BF16])
def test_batch_equals_one_by_one(precision):
    ws = blocks()
    ref = []
    for w in ws:
        a = make(w, precision)
        for item in lists_of(w):
            a.gen_matrix(*item)
        ref.append((a.get_matrix(), a.get_acf()))
        a.close()
    asm = [make(w, precision) for w in ws]
    gen_batch(asm, [lists_of(w) for w in ws])
    for a, (h, acf) in zip(asm, ref):
        assert np.array_equal(a.get_matrix(), h)
        assert np.array_equal(a.get_acf(), acf)
        a.close()


def test_batch_reports_a_bad_block():
    ws = blocks()
    asm = [make(w, SPLIT_BF16) for w in ws]
    lists = [lists_of(w) for w in ws]
    bad = list(lists[1][1])
    bad[3] = bad[3].copy()
    bad[3][0] = 10 ** 6  # K1 with a channel outside the matrix
    lists[1][1] = tuple(bad)
    with pytest.raises(DbsrgError):
        gen_batch(asm, lists)
    # the other blocks were assembled in full
    a0 = make(ws[0], SPLIT_BF16)
    for item in lists_of(ws[0]):
        a0.gen_matrix(*item)
    assert np.array_equal(asm[0].get_matrix(), a0.get_matrix())
    for a in asm + [a0]:
        a.close()
