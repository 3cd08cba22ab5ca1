"""Asynchronous mode of the C-ABI (dbsrg_set_async): the set-up of each R/S
list runs on a second stream into one of two list-state buffers while the
kernels of the previous list run.  The assembled matrix must be the same,
bit for bit, as in the synchronous mode (the same kernels in the same order
on the contraction stream), for every precision form, and errors found
while a list is set up must still be raised by the call itself."""
import numpy as np
import pytest

from dbsr_gb300 import FACTOR_FP64, PLAIN_FP64, SPLIT_BF16, Assembler, synth
from dbsr_gb300._lib import DbsrgError

pytestmark = pytest.mark.gpu


def assemble(w, precision, asynchronous, repeat=1):
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.set_precision(precision)
    a.set_async(asynchronous)
    for _ in range(repeat):
        a.zero_matrix()
        for L in w.lists:
            # fresh copies, dropped right after the call: the library copies
            # the lists during the call
            a.gen_matrix(L.icase, L.itype, L.kpol, L.k1.copy(), L.k2.copy(), L.k3.copy(),
                         L.k4.copy(), L.c.copy())
    a.sync()
    h, acf = a.get_matrix(), a.get_acf()
    a.close()
    return h, acf


@pytest.mark.parametrize("precision", [PLAIN_FP64, FACTOR_FP64, SPLIT_BF16])
def test_async_equals_sync(precision):
    w = synth.small(ns=70, nch=5, mk=4, n_entries=3000, seed=41)
    h0, a0 = assemble(w, precision, False)
    h1, a1 = assemble(w, precision, True)
    assert np.array_equal(h0, h1)
    assert np.array_equal(a0, a1)


def test_async_repeated_assembly_config1_slice():
    # many lists back to back, the two list-state buffers reused in turn
    w = synth.config1(scale=0.01, nch=24)
    h0, _ = assemble(w, SPLIT_BF16, False)
    h1, _ = assemble(w, SPLIT_BF16, True, repeat=2)
    assert np.array_equal(h0, h1)


def test_async_setup_errors_raised_by_the_call():
    w = synth.small(ns=60, nch=3, mk=3, n_entries=300, seed=42)
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.set_precision(SPLIT_BF16)
    a.set_async(True)
    L = next(L for L in w.lists if L.icase == 2)
    a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    bad = L.k1.copy()
    bad[0] = (w.nch + 1) * 2 ** 15 + 1  # channel beyond nch
    with pytest.raises(DbsrgError, match="ERANGE"):
        a.gen_matrix(L.icase, L.itype, L.kpol, bad, L.k2, L.k3, L.k4, L.c)
    a.sync()  # the first list's kernels completed without error
    a.close()


def test_invalidated_and_released_tables_rebuild_identically():
    w = synth.small(ns=70, nch=5, mk=4, n_entries=3000, seed=43)
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.set_precision(SPLIT_BF16)
    out = []
    for how in (None, "invalidate", "invalidate", "release", "invalidate"):
        if how == "invalidate":
            a.invalidate_tables()  # rebuilt from the pooled buffers
        elif how == "release":
            a.release_tables()
        a.zero_matrix()
        for L in w.lists:
            a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
        out.append(a.get_matrix())
    a.close()
    for h in out[1:]:
        assert np.array_equal(h, out[0])


def test_tuning_does_not_change_results():
    w = synth.small(ns=70, nch=6, mk=4, n_entries=4000, seed=44)
    outs = []
    for tune in ({}, {"xchunk": 2, "dchunk": 3}, {"xchunk": 1024, "dchunk": 65535}):
        a = Assembler(w.t, w.ks, w.ksp, w.ksq, tuning=tune)
        a.set_orbitals(w.pq, w.ipbs)
        a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
        for prec in (SPLIT_BF16, FACTOR_FP64):
            a.set_precision(prec)
            a.zero_matrix()
            for L in w.lists:
                a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
            outs.append((tune, prec, a.get_matrix()))
        a.close()
    for tune, prec, h in outs[2:]:
        ref = next(x for t, p, x in outs if p == prec)
        assert np.array_equal(h, ref), (tune, prec)
