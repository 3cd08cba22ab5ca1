"""Failure handling without a GPU fault (the reference Stops on any
inconsistency; here every call returns a status and the context stays
usable):

* a list with a non-finite coefficient is refused by the call (EINVAL)
  before any contraction, in every form, for R/S and overlap lists;
* the tensor-core exchange's bounded waits: with the test switch the
  epilogue warps wait on an mbarrier that nothing completes, the wait runs
  out after a short limit, the kernel drains its own copies and MMAs, frees
  its TMEM and returns, the call reports ETIMEOUT, and the next assembly on
  the same context is exact."""
import numpy as np
import pytest

from dbsr_gb300 import FACTOR_FP64, PLAIN_FP64, SPLIT_BF16, Assembler, synth
from dbsr_gb300._lib import DbsrgError

pytestmark = pytest.mark.gpu


def fresh(w, precision):
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.set_precision(precision)
    return a


def assemble(a, w):
    a.zero_matrix()
    for L in w.lists:
        a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    return a.get_matrix()


@pytest.mark.parametrize("precision", [PLAIN_FP64, FACTOR_FP64, SPLIT_BF16])
@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_non_finite_coefficient_is_refused(precision, bad):
    w = synth.small(ns=50, nch=3, mk=2, n_entries=400, breit=True, seed=101)
    a = fresh(w, precision)
    ref = assemble(a, w)
    for L in w.lists:
        c = L.c.copy()
        c[len(c) // 2] = bad
        with pytest.raises(DbsrgError, match="EINVAL"):
            a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, c)
    assert np.array_equal(a.get_matrix(), ref)  # nothing was added
    assert np.array_equal(assemble(a, w), ref)
    a.close()


def test_injected_wait_timeout_is_reported_and_the_context_recovers():
    w = synth.small(ns=70, nch=4, mk=3, n_entries=1200, breit=True, seed=102)
    a = fresh(w, SPLIT_BF16)
    ref = assemble(a, w)
    X = next(L for L in w.lists if L.icase == 2 and L.itype == 4)  # tensor-core exchange
    a.set_wait_limit(2_000_000)  # 2 ms
    a.inject_wait_timeout(True)
    a.zero_matrix()
    with pytest.raises(DbsrgError, match="ETIMEOUT"):
        a.gen_matrix(X.icase, X.itype, X.kpol, X.k1, X.k2, X.k3, X.k4, X.c)
    # asynchronous mode: reported by the next call that waits
    a.set_async(True)
    a.gen_matrix(X.icase, X.itype, X.kpol, X.k1, X.k2, X.k3, X.k4, X.c)
    with pytest.raises(DbsrgError, match="ETIMEOUT"):
        a.sync()
    a.set_async(False)
    a.inject_wait_timeout(False)
    a.set_wait_limit(2_000_000_000)
    assert np.array_equal(assemble(a, w), ref)
    a.close()
