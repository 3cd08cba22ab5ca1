"""GPU parity of the cell-factored contraction (the chosen form) against the
CPU oracle on identical seeded inputs.

FACTOR_FP64 is the factored algorithm in FP64 throughout: it sums the same
cell contributions as the reference in another order, so the plain bar
(1e-12 of the largest element of each block) applies.  SPLIT_BF16 runs the
far-field products as split-BF16 tensor-core products (FP32 accumulation,
FP64 recombination) and is held to the 1e-10 bound of the precision form.
"""
import numpy as np
import pytest

from dbsr_gb300 import FACTOR_FP64, PLAIN_FP64, SPLIT_BF16, Assembler, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def run(w, precision, lists=None):
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.set_precision(precision)
    for L in (lists if lists is not None else w.lists):
        a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    h, acf = a.get_matrix(), a.get_acf()
    a.close()
    return h, acf


def oracle(w, lists=None):
    g = O.Grid(w.t, w.ks, w.ksp, w.ksq)
    m = O.Matrix(g, w.pq, w.ipbs, w.nch, w.icc, w.mk)
    for L in (lists if lists is not None else w.lists):
        m.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    return m.hch.copy(), m.acf.copy()


def check(h, ref, tol):
    worst = 0.0
    for b in range(ref.shape[2]):
        r = ref[:, :, b]
        if np.abs(r).max() == 0:
            assert np.abs(h[:, :, b]).max() == 0, b
            continue
        e = relmax(h[:, :, b], r)
        worst = max(worst, e)
        assert e <= tol, (b, e)
    return worst


@pytest.mark.parametrize("precision,tol", [(FACTOR_FP64, 1e-12), (SPLIT_BF16, 1e-10)])
def test_factored_config0(precision, tol):
    w = synth.config0()
    h, acf = run(w, precision)
    ref, racf = oracle(w)
    check(h, ref, tol)
    assert relmax(acf, racf) <= 1e-12


@pytest.mark.parametrize("precision,tol", [(FACTOR_FP64, 1e-12), (SPLIT_BF16, 1e-10)])
def test_factored_each_list_kind(precision, tol):
    w = synth.small(ns=60, nch=3, mk=3, n_entries=500, breit=True, seed=11)
    kinds = {}
    for L in w.lists:
        kinds.setdefault((L.icase, L.itype), L)
    assert (2, 3) in kinds and (2, 4) in kinds and (3, 8) in kinds and (3, 6) in kinds
    for key, L in sorted(kinds.items()):
        h, _ = run(w, precision, [L])
        ref, _ = oracle(w, [L])
        check(h, ref, tol)


def test_factored_whole_small_workload_matches_plain():
    w = synth.small(ns=70, nch=4, mk=4, n_entries=800, breit=True, seed=5)
    hp, ap = run(w, PLAIN_FP64)
    hf, af = run(w, FACTOR_FP64)
    check(hf, hp, 1e-12)
    assert relmax(af, ap) <= 1e-12


def test_factored_case4_and_case2_structures():
    # S^k itypes 7 (convol case 2) and 9 (case 4) built from the itype 6/8
    # lists of the small workload by relabelling the structure
    w = synth.small(ns=55, nch=2, mk=2, n_entries=300, breit=True, seed=23)
    extra = []
    for L in w.lists:
        if L.icase == 3 and L.itype % 10 in (6, 8):
            extra.append(synth.CList(3, L.itype + 1, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c))
    assert extra
    for L in extra:
        for prec, tol in ((FACTOR_FP64, 1e-12), (SPLIT_BF16, 1e-10)):
            h, _ = run(w, prec, [L])
            ref, _ = oracle(w, [L])
            check(h, ref, tol)


@pytest.mark.parametrize("ns", [151, 160])
def test_split_multi_tile_rows_against_plain(ns):
    """ns above 128: quadrants of several 128-row tiles in the tensor-core
    exchange (odd ns: the 8-byte staging path, even: bulk copies), every list
    kind, 12 bound orbitals, per block against the plain FP64 assembly (held
    to the oracle at 1e-12 by test_gpu_parity)."""
    w = synth.small(ns=ns, nch=4, mk=3, n_entries=1500, breit=True, seed=70 + ns, norb=12,
                    rmax=40.0, z=12.0)
    hp, ap = run(w, PLAIN_FP64)
    hs, as_ = run(w, SPLIT_BF16)
    check(hs, hp, 1e-10)
    assert np.abs(as_ - ap).max() <= 1e-12 * max(np.abs(ap).max(), 1e-300)


def _many_orbitals(nb, seed):
    """A small grid with nb bound orbitals (hydrogenic shapes with n up to 12
    over the kappas of the target list) and two channels; R^k and S^k lists
    whose entries draw bound orbitals from all of them."""
    base = synth.TARGET_ORBITALS
    orbitals = [(n + 1 + i // len(base), k) for i, (n, k) in enumerate(base * 5)][:nb]
    return synth._build(f"{nb} bound orbitals", seed, 60, 20.0, 8.0, orbitals, [-1, 2], 2,
                        900, 1.0, breit=True, o_entries=6)


@pytest.mark.parametrize("nb", [48, 96])
@pytest.mark.parametrize("precision,tol", [(FACTOR_FP64, 1e-12), (SPLIT_BF16, 1e-10)])
def test_factored_forms_with_many_bound_orbitals(nb, precision, tol):
    """More than 32 bound orbitals: the split exchange takes one product per
    chunk of 32 orbitals (48: two chunks, 96: three), the factored FP64 path
    any number up to 128; every block against the oracle."""
    w = _many_orbitals(nb, 300 + nb)
    used = set()
    for L in w.lists:
        if L.icase in (2, 3):
            used |= set(L.k2.tolist()) | set(L.k3.tolist())
    assert max(used) > 64 if nb > 64 else max(used) > 32
    h, acf = run(w, precision)
    ref, racf = oracle(w)
    check(h, ref, tol)
    assert relmax(acf, racf) <= 1e-12


def test_bound_orbital_limit_of_the_factored_forms():
    """129 bound orbitals are beyond the factored forms (EINVAL from the
    call); the plain form still assembles the list."""
    from dbsr_gb300._lib import DbsrgError

    w = _many_orbitals(129, 81)
    L = next(L for L in w.lists if L.icase == 2 and L.itype == 4)
    for prec in (SPLIT_BF16, FACTOR_FP64):
        a = Assembler(w.t, w.ks, w.ksp, w.ksq)
        a.set_orbitals(w.pq, w.ipbs)
        a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
        a.set_precision(prec)
        with pytest.raises(DbsrgError, match="EINVAL"):
            a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
        a.close()
    h, _ = run(w, PLAIN_FP64, [L])
    ref, _ = oracle(w, [L])
    check(h, ref, 1e-12)
