"""GPU parity: every layer of the sm_103a library against the CPU oracle
on identical seeded inputs, through the C ABI.

Tolerances: grid, moments, diagonal cells and tables are computed with the
reference's operation order and explicit round-to-nearest arithmetic, so
they are compared at 1e-14 relative to the largest entry; the assembled
matrices at 1e-12 relative to the largest entry of each block (the plain
FP64 bar).
"""
import numpy as np
import pytest

from dbsr_gb300 import RK, SK, Assembler, DbsrgError, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TIGHT = 1e-14
PLAIN = 1e-12


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def pair():
    t = synth.knots(60, 20.0, 8.0)
    return Assembler(t), O.Grid(t)


def test_grid_arrays(pair):
    a, g = pair
    for name in ("gx", "gw", "gr", "grw", "grm", "pbsp", "qbsp", "fpbs", "fqbs", "fppqq"):
        assert relmax(a.grid_array(name), g.array(name)) <= TIGHT, name


@pytest.mark.parametrize("which", [0, 1, 2, 3])
@pytest.mark.parametrize("k", [0, 1, 4, -1, -6])
def test_moments(pair, which, k):
    a, g = pair
    assert relmax(a.get_moments(which, k), g.moments(which, k)) <= TIGHT


@pytest.mark.parametrize("typ", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("k", [0, 2, 7])
def test_diag_cells(pair, typ, k):
    a, g = pair
    assert relmax(a.get_diag_cells(typ, k), g.triang(typ, k)) <= TIGHT


@pytest.mark.parametrize("typ", [0, 1, 2, 3])
@pytest.mark.parametrize("k", [0, 1, 3, 6])
def test_rk_tables(pair, typ, k):
    a, g = pair
    assert relmax(a.get_table(RK, typ, k), g.mrk(typ, k)) <= TIGHT


@pytest.mark.parametrize("typ", [0, 1])
@pytest.mark.parametrize("k", [0, 2, 5])
def test_sk_tables(pair, typ, k):
    a, g = pair
    assert relmax(a.get_table(SK, typ, k), g.msk(typ, k)) <= TIGHT


def run_both(w, lists=None):
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    g = O.Grid(w.t, w.ks, w.ksp, w.ksq)
    m = O.Matrix(g, w.pq, w.ipbs, w.nch, w.icc, w.mk)
    for L in (lists if lists is not None else w.lists):
        a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
        m.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    return a, m


def check_blocks(a, m, w, tol=PLAIN):
    h = a.get_matrix()
    for b in range(w.iicc):
        ref = m.hch[:, :, b]
        if np.abs(ref).max() == 0:
            assert np.abs(h[:, :, b]).max() == 0, b
            continue
        assert relmax(h[:, :, b], ref) <= tol, b
    acf = a.get_acf()
    if np.abs(m.acf).max() > 0:
        assert relmax(acf, m.acf) <= tol


def test_config0_assembly():
    w = synth.config0()
    a, m = run_both(w)
    check_blocks(a, m, w)
    assert a.launches > 0


def test_small_with_breit_and_swapped_pairs():
    w = synth.small(ns=50, nch=3, mk=3, n_entries=400, breit=True, seed=11)
    assert any(L.icase == 3 for L in w.lists)
    a, m = run_both(w)
    check_blocks(a, m, w)


def test_each_list_kind_separately():
    w = synth.small(ns=45, nch=2, mk=2, n_entries=200, breit=True, seed=21)
    for L in w.lists:
        a, m = run_both(w, [L])
        check_blocks(a, m, w)


def test_ipt_permutation_is_honoured():
    w = synth.small(ns=45, nch=2, mk=2, n_entries=150, breit=False, seed=31)
    L = [x for x in w.lists if x.icase == 2][0]
    rng = np.random.default_rng(0)
    perm = rng.permutation(L.n)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(L.n)
    # store the list scrambled and pass IPT that restores sorted order
    k1, k2, k3, k4, c = (x[perm] for x in (L.k1, L.k2, L.k3, L.k4, L.c))
    ipt = (inv + 1).astype(np.int32)
    a = Assembler(w.t); a.set_orbitals(w.pq, w.ipbs); a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.gen_matrix(L.icase, L.itype, L.kpol, k1, k2, k3, k4, c, ipt=ipt)
    b = Assembler(w.t); b.set_orbitals(w.pq, w.ipbs); b.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    b.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    assert np.array_equal(a.get_matrix(), b.get_matrix())


def test_deterministic_bitwise():
    w = synth.small(ns=45, nch=3, mk=2, n_entries=300, breit=True, seed=41)
    outs = []
    for _ in range(2):
        a, _m = run_both(w)
        outs.append(a.get_matrix())
    assert np.array_equal(outs[0], outs[1])


def test_out_of_range_channel_is_an_error_not_a_fault():
    w = synth.config0()
    a = Assembler(w.t); a.set_orbitals(w.pq, w.ipbs); a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    L = [x for x in w.lists if x.icase == 2][0]
    k1 = L.k1.copy()
    k1[0] = 7 * 32768 + 1  # channel 7 of 2
    with pytest.raises(DbsrgError, match="ERANGE"):
        a.gen_matrix(L.icase, L.itype, L.kpol, k1, L.k2, L.k3, L.k4, L.c)
    # the context stays usable
    a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)


def test_update_hx_matches_oracle():
    w = synth.config0()
    a = Assembler(w.t); a.set_orbitals(w.pq, w.ipbs); a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    g = O.Grid(w.t)
    m = O.Matrix(g, w.pq, w.ipbs, w.nch, w.icc, w.mk)
    fppqq = g.array("fppqq")
    for ich in range(1, w.nch + 1):
        a.update_hx(ich, ich, fppqq, 1.0)
    a.update_hx(1, 2, fppqq * 0.5, 2.0)
    ref = np.zeros_like(m.hch)
    for ich in range(1, w.nch + 1):
        ref[:, :, w.icc[ich - 1, ich - 1] - 1] += fppqq
    ref[:, :, w.icc[0, 1] - 1] += (2.0 * (0.5 * fppqq)).T
    assert relmax(a.get_matrix(), ref) <= TIGHT
