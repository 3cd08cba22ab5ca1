"""GPU parity against the CPU oracle at the shape the headline metric is
quoted on: 400 B-splines to r_max = 40 a.u., Z = 26 with the first knot at
0.25/Z (values spanning many decades near the nucleus), 20 bound orbitals,
R^k for k = 0..10 and S^k up to v = 11.

Tables and diagonal cells: 1e-14 of the largest element (same operation
order as the oracle).  Assembled blocks: a sample of the lists (R^k direct
and exchange at k = 0, 5, 10; S^k structures 6 and 8 of both PQ types at
v = 5 and 11; three segments of each -- the first, the middle and the last
channel pair -- plus the overlap list) in
all three forms, per block against the oracle's assembly of the same
lists: max relative error max|d|/max|ref| and RMS relative error
||d||_2/||ref||_2, at most 1e-12 for the FP64 forms (the plain bar) and
1e-10 for the split-BF16 form (the precision form's bar).
"""
import numpy as np
import pytest

from dbsr_gb300 import FACTOR_FP64, PLAIN_FP64, RK, SK, SPLIT_BF16, Assembler, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TIGHT = 1e-14


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def wl():
    return synth.config1_shape()


@pytest.fixture(scope="module")
def pair(wl):
    a = Assembler(wl.t, wl.ks, wl.ksp, wl.ksq)
    yield a, O.Grid(wl.t, wl.ks, wl.ksp, wl.ksq)
    a.close()


@pytest.mark.parametrize("typ", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("k", [0, 8, 10])
def test_diag_cells_config1(pair, typ, k):
    a, g = pair
    assert relmax(a.get_diag_cells(typ, k), g.triang(typ, k)) <= TIGHT


@pytest.mark.parametrize("which", [0, 1, 2, 3])
@pytest.mark.parametrize("k", [10, -11])
def test_moments_config1(pair, which, k):
    a, g = pair
    assert relmax(a.get_moments(which, k), g.moments(which, k)) <= TIGHT


@pytest.mark.parametrize("typ", [0, 1, 2, 3])
@pytest.mark.parametrize("k", [0, 8, 10])
def test_rk_tables_config1(pair, typ, k):
    a, g = pair
    assert relmax(a.get_table(RK, typ, k), g.mrk(typ, k)) <= TIGHT


@pytest.mark.parametrize("typ", [0, 1])
@pytest.mark.parametrize("k", [0, 10, 11])
def test_sk_tables_config1(pair, typ, k):
    a, g = pair
    assert relmax(a.get_table(SK, typ, k), g.msk(typ, k)) <= TIGHT


def sampled_lists(w):
    """Three segments (runs of one K1: first, middle, last) of the sampled
    lists, in list order."""
    want = {(2, 3, k) for k in (0, 5, 10)} | {(2, 4, k) for k in (0, 5, 10)}
    want |= {(3, it, v) for it in (6, 8, 16, 18) for v in (5, 11)}
    out = []
    for L in w.lists:
        if L.icase == 0:
            out.append(L)
            continue
        if (L.icase, L.itype, L.kpol) not in want:
            continue
        starts = np.flatnonzero(np.r_[True, L.k1[1:] != L.k1[:-1]])
        ends = np.r_[starts[1:], L.n]
        pick = sorted({0, starts.size // 2, starts.size - 1})
        s = np.concatenate([np.arange(starts[i], ends[i]) for i in pick])
        out.append(synth.CList(L.icase, L.itype, L.kpol, L.k1[s], L.k2[s], L.k3[s], L.k4[s],
                               L.c[s]))
    assert len(out) == 1 + 6 + 8
    return out


@pytest.fixture(scope="module")
def oracle_blocks(wl):
    lists = sampled_lists(wl)
    g = O.Grid(wl.t, wl.ks, wl.ksp, wl.ksq)
    m = O.Matrix(g, wl.pq, wl.ipbs, wl.nch, wl.icc, wl.mk)
    for L in lists:
        m.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    return lists, m.hch.copy(order="F"), m.acf.copy(order="F")


@pytest.mark.parametrize("precision,tol", [(PLAIN_FP64, 1e-12), (FACTOR_FP64, 1e-12),
                                           (SPLIT_BF16, 1e-10)])
def test_sampled_blocks_against_oracle_config1(wl, oracle_blocks, precision, tol):
    lists, ref, racf = oracle_blocks
    a = Assembler(wl.t, wl.ks, wl.ksp, wl.ksq)
    a.set_orbitals(wl.pq, wl.ipbs)
    a.alloc_matrix(wl.nch, wl.icc, wl.iicc, wl.mk)
    a.set_precision(precision)
    for L in lists:
        a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    h, acf = a.get_matrix(), a.get_acf()
    a.close()
    rows = []
    for b in range(wl.iicc):
        r = ref[:, :, b]
        if not np.abs(r).max() > 0:
            assert not np.abs(h[:, :, b]).max() > 0, b
            continue
        d = h[:, :, b] - r
        emax = np.abs(d).max() / np.abs(r).max()
        erms = np.sqrt((d * d).sum() / (r * r).sum())
        rows.append((b + 1, emax, erms))
    print(f"\nprecision {precision}: block, max rel, rms rel")
    for b, e1, e2 in rows:
        print(f"  {b:3d} {e1:.3e} {e2:.3e}")
    worst = max(e for _, e, _ in rows)
    assert worst <= tol, rows
    assert max(e for _, _, e in rows) <= tol
    assert relmax(acf, racf) <= 1e-12
