"""The CPU oracle against the reference's own shipped numbers (no GPU).

* knot sequences of knot.dat / <name>.knot reproduced by the mkgrid_01
  restatement digit for digit at the printed precision (D24.16);
* R^k table dimensions through the table-memory lines of the reference
  logs (memory_DBS_integrals, dbsr_lib_dbs.f90:1619-1620);
* structural identities of the tables and an independent numpy restatement
  of the cell quadrature for sampled table elements.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O


def test_knots_reproduce_reference_files(golden):
    for k in golden["knots"]:
        z, hi = k["atomic_number"], k["hi"]
        hs = hi / z if k["nuclear"] == "point" else 4.0 * math.log(3.0) * k["a_fermi"] * hi
        ns, t = O.mkgrid_01(k["ks"], k["ml"], hs, k["he"], k["hmax"], k["rmax"])
        assert ns == k["ns"], k["file"]
        for a, b in zip(t, k["t"]):
            assert f"{a:.15e}" == f"{b:.15e}", (k["file"], a, b)


def _memory_mb(ns, ks, kmin, kmax, ntype):
    # memory_DBS_integrals expression, dbsr_lib_dbs.f90:1619-1620, with the
    # table shape produced by the oracle's mrk
    return ((kmax - kmin + 1) * ntype * 4 + ns * ns * ks * ks * (kmax - kmin + 1) * ntype * 8) / (
        1024.0 * 1024.0)


def test_table_memory_matches_reference_logs(golden):
    t = O.mkgrid_01(9, 1, 0.25 / 10.0, 0.25, 1.0, 5.0)[1]
    g = O.Grid(t)
    tab = g.mrk(0, 0)
    assert tab.shape == (g.ns, g.ns, g.ks, g.ks)
    m = golden["mat_memory"]
    val = float(m["line"].split(":")[1].split()[0])
    assert round(_memory_mb(m["ns"], m["ks"], 0, m["kmax"], m["ntype"]), 2) == val
    for h in golden["hf"]:
        assert round(_memory_mb(h["bsw"]["ns"], 9, 0, h["kmax"], 4), 2) == h["memory_mb"]


def test_gauleg_matches_legendre():
    x, w = O.gauleg(9)
    xr, wr = np.polynomial.legendre.leggauss(9)
    assert np.allclose(x, 0.5 * (xr + 1), atol=1e-15)
    assert np.allclose(w, 0.5 * wr, atol=1e-15)


@pytest.fixture(scope="module")
def grid():
    from dbsr_gb300 import synth

    return O.Grid(synth.knots(40, 12.0, 6.0))


def test_rk_table_electron_swap_symmetry(grid):
    # R^k(i,j;i',j') = R^k(j,i;j',i'): pppp/qqqq are symmetric under the
    # swap of the two electrons, pqpq and qpqp are each other's swap
    for k in (0, 1, 3):
        pp = grid.mrk(0, k)
        assert np.allclose(pp, pp.transpose(1, 0, 3, 2), rtol=1e-13, atol=1e-300)
        qq = grid.mrk(1, k)
        assert np.allclose(qq, qq.transpose(1, 0, 3, 2), rtol=1e-13, atol=1e-300)
        pq = grid.mrk(2, k)
        qp = grid.mrk(3, k)
        assert np.allclose(pq, qp.transpose(1, 0, 3, 2), rtol=1e-13, atol=1e-300)


def test_rk_table_against_numpy_cell_quadrature(grid):
    """Independent numpy evaluation of rkb elements by the cell rule:
    off-diagonal cells from products of 1-D Gauss moments, diagonal cells
    from the nested rule (inner Gauss on [t_iv, r])."""
    from dbsr_gb300 import synth

    g = grid
    t = g.array("t")
    ks, ksp = g.ks, g.ksp
    k = 2
    tab = g.mrk(0, k)
    xg, wg = np.polynomial.legendre.leggauss(ks)
    xg, wg = 0.5 * (xg + 1), 0.5 * wg
    nv = g.nv

    def B(x):  # P basis values (len(x), nsp)
        return synth._basis_at(t, ks, ksp, np.atleast_1d(x))

    def cell_points(iv):
        a, b = t[ks - 1 + iv], t[ks + iv]
        return a + (b - a) * xg, (b - a) * wg

    rng = np.random.default_rng(5)
    for _ in range(25):
        i = int(rng.integers(0, g.nsp)); j = int(rng.integers(0, g.nsp))
        ip = int(rng.integers(0, ksp)); jp = int(rng.integers(0, ksp))
        i2, j2 = i + ip, j + jp
        if i2 >= g.nsp or j2 >= g.nsp:
            continue
        val = 0.0
        for iv in range(max(0, i2 - ksp + 1), min(nv, i + 1)):
            r1, w1 = cell_points(iv)
            b1 = B(r1)
            f1 = b1[:, i] * b1[:, i2]
            for jv in range(max(0, j2 - ksp + 1), min(nv, j + 1)):
                r2, w2 = cell_points(jv)
                b2 = B(r2)
                f2 = b2[:, j] * b2[:, j2]
                if iv < jv:
                    val += np.sum(w1 * f1 * r1 ** k) * np.sum(w2 * f2 * r2 ** (-k - 1))
                elif iv > jv:
                    val += np.sum(w2 * f2 * r2 ** k) * np.sum(w1 * f1 * r1 ** (-k - 1))
                else:
                    a0 = t[ks - 1 + iv]
                    s = 0.0
                    for ro, wo, fo, fi_ in ((r1, w1, f1, (j, j2)), (r2, w2, f2, (i, i2))):
                        for m in range(ks):
                            ri = a0 + (ro[m] - a0) * xg
                            wi = (ro[m] - a0) * wg
                            bi = B(ri)
                            inner = np.sum(wi * bi[:, fi_[0]] * bi[:, fi_[1]] * ri ** k)
                            s += wo[m] * fo[m] * ro[m] ** (-k - 1) * inner
                    val += s
        ref = tab[i, j, ip, jp]
        assert abs(val - ref) <= 1e-12 * max(abs(ref), 1e-30) + 1e-300, (i, j, ip, jp, val, ref)


def test_sort_merge_matches_insertion_semantics():
    from dbsr_gb300 import synth

    rng = np.random.default_rng(1)
    n = 3000
    k1 = rng.integers(1, 30, n) * 32768 + rng.integers(1, 30, n)
    k2 = rng.integers(1, 6, n)
    k3 = rng.integers(1, 6, n)
    k4 = np.zeros(n, int)
    c = rng.uniform(-1, 1, n)
    a = O.sort_merge(k1, k2, k3, k4, c)
    b = synth.sort_merge(k1, k2, k3, k4, c)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    # a direct emulation of the binary-search insertion of Add_cdata
    keys, vals = [], []
    import bisect

    for e in range(n):
        key = (int(k1[e]), int(k2[e]), int(k3[e]), 0)
        p = bisect.bisect_left(keys, key)
        if p < len(keys) and keys[p] == key:
            vals[p] = vals[p] + c[e]
        else:
            keys.insert(p, key)
            vals.insert(p, c[e])
    assert np.array_equal(np.array([kk[0] for kk in keys]), a[0])
    assert np.array_equal(np.array(vals), a[4])


def test_oracle_config0_runs_and_is_symmetric():
    from dbsr_gb300 import synth

    w = synth.config0()
    g = O.Grid(w.t)
    m = O.Matrix(g, w.pq, w.ipbs, w.nch, w.icc, w.mk)
    for L in w.lists:
        m.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    assert np.isfinite(m.hch).all() and np.abs(m.hch).max() > 0
    # diagonal channel blocks receive y/2 + (y/2)^T: they are symmetric
    for ich in range(1, w.nch + 1):
        b = m.hch[:, :, w.icc[ich - 1, ich - 1] - 1]
        assert np.allclose(b, b.T, rtol=0, atol=1e-15 * np.abs(b).max())


def test_threej_against_sympy():
    sympy = pytest.importorskip("sympy")
    from sympy.physics.wigner import wigner_3j

    import config_energy as CE

    for j1, k, j2 in ((3, 2, 3), (5, 2, 5), (5, 4, 5), (3, 2, 5), (3, 4, 5), (1, 2, 3)):
        ref = wigner_3j(sympy.Rational(j1, 2), k, sympy.Rational(j2, 2), sympy.Rational(1, 2), 0,
                        sympy.Rational(-1, 2)) ** 2
        assert CE.threej_sq(j1, 2 * k, j2, 1, 0, -1) == sympy.Rational(ref)


def test_rk_pinned_by_configuration_energies(golden):
    """R^k of the reference's own DHF orbitals (B 2p-/2p; Fe 3d-/3d, four
    runs) against the second differences of the configuration energies the
    DBSR_HF logs print (27 energies, 13 second differences)."""
    import config_energy as CE

    n = 0
    for rec in golden["configs"]:
        lm, lp = CE.CASES[rec["log"]]
        t, pq, labels = CE.bsw_orbitals(rec["orbitals"])
        b = rec["orbitals"]
        g = O.Grid(t, b["ks"], b["ksp"], b["ksq"])
        ent = CE.second_coefficient_entries(labels.index(lm) + 1, labels.index(lp) + 1, lm, lp)
        a, _ = g.rk_energy_grad(*ent, pq, grad=False)
        refs = CE.reference_second_coefficients(rec["energies"], lm, lp)
        assert refs, rec["log"]
        for key, r in refs:
            assert abs(a - r) <= 2e-11, (rec["log"], key, a, r)
            n += 1
    assert n == 13
