"""Second differences of Dirac-Fock configuration energies as a pin of the
R^k integrals (test helper).

The average energy of a jj configuration (Grant's average-level formula) is

  E = sum_a q_a I_a
      + sum_a q_a (q_a - 1)/2 [F0(aa) - (2j_a+1)/(2j_a) sum_{k>0} g(a,k,a) F^k(aa)]
      + sum_{a<b} q_a q_b [F0(ab) - sum_k g(a,k,b) G^k(ab)],
  g(a,k,b) = (j_a k j_b; 1/2 0 -1/2)^2 when l_a + k + l_b is even, else 0,

with F^k(ab) = R^k(ab;ab), G^k(ab) = R^k(ab;ba) (rk, dbsr_lib_dbs.f90:
3981-4022).  Along a family of configurations that moves electrons between
the two subshells j- and j+ of one nl shell, everything else fixed, E is a
quadratic in q(j-) whose second coefficient is

  (E(--) + E(++) - 2 E(-+)) / 2

(E(--), E(++) the brackets of the same-subshell pairs, E(-+) of the cross
pairs): one-electron terms and interactions with the other subshells are
linear in q(j-) and drop out.  The DBSR_HF logs print the configuration
energies with the final orbitals of the run, so the second divided
differences of the printed energies pin that combination of R^k integrals
of the run's own orbitals.
"""
from __future__ import annotations

from fractions import Fraction
from math import factorial

import numpy as np

L_OF = {"s": 0, "p": 1, "d": 2, "f": 3}


def subshell(label: str):
    """(l, 2j) of a subshell label such as '3d-' or '2p'."""
    lab = label.strip()
    l = L_OF[lab.rstrip("-")[-1]]
    return l, (2 * l - 1 if lab.endswith("-") else 2 * l + 1)


def threej_sq(j1x2, j2x2, j3x2, m1x2, m2x2, m3x2) -> Fraction:
    """Square of the Wigner 3j symbol by Racah's formula (arguments doubled)."""
    if m1x2 + m2x2 + m3x2 != 0:
        return Fraction(0)
    if not (abs(j1x2 - j2x2) <= j3x2 <= j1x2 + j2x2) or (j1x2 + j2x2 + j3x2) % 2:
        return Fraction(0)
    if any(abs(m) > j for m, j in ((m1x2, j1x2), (m2x2, j2x2), (m3x2, j3x2))):
        return Fraction(0)
    h = lambda x: x // 2  # noqa: E731  (all combinations below are even)
    tri = Fraction(factorial(h(j1x2 + j2x2 - j3x2)) * factorial(h(j1x2 - j2x2 + j3x2)) *
                   factorial(h(-j1x2 + j2x2 + j3x2)), factorial(h(j1x2 + j2x2 + j3x2) + 1))
    pre = (factorial(h(j1x2 + m1x2)) * factorial(h(j1x2 - m1x2)) * factorial(h(j2x2 + m2x2)) *
           factorial(h(j2x2 - m2x2)) * factorial(h(j3x2 + m3x2)) * factorial(h(j3x2 - m3x2)))
    s = Fraction(0)
    for t in range(0, h(j1x2 + j2x2 - j3x2) + 1):
        a = [t, h(j3x2 - j2x2 + m1x2) + t, h(j3x2 - j1x2 - m2x2) + t, h(j1x2 + j2x2 - j3x2) - t,
             h(j1x2 - m1x2) - t, h(j2x2 + m2x2) - t]
        if min(a) < 0:
            continue
        d = 1
        for x in a:
            d *= factorial(x)
        s += Fraction((-1) ** t, d)
    return tri * pre * s * s


def gcoef(la, ja2, k, lb, jb2) -> float:
    if (la + k + lb) % 2:
        return 0.0
    return float(threej_sq(ja2, 2 * k, jb2, 1, 0, -1))


def second_coefficient_entries(im: int, ip: int, lm: str, lp: str):
    """R^k entries (k, i1, i2, i3, i4, coef) whose sum is the quadratic
    coefficient (E(--) + E(++) - 2 E(-+)) / 2 for orbitals im (j-) and ip (j+)
    (1-based indices into pq)."""
    l, jm2 = subshell(lm)
    _, jp2 = subshell(lp)
    ent = []

    def same(i, j2, w):
        ent.append((0, i, i, i, i, w))
        for k in range(2, j2 + 1, 2):
            g = gcoef(l, j2, k, l, j2)
            if g:
                ent.append((k, i, i, i, i, -w * (j2 + 1) / j2 * g))

    same(im, jm2, 0.5)
    same(ip, jp2, 0.5)
    ent.append((0, im, ip, im, ip, -1.0))
    for k in range(abs(jm2 - jp2) // 2, (jm2 + jp2) // 2 + 1):
        g = gcoef(l, jm2, k, l, jp2)
        if g:
            ent.append((k, im, ip, ip, im, +1.0 * g))
    cols = list(zip(*ent))
    return (np.array(cols[0], dtype=np.int32),) + tuple(
        np.array(c, dtype=np.int32) for c in cols[1:5]) + (np.array(cols[5]),)


def reference_second_coefficients(energies, lm: str, lp: str):
    """Quadratic coefficients in q(j-) from every run of three configurations
    of one family (the other occupations and q(j-) + q(j+) fixed)."""
    fam = {}
    for occ, e in energies:
        qm, qp = occ.get(lm.strip(), 0), occ.get(lp.strip(), 0)
        key = (qm + qp, tuple(sorted((k, v) for k, v in occ.items()
                                     if k not in (lm.strip(), lp.strip()))))
        fam.setdefault(key, []).append((qm, e))
    out = []
    for key, pts in fam.items():
        pts.sort()
        for (x0, y0), (x1, y1), (x2, y2) in zip(pts, pts[1:], pts[2:]):
            out.append((key, ((y2 - y1) / (x2 - x1) - (y1 - y0) / (x1 - x0)) / (x2 - x0)))
    return out


def bsw_orbitals(rec):
    """(t, pq(ns,2,norb), labels) of a golden .bsw record."""
    ns = rec["ns"]
    orbs = rec["orbitals"]
    pq = np.zeros((ns, 2, len(orbs)), order="F")
    for i, o in enumerate(orbs):
        pq[: o["mbs"], 0, i] = o["p"][: o["mbs"]]
        pq[: o["mbs"], 1, i] = o["q"][: o["mbs"]]
    return np.array(rec["t"]), pq, [o["label"].strip() for o in orbs]


CASES = {"B.log": ("2p-", "2p"), "Fe/Fe.log": ("3d-", "3d"), "Fe/2.log": ("3d-", "3d"),
         "Fe/3.log": ("3d-", "3d"), "Fe/4.log": ("3d-", "3d")}
