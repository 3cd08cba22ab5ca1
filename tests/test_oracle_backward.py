"""The oracle's energy functional and gradient (CPU, no GPU): the energy
equals the sum of rk (dbsr_lib_dbs.f90:3981-4022) values, and the gradient
built from the pair-density potentials matches central finite differences."""
import numpy as np

from dbsr_gb300 import synth
from oracle import oracle as O


def test_oracle_energy_is_sum_of_rk_and_gradient_matches_fd():
    w = synth.energy_workload("tiny energy", 31, 40, 8.0, 6.0, 4, 3, 10)
    g = O.Grid(w.t, w.ks, w.ksp, w.ksq)
    E, G = g.rk_energy_grad(w.k, w.i1, w.i2, w.i3, w.i4, w.coef, w.pq)
    ref = sum(w.coef[e] * g.rk(w.pq[:, :, w.i1[e] - 1], w.pq[:, :, w.i2[e] - 1],
                               w.pq[:, :, w.i3[e] - 1], w.pq[:, :, w.i4[e] - 1], int(w.k[e]))
              for e in range(len(w.coef)))
    assert abs(E - ref) <= 1e-13 * abs(ref)
    scale = np.abs(w.pq).max()
    worst = 0.0
    for f in np.argsort(-np.abs(G).ravel(order="F"))[:6]:
        idx = np.unravel_index(f, G.shape, order="F")
        h = 1e-6 * scale  # central differences, step 1e-6 of the coefficient scale
        p1 = w.pq.copy(order="F"); p1[idx] += h
        p2 = w.pq.copy(order="F"); p2[idx] -= h
        fd = (g.rk_energy_grad(w.k, w.i1, w.i2, w.i3, w.i4, w.coef, p1, grad=False)[0] -
              g.rk_energy_grad(w.k, w.i1, w.i2, w.i3, w.i4, w.coef, p2, grad=False)[0]) / (2 * h)
        worst = max(worst, abs(fd - G[idx]))
    assert worst <= 1e-7 * np.abs(G).max()
