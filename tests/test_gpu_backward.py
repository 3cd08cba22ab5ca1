"""Energy functional E = sum c R^k(a,b;c,d) and its gradient on the GPU
(dbsrg_backward) against the CPU oracle (rk, dbsr_lib_dbs.f90:3981-4022, and
the potentials of the pair densities) and against central finite
differences at the 300-spline, 30-orbital, 5e4-entry size."""
import numpy as np
import pytest

from dbsr_gb300 import Assembler, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def assembler(w):
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    return a


def test_backward_matches_oracle_small():
    w = synth.energy_workload("small energy", 77, 60, 12.0, 8.0, 6, 4, 60)
    a = assembler(w)
    E, G = a.backward(w.k, w.i1, w.i2, w.i3, w.i4, w.coef)
    g = O.Grid(w.t, w.ks, w.ksp, w.ksq)
    Er, Gr = g.rk_energy_grad(w.k, w.i1, w.i2, w.i3, w.i4, w.coef, w.pq)
    a.close()
    assert abs(E - Er) <= 1e-12 * max(abs(Er), 1.0)
    assert np.abs(G - Gr).max() <= 1e-12 * np.abs(Gr).max()


def test_backward_recomputes_moments_identically():
    w = synth.energy_workload("small energy", 78, 60, 12.0, 8.0, 5, 3, 40)
    a = assembler(w)
    E1, G1 = a.backward(w.k, w.i1, w.i2, w.i3, w.i4, w.coef)
    a.release_tables()  # moments, diagonal cells and pair potentials rebuilt
    E2, G2 = a.backward(w.k, w.i1, w.i2, w.i3, w.i4, w.coef)
    a.close()
    assert E1 == E2
    assert np.array_equal(G1, G2)


def test_backward_finite_differences_config4():
    w = synth.config4()
    a = assembler(w)
    E, G = a.backward(w.k, w.i1, w.i2, w.i3, w.i4, w.coef)
    rng = np.random.default_rng(5)
    # coefficients with sizeable gradients and a few random ones
    flat = np.argsort(-np.abs(G).ravel(order="F"))[:12].tolist()
    flat += rng.integers(0, G.size, 8).tolist()
    scale = np.abs(w.pq).max()
    worst = 0.0
    for f in flat:
        idx = np.unravel_index(f, G.shape, order="F")
        h = 1e-6 * scale  # central differences, step 1e-6 of the coefficient scale
        vals = []
        for s in (+1, -1):
            p = w.pq.copy(order="F")
            p[idx] += s * h
            a.set_orbitals(p, w.ipbs)
            vals.append(a.backward(w.k, w.i1, w.i2, w.i3, w.i4, w.coef, grad=False)[0])
        fd = (vals[0] - vals[1]) / (2 * h)
        worst = max(worst, abs(fd - G[idx]))
    a.close()
    assert worst <= 1e-7 * np.abs(G).max(), worst / np.abs(G).max()


def test_backward_finite_differences_config4_wide():
    """Central differences on 220 gradient entries of the config-4 size
    (300 splines, 30 orbitals, Z = 18, k = 0..8, 5e4 entries): the 80
    largest P and the 60 largest Q components, 40 of middle magnitude and
    40 random ones.  Every entry within 1e-7 of max|G|; entries with
    |G| >= 1e-3 max|G| also within 1e-6 of their own value."""
    w = synth.config4()
    a = assembler(w)
    E, G = a.backward(w.k, w.i1, w.i2, w.i3, w.i4, w.coef)
    gmax = np.abs(G).max()
    rng = np.random.default_rng(11)
    ns, _, nb = G.shape
    order = np.argsort(-np.abs(G).ravel(order="F"))
    comp = np.unravel_index(order, G.shape, order="F")[1]
    pick = order[comp == 0][:80].tolist() + order[comp == 1][:60].tolist()
    mid = order[(np.abs(G).ravel(order="F")[order] < 1e-2 * gmax) &
                (np.abs(G).ravel(order="F")[order] > 1e-5 * gmax)]
    pick += rng.choice(mid, min(40, mid.size), replace=False).tolist()
    pick += rng.integers(0, G.size, 40).tolist()
    assert len(pick) >= 200
    scale = np.abs(w.pq).max()
    h = 1e-6 * scale
    worst_abs, worst_rel, nq = 0.0, 0.0, 0
    for f in pick:
        idx = np.unravel_index(f, G.shape, order="F")
        nq += idx[1] == 1
        vals = []
        for sgn in (+1, -1):
            p = w.pq.copy(order="F")
            p[idx] += sgn * h
            a.set_orbitals(p, w.ipbs)
            vals.append(a.backward(w.k, w.i1, w.i2, w.i3, w.i4, w.coef, grad=False)[0])
        fd = (vals[0] - vals[1]) / (2 * h)
        worst_abs = max(worst_abs, abs(fd - G[idx]) / gmax)
        if abs(G[idx]) >= 1e-3 * gmax:
            worst_rel = max(worst_rel, abs(fd - G[idx]) / abs(G[idx]))
    a.close()
    assert nq >= 60
    assert worst_abs <= 1e-7, worst_abs
    assert worst_rel <= 1e-6, worst_rel


def test_autograd_function():
    torch = pytest.importorskip("torch")
    from dbsr_gb300.autograd import RkEnergy

    w = synth.energy_workload("small energy", 79, 60, 12.0, 8.0, 5, 3, 30)
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    pq = torch.tensor(np.ascontiguousarray(w.pq), dtype=torch.float64, requires_grad=True)
    E = RkEnergy.apply(pq, a, w.k, w.i1, w.i2, w.i3, w.i4, w.coef)
    E.backward()
    a.set_orbitals(w.pq, w.ipbs)
    Er, Gr = a.backward(w.k, w.i1, w.i2, w.i3, w.i4, w.coef)
    a.close()
    assert abs(E.item() - Er) == 0.0
    assert np.array_equal(pq.grad.numpy(), np.ascontiguousarray(Gr))


def test_rk_on_reference_orbitals_pinned_by_configuration_energies(golden):
    """The GPU energy functional on the reference's own DHF orbitals (B 2p-/2p
    and four Fe runs, 3d-/3d) against the second differences of the
    configuration energies DBSR_HF prints (the pin of config_energy.py)."""
    import config_energy as CE

    n = 0
    for rec in golden["configs"]:
        lm, lp = CE.CASES[rec["log"]]
        t, pq, labels = CE.bsw_orbitals(rec["orbitals"])
        b = rec["orbitals"]
        a = Assembler(t, b["ks"], b["ksp"], b["ksq"])
        a.set_orbitals(pq, np.zeros(pq.shape[2], dtype=np.int32))
        ent = CE.second_coefficient_entries(labels.index(lm) + 1, labels.index(lp) + 1, lm, lp)
        val, _ = a.backward(*ent, grad=False)
        a.close()
        for key, r in CE.reference_second_coefficients(rec["energies"], lm, lp):
            assert abs(val - r) <= 2e-11, (rec["log"], key, val, r)
            n += 1
    assert n == 13
