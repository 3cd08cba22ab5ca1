"""GPU parity of the list structures that are not channel-pair contractions
against the oracle, through the C ABI: R_data itypes 1/2, S_data ktypes 1-5
and 11-15, L_data itypes 1-3, O_data itypes 1/2/4, every routing of their
K3/K4 codes (UPDATE_HB, UPDATE_HV, UPDATE_HW, Target_h and UPDATE_HX of the
target structures), with perturbers (hcp, hp), targets (htarg, otarg) and
one-electron matrices.  These run in FP64 in every precision form, so the
bar is 1e-12 of the largest element of each block, perturber column and
target matrix -- or, where a structure's sums cancel, 20 times the block's
own sensitivity: the relative change of the oracle's block when the
orbitals are perturbed by 1e-15 relative (the S^k pqqp integrals of this
workload change by 1e-12 relative under that perturbation, so no FP64
evaluation in another order can agree with the oracle better than that).
"""
import numpy as np
import pytest

from dbsr_gb300 import FACTOR_FP64, PLAIN_FP64, SPLIT_BF16, Assembler, DbsrgError, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-12


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def wl():
    return synth.structures_case()


def make_gpu(w, precision=PLAIN_FP64):
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.alloc_perturbers(w.npert, w.icb, w.ibb)
    a.set_targets(w.ntarg, w.iptar, w.iitar, 1)
    a.set_dhl(w.kap_list, w.hd, w.kbs)
    a.set_precision(precision)
    return a


def make_oracle(w):
    g = O.Grid(w.t, w.ks, w.ksp, w.ksq)
    m = O.Matrix(g, w.pq, w.ipbs, w.nch, w.icc, w.mk)
    m.set_perturbers(w.npert, w.icb, w.ibb)
    m.set_targets(w.ntarg, w.iptar, w.iitar, 1)
    m.set_dhl(w.kap_list, w.hd, w.kbs)
    return g, m


def parts(m):
    """The oracle's results as named arrays: blocks, perturber columns,
    hp, htarg, otarg."""
    out = {("hch", b): m.hch[:, :, b] for b in range(m.hch.shape[2])}
    out.update({("hcp", c): m.hcp[:, c] for c in range(m.hcp.shape[1])})
    out.update({("hp",): m.hp, ("htarg",): m.htarg, ("otarg",): m.otarg})
    return out


def sensitivity(w, lists):
    """Relative change of every part of the oracle's result when the
    orbitals are perturbed by 1e-15 relative (seeded)."""
    rng = np.random.default_rng(123)
    pq2 = np.asfortranarray(w.pq * (1.0 + 1e-15 * rng.uniform(-1.0, 1.0, w.pq.shape)))
    w2 = synth.Workload(**{**w.__dict__, "pq": pq2})
    _, m1 = make_oracle(w)
    _, m2 = make_oracle(w2)
    for L in lists:
        m1.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
        m2.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    p1, p2 = parts(m1), parts(m2)
    return {k: (relmax(p2[k], p1[k]) if np.abs(p1[k]).max() > 0 else 0.0) for k in p1}


def compare(a, m, w, lists, tol=TOL):
    sens = sensitivity(w, lists)
    hcp, hp = a.get_perturbers()
    ht, ot = a.get_targets()
    h = a.get_matrix()
    got = {("hch", b): h[:, :, b] for b in range(w.iicc)}
    got.update({("hcp", c): hcp[:, c] for c in range(hcp.shape[1])})
    got.update({("hp",): hp, ("htarg",): ht, ("otarg",): ot})
    for k, r in parts(m).items():
        if np.abs(r).max() == 0:
            assert np.abs(got[k]).max() == 0, k
        else:
            assert relmax(got[k], r) <= max(tol, 20.0 * sens[k]), (k, relmax(got[k], r), sens[k])


def run_both(w, lists, precision=PLAIN_FP64):
    a = make_gpu(w, precision)
    g, m = make_oracle(w)
    for L in lists:
        a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
        m.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    return a, m


def test_each_structure_list_against_oracle(wl):
    seen = set()
    for L in wl.lists:
        a, m = run_both(wl, [L])
        compare(a, m, wl, [L])
        a.close()
        seen.add((L.icase, L.itype))
    assert {(2, 1), (2, 2), (1, 1), (1, 2), (1, 3), (0, 1), (0, 2), (0, 4)} <= seen
    assert {(3, t) for t in (1, 2, 3, 4, 5, 11, 12, 13, 14, 15)} <= seen


@pytest.mark.parametrize("precision", [PLAIN_FP64, FACTOR_FP64, SPLIT_BF16])
def test_every_list_kind_together_in_every_form(precision):
    """The drop-in with the whole mix of Gen_matrix lists: the contraction
    structures (O itype 3, R itypes 3/4, S 6-9) interleaved with all the
    others, in each precision form."""
    w = synth.structures_case(seed=91)
    base = synth.small(ns=w.ns, nch=w.nch, mk=w.mk, n_entries=300, breit=True, seed=91,
                       rmax=20.0, z=8.0, norb=w.nbound)
    lists = []
    for L in base.lists + w.lists:
        lists.append(L)
    lists.sort(key=lambda L: (L.icase, L.kpol, L.itype))  # State_res order per icase
    a, m = run_both(w, lists, precision)
    compare(a, m, w, lists, 1e-10 if precision == SPLIT_BF16 else TOL)
    a.close()


def test_windowed_assembly_adds_perturber_terms_once(wl):
    """Through dbsrg_assemble_to_host (lists once per window): the blocks
    window by window, hcp/hp/htarg/otarg once."""
    a = make_gpu(wl)
    a.alloc_matrix(wl.nch, wl.icc, wl.iicc, wl.mk, window=2)
    a.alloc_perturbers(wl.npert, wl.icb, wl.ibb)
    a.set_targets(wl.ntarg, wl.iptar, wl.iitar, 1)
    out = np.zeros((a.ms, a.ms, wl.iicc), order="F")
    lists = [(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c) for L in wl.lists]
    a.assemble_to_host(lists, out=out, nwin=1)
    g, m = make_oracle(wl)
    for L in wl.lists:
        m.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    sens = sensitivity(wl, wl.lists)
    for b in range(wl.iicc):
        r = m.hch[:, :, b]
        if np.abs(r).max() > 0:
            assert relmax(out[:, :, b], r) <= max(TOL, 20 * sens[("hch", b)]), b
    hcp, hp = a.get_perturbers()
    ht, ot = a.get_targets()
    for k, got in ((("hp",), hp), (("htarg",), ht), (("otarg",), ot)):
        assert relmax(got, parts(m)[k]) <= max(TOL, 20 * sens[k]), k
    for col in range(hcp.shape[1]):
        assert relmax(hcp[:, col], m.hcp[:, col]) <= max(TOL, 20 * sens[("hcp", col)]), col
    a.close()


def test_single_term_updates_against_oracle(wl):
    a = make_gpu(wl)
    g, m = make_oracle(wl)
    rng = np.random.default_rng(5)
    ms = a.ms
    for ich, jch in ((2, 1), (1, 2), (3, 3)):
        v, w_ = rng.uniform(-1, 1, ms), rng.uniform(-1, 1, ms)
        a.update_hw(ich, jch, v, w_, 0.7)
        O.lib().orc_update_hw(m._m, ich, jch, O._d(v), O._d(w_), 0.7)
    v = rng.uniform(-1, 1, ms)
    a.update_hv(2, 3, v, -1.5)
    assert O.lib().orc_update_hv(m._m, 2, 3, O._d(v), -1.5) == 0
    a.update_hb(3, 1, 2.5)
    assert O.lib().orc_update_hb(m._m, 3, 1, 2.5) == 0
    compare(a, m, wl, [])
    with pytest.raises(DbsrgError, match="ERANGE"):
        a.update_hb(4, 1, 1.0)
    a.close()


def test_errors_leave_the_context_usable(wl):
    L = next(L for L in wl.lists if (L.icase, L.itype) == (0, 1))
    a = Assembler(wl.t, wl.ks, wl.ksp, wl.ksq)
    a.set_orbitals(wl.pq, wl.ipbs)
    a.alloc_matrix(wl.nch, wl.icc, wl.iicc, wl.mk)
    with pytest.raises(DbsrgError, match="ERANGE"):  # no perturbers allocated
        a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    Ll = next(L for L in wl.lists if (L.icase, L.itype) == (1, 3))
    with pytest.raises(DbsrgError, match="ESTATE"):  # no one-electron matrices
        a.gen_matrix(Ll.icase, Ll.itype, Ll.kpol, Ll.k1, Ll.k2, Ll.k3, Ll.k4, Ll.c)
    Lr = next(L for L in wl.lists if (L.icase, L.itype) == (2, 2))
    k4 = Lr.k4.copy()
    k4[:] = 0  # io = 0: unknown structure
    a.alloc_perturbers(wl.npert, wl.icb, wl.ibb)
    with pytest.raises(DbsrgError, match="EINVAL"):
        a.gen_matrix(Lr.icase, Lr.itype, Lr.kpol, Lr.k1, Lr.k2, Lr.k3, k4, Lr.c)
    assert np.abs(a.get_matrix()).max() == 0  # nothing of a failed list was added
    a.gen_matrix(Lr.icase, Lr.itype, Lr.kpol, Lr.k1, Lr.k2, Lr.k3, Lr.k4, Lr.c)
    assert np.abs(a.get_perturbers()[0]).max() > 0
    a.close()


def _records(rng, w, icase, n, npert):
    """Decoded coefficients (k, i1..i4, c, ic, jc, io, jo) of every structure
    Idef_Otype / Idef_Ltype / Idef_Rtype / Idef_itype route (idef_type.f90),
    with overlap codes io = (channel orbital, bound orbital) and target codes
    (channel orbital, channel orbital) as Det_fact_new hands them over."""
    nb, nch = w.nbound, w.nch
    IBO = synth.IBO
    b = lambda: int(rng.integers(1, nb + 1))  # noqa: E731
    ch = lambda: nb + int(rng.integers(1, nch + 1))  # noqa: E731
    ovl = lambda: ch() * IBO + b()  # noqa: E731
    tgt = lambda: ch() * IBO + ch()  # noqa: E731
    pert = lambda: sorted((int(x) for x in rng.integers(1, npert + 1, 2)), reverse=True)  # noqa
    out = []
    for _ in range(n):
        k = int(rng.integers(0, w.mk + 1))
        o = [b(), b(), b(), b()]
        ic = jc = io = jo = 0
        if icase in (2, 3):
            kind = int(rng.integers(0, 7))
            if kind == 0:  # channel-channel
                a, bb = ((0, 2), (1, 3), (0, 3), (1, 2))[int(rng.integers(0, 4))]
                o[a], o[bb] = ch(), ch()
            elif kind == 1:
                ic, jc = pert()
            elif kind == 2:
                o[int(rng.integers(0, 4))] = ch()
                ic = pert()[0]
            elif kind == 3:
                o[int(rng.integers(0, 4))] = ch()
                io = ovl()
            elif kind == 4:
                io, jo = ovl(), ovl()
            elif kind == 5:
                ic, io = pert()[0], ovl()
            else:
                io = tgt()
        elif icase == 1:
            kind = int(rng.integers(0, 6))
            if kind == 0:
                ic, jc = pert()
            elif kind == 1:
                ic, io = pert()[0], ovl()
            elif kind == 2:
                io, jo = ovl(), ovl()
            elif kind == 3:
                o[0] = ch()
                io = ovl()
            elif kind == 4:  # L(i j): two channel orbitals of one kappa
                i = ch()
                same = [q for q in range(w.nbound + 1, w.nbf + 1) if w.kbs[q - 1] == w.kbs[i - 1]]
                o[0], o[2] = i, int(rng.choice(same))
            else:
                ic, io = 0, tgt()
            if kind in (0, 1, 2, 5):  # L(. .): two bound orbitals of one kappa
                same = [q for q in range(1, nb + 1) if w.kbs[q - 1] == w.kbs[o[0] - 1]]
                o[2] = int(rng.choice(same))
        else:
            kind = int(rng.integers(0, 4))
            if kind == 0:
                ic, jc = pert()
            elif kind == 1:
                ic, io = pert()[0], ovl()
            elif kind == 2:
                io, jo = ovl(), ovl()
            else:
                io = tgt()
        out.append((k, *o, float(rng.uniform(-1, 1)), ic, jc, io, jo))
    return [np.array([r[q] for r in out], dtype=np.float64 if q == 5 else np.int64)
            for q in range(10)]


def test_produced_lists_of_every_structure_assemble_like_the_oracle():
    """The whole hand-off of State_res (Add_integral, the Idef_* routing,
    Add_cdata merging, Add_matrix -> Gen_matrix) for O, L, R and S
    coefficients of every structure, through dbsrg_lists_* and
    dbsrg_gen_matrix, against the oracle's lists assembled by the oracle."""
    from dbsr_gb300.api import Lists
    from oracle import lists as OL

    w = synth.structures_case(seed=93, npert=4)
    kap = np.asarray(w.kbs, dtype=np.int32)
    lbs = np.array([synth.l_kappa(int(k)) for k in kap], dtype=np.int32)
    ipbs = np.asarray(w.ipbs, dtype=np.int32)
    rng = np.random.default_rng(44)
    a = make_gpu(w)
    g, m = make_oracle(w)
    used = []
    for icase in (0, 1, 2, 3):
        recs = _records(rng, w, icase, 300, w.npert)
        prod = Lists(icase, ipbs, lbs, kap, w.mk)
        prod.add(*recs)
        prod.gen_matrix(a)
        prod.close()
        ol = OL.Lists(icase, ipbs, lbs, kap, w.mk)
        for e in range(len(recs[5])):
            ol.add_integral(*[x[e].item() for x in recs])
        for kp, it in ol.keys():
            ref = ol.get(kp, it)
            L = synth.CList(icase, it, kp, *[np.array([e[j] for e in ref], dtype=np.int32)
                                             for j in range(4)],
                            np.array([e[4] for e in ref]))
            m.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
            used.append(L)
    kinds = {(L.icase, L.itype % 10) for L in used}
    assert {(0, 1), (0, 2), (0, 3), (0, 4), (1, 1), (1, 2), (1, 3), (2, 1), (2, 2), (2, 3),
            (2, 4), (3, 1), (3, 2), (3, 6), (3, 8)} <= kinds, kinds
    compare(a, m, w, used)
    a.close()


def test_core_energy_shift_scales_hch_hcp_hp(wl):
    """SUB1's shifts between the overlap and Hamiltonian passes
    (sub1.f90:96, 222-223) on the device: hch, hcp, hp times Ecore, then more
    lists on top."""
    lists = [L for L in wl.lists if L.icase == 0] + [L for L in wl.lists if L.icase == 2][:2]
    a = make_gpu(wl)
    g, m = make_oracle(wl)
    for L in lists[:3]:
        a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
        m.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    a.scale_matrix(-1.75)
    m.hch *= -1.75
    m.hcp *= -1.75
    m.hp *= -1.75
    for L in lists[3:]:
        a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
        m.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    compare(a, m, wl, lists)
    a.close()
