"""The list producer (dbsrg_lists_*: Add_integral, Idef_*, Add_cdata, Add_matrix)
against the Python restatement of the reference routines with Add_cdata's
literal binary-search insertion (oracle/lists.py): every (kpol, itype) list
equal key for key and coefficient for coefficient (equal keys are summed in
arrival order by both), for R, S, O and L coefficients with every structure
(bound-bound, bound-channel, channel-channel, overlap factors) and repeated
integrals.  The GPU test assembles the produced R and S lists and compares
the matrix with the oracle's assembly of the oracle's lists."""
import numpy as np
import pytest

from dbsr_gb300 import synth
from dbsr_gb300.api import Lists
from oracle import lists as OL

IBO = 2 ** 15


def _orbitals(w):
    kap = list(w.kappa_bound) + list(w.kappa_ch)
    lbs = np.array([synth.l_kappa(k) for k in kap], dtype=np.int32)
    return np.asarray(w.ipbs, dtype=np.int32), lbs, np.array(kap, dtype=np.int32)


def _records(rng, w, n, mk, structures=True):
    """Decoded coefficients: random orbitals (bound and channel), multipoles,
    coefficients, and (ic, jc, io, jo) patterns of every structure, a fifth
    of them repeated to exercise the merging."""
    nb, nbf, nch = w.nbound, w.nbf, w.nch
    k = rng.integers(0, mk + 2, n)
    orb = rng.integers(1, nbf + 1, (4, n))
    c = rng.uniform(-1, 1, n)
    ic = np.zeros(n, np.int32)
    jc = np.zeros(n, np.int32)
    io = np.zeros(n, np.int32)
    jo = np.zeros(n, np.int32)
    if structures:
        kind = rng.integers(0, 6, n)
        pair = lambda: int(rng.integers(1, nb + 1)) * IBO + int(rng.integers(1, nb + 1))
        for e in range(n):
            if kind[e] == 1:  # bound-bound: only bound orbitals, two configurations
                orb[:, e] = rng.integers(1, nb + 1, 4)
                ic[e], jc[e] = sorted(rng.integers(1, 5, 2), reverse=True)
            elif kind[e] == 2:  # bound-channel, one channel orbital
                orb[:, e] = rng.integers(1, nb + 1, 4)
                orb[int(rng.integers(0, 4)), e] = nb + int(rng.integers(1, nch + 1))
                ic[e] = int(rng.integers(1, 5))
            elif kind[e] == 3:  # one overlap factor
                io[e] = pair()
            elif kind[e] == 4:  # two overlap factors, bound orbitals only
                orb[:, e] = rng.integers(1, nb + 1, 4)
                io[e], jo[e] = pair(), pair()
    # channel-channel records: one channel orbital in the bra and one in the
    # ket, (i1,i3), (i2,i4), (i1,i4) or (i2,i3) (any other placement is not a
    # structure of Idef_Rtype / Idef_itype)
    valid = [(0, 2), (1, 3), (0, 3), (1, 2)]
    for e in range(n):
        if ic[e] == 0 and io[e] == 0:
            a, b = valid[int(rng.integers(0, 4))]
            orb[a, e] = nb + int(rng.integers(1, nch + 1))
            orb[b, e] = nb + int(rng.integers(1, nch + 1))
            for q in range(4):
                if q not in (a, b):
                    orb[q, e] = int(rng.integers(1, nb + 1))
    rep = rng.choice(n, n // 5)
    cat = lambda x: np.concatenate([x, x[rep]])
    c2 = np.concatenate([c, rng.uniform(-1, 1, rep.size)])
    return (cat(k), cat(orb[0]), cat(orb[1]), cat(orb[2]), cat(orb[3]), c2, cat(ic), cat(jc),
            cat(io), cat(jo))


def _compare(icase, w, recs, mk):
    ipbs, lbs, kbs = _orbitals(w)
    prod = Lists(icase, ipbs, lbs, kbs, mk)
    prod.add(*recs)
    orc = OL.Lists(icase, ipbs, lbs, kbs, mk)
    for e in range(len(recs[5])):
        orc.add_integral(*[x[e].item() for x in recs])
    keys = orc.keys()
    assert keys, "no lists produced"
    total = 0
    for kp, it in keys:
        ref = orc.get(kp, it)
        got = prod.get(kp, it)
        assert len(got[0]) == len(ref), (kp, it)
        for j in range(4):
            assert np.array_equal(got[j], [e[j] for e in ref]), (kp, it, j)
        assert np.array_equal(got[4], np.array([e[4] for e in ref])), (kp, it)
        total += len(ref)
    # and nothing beyond the oracle's lists
    for kp in range(-1, mk + 3):
        for it in range(0, 30):
            if (kp, it) not in keys:
                assert len(prod.get(kp, it)[0]) == 0, (kp, it)
    prod.close()
    return total


def test_decode_follows_the_bank_bit_layout():
    rng = np.random.default_rng(1)
    n = 500
    jcase, kpol = rng.integers(0, 4, n), rng.integers(0, 1024, n)
    i = rng.integers(0, 32, (4, n))
    i[0] = rng.integers(0, 16, n)  # a 4-byte code holds i1 < 16
    code = ((((i[0] * 32 + i[1]) * 32 + i[2]) * 32 + i[3]) * 1024 + kpol) * 4 + jcase
    out = Lists.decode(code)
    for got, ref in zip(out, (jcase, kpol, i[0], i[1], i[2], i[3])):
        assert np.array_equal(got, ref)


@pytest.mark.parametrize("icase", [2, 3])
def test_r_and_s_lists_match_the_insertion_oracle(icase):
    w = synth.small(ns=40, nch=4, mk=3, n_entries=10, breit=False, seed=5, norb=6)
    rng = np.random.default_rng(10 + icase)
    n = _compare(icase, w, _records(rng, w, 1500, 3), 3)
    assert n > 200


def _records_ol(rng, w, n, icase):
    """Overlap (icase 0) and one-electron (icase 1) coefficients of every
    structure Idef_Otype / Idef_Ltype accept (idef_type.f90:2-137)."""
    nb, nbf, nch = w.nbound, w.nbf, w.nch
    pair = lambda: int(rng.integers(1, nb + 1)) * IBO + int(rng.integers(1, nb + 1))
    recs = [[] for _ in range(10)]
    for _ in range(n):
        i1, i3 = (int(x) for x in rng.integers(1, nb + 1, 2))
        ic = jc = io = jo = 0
        kind = int(rng.integers(0, 6 if icase == 1 else 4))
        if kind == 0:
            ic, jc = sorted((int(x) for x in rng.integers(1, 5, 2)), reverse=True)
        elif kind == 1:
            ic, io = int(rng.integers(1, 5)), pair()
        elif kind == 2:
            io, jo = pair(), pair()
        elif kind == 3:
            io = pair()
            if icase == 1 and rng.uniform() < 0.5:
                i1 = nb + int(rng.integers(1, nch + 1))  # one channel orbital
        elif kind == 4:  # L: no factor, any two orbitals
            i1, i3 = (int(x) for x in rng.integers(1, nbf + 1, 2))
        else:  # L: one configuration, one channel orbital
            ic = int(rng.integers(1, 5))
            i3 = nb + int(rng.integers(1, nch + 1))
        for lst, v in zip(recs, (0, i1, 0, i3, 0, float(rng.uniform(-1, 1)), ic, jc, io, jo)):
            lst.append(v)
    out = [np.array(x, dtype=np.float64 if q == 5 else np.int64) for q, x in enumerate(recs)]
    rep = rng.choice(n, n // 5)
    return tuple(np.concatenate([x, x[rep]]) for x in out)


@pytest.mark.parametrize("icase", [0, 1])
def test_overlap_and_one_electron_lists_match_the_insertion_oracle(icase):
    w = synth.small(ns=40, nch=3, mk=1, n_entries=10, breit=False, seed=6, norb=5)
    rng = np.random.default_rng(20 + icase)
    n = _compare(icase, w, _records_ol(rng, w, 800, icase), 0)
    assert n > 50


@pytest.mark.gpu
def test_produced_lists_assemble_like_the_oracle():
    from dbsr_gb300 import PLAIN_FP64, Assembler
    from oracle import oracle as orc

    w = synth.small(ns=48, nch=3, mk=3, n_entries=10, breit=False, seed=7, norb=5)
    ipbs, lbs, kbs = _orbitals(w)
    rng = np.random.default_rng(33)
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.set_precision(PLAIN_FP64)
    g = orc.Grid(w.t, w.ks, w.ksp, w.ksq)
    m = orc.Matrix(g, w.pq, w.ipbs, w.nch, w.icc, w.mk)
    for icase in (2, 3):
        recs = _records(rng, w, 600, w.mk, structures=False)
        prod = Lists(icase, ipbs, lbs, kbs, w.mk)
        prod.add(*recs)
        prod.gen_matrix(a)
        prod.close()
        ol = OL.Lists(icase, ipbs, lbs, kbs, w.mk)
        for e in range(len(recs[5])):
            ol.add_integral(*[x[e].item() for x in recs])
        for kp, it in ol.keys():
            if (icase == 2 and it in (3, 4)) or (icase == 3 and it % 10 in (6, 7, 8, 9)):
                ref = ol.get(kp, it)
                m.gen_matrix(icase, it, kp, *[np.array([e[j] for e in ref]) for j in range(5)])
    got = a.get_matrix()
    a.close()
    err = max(np.abs(got[:, :, b] - m.hch[:, :, b]).max() / max(np.abs(m.hch[:, :, b]).max(), 1e-300)
              for b in range(w.iicc))
    assert np.abs(m.hch).max() > 0
    assert err <= 1e-12, err


def test_bad_arguments_are_errors_not_faults():
    import ctypes

    from dbsr_gb300 import DbsrgError, _lib

    L = _lib.load()
    h = ctypes.c_void_p()
    ipbs = np.zeros(4, np.int32)
    lbs = np.zeros(4, np.int32)
    assert L.dbsrg_lists_create(ctypes.byref(h), 5, 4, ipbs.ctypes.data, lbs.ctypes.data, None,
                                3, 1e-10, 1) == -1  # unknown icase
    assert L.dbsrg_lists_create(ctypes.byref(h), 2, 4, ipbs.ctypes.data, None, None, 3, 1e-10,
                                1) == -1  # R lists need lbs
    assert L.dbsrg_lists_create(ctypes.byref(h), 3, 4, ipbs.ctypes.data, lbs.ctypes.data, None,
                                3, 1e-10, 1) == -1  # S lists need kbs
    lists = Lists(2, ipbs, lbs, None, 3)
    one = np.ones(1, np.int32)
    with pytest.raises(DbsrgError):  # orbital 9 of 4
        lists.add(one * 0, one, one, one * 9, one, np.ones(1))
    with pytest.raises(DbsrgError):  # negative multipole
        lists.add(-one, one, one, one, one, np.ones(1))
    with pytest.raises(DbsrgError):  # jc > 0 with ic = 0: no structure
        lists.add(one * 0, one, one, one, one, np.ones(1), ic=one * 0, jc=one)
    assert len(lists.get(0, 1)[0]) == 0
    lists.close()
