"""Seeded synthetic workloads of the assembly benchmarks.

No public dataset is involved: every input is generated here from a
Philox stream (seed = 1234 + workload id) so that the GPU library and the
CPU oracle see identical data.

Basis: ks=9 knots, P order 8, Q order 9.  Knots: ks-fold zero, one first
interval [0, r_min], a geometric region up to r = 1 a.u., a linear region
with step 0.5 a.u. up to r_max, ks-fold r_max.  With nv = ns-ks+1
intervals, n_lin = 2(r_max-1) and n_exp = nv - n_lin - 1.  The ln-step is
0.1 when that keeps r_min >= 0.25/Z, otherwise ln(Z/0.25)/n_exp, so that
r_min = 0.25/Z (the first-step rule hs = hi/Z of mkgrid_01 with hi=0.25).

Orbitals: l = l(kappa), P = r^(l+1) exp(-Z r/n), Q = (alpha Z/2n) dP/dr,
least-squares projected on the P/Q bases, perturbed by U(-1e-3, 1e-3) and
normalised so that <P|P> + <Q|Q> = 1.  Channel orbitals follow the bound
ones in the orbital list, with zero coefficients and ipbs = channel.

Angular lists: entries (k, structure, channel pair, bound orbitals, c ~
U[-1,1]) routed as in Idef_Rtype / Idef_itype (DBSR_MAT3/idef_type.f90)
and merged like Add_cdata (MOD_c_data.f90:177-236): sorted by (K1,K2,K3,
K4), equal keys summed in arrival order.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

IBO = 32768
ALPHA = 7.297352533e-3  # fine-structure constant, dbsr_lib_zcom.f90:79
TARGET_ORBITALS = [  # (n, kappa) in the usual order
    (1, -1), (2, -1), (2, 1), (2, -2), (3, -1), (3, 1), (3, -2), (3, 2), (3, -3), (4, -1),
    (4, 1), (4, -2), (4, 2), (4, -3), (4, 3), (4, -4), (5, -1), (5, 1), (5, -2), (5, 2),
    (5, -3), (6, -1), (5, 3), (5, -4), (6, 1), (6, -2), (5, 4), (5, -5), (6, 2), (6, -3),
]


def l_kappa(kappa: int) -> int:
    """l of a relativistic orbital (l_kappa, dbsr_lib_zcom.f90:500-512)."""
    return -kappa - 1 if kappa < 0 else kappa


def j2_kappa(kappa: int) -> int:
    return 2 * abs(kappa) - 1


def knots(ns: int, rmax: float, z: float, ks: int = 9, lnstep: float = 0.1) -> np.ndarray:
    nv = ns - ks + 1
    n_lin = int(round(2 * (rmax - 1.0)))
    n_exp = nv - n_lin - 1
    if n_exp < 1:
        raise ValueError("ns too small for rmax")
    if math.exp(-lnstep * n_exp) < 0.25 / z:
        lnstep = math.log(z / 0.25) / n_exp
    pts = [0.0]
    pts += [math.exp(-lnstep * (n_exp - i)) for i in range(n_exp + 1)]  # r_min .. 1
    pts += [1.0 + 0.5 * i for i in range(1, n_lin + 1)]
    assert len(pts) == nv + 1
    t = np.concatenate([np.zeros(ks - 1), np.array(pts), np.full(ks - 1, pts[-1])])
    assert t.size == ns + ks
    return t


def _basis_at(t: np.ndarray, ks: int, kx: int, x: np.ndarray) -> np.ndarray:
    """Values of the order-kx B-splines on the component knots at x:
    (len(x), nv+kx-1), by the Cox-de Boor recursion."""
    ns = t.size - ks
    nv = ns - ks + 1
    nsx = nv + kx - 1
    tx = np.concatenate([np.full(kx, t[0]), t[ks:ns], t[ns:ns + kx]])
    assert tx.size == nsx + kx
    # order-1 indicator on [tx_i, tx_{i+1}) (last interval closed)
    B = np.zeros((x.size, tx.size - 1))
    for i in range(tx.size - 1):
        if tx[i + 1] > tx[i]:
            m = (x >= tx[i]) & (x < tx[i + 1])
            if i + 1 == nsx and True:
                m |= (x == tx[i + 1]) & (tx[i + 1] == tx[-1])
            B[m, i] = 1.0
    for k in range(2, kx + 1):
        Bn = np.zeros((x.size, tx.size - k))
        for i in range(tx.size - k):
            d1 = tx[i + k - 1] - tx[i]
            d2 = tx[i + k] - tx[i + 1]
            a = (x - tx[i]) / d1 * B[:, i] if d1 > 0 else 0.0
            b = (tx[i + k] - x) / d2 * B[:, i + 1] if d2 > 0 else 0.0
            Bn[:, i] = a + b
        B = Bn
    return B[:, :nsx]


def _gauss(t: np.ndarray, ks: int):
    ns = t.size - ks
    nv = ns - ks + 1
    xg, wg = np.polynomial.legendre.leggauss(ks)
    xg = 0.5 * (xg + 1.0)
    wg = 0.5 * wg
    a = t[ks - 1:ks - 1 + nv]
    b = t[ks:ks + nv]
    r = (a[:, None] + (b - a)[:, None] * xg[None, :]).ravel()
    w = ((b - a)[:, None] * wg[None, :]).ravel()
    return r, w


def orbital_coefficients(t, ks, ksp, ksq, z, orbitals, rng) -> np.ndarray:
    """pq(ns,2,nbound) for hydrogenic-shaped orbitals (see module doc)."""
    ns = t.size - ks
    r, w = _gauss(t, ks)
    BP = _basis_at(t, ks, ksp, r)
    BQ = _basis_at(t, ks, ksq, r)
    GP = (BP * w[:, None]).T @ BP
    GQ = (BQ * w[:, None]).T @ BQ
    out = np.zeros((ns, 2, len(orbitals)), order="F")
    for o, (n, kappa) in enumerate(orbitals):
        l = l_kappa(kappa)
        zr = z * r / n
        P = r ** (l + 1) * np.exp(-zr)
        dP = ((l + 1) * r ** l - (z / n) * r ** (l + 1)) * np.exp(-zr)
        Q = (ALPHA * z / (2 * n)) * dP
        cp = np.linalg.solve(GP, BP.T @ (w * P))
        cq = np.linalg.solve(GQ, BQ.T @ (w * Q))
        cp = cp * (1.0 + rng.uniform(-1e-3, 1e-3, cp.size))
        cq = cq * (1.0 + rng.uniform(-1e-3, 1e-3, cq.size))
        nrm = cp @ GP @ cp + cq @ GQ @ cq
        s = 1.0 / math.sqrt(nrm)
        out[: cp.size, 0, o] = cp * s
        out[: cq.size, 1, o] = cq * s
    return out


def sort_merge(k1, k2, k3, k4, c):
    """Add_cdata list semantics: sorted unique keys, duplicates summed in
    arrival order (stable sort + sequential reduction)."""
    k1, k2, k3, k4 = (np.asarray(a, dtype=np.int64) for a in (k1, k2, k3, k4))
    c = np.asarray(c, dtype=np.float64)
    if k1.size == 0:
        z = np.zeros(0, np.int32)
        return z, z, z, z, np.zeros(0)
    order = np.lexsort((k4, k3, k2, k1))  # stable
    s1, s2, s3, s4, sc = k1[order], k2[order], k3[order], k4[order], c[order]
    new = np.ones(s1.size, bool)
    new[1:] = (s1[1:] != s1[:-1]) | (s2[1:] != s2[:-1]) | (s3[1:] != s3[:-1]) | (s4[1:] != s4[:-1])
    starts = np.flatnonzero(new)
    # sequential sum within each run, in arrival order: level l adds the
    # l-th element of every run that is long enough
    ends = np.append(starts[1:], s1.size)
    lens = ends - starts
    out_c = sc[starts].copy()
    for lvl in range(1, int(lens.max())):
        m = lens > lvl
        out_c[m] = out_c[m] + sc[starts[m] + lvl]
    return (s1[starts].astype(np.int32), s2[starts].astype(np.int32),
            s3[starts].astype(np.int32), s4[starts].astype(np.int32), out_c)


@dataclass
class CList:
    """One coefficient list ready for Gen_matrix(icase,itype,kpol)."""
    icase: int
    itype: int
    kpol: int
    k1: np.ndarray
    k2: np.ndarray
    k3: np.ndarray
    k4: np.ndarray
    c: np.ndarray

    @property
    def n(self):
        return int(self.k1.size)


@dataclass
class Workload:
    name: str
    t: np.ndarray
    z: float
    ks: int
    ksp: int
    ksq: int
    nbound: int
    kappa_bound: list
    kappa_ch: list
    pq: np.ndarray            # (ns,2,nbf) bound + channel orbitals
    ipbs: np.ndarray          # (nbf,)
    nch: int
    icc: np.ndarray           # (nch,nch) 1-based block numbers
    iicc: int
    mk: int
    lists: list = field(default_factory=list)  # of CList
    # perturbers (hcp/hp numbering), targets and one-electron matrices, for
    # the workloads that carry the bound-bound and bound-channel structures
    npert: int = 0
    icb: np.ndarray = None    # (nch, npert)
    ibb: np.ndarray = None    # (npert, npert)
    ntarg: int = 0
    iptar: np.ndarray = None  # (nch,)
    iitar: int = 0
    kap_list: np.ndarray = None
    hd: np.ndarray = None     # (ms, ms, nkap)
    kbs: np.ndarray = None    # (nbf,)

    @property
    def ns(self):
        return self.t.size - self.ks

    @property
    def nbf(self):
        return self.pq.shape[2]


def block_numbering(nch: int) -> np.ndarray:
    """icc for all channel pairs: diagonal blocks first, then the lower
    triangle row by row (Alloc_dbsr_matrix with idiag=0, updates.f90:20-37)."""
    icc = np.zeros((nch, nch), dtype=np.int32, order="F")
    i = 0
    for ich in range(nch):
        i += 1
        icc[ich, ich] = i
    for ich in range(1, nch):
        for jch in range(ich):
            i += 1
            icc[ich, jch] = i
            icc[jch, ich] = i
    return icc


def _build(name, seed, ns, rmax, z, orbitals, kappa_ch, mk, n_entries, occupancy, breit,
           o_entries=0):
    rng = np.random.Generator(np.random.Philox(seed))
    ks, ksp, ksq = 9, 8, 9
    t = knots(ns, rmax, z, ks)
    nb = len(orbitals)
    pq_b = orbital_coefficients(t, ks, ksp, ksq, z, orbitals, rng)
    nch = len(kappa_ch)
    pq = np.zeros((ns, 2, nb + nch), order="F")
    pq[:, :, :nb] = pq_b
    ipbs = np.zeros(nb + nch, dtype=np.int32)
    ipbs[nb:] = np.arange(1, nch + 1)
    icc = block_numbering(nch)
    iicc = nch * (nch + 1) // 2
    lb = np.array([l_kappa(k) for _, k in orbitals])
    lc = np.array([l_kappa(k) for k in kappa_ch])
    # occupied (channel pair, k) slots
    pairs = [(i, j) for i in range(1, nch + 1) for j in range(1, i + 1)]
    slots = [(i, j, k) for (i, j) in pairs for k in range(mk + 1)]
    if occupancy >= 1.0:
        occ = slots
    else:
        m = max(1, int(round(occupancy * len(slots))))
        sel = np.sort(rng.choice(len(slots), size=m, replace=False))
        occ = [slots[s] for s in sel]
    chunks = {}  # (icase,itype,kpol) -> list of (k1,k2,k3,c) arrays in arrival order

    def add(key, k1, k2, k3, c):
        if k1.size:
            chunks.setdefault(key, []).append((k1, k2, k3, c))

    per_slot = max(1, n_entries // max(1, len(occ)))
    nkind = 4 if breit else 2
    for (ich, jch, k) in occ:
        li, lj = lc[ich - 1], lc[jch - 1]
        # candidates in one draw; the first per_slot that pass the parity
        # filter of add_integral.f90:30-32 are kept, in draw order
        m = 4 * per_slot + 8
        a = rng.integers(1, nb + 1, size=m)
        b = rng.integers(1, nb + 1, size=m)
        kind = rng.integers(0, nkind, size=m)
        cs = rng.uniform(-1.0, 1.0, size=m)
        vsh = rng.integers(0, 2, size=m)
        at = rng.integers(0, 2, size=m)
        flip = rng.integers(0, 2, size=m)
        la, lb_ = lb[a - 1], lb[b - 1]
        ok = np.where(kind == 0, ((li + lj + k) % 2 == 0) & ((la + lb_ + k) % 2 == 0),
                      np.where(kind == 1, ((li + la + k) % 2 == 0) & ((lb_ + lj + k) % 2 == 0),
                               True))
        sel = np.flatnonzero(ok)[:per_slot]
        a, b, kind, cs, vsh, at, flip = (x[sel] for x in (a, b, kind, cs, vsh, at, flip))
        key_ij = ich * IBO + jch
        # direct R^k(i a; j b): Idef_Rtype itype 3, K2 <= K3
        d = kind == 0
        add((2, 3, k), np.full(d.sum(), key_ij), np.minimum(a, b)[d], np.maximum(a, b)[d], cs[d])
        # exchange R^k(i a; b j): Idef_Rtype itype 4
        x = kind == 1
        add((2, 4, k), np.full(x.sum(), key_ij), a[x], b[x], cs[x])
        # Breit S^v: Idef_itype structures 6 / 8 for atype 0 / 1
        if breit:
            for it, kd in ((6, 2), (8, 3)):
                for atv in (0, 1):
                    for vv in (0, 1):
                        s = (kind == kd) & (at == atv) & (vsh == vv)
                        if not s.any():
                            continue
                        keys = np.where((it == 6) & (flip[s] == 1), jch * IBO + ich, key_ij)
                        add((3, 10 * atv + it, k + vv), keys, a[s], b[s], cs[s])
    lists = []
    for key in sorted(chunks):
        parts = chunks[key]
        k1 = np.concatenate([p[0] for p in parts])
        k2 = np.concatenate([p[1] for p in parts])
        k3 = np.concatenate([p[2] for p in parts])
        c = np.concatenate([p[3] for p in parts])
        k1, k2, k3, k4, c = sort_merge(k1, k2, k3, np.zeros_like(k1), c)
        lists.append(CList(key[0], key[1], key[2], k1, k2, k3, k4, c))
    if o_entries:
        # overlaps <i|.><.|j>: k1 = (channel orbital i, bound a), k2 = (channel orbital j, bound b)
        ch_orb = np.arange(nb + 1, nb + nch + 1)
        r = ([], [], [], [], [])
        for e in range(o_entries):
            i = int(rng.integers(0, nch)); j = int(rng.integers(0, nch))
            a = int(rng.integers(1, nb + 1)); b = int(rng.integers(1, nb + 1))
            r[0].append(int(ch_orb[i]) * IBO + a); r[1].append(int(ch_orb[j]) * IBO + b)
            r[2].append(0); r[3].append(0); r[4].append(float(rng.uniform(-1, 1)))
        k1, k2, k3, k4, c = sort_merge(*r)
        lists.insert(0, CList(0, 3, 0, k1, k2, k3, k4, c))
    return Workload(name, t, z, ks, ksp, ksq, nb, [k for _, k in orbitals], list(kappa_ch), pq,
                    ipbs, nch, icc, iicc, mk, lists)


def config0() -> Workload:
    """ns=80, r_max=25, Z=10; 1s,2s,2p-,2p; k=0..3; channels kappa -1,+1;
    40 angular entries; plain FP64."""
    orbitals = [(1, -1), (2, -1), (2, 1), (2, -2)]
    return _build("config0: ns=80 Z=10 nch=2 k=0..3 R^k", 1234, 80, 25.0, 10.0, orbitals, [-1, 1],
                  3, 40, 1.0, breit=False, o_entries=8)


def config1(scale: float = 1.0, nch: int = 120, breit: bool = True) -> Workload:
    """ns=400, r_max=40, Z=26; 20 target orbitals; k=0..10 R^k + S^k;
    120 channels with kappa uniform over +-1..+-6; 2e6 entries over ~5% of
    the (channel pair, k) slots.  ``scale`` shrinks the entry count and
    ``nch`` the channel count for reduced test cases."""
    rng = np.random.Generator(np.random.Philox(1235))
    kap = [int(k) * int(s) for k, s in zip(rng.integers(1, 7, nch), rng.choice([-1, 1], nch))]
    return _build(f"config1: ns=400 Z=26 nch={nch} k=0..10 R^k+S^k", 1235, 400, 40.0, 26.0,
                  TARGET_ORBITALS[:20], kap, 10, int(2e6 * scale), 0.05, breit=breit,
                  o_entries=int(2000 * scale))


def config1_shape(nch: int = 4, per_slot: int = 300, seed: int = 1240) -> Workload:
    """The grid, orbitals and multipoles of config1 (ns=400, r_max=40, Z=26,
    first knot 0.25/Z, 20 target orbitals, k=0..10 R^k and S^k up to v=11)
    with a few channels (kappa uniform over +-1..+-6) and every (channel
    pair, k) slot occupied by about ``per_slot`` entries: the lists the
    120-channel workload holds, at a size whose blocks the CPU oracle can
    assemble."""
    rng = np.random.Generator(np.random.Philox(seed))
    kap = [int(k) * int(s) for k, s in zip(rng.integers(1, 7, nch), rng.choice([-1, 1], nch))]
    slots = nch * (nch + 1) // 2 * 11
    return _build(f"config1 shape: ns=400 Z=26 nch={nch} k=0..10 R^k+S^k", seed, 400, 40.0, 26.0,
                  TARGET_ORBITALS[:20], kap, 10, per_slot * slots, 1.0, breit=True,
                  o_entries=4 * nch)


def small(ns=60, nch=3, mk=3, n_entries=300, breit=True, seed=99, rmax=20.0, z=8.0,
          occupancy=1.0, norb=4) -> Workload:
    """Reduced workloads for parity tests."""
    orbitals = TARGET_ORBITALS[:norb]
    # keep at least 10 geometric intervals below r = 1
    rmax = min(rmax, 1.0 + 0.5 * ((ns - 9 + 1) - 11))
    rng = np.random.Generator(np.random.Philox(seed + 7))
    kap = [int(k) * int(s) for k, s in zip(rng.integers(1, 4, nch), rng.choice([-1, 1], nch))]
    return _build(f"small ns={ns} nch={nch}", seed, ns, rmax, z, orbitals, kap, mk, n_entries,
                  occupancy, breit=breit, o_entries=20)


def config3_block(index: int, nch_max: int = 300, rows_entries: float = 1e4,
                  seed: int = 1237) -> Workload:
    """Block `index` of config3(nch_max=nch_max, ...), built alone (the draws of
    the earlier blocks are replayed without building them)."""
    rng = np.random.Generator(np.random.Philox(seed))
    for b in range(index + 1):
        ns = int(rng.integers(150, 451))
        nch = int(round(math.exp(rng.uniform(math.log(10), math.log(nch_max)))))
        kap = [int(k) * int(s) for k, s in zip(rng.integers(1, 7, nch), rng.choice([-1, 1], nch))]
    return _build(f"config3 block {index}: ns={ns} nch={nch} k=0..8", seed + 17 * (index + 1), ns,
                  40.0, 26.0, TARGET_ORBITALS[:20], kap, 8, max(1, int(rows_entries * nch)), 0.05,
                  breit=True, o_entries=max(1, nch))


def config3(nblocks: int = 64, nch_max: int = 300, rows_entries: float = 1e4,
            seed: int = 1237) -> list:
    """Batched form: ``nblocks`` independent J-parity blocks, each with its own
    grid (ns uniform in 150..450, r_max=40, Z=26), the 20 target orbitals
    projected on it, channel counts log-uniform in 10..nch_max, k=0..8, and
    about ``rows_entries`` entries per channel-pair row (nch * rows_entries
    per block) over 5% of the (channel pair, k) slots.  The full size
    (nch up to 300) exceeds one GPU's memory in the reference layout; the
    arguments scale it."""
    rng = np.random.Generator(np.random.Philox(seed))
    out = []
    for b in range(nblocks):
        ns = int(rng.integers(150, 451))
        nch = int(round(math.exp(rng.uniform(math.log(10), math.log(nch_max)))))
        kap = [int(k) * int(s) for k, s in zip(rng.integers(1, 7, nch), rng.choice([-1, 1], nch))]
        out.append(_build(f"config3 block {b}: ns={ns} nch={nch} k=0..8", seed + 17 * (b + 1), ns,
                          40.0, 26.0, TARGET_ORBITALS[:20], kap, 8,
                          max(1, int(rows_entries * nch)), 0.05, breit=True,
                          o_entries=max(1, nch)))
    return out


@dataclass
class EnergyWorkload:
    """E = sum_e coef[e] R^k[e](i1,i2;i3,i4) over bound orbitals pq(ns,2,nbf)."""
    name: str
    t: np.ndarray
    z: float
    ks: int
    ksp: int
    ksq: int
    pq: np.ndarray
    ipbs: np.ndarray
    k: np.ndarray
    i1: np.ndarray
    i2: np.ndarray
    i3: np.ndarray
    i4: np.ndarray
    coef: np.ndarray

    @property
    def ns(self) -> int:
        return self.t.size - self.ks


def energy_workload(name, seed, ns, rmax, z, norb, kmax, n_entries) -> EnergyWorkload:
    """Random R^k entries over the first ``norb`` target orbitals: k uniform in
    0..kmax subject to the parity rule of both pairs (l_a + l_c + k and
    l_b + l_d + k even, the condition of the angular coefficients),
    coefficients uniform in [-1, 1]."""
    rng = np.random.Generator(np.random.Philox(seed))
    ks, ksp, ksq = 9, 8, 9
    t = knots(ns, rmax, z, ks)
    orbitals = TARGET_ORBITALS[:norb]
    pq = orbital_coefficients(t, ks, ksp, ksq, z, orbitals, rng)
    ls = np.array([l_kappa(kp) for _, kp in orbitals])
    out = [[], [], [], [], [], []]
    while len(out[0]) < n_entries:
        m = 4 * (n_entries - len(out[0])) + 64
        k = rng.integers(0, kmax + 1, m)
        a, b, c, d = (rng.integers(1, norb + 1, m) for _ in range(4))
        ok = ((ls[a - 1] + ls[c - 1] + k) % 2 == 0) & ((ls[b - 1] + ls[d - 1] + k) % 2 == 0)
        idx = np.flatnonzero(ok)[: n_entries - len(out[0])]
        for lst, v in zip(out, (k, a, b, c, d, rng.uniform(-1.0, 1.0, m))):
            lst.extend(v[idx].tolist())
    k, i1, i2, i3, i4 = (np.asarray(v, dtype=np.int32) for v in out[:5])
    return EnergyWorkload(name, t, z, ks, ksp, ksq, pq, np.zeros(norb, dtype=np.int32), k, i1,
                          i2, i3, i4, np.asarray(out[5], dtype=np.float64))


def config4(n_entries: int = 50000) -> EnergyWorkload:
    """ns=300, Z=18, 30 bound orbitals, k=0..8, 5e4 entries of
    E = sum c R^k(a,b;c,d)."""
    return energy_workload(f"config4: ns=300 Z=18 30 orbitals k=0..8 {n_entries} entries", 1238,
                           300, 30.0, 18.0, 30, 8, n_entries)


def algorithmic_flops(w: Workload) -> dict:
    """Reference loop FLOPs of the contraction (2 x multiply-adds):
    T_s^2 per direct 's' convol, T_n^2 per 'n' or exchange convol, one
    convol per (segment, PQ type), plus the density accumulations."""
    ns, ks = w.ns, w.ks
    Ts = ks * ns - ks * (ks - 1) // 2
    Tn = (2 * ks - 1) * ns - ks * (ks - 1)
    fl = {"convol": 0, "density": 0}
    for L in w.lists:
        nseg = int(np.unique(L.k1).size) if L.n else 0
        if L.icase == 2:
            if L.itype == 3:
                fl["convol"] += 4 * nseg * 2 * Ts * Ts
                fl["density"] += 4 * L.n * 2 * ns * ks
            else:
                fl["convol"] += 4 * nseg * 2 * Tn * Tn
                fl["density"] += 4 * L.n * 2 * ns * ns
        elif L.icase == 3:
            fl["convol"] += nseg * 2 * Tn * Tn
            it = L.itype % 10
            fl["density"] += L.n * 2 * ns * ((2 * ks - 1) if it <= 7 else ns)
    fl["total"] = fl["convol"] + fl["density"]
    return fl


def perturber_numbering(nch: int, npert: int):
    """icb(nch,npert) row by row and ibb(npert,npert) over the lower triangle
    (Alloc_dbsr_matrix with one process, updates.f90:50-70)."""
    icb = np.zeros((nch, npert), dtype=np.int32, order="F")
    i = 0
    for ich in range(nch):
        for jp in range(npert):
            i += 1
            icb[ich, jp] = i
    ibb = np.zeros((npert, npert), dtype=np.int32, order="F")
    i = 0
    for ip in range(npert):
        for jp in range(ip + 1):
            i += 1
            ibb[ip, jp] = i
            ibb[jp, ip] = i
    return icb, ibb


def structures_case(seed: int = 77, ns: int = 50, nch: int = 3, norb: int = 4, npert: int = 3,
                    ntarg: int = 2, per_list: int = 24, mk: int = 2, iitar: int = 2,
                    rmax: float = 20.0, z: float = 8.0) -> Workload:
    """Lists of every structure that is not a channel-pair contraction --
    R^k itypes 1 and 2 (R_data.f90:92-211), S^k ktypes 1-5 and 11-15
    (S_data.f90:115-236), L itypes 1-3 (L_data.f90:46-132), O itypes 1, 2 and
    4 (O_data.f90:33-78) -- with every routing of their K3/K4 codes
    (Idef_Rtype / Idef_itype / Idef_Ltype / Idef_Otype, idef_type.f90), on a
    small grid with perturbers, targets and seeded symmetric one-electron
    matrices.  Coefficients uniform in [-1, 1]."""
    w = small(ns=ns, nch=nch, mk=mk, n_entries=8, breit=False, seed=seed, rmax=rmax, z=z,
              norb=norb)
    rng = np.random.Generator(np.random.Philox(seed + 500))
    nb = w.nbound
    ch_orb = np.arange(nb + 1, nb + nch + 1)  # channel orbitals follow the bound ones
    kbs = np.array(list(w.kappa_bound) + list(w.kappa_ch), dtype=np.int32)
    kap_list = np.array(sorted(set(kbs.tolist())), dtype=np.int32)
    ms = 2 * w.ns
    hd = np.zeros((ms, ms, kap_list.size), order="F")
    for k in range(kap_list.size):
        a = rng.uniform(-1.0, 1.0, (ms, ms))
        hd[:, :, k] = 0.5 * (a + a.T)
    icb, ibb = perturber_numbering(nch, npert)
    iptar = rng.integers(1, ntarg + 1, nch).astype(np.int32)

    def bound():
        return int(rng.integers(1, nb + 1))

    def pair():
        a, b = bound(), bound()
        return min(a, b) * IBO + max(a, b)

    def ovl():  # <channel orbital | bound orbital> code io = io1*ibo + io2
        return int(ch_orb[rng.integers(0, nch)]) * IBO + bound()

    def tgt():  # <channel orbital | channel orbital> code
        return int(ch_orb[rng.integers(0, nch)]) * IBO + int(ch_orb[rng.integers(0, nch)])

    def pert():
        return int(rng.integers(1, npert + 1))

    def chan():
        return int(rng.integers(1, nch + 1))

    def c():
        return float(rng.uniform(-1.0, 1.0))

    lists = []

    def add(icase, itype, kpol, rows):
        if rows:
            k1, k2, k3, k4, cc = sort_merge(*zip(*rows))
            lists.append(CList(icase, itype, kpol, k1, k2, k3, k4, cc))

    # R^k / S^k itype 1: K1, K2 bound pairs; K3/K4 = (-ic,-jc), (io,-ic), (io,jo), (io,0)
    def bound_rows():
        rows = []
        for _ in range(per_list):
            r = int(rng.integers(0, 4))
            k3, k4 = ((-pert(), -pert()), (ovl(), -pert()), (ovl(), ovl()), (tgt(), 0))[r]
            rows.append((pair(), pair(), k3, k4, c()))
        return rows

    # itype 2: K1 bound pair, K2 bound orbital, K3 channel, K4 = io or -ic
    def channel_rows():
        rows = []
        for _ in range(per_list):
            k4 = ovl() if rng.integers(0, 2) else -pert()
            rows.append((pair(), bound(), chan(), k4, c()))
        return rows

    for k in range(mk + 1):
        add(2, 1, k, bound_rows())
        add(2, 2, k, channel_rows())
    for v in (0, mk + 1):
        for at in (0, 1):
            add(3, 10 * at + 1, v, bound_rows())
            for it in (2, 3, 4, 5):
                add(3, 10 * at + it, v, channel_rows())
    # L itype 1: K1 <= K2 bound orbitals of one kappa; K3/K4 = (ic,jc), (-io,ic),
    # (-io,-jo), (-io,0)
    by_kappa = {}
    for o in range(1, nb + 1):
        by_kappa.setdefault(int(kbs[o - 1]), []).append(o)
    rows = []
    for _ in range(per_list):
        grp = list(by_kappa.values())[int(rng.integers(0, len(by_kappa)))]
        a, b = (int(x) for x in rng.choice(grp, 2))
        r = int(rng.integers(0, 4))
        k3, k4 = ((pert(), pert()), (-ovl(), pert()), (-ovl(), -ovl()), (-tgt(), 0))[r]
        rows.append((min(a, b), max(a, b), k3, k4, c()))
    add(1, 1, 0, rows)
    # L itype 2: K1 bound orbital, K2 channel, K3 = ic or -io
    rows = [(bound(), chan(), (pert() if rng.integers(0, 2) else -ovl()), 0, c())
            for _ in range(per_list)]
    add(1, 2, 0, rows)
    # L itype 3: channel orbitals of one kappa
    rows = []
    for _ in range(per_list):
        i, j = (int(x) for x in rng.integers(0, nch, 2))
        if kbs[ch_orb[i] - 1] != kbs[ch_orb[j] - 1]:
            j = i
        rows.append((int(ch_orb[i]), int(ch_orb[j]), 0, 0, c()))
    add(1, 3, 0, rows)
    # O itypes 1, 2, 4
    add(0, 1, 0, [(pert(), pert(), 0, 0, c()) for _ in range(per_list)])
    add(0, 2, 0, [(ovl(), pert(), 0, 0, c()) for _ in range(per_list)])
    add(0, 4, 0, [(tgt(), 0, 0, 0, c()) for _ in range(per_list)])
    w.name = f"structures ns={w.ns} nch={nch} npert={npert} ntarg={ntarg}"
    w.lists = lists
    w.npert, w.icb, w.ibb = npert, icb, ibb
    w.ntarg, w.iptar, w.iitar = ntarg, iptar, iitar
    w.kap_list, w.hd, w.kbs = kap_list, hd, kbs
    return w
