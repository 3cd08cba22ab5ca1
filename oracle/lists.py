"""Pure-Python restatement of DBSR_MAT3's list producer (test infrastructure
only, small cases): Add_integral (add_integral.f90:17-49), SMU
(DBSR_HF/hf_energy_BR.f90:58-121), Idef_Otype / Idef_Ltype / Idef_Rtype /
Idef_itype (idef_type.f90:1-437) and Add_cdata's sorted insertion with
binary search (MOD_c_data.f90:177-236), one unbounded block per
(kpol, itype); Merge_cdata's drop of |c| <= eps_c (MOD_c_data.f90:300) is
applied when a list is read.  Orbital and channel numbers are 1-based as in
the reference.

Parity unpinned: the reference ships no int_bnk bank and no list dump, so
these lists are checked against this restatement only."""
from __future__ import annotations

IBO = 2 ** 15
IBTYPE = 10


def l_kappa(k: int) -> int:
    return -k - 1 if k < 0 else k


def smu(ka, kb, kc, kd, L, v):
    """(SMU, S(1:8)) of hf_energy_BR.f90:58-121."""
    S = [0.0] * 8
    if L < 0 or v < 0:
        return 0.0, S
    la, lc = l_kappa(ka), l_kappa(kc)
    if (la + lc + v) % 2 == 0:
        return 0.0, S
    lb, ld = l_kappa(kb), l_kappa(kd)
    if (lb + ld + v) % 2 == 0:
        return 0.0, S
    if v == L:
        if L == 0:
            return 0.0, S
        r = float(-(ka + kc) * (kb + kd))
        r = r / L / (L + 1)
        return r, [r] * 8
    K, Kp = kc - ka, kd - kb
    if v == L - 1:
        bp = float(L + 1)
        bp = bp / 2 / (L + L - 1)
        cp = float(-(L - 2))
        cp = cp / 2 / L / (L + L - 1)
        S = [(L + K) * (bp + cp * Kp), (L + Kp) * (bp + cp * K), (L - K) * (bp - cp * Kp),
             (L - Kp) * (bp - cp * K), -(L + K) * (bp - cp * Kp), -(L - Kp) * (bp + cp * K),
             -(L - K) * (bp + cp * Kp), -(L + Kp) * (bp - cp * K)]
    elif v == L + 1:
        i = -L - 1
        b = float(L)
        b = b / 2 / (L + L + 3)
        c = float(L + 3)
        c = c / (L + L + 2) / (L + L + 3)
        S = [(i + Kp) * (b + c * K), (i + K) * (b + c * Kp), (i - Kp) * (b - c * K),
             (i - K) * (b - c * Kp), -(i - Kp) * (b + c * K), -(i + K) * (b - c * Kp),
             -(i + Kp) * (b - c * K), -(i - K) * (b + c * Kp)]
    r = 0.0
    for x in S:
        r = r + abs(x)
    return r, S


class Lists:
    def __init__(self, icase, ipbs, lbs, kbs, mk, eps_c=1e-10, check_target=1):
        self.icase, self.mk, self.eps_c, self.check_target = icase, mk, eps_c, check_target
        self.ipbs = [int(x) for x in ipbs]
        self.lbs = [int(x) for x in lbs] if lbs is not None else None
        self.kbs = [int(x) for x in kbs] if kbs is not None else None
        self.data = {}  # (kpol, itype) -> sorted list of [k1, k2, k3, k4, c]

    def ip(self, i):
        return self.ipbs[i - 1]

    # Add_coef + Add_cdata: binary search on (K1,K2,K3,K4), sum or insert
    def add_coef(self, C, kpol, k1, k2, k3, k4, itype):
        lst = self.data.setdefault((kpol, itype), [])
        key = (k1, k2, k3, k4)
        lo, hi = 0, len(lst) - 1
        while lo <= hi:
            m = (lo + hi) // 2
            km = tuple(lst[m][:4])
            if key < km:
                hi = m - 1
            elif key > km:
                lo = m + 1
            else:
                lst[m][4] = lst[m][4] + C
                return
        lst.insert(lo, [k1, k2, k3, k4, C])

    def idef_otype(self, C, ic, jc, io, jo):
        if abs(C) < self.eps_c:
            return
        itype = 0
        if jc > 0:
            k1, k2, itype = ic, jc, 1
        elif ic > 0 and io > 0:
            k1, k2, itype = io, ic, 2
        elif io > 0 and jo > 0:
            k1, k2, itype = io, jo, 3
        elif io > 0 and jo == 0:
            k1, k2, itype = io, 0, 4
        if itype == 0:
            raise ValueError("Idef_Otype: itype=0")
        if self.check_target == 0 and itype == 4:
            return
        self.add_coef(C, 0, k1, k2, 0, 0, itype)

    def idef_ltype(self, ii, jj, C, ic, jc, io, jo):
        if abs(C) < self.eps_c:
            return
        i, j = min(ii, jj), max(ii, jj)
        ich, jch = self.ip(i), self.ip(j)
        itype = 0
        if jc > 0:
            k1, k2, k3, k4, itype = i, j, ic, jc, 1
        elif ic > 0:
            if io == 0:
                if ich != 0 and jch == 0:
                    k1, k2, k3, k4, itype = j, ich, ic, 0, 2
                elif ich == 0 and jch != 0:
                    k1, k2, k3, k4, itype = i, jch, ic, 0, 2
            elif io > 0:
                k1, k2, k3, k4, itype = i, j, -io, ic, 1
        elif io == 0:
            k1, k2, k3, k4, itype = j, i, 0, 0, 3
        elif io > 0 and jo == 0:
            if ich != 0 and jch == 0:
                k1, k2, k3, k4, itype = j, ich, -io, 0, 2
            elif jch != 0 and ich == 0:
                k1, k2, k3, k4, itype = i, jch, -io, 0, 2
            elif ich == 0 and jch == 0:
                k1, k2, k3, k4, itype = i, j, -io, 0, 1
                if self.check_target == 0:
                    return
        elif io > 0 and jo > 0:
            k1, k2, k3, k4, itype = i, j, -io, -jo, 1
        if itype == 0:
            raise ValueError("Idef_Ltype: itype=0")
        self.add_coef(C, 0, k1, k2, k3, k4, itype)

    def idef_rtype(self, k, j1, j2, j3, j4, C, ic, jc, io, jo):
        if abs(C) < self.eps_c:
            return
        ip = self.ip
        if ip(j1) + ip(j2) == 0 or ip(j3) + ip(j4) == 0:
            i1, i3 = (j3, j1) if j1 > j3 else (j1, j3)
            i2, i4 = (j4, j2) if j2 > j4 else (j2, j4)
            if i1 > i2:
                i1, i2, i3, i4 = i2, i1, i4, i3
        else:
            i1, i2, i3, i4 = j1, j2, j3, j4
        itype, k4 = 0, 0
        if jc > 0:
            k1, k2, k3, k4, itype = i1 * IBO + i3, i2 * IBO + i4, -ic, -jc, 1
        elif ic > 0:
            if io == 0:
                if ip(i1) > 0:
                    k1, k2, k3, k4, itype = i2 * IBO + i4, i3, ip(i1), -ic, 2
                elif ip(i2) > 0:
                    k1, k2, k3, k4, itype = i1 * IBO + i3, i4, ip(i2), -ic, 2
                elif ip(i3) > 0:
                    k1, k2, k3, k4, itype = i2 * IBO + i4, i1, ip(i3), -ic, 2
                elif ip(i4) > 0:
                    k1, k2, k3, k4, itype = i1 * IBO + i3, i2, ip(i4), -ic, 2
            elif io > 0:
                k1, k2, k3, k4, itype = i1 * IBO + i3, i2 * IBO + i4, io, -ic, 1
        elif io == 0:
            if ip(i1) > 0 and ip(i3) > 0:
                if ip(i1) >= ip(i3):
                    k1, k2, k3, itype = ip(i1) * IBO + ip(i3), i2, i4, 3
                    if k2 > k3:
                        k2, k3 = i4, i2
                else:
                    k1, k2, k3, itype = ip(i3) * IBO + ip(i1), i4, i2, 3
                    if k2 > k3:
                        k2, k3 = i2, i4
            elif ip(i2) > 0 and ip(i4) > 0:
                if ip(i2) >= ip(i4):
                    k1, k2, k3, itype = ip(i2) * IBO + ip(i4), i1, i3, 3
                    if k2 > k3:
                        k2, k3 = i3, i1
                else:
                    k1, k2, k3, itype = ip(i4) * IBO + ip(i2), i3, i1, 3
                    if k2 > k3:
                        k2, k3 = i1, i3
            elif ip(i1) > 0 and ip(i4) > 0:
                if ip(i1) >= ip(i4):
                    k1, k2, k3, itype = ip(i1) * IBO + ip(i4), i3, i2, 4
                else:
                    k1, k2, k3, itype = ip(i4) * IBO + ip(i1), i2, i3, 4
            elif ip(i2) > 0 and ip(i3) > 0:
                if ip(i3) >= ip(i2):
                    k1, k2, k3, itype = ip(i3) * IBO + ip(i2), i1, i4, 4
                else:
                    k1, k2, k3, itype = ip(i2) * IBO + ip(i3), i4, i1, 4
            k4 = 0
        elif io > 0 and jo == 0:
            if ip(i1) > 0:
                k1, k2, k3, k4, itype = i2 * IBO + i4, i3, ip(i1), io, 2
            elif ip(i2) > 0:
                k1, k2, k3, k4, itype = i1 * IBO + i3, i4, ip(i2), io, 2
            elif ip(i3) > 0:
                k1, k2, k3, k4, itype = i2 * IBO + i4, i1, ip(i3), io, 2
            elif ip(i4) > 0:
                k1, k2, k3, k4, itype = i1 * IBO + i3, i2, ip(i4), io, 2
            else:
                k1, k2, k3, k4, itype = i1 * IBO + i3, i2 * IBO + i4, io, 0, 1
                if self.check_target == 0:
                    return
        elif io > 0 and jo > 0:
            k1, k2, k3, k4, itype = i1 * IBO + i3, i2 * IBO + i4, io, jo, 1
        if itype == 0:
            raise ValueError("Idef_Rtype: itype=0")
        self.add_coef(C, k, k1, k2, k3, k4, itype)

    def idef_itype(self, atype, k, i1, i2, i3, i4, C, ic, jc, io, jo):
        if C == 0.0:
            return
        ip = self.ip
        itype, k4 = 0, 0
        if jc > 0:
            k1, k2, k3, k4, itype = i1 * IBO + i3, i2 * IBO + i4, -ic, -jc, 1
        elif ic > 0:
            if io == 0:
                if ip(i1) > 0:
                    k1, k2, k3, k4, itype = i2 * IBO + i4, i3, ip(i1), -ic, 2
                elif ip(i2) > 0:
                    k1, k2, k3, k4, itype = i1 * IBO + i3, i4, ip(i2), -ic, 3
                elif ip(i3) > 0:
                    k1, k2, k3, k4, itype = i2 * IBO + i4, i1, ip(i3), -ic, 4
                elif ip(i4) > 0:
                    k1, k2, k3, k4, itype = i1 * IBO + i3, i2, ip(i4), -ic, 5
            elif io > 0:
                k1, k2, k3, k4, itype = i1 * IBO + i3, i2 * IBO + i4, io, -ic, 1
        elif io == 0:
            if ip(i1) > 0 and ip(i3) > 0:
                k1, k2, k3, itype = ip(i1) * IBO + ip(i3), i2, i4, 6
            elif ip(i2) > 0 and ip(i4) > 0:
                k1, k2, k3, itype = ip(i2) * IBO + ip(i4), i1, i3, 7
            elif ip(i1) > 0 and ip(i4) > 0:
                k1, k2, k3, itype = ip(i1) * IBO + ip(i4), i3, i2, 8
            elif ip(i2) > 0 and ip(i3) > 0:
                k1, k2, k3, itype = ip(i3) * IBO + ip(i2), i1, i4, 9
            k4 = 0
        elif io > 0 and jo == 0:
            if ip(i1) > 0:
                k1, k2, k3, k4, itype = i2 * IBO + i4, i3, ip(i1), io, 2
            elif ip(i2) > 0:
                k1, k2, k3, k4, itype = i1 * IBO + i3, i4, ip(i2), io, 3
            elif ip(i3) > 0:
                k1, k2, k3, k4, itype = i2 * IBO + i4, i1, ip(i3), io, 4
            elif ip(i4) > 0:
                k1, k2, k3, k4, itype = i1 * IBO + i3, i2, ip(i4), io, 5
            else:
                k1, k2, k3, k4, itype = i1 * IBO + i3, i2 * IBO + i4, io, 0, 1
        elif io > 0 and jo > 0:
            k1, k2, k3, k4, itype = i1 * IBO + i3, i2 * IBO + i4, io, jo, 1
        if itype == 0:
            raise ValueError("Idef_itype: itype=0")
        self.add_coef(C, k, k1, k2, k3, k4, atype * IBTYPE + itype)

    def add_integral(self, kpol, i1, i2, i3, i4, C, ic, jc, io, jo):
        if self.icase == 0:
            self.idef_otype(C, ic, jc, io, jo)
        elif self.icase == 1:
            self.idef_ltype(i1, i3, C, ic, jc, io, jo)
        elif self.icase == 2:
            lb = self.lbs
            m = (lb[i1 - 1] + lb[i3 - 1] + kpol) % 2 + (lb[i2 - 1] + lb[i4 - 1] + kpol) % 2
            if m == 0 and kpol <= self.mk:
                self.idef_rtype(kpol, i1, i2, i3, i4, C, ic, jc, io, jo)
        elif self.icase == 3:
            kb = self.kbs
            for v in range(kpol - 1, kpol + 2):
                if v > self.mk:
                    continue
                r, S = smu(kb[i1 - 1], kb[i2 - 1], kb[i3 - 1], kb[i4 - 1], kpol, v)
                if r == 0.0:
                    continue
                self.idef_itype(0, v, i1, i2, i3, i4, C * S[0], ic, jc, io, jo)
                self.idef_itype(0, v, i2, i1, i4, i3, C * S[1], ic, jc, io, jo)
                self.idef_itype(0, v, i3, i4, i1, i2, C * S[2], ic, jc, io, jo)
                self.idef_itype(0, v, i4, i3, i2, i1, C * S[3], ic, jc, io, jo)
                self.idef_itype(1, v, i1, i2, i3, i4, C * S[4], ic, jc, io, jo)
                self.idef_itype(1, v, i4, i3, i2, i1, C * S[5], ic, jc, io, jo)
                self.idef_itype(1, v, i3, i4, i1, i2, C * S[6], ic, jc, io, jo)
                self.idef_itype(1, v, i2, i1, i4, i3, C * S[7], ic, jc, io, jo)

    def get(self, kpol, itype):
        """The list as Merge_cdata leaves it: |c| <= eps_c dropped."""
        return [e for e in self.data.get((kpol, itype), []) if abs(e[4]) > self.eps_c]

    def keys(self):
        return sorted(k for k in self.data if self.get(*k))
