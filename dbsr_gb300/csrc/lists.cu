// lists.cu -- the list producer of DBSR_MAT3 between the decoded angular
// bank and Gen_matrix: Add_integral (add_integral.f90:2-57) with its parity
// filter and the Breit expansion over v = k-1..k+1 by SMU
// (DBSR_HF/hf_energy_BR.f90:58-121), the structure classification
// Idef_Otype / Idef_Ltype / Idef_Rtype / Idef_itype (idef_type.f90:1-437),
// and Add_coef / Add_cdata / Merge_cdata / Add_matrix (MOD_c_data.f90:117-
// 368), which keep every (kpol, itype) list sorted by (K1,K2,K3,K4) with
// equal keys summed.
//
// The reference inserts every coefficient into a sorted block by binary
// search and shifts the tail (O(n^2) per block) and merges blocks when they
// fill.  Here the coefficients are appended in arrival order and each list
// is put in order once, by a stable sort of its keys, when it is read: equal
// keys are summed in arrival order (the association of Add_cdata's running
// sum), and sums with |c| <= eps_c are dropped as Merge_cdata drops them.
// The lists are sorted on several host threads at once.  Host code only.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <thread>
#include <vector>

#include "internal.cuh"

struct dbsrg_lists {
  int icase = 0, nbf = 0, mk = 0, check_target = 1;
  double eps_c = 1e-10;
  std::vector<int> ipbs, lbs, kbs;
  struct Entry {
    int k1, k2, k3, k4;
    double c;
  };
  std::map<std::pair<int, int>, std::vector<Entry>> raw;     // (kpol, itype) -> arrival order
  std::map<std::pair<int, int>, std::vector<Entry>> merged;  // sorted, summed
  bool dirty = true;
};

namespace {

constexpr int IBO = DBSRG_IBO;
constexpr int IBTYPE = 10;  // ktype = atype * ibtype + itype (mod_dbsr_mat.f90:103)

int l_kappa(int k) { return k < 0 ? -k - 1 : k; }

// SMU: the Breit coefficients S(1:8) of the eight orderings for multipole L
// and rank v (Grant and Pyper, J. Phys. B 9 (1976) 761), hf_energy_BR.f90:
// 58-121; returns their absolute sum (0: no contribution)
double smu(int ka, int kb, int kc, int kd, int L, int v, double *S) {
  for (int i = 0; i < 8; i++) S[i] = 0.0;
  if (L < 0 || v < 0) return 0.0;
  const int la = l_kappa(ka), lc = l_kappa(kc);
  if ((la + lc + v) % 2 == 0) return 0.0;
  const int lb = l_kappa(kb), ld = l_kappa(kd);
  if ((lb + ld + v) % 2 == 0) return 0.0;
  double r = 0.0;
  if (v == L) {
    if (L == 0) return 0.0;
    r = (double)(-(ka + kc) * (kb + kd));
    r = r / L / (L + 1);
    for (int i = 0; i < 8; i++) S[i] = r;
    return r;
  }
  const int K = kc - ka, Kp = kd - kb;
  if (v == L - 1) {
    double bp = L + 1;
    bp = bp / 2 / (L + L - 1);
    double cp = -(L - 2);
    cp = cp / 2 / L / (L + L - 1);
    S[0] = (L + K) * (bp + cp * Kp);
    S[1] = (L + Kp) * (bp + cp * K);
    S[2] = (L - K) * (bp - cp * Kp);
    S[3] = (L - Kp) * (bp - cp * K);
    S[4] = -(L + K) * (bp - cp * Kp);
    S[5] = -(L - Kp) * (bp + cp * K);
    S[6] = -(L - K) * (bp + cp * Kp);
    S[7] = -(L + Kp) * (bp - cp * K);
  } else if (v == L + 1) {
    const int i = -L - 1;
    double b = L;
    b = b / 2 / (L + L + 3);
    double c = (L + 3);
    c = c / (L + L + 2) / (L + L + 3);
    S[0] = (i + Kp) * (b + c * K);
    S[1] = (i + K) * (b + c * Kp);
    S[2] = (i - Kp) * (b - c * K);
    S[3] = (i - K) * (b - c * Kp);
    S[4] = -(i - Kp) * (b + c * K);
    S[5] = -(i + K) * (b - c * Kp);
    S[6] = -(i + Kp) * (b - c * K);
    S[7] = -(i - K) * (b + c * Kp);
  }
  for (int q = 0; q < 8; q++) r = r + std::fabs(S[q]);
  return r;
}

void add_coef(dbsrg_lists *L, double c, int kpol, int k1, int k2, int k3, int k4, int itype) {
  L->raw[{kpol, itype}].push_back({k1, k2, k3, k4, c});
  L->dirty = true;
}

int ip(const dbsrg_lists *L, int i) { return L->ipbs[i - 1]; }

// Idef_Otype (idef_type.f90:2-47); 0, or a status
int idef_otype(dbsrg_lists *L, double C, int ic, int jc, int io, int jo) {
  if (std::fabs(C) < L->eps_c) return 0;
  if (jc > 0 && ic <= 0) return DBSRG_EINVAL;
  int k1 = 0, k2 = 0, itype = 0;
  if (jc > 0) {
    k1 = ic; k2 = jc; itype = 1;
  } else if (ic > 0 && io > 0) {
    k1 = io; k2 = ic; itype = 2;
  } else if (io > 0 && jo > 0) {
    k1 = io; k2 = jo; itype = 3;
  } else if (io > 0 && jo == 0) {
    k1 = io; k2 = 0; itype = 4;
  }
  if (itype == 0) return DBSRG_EINVAL;
  if (L->check_target == 0 && itype == 4) return 0;
  add_coef(L, C, 0, k1, k2, 0, 0, itype);
  return 0;
}

// Idef_Ltype (idef_type.f90:51-137)
int idef_ltype(dbsrg_lists *L, int ii, int jj, double C, int ic, int jc, int io, int jo) {
  if (std::fabs(C) < L->eps_c) return 0;
  if ((jc > 0 && ic <= 0) || (jo > 0 && io <= 0) || (io > 0 && jc != 0) || (jo > 0 && ic != 0))
    return DBSRG_EINVAL;
  const int i = std::min(ii, jj), j = std::max(ii, jj), ich = ip(L, i), jch = ip(L, j);
  int k1 = 0, k2 = 0, k3 = 0, k4 = 0, itype = 0;
  if (jc > 0) {
    k1 = i; k2 = j; k3 = ic; k4 = jc; itype = 1;
  } else if (ic > 0) {
    if (io == 0) {
      if (ich != 0 && jch == 0) {
        k1 = j; k2 = ich; k3 = ic; k4 = 0; itype = 2;
      } else if (ich == 0 && jch != 0) {
        k1 = i; k2 = jch; k3 = ic; k4 = 0; itype = 2;
      }
    } else if (io > 0) {
      k1 = i; k2 = j; k3 = -io; k4 = ic; itype = 1;
    }
  } else if (io == 0) {
    k1 = j; k2 = i; k3 = 0; k4 = 0; itype = 3;
  } else if (io > 0 && jo == 0) {
    if (ich != 0 && jch == 0) {
      k1 = j; k2 = ich; k3 = -io; k4 = 0; itype = 2;
    } else if (jch != 0 && ich == 0) {
      k1 = i; k2 = jch; k3 = -io; k4 = 0; itype = 2;
    } else if (ich == 0 && jch == 0) {
      k1 = i; k2 = j; k3 = -io; k4 = 0; itype = 1;
      if (L->check_target == 0) return 0;
    }
  } else if (io > 0 && jo > 0) {
    k1 = i; k2 = j; k3 = -io; k4 = -jo; itype = 1;
  }
  if (itype == 0) return DBSRG_EINVAL;
  add_coef(L, C, 0, k1, k2, k3, k4, itype);
  return 0;
}

// Idef_Rtype (idef_type.f90:141-296)
int idef_rtype(dbsrg_lists *L, int k, int j1, int j2, int j3, int j4, double C, int ic, int jc,
               int io, int jo) {
  if (std::fabs(C) < L->eps_c) return 0;
  if ((io != 0 && std::abs(io) <= IBO) || (jo != 0 && std::abs(jo) <= IBO) || (jc > 0 && ic <= 0))
    return DBSRG_EINVAL;
  int i1, i2, i3, i4;
  if (ip(L, j1) + ip(L, j2) == 0 || ip(L, j3) + ip(L, j4) == 0) {
    i1 = j1; i3 = j3;
    if (j1 > j3) { i1 = j3; i3 = j1; }
    i2 = j2; i4 = j4;
    if (j2 > j4) { i2 = j4; i4 = j2; }
    if (i1 > i2) {
      std::swap(i1, i2);
      std::swap(i3, i4);
    }
  } else {
    i1 = j1; i2 = j2; i3 = j3; i4 = j4;
  }
  int k1 = 0, k2 = 0, k3 = 0, k4 = 0, itype = 0;
  if (jc > 0) {
    k1 = i1 * IBO + i3; k2 = i2 * IBO + i4; k3 = -ic; k4 = -jc; itype = 1;
  } else if (ic > 0) {
    if (io == 0) {
      if (ip(L, i1) > 0) {
        k1 = i2 * IBO + i4; k2 = i3; k3 = ip(L, i1); k4 = -ic; itype = 2;
      } else if (ip(L, i2) > 0) {
        k1 = i1 * IBO + i3; k2 = i4; k3 = ip(L, i2); k4 = -ic; itype = 2;
      } else if (ip(L, i3) > 0) {
        k1 = i2 * IBO + i4; k2 = i1; k3 = ip(L, i3); k4 = -ic; itype = 2;
      } else if (ip(L, i4) > 0) {
        k1 = i1 * IBO + i3; k2 = i2; k3 = ip(L, i4); k4 = -ic; itype = 2;
      }
    } else if (io > 0) {
      k1 = i1 * IBO + i3; k2 = i2 * IBO + i4; k3 = io; k4 = -ic; itype = 1;
    }
  } else if (io == 0) {
    if (ip(L, i1) > 0 && ip(L, i3) > 0) {
      if (ip(L, i1) >= ip(L, i3)) {
        k1 = ip(L, i1) * IBO + ip(L, i3); k2 = i2; k3 = i4; itype = 3;
        if (k2 > k3) { k2 = i4; k3 = i2; }
      } else {
        k1 = ip(L, i3) * IBO + ip(L, i1); k2 = i4; k3 = i2; itype = 3;
        if (k2 > k3) { k2 = i2; k3 = i4; }
      }
    } else if (ip(L, i2) > 0 && ip(L, i4) > 0) {
      if (ip(L, i2) >= ip(L, i4)) {
        k1 = ip(L, i2) * IBO + ip(L, i4); k2 = i1; k3 = i3; itype = 3;
        if (k2 > k3) { k2 = i3; k3 = i1; }
      } else {
        k1 = ip(L, i4) * IBO + ip(L, i2); k2 = i3; k3 = i1; itype = 3;
        if (k2 > k3) { k2 = i1; k3 = i3; }
      }
    } else if (ip(L, i1) > 0 && ip(L, i4) > 0) {
      if (ip(L, i1) >= ip(L, i4)) {
        k1 = ip(L, i1) * IBO + ip(L, i4); k2 = i3; k3 = i2; itype = 4;
      } else {
        k1 = ip(L, i4) * IBO + ip(L, i1); k2 = i2; k3 = i3; itype = 4;
      }
    } else if (ip(L, i2) > 0 && ip(L, i3) > 0) {
      if (ip(L, i3) >= ip(L, i2)) {
        k1 = ip(L, i3) * IBO + ip(L, i2); k2 = i1; k3 = i4; itype = 4;
      } else {
        k1 = ip(L, i2) * IBO + ip(L, i3); k2 = i4; k3 = i1; itype = 4;
      }
    }
    k4 = 0;
  } else if (io > 0 && jo == 0) {
    if (ip(L, i1) > 0) {
      k1 = i2 * IBO + i4; k2 = i3; k3 = ip(L, i1); k4 = io; itype = 2;
    } else if (ip(L, i2) > 0) {
      k1 = i1 * IBO + i3; k2 = i4; k3 = ip(L, i2); k4 = io; itype = 2;
    } else if (ip(L, i3) > 0) {
      k1 = i2 * IBO + i4; k2 = i1; k3 = ip(L, i3); k4 = io; itype = 2;
    } else if (ip(L, i4) > 0) {
      k1 = i1 * IBO + i3; k2 = i2; k3 = ip(L, i4); k4 = io; itype = 2;
    } else {
      k1 = i1 * IBO + i3; k2 = i2 * IBO + i4; k3 = io; k4 = 0; itype = 1;
      if (L->check_target == 0) return 0;
    }
  } else if (io > 0 && jo > 0) {
    k1 = i1 * IBO + i3; k2 = i2 * IBO + i4; k3 = io; k4 = jo; itype = 1;
  }
  if (itype == 0) return DBSRG_EINVAL;
  add_coef(L, C, k, k1, k2, k3, k4, itype);
  return 0;
}

// Idef_itype (idef_type.f90:300-437); ktype = atype * ibtype + itype
int idef_itype(dbsrg_lists *L, int atype, int k, int i1, int i2, int i3, int i4, double C, int ic,
               int jc, int io, int jo) {
  if (C == 0.0) return 0;
  if ((io != 0 && std::abs(io) <= IBO) || (jo != 0 && std::abs(jo) <= IBO) || (jc > 0 && ic <= 0))
    return DBSRG_EINVAL;
  int k1 = 0, k2 = 0, k3 = 0, k4 = 0, itype = 0;
  if (jc > 0) {
    k1 = i1 * IBO + i3; k2 = i2 * IBO + i4; k3 = -ic; k4 = -jc; itype = 1;
  } else if (ic > 0) {
    if (io == 0) {
      if (ip(L, i1) > 0) {
        k1 = i2 * IBO + i4; k2 = i3; k3 = ip(L, i1); k4 = -ic; itype = 2;
      } else if (ip(L, i2) > 0) {
        k1 = i1 * IBO + i3; k2 = i4; k3 = ip(L, i2); k4 = -ic; itype = 3;
      } else if (ip(L, i3) > 0) {
        k1 = i2 * IBO + i4; k2 = i1; k3 = ip(L, i3); k4 = -ic; itype = 4;
      } else if (ip(L, i4) > 0) {
        k1 = i1 * IBO + i3; k2 = i2; k3 = ip(L, i4); k4 = -ic; itype = 5;
      }
    } else if (io > 0) {
      k1 = i1 * IBO + i3; k2 = i2 * IBO + i4; k3 = io; k4 = -ic; itype = 1;
    }
  } else if (io == 0) {
    if (ip(L, i1) > 0 && ip(L, i3) > 0) {
      k1 = ip(L, i1) * IBO + ip(L, i3); k2 = i2; k3 = i4; itype = 6;
    } else if (ip(L, i2) > 0 && ip(L, i4) > 0) {
      k1 = ip(L, i2) * IBO + ip(L, i4); k2 = i1; k3 = i3; itype = 7;
    } else if (ip(L, i1) > 0 && ip(L, i4) > 0) {
      k1 = ip(L, i1) * IBO + ip(L, i4); k2 = i3; k3 = i2; itype = 8;
    } else if (ip(L, i2) > 0 && ip(L, i3) > 0) {
      k1 = ip(L, i3) * IBO + ip(L, i2); k2 = i1; k3 = i4; itype = 9;
    }
    k4 = 0;
  } else if (io > 0 && jo == 0) {
    if (ip(L, i1) > 0) {
      k1 = i2 * IBO + i4; k2 = i3; k3 = ip(L, i1); k4 = io; itype = 2;
    } else if (ip(L, i2) > 0) {
      k1 = i1 * IBO + i3; k2 = i4; k3 = ip(L, i2); k4 = io; itype = 3;
    } else if (ip(L, i3) > 0) {
      k1 = i2 * IBO + i4; k2 = i1; k3 = ip(L, i3); k4 = io; itype = 4;
    } else if (ip(L, i4) > 0) {
      k1 = i1 * IBO + i3; k2 = i2; k3 = ip(L, i4); k4 = io; itype = 5;
    } else {
      k1 = i1 * IBO + i3; k2 = i2 * IBO + i4; k3 = io; k4 = 0; itype = 1;
    }
  } else if (io > 0 && jo > 0) {
    k1 = i1 * IBO + i3; k2 = i2 * IBO + i4; k3 = io; k4 = jo; itype = 1;
  }
  if (itype == 0) return DBSRG_EINVAL;
  add_coef(L, C, k, k1, k2, k3, k4, atype * IBTYPE + itype);
  return 0;
}

// Add_integral (add_integral.f90:17-49) for one decoded coefficient
int add_integral(dbsrg_lists *L, int kpol, int i1, int i2, int i3, int i4, double C, int ic,
                 int jc, int io, int jo) {
  auto orb = [&](int i) { return i >= 1 && i <= L->nbf; };
  switch (L->icase) {
    case 0:
      return idef_otype(L, C, ic, jc, io, jo);
    case 1:
      if (!orb(i1) || !orb(i3)) return DBSRG_ERANGE;
      return idef_ltype(L, i1, i3, C, ic, jc, io, jo);
    case 2: {
      if (!orb(i1) || !orb(i2) || !orb(i3) || !orb(i4) || kpol < 0) return DBSRG_ERANGE;
      const int m = (L->lbs[i1 - 1] + L->lbs[i3 - 1] + kpol) % 2 +
                    (L->lbs[i2 - 1] + L->lbs[i4 - 1] + kpol) % 2;
      if (m == 0 && kpol <= L->mk) return idef_rtype(L, kpol, i1, i2, i3, i4, C, ic, jc, io, jo);
      return 0;
    }
    case 3: {
      if (!orb(i1) || !orb(i2) || !orb(i3) || !orb(i4) || kpol < 0) return DBSRG_ERANGE;
      const int ka = L->kbs[i1 - 1], kb = L->kbs[i2 - 1], kc = L->kbs[i3 - 1],
                kd = L->kbs[i4 - 1];
      for (int v = kpol - 1; v <= kpol + 1; v++) {
        if (v > L->mk) continue;
        double S[8];
        if (smu(ka, kb, kc, kd, kpol, v, S) == 0.0) continue;
        int rc = 0;
        rc |= idef_itype(L, 0, v, i1, i2, i3, i4, C * S[0], ic, jc, io, jo);
        rc |= idef_itype(L, 0, v, i2, i1, i4, i3, C * S[1], ic, jc, io, jo);
        rc |= idef_itype(L, 0, v, i3, i4, i1, i2, C * S[2], ic, jc, io, jo);
        rc |= idef_itype(L, 0, v, i4, i3, i2, i1, C * S[3], ic, jc, io, jo);
        rc |= idef_itype(L, 1, v, i1, i2, i3, i4, C * S[4], ic, jc, io, jo);
        rc |= idef_itype(L, 1, v, i4, i3, i2, i1, C * S[5], ic, jc, io, jo);
        rc |= idef_itype(L, 1, v, i3, i4, i1, i2, C * S[6], ic, jc, io, jo);
        rc |= idef_itype(L, 1, v, i2, i1, i4, i3, C * S[7], ic, jc, io, jo);
        if (rc) return DBSRG_EINVAL;
      }
      return 0;
    }
  }
  return DBSRG_EINVAL;
}

// every list in (K1,K2,K3,K4) order with equal keys summed in arrival
// order and |sum| <= eps_c dropped; lists sorted on several threads
void finalize(dbsrg_lists *L) {
  if (!L->dirty) return;
  std::vector<std::pair<const std::pair<int, int>, std::vector<dbsrg_lists::Entry>> *> work;
  for (auto &kv : L->raw) work.push_back(&kv);
  std::vector<std::vector<dbsrg_lists::Entry>> out(work.size());
  auto one = [&](size_t w) {
    const auto &in = work[w]->second;
    std::vector<int> idx(in.size());
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
      const auto &x = in[a], &y = in[b];
      if (x.k1 != y.k1) return x.k1 < y.k1;
      if (x.k2 != y.k2) return x.k2 < y.k2;
      if (x.k3 != y.k3) return x.k3 < y.k3;
      return x.k4 < y.k4;
    });
    auto &o = out[w];
    for (size_t q = 0; q < idx.size();) {
      const auto &e = in[idx[q]];
      double c = e.c;
      size_t r = q + 1;
      for (; r < idx.size(); r++) {
        const auto &f = in[idx[r]];
        if (f.k1 != e.k1 || f.k2 != e.k2 || f.k3 != e.k3 || f.k4 != e.k4) break;
        c = c + f.c;
      }
      if (std::fabs(c) > L->eps_c) o.push_back({e.k1, e.k2, e.k3, e.k4, c});
      q = r;
    }
  };
  const size_t nt = std::max<size_t>(1, std::min<size_t>(work.size(),
                                                         std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (size_t t = 0; t < nt; t++)
    th.emplace_back([&, t] {
      for (size_t w = t; w < work.size(); w += nt) one(w);
    });
  for (auto &x : th) x.join();
  L->merged.clear();
  for (size_t w = 0; w < work.size(); w++) L->merged[work[w]->first] = std::move(out[w]);
  L->dirty = false;
}

}  // namespace

extern "C" int dbsrg_lists_create(dbsrg_lists **out, int icase, int nbf, const int *ipbs,
                                  const int *lbs, const int *kbs, int mk, double eps_c,
                                  int check_target) {
  if (!out || icase < 0 || icase > 3 || nbf < 1 || !ipbs || mk < 0 || !(eps_c >= 0.0))
    return DBSRG_EINVAL;
  if ((icase == 2 && !lbs) || (icase == 3 && !kbs)) return DBSRG_EINVAL;
  dbsrg_lists *L = new (std::nothrow) dbsrg_lists();
  if (!L) return DBSRG_ENOMEM;
  L->icase = icase;
  L->nbf = nbf;
  L->mk = mk;
  L->eps_c = eps_c;
  L->check_target = check_target;
  L->ipbs.assign(ipbs, ipbs + nbf);
  if (lbs) L->lbs.assign(lbs, lbs + nbf);
  if (kbs) L->kbs.assign(kbs, kbs + nbf);
  *out = L;
  return DBSRG_OK;
}

extern "C" int dbsrg_lists_destroy(dbsrg_lists *L) {
  delete L;
  return DBSRG_OK;
}

extern "C" int dbsrg_lists_add(dbsrg_lists *L, int n, const int *kpol, const int *i1,
                               const int *i2, const int *i3, const int *i4, const double *c,
                               const int *ic, const int *jc, const int *io, const int *jo) {
  if (!L || n < 0) return DBSRG_EINVAL;
  if (n > 0 && (!kpol || !i1 || !i2 || !i3 || !i4 || !c || !ic || !jc || !io || !jo))
    return DBSRG_EINVAL;
  for (int e = 0; e < n; e++) {
    const int rc = add_integral(L, kpol[e], i1[e], i2[e], i3[e], i4[e], c[e], ic[e], jc[e],
                                io[e], jo[e]);
    if (rc) return rc;
  }
  return DBSRG_OK;
}

extern "C" int dbsrg_lists_decode(int n, const int *code, int *jcase, int *kpol, int *i1,
                                  int *i2, int *i3, int *i4) {
  if (n < 0 || (n > 0 && (!code || !jcase || !kpol || !i1 || !i2 || !i3 || !i4)))
    return DBSRG_EINVAL;
  for (int e = 0; e < n; e++) {  // state_res.f90:83-96: 2, 10, 5, 5, 5 bits from the bottom
    int v = code[e];
    jcase[e] = v % 4;
    v /= 4;
    kpol[e] = v % 1024;
    v /= 1024;
    i4[e] = v % 32;
    v /= 32;
    i3[e] = v % 32;
    v /= 32;
    i2[e] = v % 32;
    i1[e] = v / 32;
  }
  return DBSRG_OK;
}

extern "C" int dbsrg_lists_count(dbsrg_lists *L, int kpol, int itype) {
  if (!L) return DBSRG_EINVAL;
  finalize(L);
  auto it = L->merged.find({kpol, itype});
  return it == L->merged.end() ? 0 : (int)it->second.size();
}

extern "C" int dbsrg_lists_get(dbsrg_lists *L, int kpol, int itype, int *k1, int *k2, int *k3,
                               int *k4, double *cdata) {
  if (!L || !k1 || !k2 || !k3 || !k4 || !cdata) return DBSRG_EINVAL;
  finalize(L);
  auto it = L->merged.find({kpol, itype});
  if (it == L->merged.end()) return DBSRG_OK;
  const auto &v = it->second;
  for (size_t q = 0; q < v.size(); q++) {
    k1[q] = v[q].k1;
    k2[q] = v[q].k2;
    k3[q] = v[q].k3;
    k4[q] = v[q].k4;
    cdata[q] = v[q].c;
  }
  return DBSRG_OK;
}

extern "C" int dbsrg_lists_gen_matrix(dbsrg_lists *L, dbsrg_ctx *ctx) {
  if (!L || !ctx) return DBSRG_EINVAL;
  finalize(L);
  // Add_matrix per (kpol, itype), kpol outer, itype inner (state_res.f90:187-191),
  // every non-empty list: Gen_matrix takes every structure of every icase
  std::vector<int> k1, k2, k3, k4;
  std::vector<double> cd;
  for (const auto &kv : L->merged) {
    const auto &v = kv.second;
    if (v.empty()) continue;
    k1.resize(v.size());
    k2.resize(v.size());
    k3.resize(v.size());
    k4.resize(v.size());
    cd.resize(v.size());
    for (size_t q = 0; q < v.size(); q++) {
      k1[q] = v[q].k1;
      k2[q] = v[q].k2;
      k3[q] = v[q].k3;
      k4[q] = v[q].k4;
      cd[q] = v[q].c;
    }
    const int rc = dbsrg_gen_matrix(ctx, L->icase, kv.first.second, kv.first.first, (int)v.size(),
                                    nullptr, k1.data(), k2.data(), k3.data(), k4.data(),
                                    cd.data());
    if (rc) return rc;
  }
  return DBSRG_OK;
}
