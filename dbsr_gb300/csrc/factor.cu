// factor.cu -- the factored contraction of the chosen form.
//
// The R^k / S^k tables are sums of cell contributions (mrk_*/msk_*,
// dbsr_lib_dbs.f90:2898-3833): for electron-1 functions on interval iv and
// electron-2 functions on interval jv, a cell with iv < jv is the product of
// two 1-D moments, lo1(pair1,iv)*hi2(pair2,jv); iv > jv gives
// lo2(pair2,jv)*hi1(pair1,iv) (R^k only); iv == jv the diagonal-cell integral
// rkd.  The contraction of a table with a segment's density uses that
// structure instead of the assembled table:
//
// exchange (convol cases 3/4, the full ns x ns block of R_data itype 4 and
// S_data itypes 8/9):  out(x,y) = sum_e c_e K_{a_e b_e}(x,y), where x, y are
// the output functions of electrons 1 and 2 and a_e, b_e the bound orbitals
// of the entry.  When y - x >= 9 every contributing cell has iv < jv and
//     K_ab(x,y) = U_a(x) V_b(y),  U_a(x) = sum_iv sum_x' lo1(x,x';iv) p_a(x'),
//                                 V_b(y) = sum_jv sum_y' hi2(y',y;jv) p_b(y'),
// so out = U C V^T on that far field (C = the segment's coefficients over
// bound-orbital pairs); likewise x - y >= 9 gives Ul C Vl^T (R^k).  The band
// |y - x| <= 8 is gathered from the table itself with a band-limited
// density (|x' - y'| <= 24 is all the band needs).
//
// direct (convol cases 1/2, the band results of R_data itype 3 and S_data
// itypes 6/7): the output band of one electron's pair is
//     sum_iv [lo1(pair;iv) Suf_hi(iv) + hi1(pair;iv) Pre_lo(iv) + sum_pair2 rkd(pair,pair2;iv) rho(pair2)]
// with Suf/Pre the suffix/prefix sums over cells of the other electron's
// moment-weighted density -- the diagonal cells are the only non-separable
// part.
//
// All of this is FP64; with job.split the far-field product runs as
// split-precision products on the tensor cores (farfield_tc.cu).
#include "internal.cuh"

#include <algorithm>

namespace {

constexpr int NB_MAX = 64;   // bound orbitals handled by the far-field kernels
constexpr int XB_HALF = 24;  // half width of the band-limited density
constexpr int XB_W = 2 * XB_HALF + 1;
constexpr int FAR = 9;       // |y - x| >= FAR is far field (spline orders <= 9)

struct PairSpec {
  int k1, k2, sym;  // orders of the first / second function; packed symmetric
};

__device__ __forceinline__ int pidx(PairSpec s, int h1, int h2) {  // 1-based locals
  if (s.sym) {
    int a = min(h1, h2), b = max(h1, h2);
    return (a - 1) * s.k1 - ((a - 1) * (a - 2)) / 2 + (b - a);
  }
  return (h1 - 1) * s.k2 + (h2 - 1);
}

// bases of the four functions of a table: 1 = P, 2 = Q
struct TableBases {
  int a1, a2, b1, b2;
  PairSpec e1, e2;
};

TableBases table_bases(const DeviceGrid &g, int family, int type) {
  TableBases t;
  auto ord = [&](int b) { return b == 1 ? g.ksp : g.ksq; };
  if (family == 0) {
    int A = (type == 0 || type == 2) ? 1 : 2, B = (type == 0 || type == 3) ? 1 : 2;
    t.a1 = t.a2 = A;
    t.b1 = t.b2 = B;
    t.e1 = {ord(A), ord(A), 1};
    t.e2 = {ord(B), ord(B), 1};
  } else {
    t.a1 = 1;
    t.a2 = 2;
    t.b1 = type == 0 ? 1 : 2;
    t.b2 = type == 0 ? 2 : 1;
    t.e1 = {g.ksp, g.ksq, 0};
    t.e2 = {ord(t.b1), ord(t.b2), 0};
  }
  return t;
}

// ---------------------------------------------------------------------------
// far-field vectors of one electron: Ulo(x,a) = sum_iv sum_xc mlo(pair;iv) p_a(xc)
// (and Uhi with mhi), x the output function, xc the contracted one.
__global__ void k_far_vectors(int ns, int nv, int kk, int nb, const int *b2o, const double *pq,
                              PairSpec e, int out_first, int ko, int kc, int ccomp,
                              const double *mlo, const double *mhi, double *Ulo, double *Uhi) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ns * nb) return;
  int x = q % ns + 1, a = q / ns;
  const double *p = pq + (size_t)ns * (ccomp - 1) + (size_t)2 * ns * (b2o[a] - 1) - 1;
  double slo = 0.0, shi = 0.0;
  for (int iv = max(1, x - ko + 1); iv <= min(nv, x); iv++) {
    int ho = x - iv + 1;
    for (int hc = 1; hc <= kc; hc++) {
      int xc = iv + hc - 1;
      if (xc > ns) break;
      int pi = out_first ? pidx(e, ho, hc) : pidx(e, hc, ho);
      size_t o = (size_t)pi + (size_t)kk * (iv - 1);
      slo = fma(mlo[o], p[xc], slo);
      if (mhi) shi = fma(mhi[o], p[xc], shi);
    }
  }
  Ulo[q] = slo;
  if (Uhi) Uhi[q] = shi;
}

// Z(a,y) = sum_{e in segment, bound(K2)=a} c_e V(y, bound(K3)), also Zl with Vl
__global__ void k_far_z(int ns, int nb, int nm, const int *members, const SegInfo *info,
                        const int *k2, const int *k3, const double *cd, const int *bmap,
                        const double *V, const double *Vl, double *Z, double *Zl) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ns * nb) return;
  int a = q % nb, y = q / nb;
  int slot = blockIdx.y;
  SegInfo si = info[members[slot]];
  double z = 0.0, zl = 0.0;
  for (int e = si.start; e < si.end; e++) {
    if (bmap[k2[e] - 1] != a) continue;
    int b = bmap[k3[e] - 1];
    z = fma(cd[e], V[(size_t)y + (size_t)ns * b], z);
    if (Vl) zl = fma(cd[e], Vl[(size_t)y + (size_t)ns * b], zl);
  }
  size_t o = (size_t)slot * nb * ns + q;  // Z[slot][a + nb*y]
  Z[o] = z;
  if (Zl) Zl[o] = zl;
}

// band-limited exchange density: Xb(xc, d) = sum_e c_e p1(xc) p2(xc+d-24)
__global__ void k_density_band(int ns, int nm, const int *members, const SegInfo *info,
                               const int *k2, const int *k3, const double *cd, const double *pq,
                               int jp1, int jp2, double *Xb) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ns * XB_W) return;
  int xc = q % ns, d = q / ns;
  int yc = xc + d - XB_HALF;
  int slot = blockIdx.y;
  SegInfo si = info[members[slot]];
  double acc = 0.0;
  if (yc >= 0 && yc < ns) {
    for (int e = si.start; e < si.end; e++) {
      double p1 = pq[(size_t)xc + (size_t)ns * (jp1 - 1) + (size_t)2 * ns * (k2[e] - 1)];
      double p2 = pq[(size_t)yc + (size_t)ns * (jp2 - 1) + (size_t)2 * ns * (k3[e] - 1)];
      acc = acc + cd[e] * (p1 * p2);
    }
  }
  Xb[(size_t)slot * ns * XB_W + q] = acc;
}

// far field out(x,y) = U(x,:) Z(:,y) for y-x >= FAR, Ul(x,:) Zl(:,y) for
// x-y >= FAR; 32x32 output tiles, 256 threads with 4 outputs each, the
// orbital dimension staged through shared memory 32 at a time.
constexpr int FK = 32;
__global__ void __launch_bounds__(256) k_far_field(int ns, int nb, const double *U,
                                                   const double *Ul, const double *Z,
                                                   const double *Zl, double *Y, size_t per) {
  __shared__ double su[32][FK + 1], sz[FK][33];
  __shared__ double sul[32][FK + 1], szl[FK][33];
  const int slot = blockIdx.z;
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
  const bool any_up = (y0 + 31) - x0 >= FAR, lo_region = (x0 + 31) - y0 >= FAR;
  const bool any_lo = Ul && lo_region;  // S^k tables have no lower field: zeros there
  if (!any_up && !lo_region) return;
  const double *Zs = Z + (size_t)slot * nb * ns;
  const double *Zls = Zl ? Zl + (size_t)slot * nb * ns : nullptr;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int a0 = 0; a0 < nb; a0 += FK) {
    const int na = min(FK, nb - a0);
    for (int q = threadIdx.x; q < 32 * FK; q += 256) {
      int r = q % 32, a = q / 32;
      int x = x0 + r, y = y0 + r;
      bool ok = a < na;
      su[r][a] = (ok && x < ns && any_up) ? U[(size_t)x + (size_t)ns * (a0 + a)] : 0.0;
      sz[a][r] = (ok && y < ns && any_up) ? Zs[(size_t)(a0 + a) + (size_t)nb * y] : 0.0;
      sul[r][a] = (ok && x < ns && any_lo) ? Ul[(size_t)x + (size_t)ns * (a0 + a)] : 0.0;
      szl[a][r] = (ok && y < ns && any_lo) ? Zls[(size_t)(a0 + a) + (size_t)nb * y] : 0.0;
    }
    __syncthreads();
    for (int t = 0; t < 4; t++) {
      int q = threadIdx.x + 256 * t;
      int r = q % 32, cc = q / 32;
      int d = (y0 + cc) - (x0 + r);
      double s = acc[t];
      if (d >= FAR)
        for (int a = 0; a < na; a++) s = fma(su[r][a], sz[a][cc], s);
      else if (d <= -FAR)
        for (int a = 0; a < na; a++) s = fma(sul[r][a], szl[a][cc], s);
      acc[t] = s;
    }
    __syncthreads();
  }
  double *Ys = Y + (size_t)slot * per;
  for (int t = 0; t < 4; t++) {
    int q = threadIdx.x + 256 * t;
    int r = q % 32, cc = q / 32;
    int x = x0 + r, y = y0 + cc;
    if (x >= ns || y >= ns) continue;
    int d = y - x;
    if (d >= FAR || d <= -FAR) Ys[(size_t)x + (size_t)ns * y] = acc[t];
  }
}

// band |y-x| <= 8 of the exchange result from the table and the band density
// (the gather of k_exchange in assemble.cu restricted to the band).
// mode 0: R table 's','s' case 3; 1: S 'n','n' case 3; 2: S 'n','n' case 4.
__global__ void __launch_bounds__(256) k_band_exchange(int ns, int ks, int mode,
                                                       const double *__restrict__ rkb,
                                                       const double *__restrict__ Xb,
                                                       double *__restrict__ Y, size_t per) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int nd = 2 * (FAR - 1) + 1;
  if (q >= ns * nd) return;
  const int slot = blockIdx.y;
  const int x = q % ns + 1, y = x + q / ns - (FAR - 1);
  if (y < 1 || y > ns) return;
  const double *D = Xb + (size_t)slot * ns * XB_W;
  auto DV = [&](int i, int j) -> double {
    return __ldg(&D[(size_t)(i - 1) + (size_t)ns * (j - i + XB_HALF)]);
  };
  double acc = 0.0;
  // band table: rkb(i, j-i+BW+1, ip, jp), |j - i| <= BW (= 16) is all that
  // the band outputs read
  constexpr int BW = DBSRG_TABLE_BAND, NJ = 2 * DBSRG_TABLE_BAND + 1;
  if (mode == 0) {
    auto TB = [&](int i, int j, int ip, int jp) -> double {
      return __ldg(&rkb[(size_t)(i - 1) + (size_t)ns * ((size_t)(j - i + BW) +
                        (size_t)NJ * ((size_t)(ip - 1) + (size_t)ks * (size_t)(jp - 1)))]);
    };
    for (int jp = 1; jp <= ks; jp++)
      for (int ip = 1; ip <= ks; ip++) {
        if (y - jp + 1 >= 1 && x + ip - 1 <= ns)
          acc = fma(TB(x, y - jp + 1, ip, jp), DV(x + ip - 1, y - jp + 1), acc);
        if (ip > 1 && x - ip + 1 >= 1 && y - jp + 1 >= 1)
          acc = fma(TB(x - ip + 1, y - jp + 1, ip, jp), DV(x - ip + 1, y - jp + 1), acc);
        if (jp > 1 && x + ip - 1 <= ns && y + jp - 1 <= ns)
          acc = fma(TB(x, y, ip, jp), DV(x + ip - 1, y + jp - 1), acc);
        if (ip > 1 && jp > 1 && x - ip + 1 >= 1 && y + jp - 1 <= ns)
          acc = fma(TB(x - ip + 1, y, ip, jp), DV(x - ip + 1, y + jp - 1), acc);
      }
  } else {
    const int kb = 2 * ks - 1;
    auto TB = [&](int i, int j, int ip, int jp) -> double {
      return __ldg(&rkb[(size_t)(i - 1) + (size_t)ns * ((size_t)(j - i + BW) +
                        (size_t)NJ * ((size_t)(ip - 1) + (size_t)kb * (size_t)(jp - 1)))]);
    };
    for (int jp = 1; jp <= kb; jp++)
      for (int ip = 1; ip <= kb; ip++) {
        if (mode == 1) {
          int j = y - jp + ks, ii = x + ip - ks;
          if (j < max(1, 1 + ks - jp) || j > min(ns, ns + ks - jp)) continue;
          if (x < max(1, 1 + ks - ip) || x > min(ns, ns + ks - ip)) continue;
          acc = fma(TB(x, j, ip, jp), DV(ii, j), acc);
        } else {
          int i = x - ip + ks, jj = y + jp - ks;
          if (y < max(1, 1 + ks - jp) || y > min(ns, ns + ks - jp)) continue;
          if (i < max(1, 1 + ks - ip) || i > min(ns, ns + ks - ip)) continue;
          acc = fma(TB(i, y, ip, jp), DV(i, jj), acc);
        }
      }
  }
  Y[(size_t)slot * per + (size_t)(x - 1) + (size_t)ns * (y - 1)] = acc;
}

// ---------------------------------------------------------------------------
// direct contraction, one thread block per (segment slot): cell sums of the
// density electron, prefix/suffix sums over cells, then the output band.
//   icv 1: output electron-1 pair band, density over electron-2 pairs
//   icv 2: output electron-2 pair band, density over electron-1 pairs (S^k)
// storage: 's' Y(x,ip) x'=x+ip-1 (R^k), 'n' Y(x,ip) x'=x+ip-ks (S^k)
__global__ void __launch_bounds__(256) k_direct(int ns, int ks, int nv, int kk, int icv,
                                                char sym, PairSpec e1, PairSpec e2,
                                                const double *lo1, const double *hi1,
                                                const double *lo2, const double *hi2,
                                                const double *rkd, const double *X, double *Y,
                                                size_t per) {
  extern __shared__ double sh[];
  double *s_a = sh;        // cell sums (hi for icv1 upper, lo1 for icv2)
  double *s_b = sh + nv;   // icv1 lower (R^k)
  const int slot = blockIdx.x;
  const double *Xs = X + (size_t)slot * per;
  const int ncol = sym == 's' ? ks : 2 * ks - 1;
  // density value of a pair of absolute indices (first, second) or 0
  auto rho = [&](int f, int s2) -> double {
    if (f < 1 || s2 < 1 || f > ns || s2 > ns) return 0.0;
    if (sym == 's') {
      int lo = min(f, s2), dd = abs(f - s2);
      if (dd >= ks) return 0.0;
      return Xs[(size_t)(lo - 1) + (size_t)ns * dd];
    }
    int c = s2 - f + ks;
    if (c < 1 || c > 2 * ks - 1) return 0.0;
    return Xs[(size_t)(f - 1) + (size_t)ns * (c - 1)];
  };
  PairSpec ed = icv == 1 ? e2 : e1;  // electron whose pairs carry the density
  // phase 1: moment-weighted density per cell of the density electron
  for (int cv = threadIdx.x + 1; cv <= nv; cv += blockDim.x) {
    double sa = 0.0, sb = 0.0;
    for (int h1 = 1; h1 <= ed.k1; h1++)
      for (int h2 = ed.sym ? h1 : 1; h2 <= ed.k2; h2++) {
        double r = rho(cv + h1 - 1, cv + h2 - 1);
        size_t o = (size_t)pidx(ed, h1, h2) + (size_t)kk * (cv - 1);
        if (icv == 1) {
          sa = fma(hi2[o], r, sa);
          if (lo2) sb = fma(lo2[o], r, sb);
        } else {
          sa = fma(lo1[o], r, sa);
        }
      }
    s_a[cv - 1] = sa;
    s_b[cv - 1] = sb;
  }
  __syncthreads();
  // phase 2: icv1 -> s_a := suffix sums sum_{jv>iv}, s_b := prefix sums
  // sum_{jv<iv}; icv2 -> s_a := prefix sums sum_{iv<jv}
  if (threadIdx.x == 0) {
    if (icv == 1) {
      double acc = 0.0;
      for (int iv = nv; iv >= 1; iv--) {
        double v = s_a[iv - 1];
        s_a[iv - 1] = acc;
        acc += v;
      }
      acc = 0.0;
      for (int iv = 1; iv <= nv; iv++) {
        double v = s_b[iv - 1];
        s_b[iv - 1] = acc;
        acc += v;
      }
    } else {
      double acc = 0.0;
      for (int iv = 1; iv <= nv; iv++) {
        double v = s_a[iv - 1];
        s_a[iv - 1] = acc;
        acc += v;
      }
    }
  }
  __syncthreads();
  // phase 3a: the separable (off-diagonal cell) terms into the output band,
  // kept in shared memory
  PairSpec eo = icv == 1 ? e1 : e2;
  double *out = sh + 2 * nv;               // ns * ncol
  double *rho_w = out + (size_t)ns * ncol; // 81 values per warp
  for (int q = threadIdx.x; q < ns * ncol; q += blockDim.x) {
    int f = q % ns + 1, col = q / ns + 1;
    int s2 = sym == 's' ? f + col - 1 : f + col - ks;
    double acc = 0.0;
    if (s2 >= 1 && s2 <= ns) {
      int lo = max(max(1, f - eo.k1 + 1), s2 - eo.k2 + 1), hi = min(min(nv, f), s2);
      for (int cv = lo; cv <= hi; cv++) {
        size_t o = (size_t)pidx(eo, f - cv + 1, s2 - cv + 1) + (size_t)kk * (cv - 1);
        if (icv == 1) {
          acc = fma(lo1[o], s_a[cv - 1], acc);
          if (hi1) acc = fma(hi1[o], s_b[cv - 1], acc);
        } else {
          acc = fma(hi2[o], s_a[cv - 1], acc);
        }
      }
    }
    out[q] = acc;
  }
  __syncthreads();
  // phase 3b: diagonal cells, one warp per cell.  Cell cv touches outputs
  // with first index in [cv, cv+8], so cells 9 apart never share an output:
  // nine phases of disjoint cells give every output one writer at a time.
  const int lane = threadIdx.x % 32, warp = threadIdx.x / 32, nwarp = blockDim.x / 32;
  const int npo = eo.sym ? eo.k1 * (eo.k1 + 1) / 2 : eo.k1 * eo.k2;
  double *rw = rho_w + 81 * warp;
  for (int ph = 0; ph < 9; ph++) {
    for (int cv = ph + 1 + 9 * warp; cv <= nv; cv += 9 * nwarp) {
      // stage the cell's density pairs, one pair per lane
      const int npd = ed.sym ? ed.k1 * (ed.k1 + 1) / 2 : ed.k1 * ed.k2;
      for (int pd = lane; pd < npd; pd += 32) {
        int g1, g2;
        if (ed.sym) {
          int r = pd, row = 0;
          while (r >= ed.k1 - row) {
            r -= ed.k1 - row;
            row++;
          }
          g1 = row + 1;
          g2 = row + 1 + r;
        } else {
          g1 = pd / ed.k2 + 1;
          g2 = pd % ed.k2 + 1;
        }
        rw[pd] = rho(cv + g1 - 1, cv + g2 - 1);
      }
      __syncwarp();
      for (int po = lane; po < npo; po += 32) {
        int h1, h2;
        if (eo.sym) {
          int r = po, row = 0;
          while (r >= eo.k1 - row) {
            r -= eo.k1 - row;
            row++;
          }
          h1 = row + 1;
          h2 = row + 1 + r;
        } else {
          h1 = po / eo.k2 + 1;
          h2 = po % eo.k2 + 1;
        }
        int f = cv + h1 - 1, s2 = cv + h2 - 1;
        if (f > ns || s2 > ns) continue;
        double acc = 0.0;
        if (icv == 1) {
          const double *rk = rkd + (size_t)po + (size_t)kk * (size_t)kk * (cv - 1);
          for (int pd = 0; pd < npd; pd++) acc = fma(rk[(size_t)kk * pd], rw[pd], acc);
        } else {
          const double *rk = rkd + (size_t)kk * ((size_t)po + (size_t)kk * (cv - 1));
          for (int pd = 0; pd < npd; pd++) acc = fma(rk[pd], rw[pd], acc);
        }
        int q = sym == 's' ? (f - 1) + ns * (s2 - f) : (f - 1) + ns * (s2 - f + ks - 1);
        out[q] += acc;
      }
      __syncwarp();
    }
    __syncthreads();
  }
  for (int q = threadIdx.x; q < ns * ncol; q += blockDim.x) Y[(size_t)slot * per + q] = out[q];
}

__global__ void k_check_bound(int n, const int *k2, const int *k3, const int *bmap, int *err) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  if (bmap[k2[e] - 1] < 0 || bmap[k3[e] - 1] < 0) atomicExch(err, 3);
}

}  // namespace

int ensure_fscratch(dbsrg_ctx *c, size_t bytes) {
  if (c->fscratch_bytes >= bytes) return DBSRG_OK;
  if (c->fscratch) {
    cudaStreamSynchronize(c->stream);
    cudaFree(c->fscratch);
    c->fscratch = nullptr;
    c->fscratch_bytes = 0;
  }
  size_t want = bytes + bytes / 4;
  if (cudaMalloc(&c->fscratch, want) != cudaSuccess) {
    cudaGetLastError();
    if (cudaMalloc(&c->fscratch, bytes) != cudaSuccess) {
      c->fscratch = nullptr;
      return set_err(c, DBSRG_ENOMEM, "factor scratch allocation failed");
    }
    want = bytes;
  }
  c->fscratch_bytes = want;
  return DBSRG_OK;
}

int check_bound_orbitals(dbsrg_ctx *c, int n, const int *k2, const int *k3, int *derr) {
  if (n <= 0) return DBSRG_OK;
  DBSRG_RUN(c, "k_check_bound",
            k_check_bound<<<(n + 255) / 256, 256, 0, c->stream>>>(n, k2, k3, c->bmap, derr));
  return DBSRG_OK;
}

// far-field vectors of (family, type, k, exchange case), cached
static int get_farfield(dbsrg_ctx *c, int family, int type, int k, int cs, const FarField **out) {
  std::vector<FarField> &v = family == 0 ? c->rfar : c->sfar;
  size_t idx = ((size_t)k * (family == 0 ? 4 : 2) + type) * 2 + (cs == 4 ? 1 : 0);
  if (v.size() <= idx) v.resize(idx + 1);
  if (v[idx].U) {
    *out = &v[idx];
    return DBSRG_OK;
  }
  const DeviceGrid &g = c->g;
  const CellData *cd;
  int rc = get_celldata(c, family, type, k, &cd);
  if (rc) return rc;
  const int ns = g.ns, nb = c->nbound, kk = g.ks * g.ks;
  size_t m = (size_t)ns * nb;
  double *base = nullptr;
  if (cudaMalloc((void **)&base, 4 * m * sizeof(double)) != cudaSuccess)
    return set_err(c, DBSRG_ENOMEM, "far-field allocation failed");
  FarField f;
  f.U = base;
  f.V = base + m;
  f.Ul = family == 0 ? base + 2 * m : nullptr;
  f.Vl = family == 0 ? base + 3 * m : nullptr;
  TableBases tb = table_bases(g, family, type);
  auto ord = [&](int b) { return b == 1 ? g.ksp : g.ksq; };
  // electron 1: case 3 output = first function, contracted = second
  int o1f = cs == 3 ? 1 : 0;
  int ko1 = ord(cs == 3 ? tb.a1 : tb.a2), kc1 = ord(cs == 3 ? tb.a2 : tb.a1);
  int cc1 = cs == 3 ? tb.a2 : tb.a1;
  // electron 2: case 3 output = second function, contracted = first
  int o2f = cs == 3 ? 0 : 1;
  int ko2 = ord(cs == 3 ? tb.b2 : tb.b1), kc2 = ord(cs == 3 ? tb.b1 : tb.b2);
  int cc2 = cs == 3 ? tb.b1 : tb.b2;
  unsigned nbk = (unsigned)((m + 127) / 128);
  DBSRG_RUN(c, "k_far_vectors",
            k_far_vectors<<<nbk, 128, 0, c->stream>>>(ns, g.nv, kk, nb, c->b2o, c->pq, tb.e1, o1f,
                                                      ko1, kc1, cc1, cd->lo1,
                                                      family == 0 ? cd->hi1 : nullptr, f.U, f.Ul));
  DBSRG_RUN(c, "k_far_vectors",
            k_far_vectors<<<nbk, 128, 0, c->stream>>>(ns, g.nv, kk, nb, c->b2o, c->pq, tb.e2, o2f,
                                                      ko2, kc2, cc2, cd->hi2,
                                                      family == 0 ? cd->lo2 : nullptr, f.V, f.Vl));
  v[idx] = f;
  *out = &v[idx];
  return DBSRG_OK;
}

int farfield_tc(dbsrg_ctx *c, int ns, int nb, int nm, const double *U, const double *Ul,
                const double *Z, const double *Zl, double *Y, size_t per);

int factored_contract(dbsrg_ctx *c, const FactorJob &j) {
  const DeviceGrid &g = c->g;
  const int ns = g.ns, ks = g.ks, nv = g.nv, kk = ks * ks, nb = c->nbound;
  cudaStream_t st = c->stream;
  int rc;
  if (j.icv >= 3) {
    if (nb < 1 || nb > NB_MAX) return set_err(c, DBSRG_EINVAL, "factored exchange: 1..64 bound orbitals");
    size_t xb = (size_t)j.nm * ns * XB_W, zs = (size_t)j.nm * nb * ns;
    if ((rc = ensure_fscratch(c, (xb + 2 * zs) * sizeof(double)))) return rc;
    double *Xb = (double *)c->fscratch, *Z = Xb + xb, *Zl = Z + zs;
    for (int a = 0; a < j.na; a++) {
      const int cs = j.icv;
      const FarField *f;
      if ((rc = get_farfield(c, j.family, j.types[a], j.kpol, cs, &f))) return rc;
      TableBases tb = table_bases(g, j.family, j.types[a]);
      int c1 = cs == 3 ? tb.a2 : tb.a1, c2 = cs == 3 ? tb.b1 : tb.b2;
      if (c1 != j.jp1[a] || c2 != j.jp2[a])
        return set_err(c, DBSRG_EINVAL, "factored exchange: component mismatch");
      double *Ya = j.Y + (size_t)a * j.nm * j.per;
      dim3 gz((unsigned)((ns * nb + 127) / 128), (unsigned)j.nm);
      DBSRG_RUN(c, "k_far_z",
                k_far_z<<<gz, 128, 0, st>>>(ns, nb, j.nm, j.members, j.info, j.k2, j.k3, j.cd,
                                            c->bmap, f->V, f->Vl, Z, f->Vl ? Zl : nullptr));
      if (j.split) {
        if ((rc = farfield_tc(c, ns, nb, j.nm, f->U, f->Ul, Z, f->Vl ? Zl : nullptr, Ya, j.per)))
          return rc;
      } else {
        dim3 gf((unsigned)((ns + 31) / 32), (unsigned)((ns + 31) / 32), (unsigned)j.nm);
        DBSRG_RUN(c, "k_far_field",
                  k_far_field<<<gf, 256, 0, st>>>(ns, nb, f->U, f->Ul, Z, f->Vl ? Zl : nullptr, Ya,
                                                  j.per));
      }
      dim3 gb((unsigned)((ns * XB_W + 255) / 256), (unsigned)j.nm);
      DBSRG_RUN(c, "k_density_band",
                k_density_band<<<gb, 256, 0, st>>>(ns, j.nm, j.members, j.info, j.k2, j.k3, j.cd,
                                                   c->pq, j.jp1[a], j.jp2[a], Xb));
      int mode = j.family == 0 ? 0 : (cs == 3 ? 1 : 2);
      dim3 gx((unsigned)((ns * (2 * FAR - 1) + 255) / 256), (unsigned)j.nm);
      DBSRG_RUN(c, "k_band_exchange",
                k_band_exchange<<<gx, 256, 0, st>>>(ns, ks, mode, j.tabs[a], Xb, Ya, j.per));
    }
    return DBSRG_OK;
  }
  // direct
  for (int a = 0; a < j.na; a++) {
    const CellData *cd;
    if ((rc = get_celldata(c, j.family, j.types[a], j.kpol, &cd))) return rc;
    TableBases tb = table_bases(g, j.family, j.types[a]);
    const double *Xa = j.X + (size_t)a * j.nm * j.per;
    double *Ya = j.Y + (size_t)a * j.nm * j.per;
    const int ncol = j.sym == 's' ? ks : 2 * ks - 1;
    size_t smem = (2 * (size_t)nv + (size_t)ns * ncol + 81 * 8) * sizeof(double);
    if (smem > 200 * 1024) return set_err(c, DBSRG_EINVAL, "direct contraction: ns too large");
    if (smem > 48 * 1024)
      DBSRG_TRY(c, cudaFuncSetAttribute(k_direct, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
    DBSRG_RUN(c, "k_direct",
              k_direct<<<j.nm, 256, smem, st>>>(ns, ks, nv, kk, j.icv, j.sym, tb.e1, tb.e2,
                                                cd->lo1, j.family == 0 ? cd->hi1 : nullptr,
                                                j.family == 0 ? cd->lo2 : nullptr, cd->hi2,
                                                cd->rkd, Xa, Ya, j.per));
  }
  return DBSRG_OK;
}
