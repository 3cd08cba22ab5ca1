// factor.cu -- the factored contraction of the chosen form.
//
// The R^k / S^k tables are sums of cell contributions (mrk_*/msk_*,
// dbsr_lib_dbs.f90:2898-3833): for electron-1 functions on interval iv and
// electron-2 functions on interval jv, a cell with iv < jv is the product of
// two 1-D moments, lo1(pair1,iv)*hi2(pair2,jv); iv > jv gives
// lo2(pair2,jv)*hi1(pair1,iv) (R^k only); iv == jv the diagonal-cell integral
// rkd.  A segment's density is a sum over its entries of orbital products,
// rho = sum_e c_e p1_{a_e} (x) p2_{b_e} with a_e, b_e the bound orbitals of
// K2, K3, so every contraction is linear in the ordered bound-orbital pairs
// (a,b).  The factored path therefore works per table with those pairs and
// per segment only with its coefficients:
//
// exchange (convol cases 3/4: R_data itype 4, S_data itypes 8/9), result
// out(x,y) over the output functions x, y of electrons 1 and 2:
//   far field |y-x| >= 9: every contributing cell has iv < jv, so
//     out = U C V^T with U_a(x) = sum_iv sum_x' lo1(x,x';iv) p_a(x'),
//     V_b(y) = sum_jv sum_y' hi2(y',y;jv) p_b(y') and C the segment's
//     coefficients over pairs (x-y >= 9: Ul C Vl^T, R^k only; zero for S^k);
//   near band |y-x| <= 8: out = sum_e c_e Kb_{a_e b_e}, where the band pair
//     potential Kb_ab(x,y) = sum_(i,j) W_xy(i,j) p1_a(i) p2_b(j) holds the
//     band-table element W_xy(i,j) that the exchange gather pairs with
//     density element (i,j) (built once per table, in two separable stages).
//
// direct (convol cases 1/2: R_data itype 3, S_data itypes 6/7): the band
// result is sum_e c_e Kd_{a_e b_e}, with the direct pair potential
//   Kd_ab(pair1) = sum_iv [lo1(pair1;iv) Suf_ab(iv) + hi1(pair1;iv) Pre_ab(iv)]
//                + sum_{pair2} rkd(pair1,pair2;iv) rho_ab(pair2)   (iv = jv)
// Suf/Pre the suffix/prefix sums over cells of the moment-weighted density of
// the pair, and rho_ab the pair density in the reference's storage (the
// symmetric 's' storage sums both orders, p1(f)p2(s)+p1(s)p2(f)).
//
// The per-segment work is then a sum of a few dozen potential rows per
// output element, fused into the scatter for the direct cases.  All of this
// is FP64; with job.split the exchange far field runs as split-precision
// products on the tensor cores, fused with the near band and the scatter
// (exchange_tc.cu).
#include "internal.cuh"
#include "ff.cuh"

#include <algorithm>
#include <type_traits>

namespace {

constexpr int NB_MAX = 128;       // bound orbitals handled by the factored path
constexpr int FAR = 9;            // |y - x| >= FAR is far field (spline orders <= 9)
constexpr int BAND = FAR - 1;     // near band |y - x| <= 8
constexpr int NDB = 2 * BAND + 1; // band diagonals
constexpr int PXC = 4;            // output rows per block of the band pair potentials
constexpr int PBC = 4;            // second-orbital chunk of the diagonal-cell stage

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

// target quadrants of the atypes of one list (UPDATE_HS)
struct QuadSpec {
  int na;
  int ii[4], jj[4];
};

// direct pair potentials of the atypes of one list (FP64, or float-float
// pairs in the split form)
struct KdSet {
  const double *K[4];
  const float2 *Kf[4];
};

// ---------------------------------------------------------------------------
// bound-orbital rows of one component: P[a*ns + x] = pq(x+1, comp, b2o[a])
__global__ void k_bound_rows(int ns, int nb, const int *b2o, const double *pq, int comp,
                             double *P) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ns * nb) return;
  int x = q % ns, a = q / ns;
  P[q] = pq[(size_t)x + (size_t)ns * (comp - 1) + (size_t)2 * ns * (b2o[a] - 1)];
}

// ordered bound-orbital pair of every entry
__global__ void k_pair_index(int n, const int *k2, const int *k3, const int *bmap, int nb,
                             int *pairs, int *err) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  int a = bmap[k2[e] - 1], b = bmap[k3[e] - 1];
  if (a < 0 || b < 0) {
    atomicExch(err, 3);
    pairs[e] = 0;
    return;
  }
  pairs[e] = a * nb + b;
}

// ---------------------------------------------------------------------------
// far-field vectors of one electron: Ulo(x,a) = sum_iv sum_xc mlo(pair;iv) p_a(xc)
// (and Uhi with mhi), x the output function, xc the contracted one.
// both electrons' vectors in one launch (blockIdx.y)
struct FarSide {
  PairSpec e;
  int out_first, ko, kc, ccomp;
  const double *mlo, *mhi;
  double *Ulo, *Uhi;
};

__global__ void k_far_vectors(int ns, int nv, int kk, int nb, const int *b2o, const double *pq,
                              const FarSide s0, const FarSide s1) {
  const FarSide &sd = blockIdx.y ? s1 : s0;
  const PairSpec e = sd.e;
  const int out_first = sd.out_first, ko = sd.ko, kc = sd.kc, ccomp = sd.ccomp;
  const double *mlo = sd.mlo, *mhi = sd.mhi;
  double *Ulo = sd.Ulo, *Uhi = sd.Uhi;
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

// Z(a,y) = sum_{e in segment, first orbital a} c_e V(y, second orbital), also Zl with Vl
__global__ void k_far_z(int ns, int nb, const int *members, const SegInfo *info,
                        const int *pairs, const double *cd, const double *V, const double *Vl,
                        double *Z, double *Zl) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ns * nb) return;
  int a = q % nb, y = q / nb;
  int slot = blockIdx.y;
  SegInfo si = info[members[slot]];
  double z = 0.0, zl = 0.0;
  for (int e = si.start; e < si.end; e++) {
    const int pr = pairs[e];
    if (pr / nb != a) continue;
    const int b = pr - a * nb;
    z = fma(cd[e], V[(size_t)y + (size_t)ns * b], z);
    if (Vl) zl = fma(cd[e], Vl[(size_t)y + (size_t)ns * b], zl);
  }
  size_t o = (size_t)slot * nb * ns + q;  // Z[slot][a + nb*y]
  Z[o] = z;
  if (Zl) Zl[o] = zl;
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
  const bool any_up = (y0 + 31) - x0 >= FAR;
  const bool any_lo = Ul && (x0 + 31) - y0 >= FAR;
  if (!any_up && !any_lo) return;
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
    if (d >= FAR || (Ul && d <= -FAR)) Ys[(size_t)x + (size_t)ns * y] = acc[t];
  }
}

// ---------------------------------------------------------------------------
// band pair potentials of an exchange table, one block per PXC output rows
// and one band diagonal d = y - x:
//   W(x; i, j)  the table element the exchange gather of output (x, y) pairs
//               with density element (i, j) (the gather of k_exchange in
//               assemble.cu, restricted to the band; every (i, j) meets one
//               element, so W needs no sums)
//   H(x; i, b)  = sum_j W(x; i, j) P2(b, j)
//   Kb(ab; x, y) = sum_i P1(a, i) H(x; i, b)
// mode 0: R table 's','s' case 3; 1: S 'n','n' case 3; 2: S 'n','n' case 4.
// Band table layout: rkb(i, j-i+BW+1, ip, jp) for |j - i| <= BW.
// FF: the windows split once into float-float pairs, both stages as
// float-float sums (ff.cuh), Kb written as float-float pairs (float2).
template <bool FF>
__global__ void __launch_bounds__(256) k_pair_band(int ns, int ks, int nb, int mode,
                                                   const double *__restrict__ rkb,
                                                   const double *__restrict__ P1,
                                                   const double *__restrict__ P2,
                                                   void *__restrict__ Kout) {
  using S = typename std::conditional<FF, float2, double>::type;
  extern __shared__ double smraw[];
  S *sm = reinterpret_cast<S *>(smraw);
  const int W = 2 * ks - 1;            // offsets -(ks-1) .. ks-1
  const int WL = PXC + W - 1;          // window of the row vectors
  const int WLP = WL | 1;              // its stride (odd: no bank conflicts across orbitals)
  const int HX = W * nb + 1;           // stride of H per output row (odd)
  const int x0 = blockIdx.x * PXC + 1; // first output row (1-based)
  const int d = (int)blockIdx.y - BAND;
  S *Wm = sm;                          // [PXC][W][W]
  S *p1w = Wm + PXC * W * W;           // [nb][WLP]: P1(a, x0-(ks-1)+t)
  S *p2w = p1w + nb * WLP;             // [nb][WLP]: P2(b, x0+d-(ks-1)+t)
  S *H = p2w + nb * WLP;               // [PXC][HX]: H(xl; u, b) at u*nb + b
  auto sv = [](double v) -> S {
    if constexpr (FF) return ffa::split(v); else return v;
  };
  const int kb = mode == 0 ? ks : 2 * ks - 1;
  constexpr int BW = DBSRG_TABLE_BAND, NJ = 2 * DBSRG_TABLE_BAND + 1;
  auto TB = [&](int i, int j, int ip, int jp) -> double {
    return rkb[(size_t)(i - 1) + (size_t)ns * ((size_t)(j - i + BW) +
               (size_t)NJ * ((size_t)(ip - 1) + (size_t)kb * (size_t)(jp - 1)))];
  };
  for (int q = threadIdx.x; q < PXC * W * W; q += blockDim.x) Wm[q] = sv(0.0);
  for (int q = threadIdx.x; q < nb * WL; q += blockDim.x) {
    const int a = q / WL, t = q % WL;
    const int xi = x0 - (ks - 1) + t, yi = x0 + d - (ks - 1) + t;
    p1w[a * WLP + t] = sv((xi >= 1 && xi <= ns) ? P1[(size_t)a * ns + xi - 1] : 0.0);
    p2w[a * WLP + t] = sv((yi >= 1 && yi <= ns) ? P2[(size_t)a * ns + yi - 1] : 0.0);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < PXC * kb * kb; q += blockDim.x) {
    const int xl = q / (kb * kb), r = q % (kb * kb), ip = r % kb + 1, jp = r / kb + 1;
    const int x = x0 + xl, y = x + d;
    if (x > ns || y < 1 || y > ns) continue;
    S *w = Wm + (size_t)xl * W * W;
    auto put = [&](int i, int j, double v) { w[(i - x + ks - 1) * W + (j - y + ks - 1)] = sv(v); };
    if (mode == 0) {
      if (y - jp + 1 >= 1 && x + ip - 1 <= ns)
        put(x + ip - 1, y - jp + 1, TB(x, y - jp + 1, ip, jp));
      if (ip > 1 && x - ip + 1 >= 1 && y - jp + 1 >= 1)
        put(x - ip + 1, y - jp + 1, TB(x - ip + 1, y - jp + 1, ip, jp));
      if (jp > 1 && x + ip - 1 <= ns && y + jp - 1 <= ns)
        put(x + ip - 1, y + jp - 1, TB(x, y, ip, jp));
      if (ip > 1 && jp > 1 && x - ip + 1 >= 1 && y + jp - 1 <= ns)
        put(x - ip + 1, y + jp - 1, TB(x - ip + 1, y, ip, jp));
    } else if (mode == 1) {
      const int j = y - jp + ks, ii = x + ip - ks;
      if (j < max(1, 1 + ks - jp) || j > min(ns, ns + ks - jp)) continue;
      if (x < max(1, 1 + ks - ip) || x > min(ns, ns + ks - ip)) continue;
      put(ii, j, TB(x, j, ip, jp));
    } else {
      const int i = x - ip + ks, jj = y + jp - ks;
      if (y < max(1, 1 + ks - jp) || y > min(ns, ns + ks - jp)) continue;
      if (i < max(1, 1 + ks - ip) || i > min(ns, ns + ks - ip)) continue;
      put(i, jj, TB(i, y, ip, jp));
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < PXC * W * nb; q += blockDim.x) {
    const int b = q % nb, r = q / nb, u = r % W, xl = r / W;
    const S *w = Wm + ((size_t)xl * W + u) * W;
    const S *p = p2w + (size_t)b * WLP + xl;
    S *hq = H + (size_t)xl * HX + (size_t)u * nb + b;
    if constexpr (FF) {
      float sh = 0.0f, sl = 0.0f;
      for (int v = 0; v < W; v++) ffa::mac(w[v], p[v], sh, sl);
      *hq = ffa::norm(sh, sl);
    } else {
      double s = 0.0;
      for (int v = 0; v < W; v++) s = fma(w[v], p[v], s);
      *hq = s;
    }
  }
  __syncthreads();
  const size_t per = (size_t)ns * NDB;
  for (int q = threadIdx.x; q < PXC * nb * nb; q += blockDim.x) {
    const int xl = q % PXC, pr = q / PXC, b = pr % nb, a = pr / nb;
    const int x = x0 + xl, y = x + d;
    if (x > ns || y < 1 || y > ns) continue;
    const S *p = p1w + (size_t)a * WLP + xl;
    const S *h = H + (size_t)xl * HX + b;
    const size_t o = (size_t)pr * per + (size_t)(x - 1) + (size_t)ns * (d + BAND);
    if constexpr (FF) {
      float sh = 0.0f, sl = 0.0f;
      for (int u = 0; u < W; u++) ffa::mac(p[u], h[(size_t)u * nb], sh, sl);
      static_cast<float2 *>(Kout)[o] = ffa::norm(sh, sl);
    } else {
      double s = 0.0;
      for (int u = 0; u < W; u++) s = fma(p[u], h[(size_t)u * nb], s);
      static_cast<double *>(Kout)[o] = s;
    }
  }
}

// ---------------------------------------------------------------------------
// direct pair potentials.  ed: pairs of the density electron, eo: of the
// output electron.  Pair densities of a symmetric storage give every ordered
// (h1, h2) the moment of the unordered pair (pidx orders them).
//
// (1) cell sums, one block per cell cv:
//   S1(ab, cv) = sum_{h1,h2} M1(h1,h2;cv) P1(a, cv+h1-1) P2(b, cv+h2-1), S2 with M2
__global__ void k_pair_cellsum(int ns, int nv, int kk, int nb, PairSpec ed, const double *M1,
                               const double *M2, const double *P1, const double *P2, double *S1,
                               double *S2) {
  extern __shared__ double sm[];
  const int cv = blockIdx.x + 1, k1 = ed.k1, k2 = ed.k2;
  double *w1 = sm, *w2 = w1 + nb * k1, *t1 = w2 + nb * k2, *t2 = t1 + nb * k1;
  for (int q = threadIdx.x; q < nb * k1; q += blockDim.x) {
    const int a = q / k1, x = cv + q % k1;
    w1[q] = x <= ns ? P1[(size_t)a * ns + x - 1] : 0.0;
  }
  for (int q = threadIdx.x; q < nb * k2; q += blockDim.x) {
    const int b = q / k2, x = cv + q % k2;
    w2[q] = x <= ns ? P2[(size_t)b * ns + x - 1] : 0.0;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nb * k1; q += blockDim.x) {
    const int b = q / k1, h1 = q % k1 + 1;
    double s1 = 0.0, s2 = 0.0;
    for (int h2 = 1; h2 <= k2; h2++) {
      const size_t o = (size_t)pidx(ed, h1, h2) + (size_t)kk * (cv - 1);
      const double p = w2[b * k2 + h2 - 1];
      s1 = fma(M1[o], p, s1);
      if (M2) s2 = fma(M2[o], p, s2);
    }
    t1[q] = s1;
    t2[q] = s2;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nb * nb; q += blockDim.x) {
    const int a = q / nb, b = q % nb;
    double s1 = 0.0, s2 = 0.0;
    for (int h = 0; h < k1; h++) {
      const double p = w1[a * k1 + h];
      s1 = fma(p, t1[b * k1 + h], s1);
      s2 = fma(p, t2[b * k1 + h], s2);
    }
    S1[(size_t)q * nv + cv - 1] = s1;
    if (S2) S2[(size_t)q * nv + cv - 1] = s2;
  }
}

// (2) exclusive suffix (sum over later cells) or prefix sums per pair, one
// warp per pair: every lane scans a run of cells, the run totals are
// scanned across the warp by shuffles
// (blockIdx.y 1: a second array S1 with its own direction, same launch)
__global__ void k_pair_scan(int nv, int npair, double *S0, int suffix0, double *S1, int suffix1) {
  double *S = blockIdx.y ? S1 : S0;
  const int suffix = blockIdx.y ? suffix1 : suffix0;
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) / 32), lane = threadIdx.x % 32;
  if (warp >= npair) return;
  double *s = S + (size_t)warp * nv;
  const int run = (nv + 31) / 32;
  const int lo = min(nv, lane * run), hi = min(nv, lo + run);
  double tot = 0.0;
  for (int i = lo; i < hi; i++) tot += s[i];
  double incl = tot;
  for (int off = 1; off < 32; off <<= 1) {
    const double v = suffix ? __shfl_down_sync(0xffffffffu, incl, off)
                            : __shfl_up_sync(0xffffffffu, incl, off);
    if (suffix ? lane + off < 32 : lane >= off) incl += v;
  }
  const double nb1 = suffix ? __shfl_down_sync(0xffffffffu, incl, 1)
                            : __shfl_up_sync(0xffffffffu, incl, 1);
  double acc = suffix ? (lane == 31 ? 0.0 : nb1) : (lane == 0 ? 0.0 : nb1);
  if (suffix) {
    for (int i = hi - 1; i >= lo; i--) {
      const double v = s[i];
      s[i] = acc;
      acc += v;
    }
  } else {
    for (int i = lo; i < hi; i++) {
      const double v = s[i];
      s[i] = acc;
      acc += v;
    }
  }
}

// (3) diagonal cells, one block per cell cv:
//   Dq[ph][ab][q(po)] = sum_{g1,g2} R(po; g1,g2; cv) P1(a, cv+g1-1) P2(b, cv+g2-1)
// with po an output pair of the cell, q its position in the ns x ncol result
// and ph = (cv-1) mod 9: a cell touches outputs with first index in
// [cv, cv+8], so cells of one phase never share an output.  Two stages:
// H(po, g1, b) = sum_g2 R P2, then sum_g1 P1 H.
template <bool FF>
__global__ void __launch_bounds__(512) k_pair_diag(int ns, int ks, int kk, int nb, int icv,
                                                   char sym, PairSpec eo, PairSpec ed,
                                                   const double *__restrict__ rkd,
                                                   const double *__restrict__ P1,
                                                   const double *__restrict__ P2,
                                                   double *__restrict__ Dq, size_t per) {
  using S = typename std::conditional<FF, float2, double>::type;
  extern __shared__ double smraw[];
  S *sm = reinterpret_cast<S *>(smraw);
  auto sv = [](double v) -> S {
    if constexpr (FF) return ffa::split(v); else return v;
  };
  const int cv = blockIdx.x + 1, k1 = ed.k1, k2 = ed.k2, kd = k1 * k2;
  const int npo = eo.sym ? eo.k1 * (eo.k1 + 1) / 2 : eo.k1 * eo.k2;
  const size_t npair = (size_t)nb * nb;
  S *w1 = sm, *w2 = w1 + nb * k1, *Rt = w2 + nb * k2;
  S *H = Rt + (size_t)npo * kd;
  int *poq = (int *)(H + (size_t)npo * k1 * PBC);
  for (int q = threadIdx.x; q < nb * k1; q += blockDim.x) {
    const int a = q / k1, x = cv + q % k1;
    w1[q] = sv(x <= ns ? P1[(size_t)a * ns + x - 1] : 0.0);
  }
  for (int q = threadIdx.x; q < nb * k2; q += blockDim.x) {
    const int b = q / k2, x = cv + q % k2;
    w2[q] = sv(x <= ns ? P2[(size_t)b * ns + x - 1] : 0.0);
  }
  for (int po = threadIdx.x; po < npo; po += blockDim.x) {
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
    const int f = cv + h1 - 1, s2 = cv + h2 - 1;
    poq[po] = (f > ns || s2 > ns) ? -1
              : (sym == 's' ? (f - 1) + ns * (s2 - f) : (f - 1) + ns * (s2 - f + ks - 1));
  }
  const double *rc = rkd + (size_t)kk * kk * (cv - 1);  // rkd(e1 pair, e2 pair; cv)
  // the cell's table slice: consecutive threads read consecutive table
  // elements (po fastest for case 1, the density pair fastest otherwise)
  for (int q = threadIdx.x; q < npo * kd; q += blockDim.x) {
    int po, r;
    if (icv == 1) {
      po = q % npo;
      r = q / npo;
    } else {
      po = q / kd;
      r = q % kd;
    }
    const int g1 = r / k2 + 1, g2 = r % k2 + 1;
    const int pd = pidx(ed, g1, g2);
    Rt[(size_t)po * kd + r] =
        sv(icv == 1 ? rc[(size_t)po + (size_t)kk * pd] : rc[(size_t)pd + (size_t)kk * po]);
  }
  __syncthreads();
  const int ph = (cv - 1) % FAR;
  for (int b0 = 0; b0 < nb; b0 += PBC) {  // chunks of second orbitals
    const int bc = min(PBC, nb - b0);
    // stage 1: a thread forms H(po, g1, b) for the bc second orbitals of the
    // chunk at once (independent sums sharing each table load)
    for (int q = threadIdx.x; q < npo * k1; q += blockDim.x) {
      const int g1 = q % k1, po = q / k1;
      const S *rt = Rt + (size_t)po * kd + (size_t)g1 * k2;
      S *hq = H + ((size_t)po * k1 + g1) * PBC;
      if constexpr (FF) {
        float sh[PBC], sl[PBC];
#pragma unroll
        for (int bb = 0; bb < PBC; bb++) sh[bb] = sl[bb] = 0.0f;
        for (int g2 = 0; g2 < k2; g2++) {
          const S r = rt[g2];
#pragma unroll
          for (int bb = 0; bb < PBC; bb++)
            if (bb < bc) ffa::mac(r, w2[(size_t)(b0 + bb) * k2 + g2], sh[bb], sl[bb]);
        }
#pragma unroll
        for (int bb = 0; bb < PBC; bb++)
          if (bb < bc) hq[bb] = ffa::norm(sh[bb], sl[bb]);
      } else {
        double acc[PBC];
#pragma unroll
        for (int bb = 0; bb < PBC; bb++) acc[bb] = 0.0;
        for (int g2 = 0; g2 < k2; g2++) {
          const S r = rt[g2];
#pragma unroll
          for (int bb = 0; bb < PBC; bb++)
            if (bb < bc) acc[bb] = fma(r, w2[(size_t)(b0 + bb) * k2 + g2], acc[bb]);
        }
#pragma unroll
        for (int bb = 0; bb < PBC; bb++)
          if (bb < bc) hq[bb] = acc[bb];
      }
    }
    __syncthreads();
    // stage 2: Dq for the bc second orbitals at once
    for (int q = threadIdx.x; q < npo * nb; q += blockDim.x) {
      const int a = q % nb, po = q / nb;
      const int qp = poq[po];
      if (qp < 0) continue;
      const S *p = w1 + (size_t)a * k1;
      const S *h = H + (size_t)po * k1 * PBC;
      const size_t d0 = ((size_t)ph * npair + (size_t)a * nb + b0) * per + qp;
      if constexpr (FF) {  // kept as float-float pairs (no FP64 conversion)
        float sh[PBC], sl[PBC];
#pragma unroll
        for (int bb = 0; bb < PBC; bb++) sh[bb] = sl[bb] = 0.0f;
        for (int g1 = 0; g1 < k1; g1++) {
          const S pv = p[g1];
#pragma unroll
          for (int bb = 0; bb < PBC; bb++)
            if (bb < bc) ffa::mac(pv, h[(size_t)g1 * PBC + bb], sh[bb], sl[bb]);
        }
        float2 *D = reinterpret_cast<float2 *>(Dq);
#pragma unroll
        for (int bb = 0; bb < PBC; bb++)
          if (bb < bc) D[d0 + (size_t)bb * per] = ffa::norm(sh[bb], sl[bb]);
      } else {
        double s[PBC];
#pragma unroll
        for (int bb = 0; bb < PBC; bb++) s[bb] = 0.0;
        for (int g1 = 0; g1 < k1; g1++) {
          const S pv = p[g1];
#pragma unroll
          for (int bb = 0; bb < PBC; bb++)
            if (bb < bc) s[bb] = fma(pv, h[(size_t)g1 * PBC + bb], s[bb]);
        }
#pragma unroll
        for (int bb = 0; bb < PBC; bb++)
          if (bb < bc) Dq[d0 + (size_t)bb * per] = s[bb];
      }
    }
    __syncthreads();
  }
}

// (4) the pair potential: separable terms from the scanned cell sums plus the
// diagonal-cell parts, cells in order (the output loop of k_direct)
template <bool FF>
__global__ void k_pair_direct_final(int ns, int ks, int nv, int kk, int nb, int icv, char sym,
                                    PairSpec eo, const double *lo1, const double *hi1,
                                    const double *hi2, const double *SA, const double *SB,
                                    const double *Dq, void *Kout, size_t per) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= per) return;
  const int pair = blockIdx.y;
  const size_t npair = (size_t)nb * nb;
  const int f = (int)(t % ns) + 1, col = (int)(t / ns) + 1;
  const int s2 = sym == 's' ? f + col - 1 : f + col - ks;
  double acc = 0.0;
  float dh = 0.0f, dl = 0.0f;  // float-float diagonal-cell parts (FF)
  if (s2 >= 1 && s2 <= ns) {
    const int lo = max(max(1, f - eo.k1 + 1), s2 - eo.k2 + 1), hi = min(min(nv, f), s2);
    const double *sa = SA + (size_t)pair * nv;
    const double *sb = SB ? SB + (size_t)pair * nv : nullptr;
    for (int cv = lo; cv <= hi; cv++) {
      const size_t o = (size_t)pidx(eo, f - cv + 1, s2 - cv + 1) + (size_t)kk * (cv - 1);
      if (icv == 1) {
        acc = fma(lo1[o], sa[cv - 1], acc);
        if (sb) acc = fma(hi1[o], sb[cv - 1], acc);
      } else {
        acc = fma(hi2[o], sa[cv - 1], acc);
      }
      const size_t dq = ((size_t)((cv - 1) % FAR) * npair + pair) * per + t;
      if constexpr (FF)
        ffa::add(reinterpret_cast<const float2 *>(Dq)[dq], dh, dl);
      else
        acc += Dq[dq];
    }
  }
  if constexpr (FF)
    static_cast<float2 *>(Kout)[(size_t)pair * per + t] = ffa::split(acc + ffa::value(dh, dl));
  else
    static_cast<double *>(Kout)[(size_t)pair * per + t] = acc;
}

// ---------------------------------------------------------------------------
// near band of the exchange results: Y(x, x+d) = sum_e c_e Kb(pair_e; x, d)
__global__ void k_band_sum(int ns, const int *members, const SegInfo *info, const int *pairs,
                           const double *cd, const double *Kb, double *Y, size_t per) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ns * NDB) return;
  const int slot = blockIdx.y;
  const int x = t % ns + 1, y = x + t / ns - BAND;
  if (y < 1 || y > ns) return;
  const SegInfo si = info[members[slot]];
  const size_t kper = (size_t)ns * NDB;
  double acc = 0.0;
  for (int e = si.start; e < si.end; e++) acc = fma(cd[e], Kb[(size_t)pairs[e] * kper + t], acc);
  Y[(size_t)slot * per + (size_t)(x - 1) + (size_t)ns * (y - 1)] = acc;
}

// Exchange scatter (UPDATE_HS, updates.f90:110-179): one 32x32 tile of one
// quadrant of an owner's block; contributions in the reference's order
// (atype-major, owner then partner), transposed reads staged through shared
// memory so that every global access is coalesced.  Without a lower far
// field (S^k) the region x - y >= 9 of every result is zero.
__global__ void __launch_bounds__(256) k_scatter_x(int ns, QuadSpec sp, int nm,
                                                   const int *members, const int *own_slots,
                                                   const SegInfo *info, const double *Y,
                                                   int lower, double *hch) {
  __shared__ double tt[32][33];
  const int ms = 2 * ns, nt = (ns + 31) / 32;
  const int quad = blockIdx.x / (nt * nt), tile = blockIdx.x % (nt * nt);
  const int qr = quad % 2 + 1, qc = quad / 2 + 1;
  const int r0 = (tile % nt) * 32, c0 = (tile / nt) * 32;
  const int oslot = own_slots[blockIdx.y];
  const SegInfo si = info[members[oslot]];
  if (si.blk < 1) return;
  const int pslot = si.partner >= 0 ? oslot + 1 : -1;
  const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
  const size_t per = (size_t)ns * ns;
  double *hb = hch + (size_t)(si.blk - 1) * ms * ms + (size_t)(qr - 1) * ns + (size_t)ms * (qc - 1) * ns;
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  bool touched = false;
  for (int a = 0; a < sp.na; a++) {
    for (int pass = 0; pass < 2; pass++) {
      const int slot = pass == 0 ? oslot : pslot;
      if (slot < 0) break;
      const SegInfo sj = info[members[slot]];
      const double *d = Y + ((size_t)a * nm + slot) * per;
      const int ii = sp.ii[a], jj = sp.jj[a];
      const bool eq = sj.ich == sj.jch;
      const bool dir = (sj.ich > sj.jch || eq) && qr == ii && qc == jj;
      const bool tra = (sj.ich < sj.jch && qr == ii && qc == jj) || (eq && qr == jj && qc == ii);
      if (!dir && !tra) continue;
      if (!touched) {
        touched = true;
        for (int k = 0; k < 4; k++) {
          const int lr = r0 + tx, lc = c0 + ty + 8 * k;
          if (lr < ns && lc < ns) v[k] = hb[(size_t)lr + (size_t)ms * lc];
        }
      }
      if (dir) {
        for (int k = 0; k < 4; k++) {
          const int lr = r0 + tx, lc = c0 + ty + 8 * k;
          if (lr >= ns || lc >= ns) continue;
          const double y = (lower || lr - lc < FAR) ? d[(size_t)lr + (size_t)ns * lc] : 0.0;
          v[k] = v[k] + (eq ? y / 2.0 : y);
        }
      }
      if (tra) {
        __syncthreads();
        for (int k = 0; k < 4; k++) {
          const int x = c0 + tx, y = r0 + ty + 8 * k;  // y(x, y) = element (lc, lr)
          tt[ty + 8 * k][tx] =
              (x < ns && y < ns && (lower || x - y < FAR)) ? d[(size_t)x + (size_t)ns * y] : 0.0;
        }
        __syncthreads();
        for (int k = 0; k < 4; k++) {
          const int lr = r0 + tx, lc = c0 + ty + 8 * k;
          if (lr >= ns || lc >= ns) continue;
          const double y = tt[tx][ty + 8 * k];
          v[k] = v[k] + (eq ? y / 2.0 : y);
        }
      }
    }
  }
  if (!touched) return;
  for (int k = 0; k < 4; k++) {
    const int lr = r0 + tx, lc = c0 + ty + 8 * k;
    if (lr < ns && lc < ns) hb[(size_t)lr + (size_t)ms * lc] = v[k];
  }
}

// position of element (i, j) (1-based) of the band result y in its ns x ncol
// storage, or -1 where the storage holds no element (yval of assemble.cu)
__device__ __forceinline__ int band_pos(int ns, int ks, char sym, int i, int j) {
  if (sym == 's') {
    const int lo = min(i, j), dl = abs(i - j);
    return dl >= ks ? -1 : (lo - 1) + ns * dl;
  }
  const int jp = j - i + ks;
  return (jp < 1 || jp > 2 * ks - 1) ? -1 : (i - 1) + ns * (jp - 1);
}

// Direct scatter: every band element of the four quadrants of an owner's
// block; each contribution is formed from the pair potentials and the
// segment's coefficients where it is added (FF: as a float-float sum).
template <bool FF>
__global__ void k_scatter_dp(int ns, int ks, char sym, QuadSpec sp, KdSet kd,
                             const int *members, const int *own_slots, const SegInfo *info,
                             const int *pairs, const double *cd, const float2 *cdf,
                             double *hch) {
  const int ms = 2 * ns, nd = 2 * ks - 1;
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (size_t)4 * ns * nd) return;
  const int oslot = own_slots[blockIdx.y];
  const SegInfo si = info[members[oslot]];
  if (si.blk < 1) return;
  const int pslot = si.partner >= 0 ? oslot + 1 : -1;
  const int quad = (int)(q / ((size_t)ns * nd));
  const int rem = (int)(q % ((size_t)ns * nd));
  const int lr = rem % ns, lc = lr + rem / ns - (ks - 1);
  if (lc < 0 || lc >= ns) return;
  const int qr = (quad & 1) + 1, qc = (quad >> 1) + 1;
  const size_t per = (size_t)ns * (sym == 's' ? ks : nd);
  double *h = hch + (size_t)(si.blk - 1) * ms * ms + (size_t)((qr - 1) * ns + lr) +
              (size_t)ms * ((qc - 1) * ns + lc);
  bool touched = false;
  double val = 0.0;
  auto ysum = [&](int a, const SegInfo &sj, int i, int j) -> double {
    const int p = band_pos(ns, ks, sym, i, j);
    if (p < 0) return 0.0;
    // entries in batches of EB: the EB potential loads are issued together
    // (they depend only on the batch's pair indices), then summed in order
    constexpr int EB = 8;
    int e = sj.start;
    if (FF) {
      const float2 *K = kd.Kf[a];
      float sh = 0.0f, sl = 0.0f;
      for (; e + EB <= sj.end; e += EB) {
        float2 kv[EB];
#pragma unroll
        for (int u = 0; u < EB; u++) kv[u] = K[(size_t)pairs[e + u] * per + p];
#pragma unroll
        for (int u = 0; u < EB; u++) ffa::mac(cdf[e + u], kv[u], sh, sl);
      }
      for (; e < sj.end; e++) ffa::mac(cdf[e], K[(size_t)pairs[e] * per + p], sh, sl);
      return ffa::value(sh, sl);
    }
    const double *K = kd.K[a];
    double acc = 0.0;
    for (; e + EB <= sj.end; e += EB) {
      double kv[EB];
#pragma unroll
      for (int u = 0; u < EB; u++) kv[u] = K[(size_t)pairs[e + u] * per + p];
#pragma unroll
      for (int u = 0; u < EB; u++) acc = fma(cd[e + u], kv[u], acc);
    }
    for (; e < sj.end; e++) acc = fma(cd[e], K[(size_t)pairs[e] * per + p], acc);
    return acc;
  };
  for (int a = 0; a < sp.na; a++) {
    for (int pass = 0; pass < 2; pass++) {
      const int slot = pass == 0 ? oslot : pslot;
      if (slot < 0) break;
      const SegInfo sj = info[members[slot]];
      const int ii = sp.ii[a], jj = sp.jj[a];
      if (sj.ich != sj.jch) {
        if (qr == ii && qc == jj) {
          if (!touched) { val = *h; touched = true; }
          val = val + (sj.ich > sj.jch ? ysum(a, sj, lr + 1, lc + 1)
                                       : ysum(a, sj, lc + 1, lr + 1));
        }
      } else {
        if (qr == ii && qc == jj) {
          if (!touched) { val = *h; touched = true; }
          val = val + ysum(a, sj, lr + 1, lc + 1) / 2.0;
        }
        if (qr == jj && qc == ii) {
          if (!touched) { val = *h; touched = true; }
          val = val + ysum(a, sj, lc + 1, lr + 1) / 2.0;
        }
      }
    }
  }
  if (touched) *h = val;
}

}  // namespace

int ensure_fscratch(dbsrg_ctx *c, size_t bytes) {
  return grow_buffer(c, &c->fscratch, &c->fscratch_bytes, bytes);
}

int pair_index(dbsrg_ctx *c, int n, const int *k2, const int *k3, int *pairs, int *derr,
               cudaStream_t s) {
  if (n <= 0) return DBSRG_OK;
  if (c->nbound < 1 || c->nbound > NB_MAX)
    return set_err(c, DBSRG_EINVAL, "factored contraction: 1..128 bound orbitals (ipbs = 0)");
  DBSRG_RUN_S(c, s, "k_pair_index",
              k_pair_index<<<(n + 255) / 256, 256, 0, s>>>(n, k2, k3, c->bmap, c->nbound, pairs,
                                                           derr));
  return DBSRG_OK;
}

// far-field vectors of (family, type, k, exchange case), cached
static int get_farfield(dbsrg_ctx *c, int family, int type, int k, int cs, const FarField **out) {
  std::map<size_t, FarField> &v = family == 0 ? c->rfar : c->sfar;
  const size_t idx = ((size_t)k * (family == 0 ? 4 : 2) + type) * 2 + (cs == 4 ? 1 : 0);
  auto it = v.find(idx);
  if (it != v.end() && it->second.U) {
    *out = &it->second;
    return DBSRG_OK;
  }
  const DeviceGrid &g = c->g;
  const CellData *cd;
  int rc = get_celldata(c, family, type, k, &cd);
  if (rc) return rc;
  const int ns = g.ns, nb = c->nbound, kk = g.ks * g.ks;
  size_t m = (size_t)ns * nb;
  double *base = nullptr;
  if (!(base = (double *)cache_alloc(c, 4 * m * sizeof(double))))
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
  const FarSide s1{tb.e1, o1f, ko1, kc1, cc1, cd->lo1, family == 0 ? cd->hi1 : nullptr, f.U, f.Ul};
  const FarSide s2{tb.e2, o2f, ko2, kc2, cc2, cd->hi2, family == 0 ? cd->lo2 : nullptr, f.V, f.Vl};
  const dim3 gv((unsigned)((m + 63) / 64), 2);
  DBSRG_RUN(c, "k_far_vectors",
            k_far_vectors<<<gv, 64, 0, c->stream>>>(ns, g.nv, kk, nb, c->b2o, c->pq, s1, s2));
  v[idx] = f;
  *out = &v.at(idx);
  return DBSRG_OK;
}

// bound-orbital rows of both components, built once per orbital set
static int ensure_brows(dbsrg_ctx *c) {
  if (c->brows) return DBSRG_OK;
  const int ns = c->g.ns, nb = c->nbound;
  const size_t m = (size_t)ns * nb;
  if (!(c->brows = (double *)cache_alloc(c, 2 * m * sizeof(double))))
    return set_err(c, DBSRG_ENOMEM, "bound-orbital rows allocation failed");
  for (int comp = 1; comp <= 2; comp++)
    DBSRG_RUN(c, "k_bound_rows",
              k_bound_rows<<<(unsigned)((m + 255) / 256), 256, 0, c->stream>>>(
                  ns, nb, c->b2o, c->pq, comp, c->brows + (size_t)(comp - 1) * m));
  return DBSRG_OK;
}

int ensure_bound_rows(dbsrg_ctx *c, bool *built) {
  if (c->brows) return DBSRG_OK;
  *built = true;
  return ensure_brows(c);
}

static long long pairpot_key(int kind, int family, int type, int k, int icv, int jp1, int jp2,
                             bool ff) {
  return (long long)kind | (long long)family << 1 | (long long)type << 2 | (long long)icv << 5 |
         (long long)jp1 << 8 | (long long)jp2 << 10 | (long long)ff << 12 | (long long)k << 13;
}

static int set_smem(dbsrg_ctx *c, const void *fn, size_t smem) {
  if (smem > 220 * 1024) return set_err(c, DBSRG_EINVAL, "pair potentials: too many bound orbitals");
  return raise_smem_limit(c, fn, smem);
}

// direct pair potentials of (family, type, k, case icv) with density
// components jp1/jp2: Kd[pair][ns*ncol], cached
int get_pairpot_direct(dbsrg_ctx *c, int family, int type, int k, int icv, int jp1,
                              int jp2, const double **out) {
  return get_pairpot_direct_any(c, family, type, k, icv, jp1, jp2, false, (const void **)out);
}

int get_pairpot_direct_ff(dbsrg_ctx *c, int family, int type, int k, int icv, int jp1, int jp2,
                          const float2 **out) {
  return get_pairpot_direct_any(c, family, type, k, icv, jp1, jp2, true, (const void **)out);
}

// ff: the diagonal-cell contraction in float-float arithmetic and the result
// stored as float-float pairs (the split form's gather-sums read those)
int get_pairpot_direct_any(dbsrg_ctx *c, int family, int type, int k, int icv, int jp1,
                           int jp2, bool ff, const void **out) {
  const long long key = pairpot_key(0, family, type, k, icv, jp1, jp2, ff);
  auto it = c->ppot.find(key);
  if (it != c->ppot.end()) {
    *out = it->second;
    return DBSRG_OK;
  }
  const DeviceGrid &g = c->g;
  const int ns = g.ns, ks = g.ks, nv = g.nv, kk = ks * ks, nb = c->nbound;
  const size_t npair = (size_t)nb * nb;
  const char sym = family == 0 ? 's' : 'n';
  const size_t per = (size_t)ns * (sym == 's' ? ks : 2 * ks - 1);
  int rc;
  const CellData *cd;
  if ((rc = get_celldata(c, family, type, k, &cd))) return rc;
  if ((rc = ensure_brows(c))) return rc;
  TableBases tb = table_bases(g, family, type);
  const PairSpec eo = icv == 1 ? tb.e1 : tb.e2, ed = icv == 1 ? tb.e2 : tb.e1;
  const double *P1 = c->brows + (size_t)(jp1 - 1) * nb * ns;
  const double *P2 = c->brows + (size_t)(jp2 - 1) * nb * ns;
  const double *M1 = icv == 1 ? cd->hi2 : cd->lo1;
  const double *M2 = (icv == 1 && family == 0) ? cd->lo2 : nullptr;
  // scratch: SA, SB (npair x nv), Dq (9 x npair x per)
  const size_t sbytes = (2 * npair * nv + (size_t)FAR * npair * per) * sizeof(double);
  const int ps = c->stream == c->bstream[1] ? 1 : 0;  // scratch of this stream
  if (c->stream != c->bstream[0] && c->stream != c->bstream[1]) c->stream_built = true;
  if ((rc = ensure_pscratch(c, ps, sbytes))) return rc;
  double *SA = (double *)c->pscratch[ps], *SB = SA + npair * nv, *Dq = SB + npair * nv;
  double *K = nullptr;  // doubles, or as many float2 pairs (same bytes)
  if (!(K = (double *)cache_alloc(c, npair * per * sizeof(double)))) {
    cudaGetLastError();
    return set_err(c, DBSRG_ENOMEM, "pair potential allocation failed");
  }
  c->ppot[key] = K;
  cudaStream_t st = c->stream;
  const size_t sm1 = (size_t)nb * (3 * ed.k1 + ed.k2) * sizeof(double);
  if ((rc = set_smem(c, (const void *)k_pair_cellsum, sm1))) return rc;
  DBSRG_RUN(c, "k_pair_cellsum",
            k_pair_cellsum<<<nv, 256, sm1, st>>>(ns, nv, kk, nb, ed, M1, M2, P1, P2, SA,
                                                 M2 ? SB : nullptr));
  const unsigned gp = (unsigned)((npair * 32 + 255) / 256);
  DBSRG_RUN(c, "k_pair_scan", k_pair_scan<<<dim3(gp, M2 ? 2 : 1), 256, 0, st>>>(
                                  nv, (int)npair, SA, icv == 1, SB, 0));
  const int npo = eo.sym ? eo.k1 * (eo.k1 + 1) / 2 : eo.k1 * eo.k2;
  const size_t sm3 = ((size_t)nb * (ed.k1 + ed.k2) + (size_t)npo * ed.k1 * ed.k2 +
                      (size_t)npo * ed.k1 * PBC) * sizeof(double) + (size_t)npo * sizeof(int);
  const double *lo1 = icv == 1 ? cd->lo1 : nullptr;
  const double *hi1 = (icv == 1 && family == 0) ? cd->hi1 : nullptr;
  dim3 gf((unsigned)((per + 127) / 128), (unsigned)npair);
  // executed work of the diagonal cells: per cell, stage 1 npo k1 k2 nb and
  // stage 2 npo nb k1 nb multiply-adds; the cell's table slice read and its
  // npo nb^2 outputs written.  The final potentials: per output element and
  // pair a few separable terms (about 4 multiply-adds) and the nine
  // diagonal-cell phases read, the potential written.
  const double dflops = 2.0 * nv * npo * ed.k1 * ((double)ed.k2 * nb + (double)nb * nb);
  const double dbytes = 8.0 * nv * ((double)npo * ed.k1 * ed.k2 + (double)npo * nb * nb);
  const double fflops = 8.0 * (double)per * npair;
  const double fbytes = 8.0 * (double)per * npair * (FAR + 1);
  if (ff) {
    if ((rc = set_smem(c, (const void *)k_pair_diag<true>, sm3))) return rc;
    DBSRG_RUN_W(c, "k_pair_diag", dbytes, dflops,
                k_pair_diag<true><<<nv, 512, sm3, st>>>(
                    ns, ks, kk, nb, icv, sym, eo, ed, cd->rkd, P1, P2, Dq, per));
    DBSRG_RUN_W(c, "k_pair_direct_final", fbytes, fflops,
                k_pair_direct_final<true><<<gf, 128, 0, st>>>(ns, ks, nv, kk, nb, icv, sym, eo,
                                                              lo1, hi1, cd->hi2, SA,
                                                              M2 ? SB : nullptr, Dq, K, per));
  } else {
    if ((rc = set_smem(c, (const void *)k_pair_diag<false>, sm3))) return rc;
    DBSRG_RUN_W(c, "k_pair_diag", dbytes, dflops,
                k_pair_diag<false><<<nv, 512, sm3, st>>>(
                    ns, ks, kk, nb, icv, sym, eo, ed, cd->rkd, P1, P2, Dq, per));
    DBSRG_RUN_W(c, "k_pair_direct_final", fbytes, fflops,
                k_pair_direct_final<false><<<gf, 128, 0, st>>>(ns, ks, nv, kk, nb, icv, sym, eo,
                                                               lo1, hi1, cd->hi2, SA,
                                                               M2 ? SB : nullptr, Dq, K, per));
  }
  *out = K;
  return DBSRG_OK;
}

// exchange band pair potentials of (family, type, k, case) with density
// components jp1/jp2: Kb[pair][ns*17], cached
// ff: both stages in float-float arithmetic, the result stored as
// float-float pairs (float2, same bytes) for the split form's Z digits
static int get_pairpot_band(dbsrg_ctx *c, int family, int type, int k, int cs, int jp1, int jp2,
                            const double *tab, bool ff, const void **out) {
  const long long key = pairpot_key(1, family, type, k, cs, jp1, jp2, ff);
  auto it = c->ppot.find(key);
  if (it != c->ppot.end()) {
    *out = it->second;
    return DBSRG_OK;
  }
  const DeviceGrid &g = c->g;
  const int ns = g.ns, ks = g.ks, nb = c->nbound;
  const size_t npair = (size_t)nb * nb, per = (size_t)ns * NDB;
  int rc;
  if ((rc = ensure_brows(c))) return rc;
  double *K = nullptr;
  if (!(K = (double *)cache_alloc(c, npair * per * sizeof(double)))) {
    cudaGetLastError();
    return set_err(c, DBSRG_ENOMEM, "pair potential allocation failed");
  }
  c->ppot[key] = K;
  // positions past the ends of the band are never written by k_pair_band
  DBSRG_TRY(c, cudaMemsetAsync(K, 0, npair * per * sizeof(double), c->stream));
  const double *P1 = c->brows + (size_t)(jp1 - 1) * nb * ns;
  const double *P2 = c->brows + (size_t)(jp2 - 1) * nb * ns;
  const int W = 2 * ks - 1, WLP = (PXC + W - 1) | 1;
  const size_t smem =
      ((size_t)PXC * W * W + 2 * (size_t)nb * WLP + (size_t)PXC * (W * nb + 1)) * sizeof(double);
  const int mode = family == 0 ? 0 : (cs == 3 ? 1 : 2);
  dim3 gb((unsigned)((ns + PXC - 1) / PXC), (unsigned)NDB);
  // executed work: per output row and band diagonal W^2 nb (stage 1) and
  // W nb^2 (stage 2) multiply-adds; the band table read, the potentials
  // written
  const double kb = family == 0 ? ks : W;
  const double bflops = 2.0 * ns * NDB * ((double)W * W * nb + (double)W * nb * nb);
  const double bbytes = 8.0 * ns * NDB * (kb * kb + (double)npair);
  if (ff) {
    if ((rc = set_smem(c, (const void *)k_pair_band<true>, smem))) return rc;
    DBSRG_RUN_W(c, "k_pair_band", bbytes, bflops,
                k_pair_band<true><<<gb, 256, smem, c->stream>>>(ns, ks, nb, mode, tab, P1, P2,
                                                                K));
  } else {
    if ((rc = set_smem(c, (const void *)k_pair_band<false>, smem))) return rc;
    DBSRG_RUN_W(c, "k_pair_band", bbytes, bflops,
                k_pair_band<false><<<gb, 256, smem, c->stream>>>(ns, ks, nb, mode, tab, P1, P2,
                                                                 K));
  }
  *out = K;
  return DBSRG_OK;
}

void free_orbital_products(dbsrg_ctx *c) {
  graph_drop(c);
  if (!c->rfar.empty() || !c->sfar.empty() || !c->ppot.empty() || c->brows || !c->ffc.empty())
    cudaStreamSynchronize(c->stream);
  for (auto *v : {&c->rfar, &c->sfar})
    for (auto &kv : *v) {
      cache_free(c, kv.second.U);
      cache_free(c, kv.second.Ud);
    }
  c->rfar.clear();
  c->sfar.clear();
  for (auto &kv : c->ppot)
    cache_free(c, kv.second);
  c->ppot.clear();
  cache_free(c, c->brows);
  c->brows = nullptr;
  for (auto &kv : c->ffc) cache_free(c, kv.second);
  c->ffc.clear();
}

namespace {
__global__ void k_to_ff(size_t n, const double *src, float2 *dst) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = ffa::split(src[i]);
}
}  // namespace

int ff_of(dbsrg_ctx *c, const double *src, size_t n, const float2 **out) {
  auto it = c->ffc.find(src);
  if (it != c->ffc.end()) {
    *out = it->second;
    return DBSRG_OK;
  }
  float2 *d = (float2 *)cache_alloc(c, n * sizeof(float2));
  if (!d) return set_err(c, DBSRG_ENOMEM, "float-float copy allocation failed");
  c->ffc[src] = d;
  DBSRG_RUN(c, "k_to_ff",
            k_to_ff<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, src, d));
  *out = d;
  return DBSRG_OK;
}

int factored_contract(dbsrg_ctx *c, const FactorJob &j) {
  const DeviceGrid &g = c->g;
  const int ns = g.ns, ks = g.ks, nb = c->nbound;
  cudaStream_t st = c->stream;
  int rc;
  if (nb < 1 || nb > NB_MAX)
    return set_err(c, DBSRG_EINVAL, "factored contraction: 1..128 bound orbitals (ipbs = 0)");
  if (ks > FAR) return set_err(c, DBSRG_EINVAL, "factored contraction: spline order above 9");
  if (j.nown < 1) return DBSRG_OK;
  QuadSpec qs{};
  qs.na = j.na;
  for (int a = 0; a < j.na; a++) {
    qs.ii[a] = j.ii[a];
    qs.jj[a] = j.jj[a];
  }
  if (j.icv >= 3 && j.split) {
    SplitExchange x{};
    x.na = j.na;
    x.nm = j.nm;
    x.lower = j.family == 0 ? 1 : 0;
    for (int a = 0; a < j.na; a++) {
      const int cs = j.icv;
      if ((rc = get_farfield(c, j.family, j.types[a], j.kpol, cs, &x.far[a]))) return rc;
      TableBases tb = table_bases(g, j.family, j.types[a]);
      int c1 = cs == 3 ? tb.a2 : tb.a1, c2 = cs == 3 ? tb.b1 : tb.b2;
      if (c1 != j.jp1[a] || c2 != j.jp2[a])
        return set_err(c, DBSRG_EINVAL, "factored exchange: component mismatch");
      if ((rc = get_pairpot_band(c, j.family, j.types[a], j.kpol, cs, j.jp1[a], j.jp2[a],
                                 j.tabs[a], true, (const void **)&x.Kbf[a])))
        return rc;
    }
    x.members = j.members;
    x.xq = j.xq;
    x.hxq = j.hxq;
    x.nxq = j.nxq;
    x.info = j.info;
    x.pairs = j.pairs;
    x.cd = j.cd;
    x.cdf = j.cdf;
    x.prep = j.prep;
    x.nent = j.nent;
    return split_exchange(c, x);
  }
  if (j.icv >= 3 && j.prep) {
    for (int a = 0; a < j.na; a++) {
      const FarField *f;
      const void *Kb;
      if ((rc = get_farfield(c, j.family, j.types[a], j.kpol, j.icv, &f))) return rc;
      if ((rc = get_pairpot_band(c, j.family, j.types[a], j.kpol, j.icv, j.jp1[a], j.jp2[a],
                                 j.tabs[a], false, &Kb)))
        return rc;
    }
    return DBSRG_OK;
  }
  if (j.icv >= 3) {
    const size_t per = (size_t)ns * ns;
    size_t zs = (size_t)j.nm * nb * ns;
    if ((rc = ensure_fscratch(c, 2 * zs * sizeof(double)))) return rc;
    double *Z = (double *)c->fscratch, *Zl = Z + zs;
    for (int a = 0; a < j.na; a++) {
      const int cs = j.icv;
      const FarField *f;
      if ((rc = get_farfield(c, j.family, j.types[a], j.kpol, cs, &f))) return rc;
      TableBases tb = table_bases(g, j.family, j.types[a]);
      int c1 = cs == 3 ? tb.a2 : tb.a1, c2 = cs == 3 ? tb.b1 : tb.b2;
      if (c1 != j.jp1[a] || c2 != j.jp2[a])
        return set_err(c, DBSRG_EINVAL, "factored exchange: component mismatch");
      const double *Kb;
      if ((rc = get_pairpot_band(c, j.family, j.types[a], j.kpol, cs, j.jp1[a], j.jp2[a],
                                 j.tabs[a], false, (const void **)&Kb)))
        return rc;
      double *Ya = j.Y + (size_t)a * j.nm * per;
      dim3 gz((unsigned)((ns * nb + 127) / 128), (unsigned)j.nm);
      DBSRG_RUN(c, "k_far_z",
                k_far_z<<<gz, 128, 0, st>>>(ns, nb, j.members, j.info, j.pairs, j.cd, f->V,
                                            f->Vl, Z, f->Vl ? Zl : nullptr));
      dim3 gf((unsigned)((ns + 31) / 32), (unsigned)((ns + 31) / 32), (unsigned)j.nm);
      DBSRG_RUN(c, "k_far_field",
                k_far_field<<<gf, 256, 0, st>>>(ns, nb, f->U, f->Ul, Z, f->Vl ? Zl : nullptr, Ya,
                                                per));
      dim3 gb((unsigned)((ns * NDB + 255) / 256), (unsigned)j.nm);
      DBSRG_RUN(c, "k_band_sum",
                k_band_sum<<<gb, 256, 0, st>>>(ns, j.members, j.info, j.pairs, j.cd, Kb, Ya, per));
    }
    const int nt = (ns + 31) / 32;
    dim3 gs((unsigned)(4 * nt * nt), (unsigned)j.nown);
    DBSRG_RUN(c, "k_scatter_x",
              k_scatter_x<<<gs, 256, 0, st>>>(ns, qs, j.nm, j.members, j.own, j.info, j.Y,
                                              j.family == 0 ? 1 : 0, hch_base(c)));
    return DBSRG_OK;
  }
  // direct
  KdSet kd{};
  for (int a = 0; a < j.na; a++) {
    if (j.split && j.cdf)
      rc = get_pairpot_direct_ff(c, j.family, j.types[a], j.kpol, j.icv, j.jp1[a], j.jp2[a],
                                 &kd.Kf[a]);
    else
      rc = get_pairpot_direct(c, j.family, j.types[a], j.kpol, j.icv, j.jp1[a], j.jp2[a],
                              &kd.K[a]);
    if (rc) return rc;
  }
  if (j.prep) return DBSRG_OK;
  const size_t space = (size_t)4 * ns * (2 * ks - 1);
  dim3 gs((unsigned)((space + 127) / 128), (unsigned)j.nown);
  // executed work: per PQ type every band element of its quadrant (about
  // ns (2ks-1)) sums one pair-potential value per entry of the owner and
  // partner segments (one multiply-add, float-float in the split form), and
  // is read and written once in hch; the potentials are read per entry
  const double nd = 2.0 * ks - 1.0, band = ns * nd;
  const double wflops = 2.0 * j.na * band * (double)j.nent;
  const double wbytes = 16.0 * j.na * band * j.nown + 8.0 * j.na * band * (double)j.nent;
  if (j.split && j.cdf)
    DBSRG_RUN_W(c, "k_scatter_dp", wbytes, wflops,
                k_scatter_dp<true><<<gs, 128, 0, st>>>(ns, ks, j.sym, qs, kd, j.members, j.own,
                                                       j.info, j.pairs, j.cd, j.cdf, hch_base(c)));
  else
    DBSRG_RUN_W(c, "k_scatter_dp", wbytes, wflops,
                k_scatter_dp<false><<<gs, 128, 0, st>>>(ns, ks, j.sym, qs, kd, j.members, j.own,
                                                        j.info, j.pairs, j.cd, j.cdf,
                                                        hch_base(c)));
  return DBSRG_OK;
}
