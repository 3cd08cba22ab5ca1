// tables.cu -- B-spline grid, cell moments, diagonal-cell integrals and the
// assembled R^k / S^k tables, all computed on the device in FP64.
//
// Operation order follows the reference routines (cited per kernel) and
// uses explicit round-to-nearest intrinsics where the reference forms a
// product and then a sum, so the tables reproduce the reference's loop
// arithmetic instead of a contracted variant.
#include "internal.cuh"

#include <cmath>

#define IDX2(i, j, n1) ((size_t)(i) + (size_t)(n1) * (size_t)(j))
#define IDX3(i, j, k, n1, n2) ((size_t)(i) + (size_t)(n1) * ((size_t)(j) + (size_t)(n2) * (size_t)(k)))

// ----------------------------------------------------------------------------
// gauleg on [0,1]: dbsr_lib_zcom.f90:1990-2039 (Newton on the Legendre
// recurrence).  One thread; n is the spline order.
__global__ void k_gauleg(int n, double *x, double *w) {
  const double EPS = 1.0e-14;
  int m = (n + 1) / 2;
  double xm = 0.5, xl = 0.5;
  for (int i = 1; i <= m; i++) {
    double z = cos(__ddiv_rn(__dmul_rn(3.141592654, (i - 0.25)), (n + 0.5)));
    double z1, pp, p1, p2, p3;
    do {
      p1 = 1.0;
      p2 = 0.0;
      for (int j = 1; j <= n; j++) {
        p3 = p2;
        p2 = p1;
        p1 = __ddiv_rn(__dsub_rn(__dmul_rn(__dmul_rn(2.0 * j - 1.0, z), p2),
                                 __dmul_rn(j - 1.0, p3)),
                       (double)j);
      }
      pp = __ddiv_rn(__dmul_rn((double)n, __dsub_rn(__dmul_rn(z, p1), p2)),
                     __dsub_rn(__dmul_rn(z, z), 1.0));
      z1 = z;
      z = __dsub_rn(z1, __ddiv_rn(p1, pp));
    } while (fabs(z - z1) > EPS);
    x[i - 1] = __dsub_rn(xm, __dmul_rn(xl, z));
    x[n - i] = __dadd_rn(xm, __dmul_rn(xl, z));
    w[i - 1] = __ddiv_rn(2.0 * xl, __dmul_rn(__dmul_rn(__dsub_rn(1.0, __dmul_rn(z, z)), pp), pp));
    w[n - i] = w[i - 1];
  }
}

// Gauss points per interval: alloc_DBS_gauss, dbsr_lib_dbs.f90:929-936.
__global__ void k_gauss_points(int nv, int ks, const double *t, const double *gx,
                               const double *gw, double *gr, double *grm, double *grw) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nv * ks) return;
  int iv = q % nv, m = q / nv;  // 0-based
  double tl = t[ks + iv - 1], tr = t[ks + iv];
  double h = __dsub_rn(tr, tl);
  double r = __dadd_rn(__dmul_rn(h, gx[m]), tl);
  gr[q] = r;
  grm[q] = __ddiv_rn(1.0, r);
  grw[q] = __dmul_rn(h, gw[m]);
}

// Knots of a component basis: Def_pbsp / Def_qbsp, dbsr_lib_dbs.f90:997-999.
__global__ void k_sub_knots(int ns, int ks, int kx, int nsx, const double *t, double *tx) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1;  // 1-based
  if (i > nsx + kx) return;
  double v;
  if (i <= kx)
    v = t[0];
  else if (i <= nsx)
    v = t[ks + (i - kx) - 1];
  else
    v = t[ns + (i - nsx) - 1];
  tx[i - 1] = v;
}

// B-spline values at the Gauss points, bsp(nv+1,ks,kx): Def_pbsp /
// Def_qbsp (dbsr_lib_dbs.f90:1003-1020); row nv+1 holds the values at the
// last knot in its first column.
__global__ void k_bsp_values(int nv, int ks, int kx, int nsx, const double *tx,
                             const double *gr, double *bsp) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int nw = nv + 1;
  if (q >= nw * ks) return;
  int iv = q % nw, m = q / nw;
  double v[DBSRG_MAXK];
  if (iv < nv) {
    bspline_values(tx, kx, kx + iv, gr[IDX2(iv, m, nv)], v);
  } else if (m == 0) {
    bspline_values(tx, kx, nsx, tx[nsx], v);
  } else {
    for (int j = 0; j < kx; j++) v[j] = 0.0;
  }
  for (int j = 0; j < kx; j++) bsp[IDX3(iv, m, j, nw, ks)] = v[j];
}

// Banded Gram matrix ym(i,j) = <B1_i|y|B2_j>: ZINTYM, dbsr_lib_dbs.f90:4472-4497.
// ym has leading dimension ld and is written at offset (off,off).
__global__ void k_gram(int ns, int nv, int ks, int kx, const double *b, const double *ygr,
                       double *ym, int ld, int off) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ns * ns) return;
  int i = q % ns + 1, j = q / ns + 1;  // 1-based
  const int nw = nv + 1;
  double acc = 0.0;
  int lo = max(max(1, i - kx + 1), j - kx + 1), hi = min(min(nv, i), j);
  for (int iv = lo; iv <= hi; iv++) {
    int ith = i - iv + 1, jth = j - iv + 1;
    double s = 0.0;
    for (int m = 0; m < ks; m++) {
      double p = __dmul_rn(__dmul_rn(ygr[IDX2(iv - 1, m, nv)], b[IDX3(iv - 1, m, ith - 1, nw, ks)]),
                           b[IDX3(iv - 1, m, jth - 1, nw, ks)]);
      s = __dadd_rn(s, p);
    }
    acc = __dadd_rn(acc, s);
  }
  ym[IDX2(off + i - 1, off + j - 1, ld)] = acc;
}

static int build_triang_points(dbsrg_ctx *c);

int build_grid(dbsrg_ctx *c, const double *t_in) {
  DeviceGrid &g = c->g;
  const int ns = g.ns, ks = g.ks, nv = g.nv, nw = nv + 1, ms = g.ms;
  auto alloc = [&](double **p, size_t n) -> cudaError_t {
    return cudaMalloc((void **)p, sizeof(double) * (n > 0 ? n : 1));
  };
  DBSRG_TRY(c, alloc(&g.t, ns + ks));
  DBSRG_TRY(c, alloc(&g.tp, g.nsp + g.ksp));
  DBSRG_TRY(c, alloc(&g.tq, g.nsq + g.ksq));
  DBSRG_TRY(c, alloc(&g.gx, ks));
  DBSRG_TRY(c, alloc(&g.gw, ks));
  DBSRG_TRY(c, alloc(&g.gr, (size_t)nv * ks));
  DBSRG_TRY(c, alloc(&g.grw, (size_t)nv * ks));
  DBSRG_TRY(c, alloc(&g.grm, (size_t)nv * ks));
  DBSRG_TRY(c, alloc(&g.pbsp, (size_t)nw * ks * g.ksp));
  DBSRG_TRY(c, alloc(&g.qbsp, (size_t)nw * ks * g.ksq));
  DBSRG_TRY(c, alloc(&g.fpbs, (size_t)ns * ns));
  DBSRG_TRY(c, alloc(&g.fqbs, (size_t)ns * ns));
  DBSRG_TRY(c, alloc(&g.fppqq, (size_t)ms * ms));
  int rc = copy_in(c, g.t, t_in, sizeof(double) * (ns + ks));
  if (rc) return rc;
  cudaStream_t s = c->stream;
  DBSRG_RUN(c, "k_gauleg", k_gauleg<<<1, 1, 0, s>>>(ks, g.gx, g.gw));
  int nt = nv * ks;
  DBSRG_RUN(c, "k_gauss_points", k_gauss_points<<<(nt + 127) / 128, 128, 0, s>>>(nv, ks, g.t, g.gx, g.gw, g.gr, g.grm, g.grw));
  DBSRG_RUN(c, "k_sub_knots", k_sub_knots<<<(g.nsp + g.ksp + 127) / 128, 128, 0, s>>>(ns, ks, g.ksp, g.nsp, g.t, g.tp));
  DBSRG_RUN(c, "k_sub_knots", k_sub_knots<<<(g.nsq + g.ksq + 127) / 128, 128, 0, s>>>(ns, ks, g.ksq, g.nsq, g.t, g.tq));
  int nb = nw * ks;
  DBSRG_RUN(c, "k_bsp_values", k_bsp_values<<<(nb + 127) / 128, 128, 0, s>>>(nv, ks, g.ksp, g.nsp, g.tp, g.gr, g.pbsp));
  DBSRG_RUN(c, "k_bsp_values", k_bsp_values<<<(nb + 127) / 128, 128, 0, s>>>(nv, ks, g.ksq, g.nsq, g.tq, g.gr, g.qbsp));
  int nn = ns * ns;
  DBSRG_RUN(c, "k_gram", k_gram<<<(nn + 255) / 256, 256, 0, s>>>(ns, nv, ks, g.ksp, g.pbsp, g.grw, g.fpbs, ns, 0));
  DBSRG_RUN(c, "k_gram", k_gram<<<(nn + 255) / 256, 256, 0, s>>>(ns, nv, ks, g.ksq, g.qbsp, g.grw, g.fqbs, ns, 0));
  DBSRG_TRY(c, cudaMemsetAsync(g.fppqq, 0, sizeof(double) * (size_t)ms * ms, s));
  DBSRG_RUN(c, "k_gram", k_gram<<<(nn + 255) / 256, 256, 0, s>>>(ns, nv, ks, g.ksp, g.pbsp, g.grw, g.fppqq, ms, 0));
  DBSRG_RUN(c, "k_gram", k_gram<<<(nn + 255) / 256, 256, 0, s>>>(ns, nv, ks, g.ksq, g.qbsp, g.grw, g.fppqq, ms, ns));
  if ((rc = build_triang_points(c))) return rc;
  DBSRG_TRY(c, cudaStreamSynchronize(s));
  return DBSRG_OK;
}

// ----------------------------------------------------------------------------
// Cell moments <B_i|r^k|B_j> per interval: moment_pp/qq/pq/qp,
// dbsr_lib_dbs.f90:1401-1564.  rkm(ks*ks,nv); pp/qq packed i<=j.
// up to four moment arrays per launch (blockIdx.y): the moments of one cell
// data set
struct MomentSet {
  const double *b1s[4], *b2s[4];
  int k1[4], k2[4], sym[4], k[4];
  double *rkm[4];
};

__global__ void k_moments(int nv, int ks, const MomentSet ms, const double *gr,
                          const double *grm, const double *grw) {
  const int y = blockIdx.y;
  const double *b1s = ms.b1s[y], *b2s = ms.b2s[y];
  const int k1 = ms.k1[y], k2 = ms.k2[y], sym = ms.sym[y], k = ms.k[y];
  double *rkm = ms.rkm[y];
  int kk = ks * ks;
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= kk * nv) return;
  int ii = q % kk, iv = q / kk;
  int npair = sym ? k1 * (k1 + 1) / 2 : k1 * k2;
  if (ii >= npair) {
    rkm[q] = 0.0;
    return;
  }
  int i, j;
  if (sym) {  // invert the packed upper-triangular index
    int r = ii, row = 0;
    while (r >= k1 - row) {
      r -= k1 - row;
      row++;
    }
    i = row;
    j = row + r;
  } else {
    i = ii / k2;
    j = ii % k2;
  }
  const int nw = nv + 1;
  double s = 0.0;
  for (int m = 0; m < ks; m++) {
    double w = grw[IDX2(iv, m, nv)];
    if (k > 0) w = __dmul_rn(grw[IDX2(iv, m, nv)], ipow_d(gr[IDX2(iv, m, nv)], k));
    if (k < 0) w = __dmul_rn(grw[IDX2(iv, m, nv)], ipow_d(grm[IDX2(iv, m, nv)], -k));
    const double b2 = __dmul_rn(b2s[IDX3(iv, m, j, nw, ks)], w);
    s = fma(b1s[IDX3(iv, m, i, nw, ks)], b2, s);
  }
  rkm[q] = s;
}

static void basis_of(const DeviceGrid &g, int which, const double **b1, const double **b2,
                     int *k1, int *k2, int *sym) {
  switch (which) {
    case 0: *b1 = g.pbsp; *b2 = g.pbsp; *k1 = g.ksp; *k2 = g.ksp; *sym = 1; break;
    case 1: *b1 = g.qbsp; *b2 = g.qbsp; *k1 = g.ksq; *k2 = g.ksq; *sym = 1; break;
    case 2: *b1 = g.pbsp; *b2 = g.qbsp; *k1 = g.ksp; *k2 = g.ksq; *sym = 0; break;
    default: *b1 = g.qbsp; *b2 = g.pbsp; *k1 = g.ksq; *k2 = g.ksp; *sym = 0; break;
  }
}

// n (1..4) moment arrays in one launch: basis pair which[i], power k[i]
static int compute_moment_set(dbsrg_ctx *c, int n, const int *which, const int *k,
                              double *const *rkm) {
  const DeviceGrid &g = c->g;
  MomentSet ms{};
  for (int i = 0; i < n; i++) {
    basis_of(g, which[i], &ms.b1s[i], &ms.b2s[i], &ms.k1[i], &ms.k2[i], &ms.sym[i]);
    ms.k[i] = k[i];
    ms.rkm[i] = rkm[i];
  }
  const int m = g.ks * g.ks * g.nv;
  DBSRG_RUN(c, "k_moments", k_moments<<<dim3((m + 127) / 128, n), 128, 0, c->stream>>>(
                                g.nv, g.ks, ms, g.gr, g.grm, g.grw));
  return DBSRG_OK;
}

int compute_moments(dbsrg_ctx *c, int which, int k, double *rkm) {
  return compute_moment_set(c, 1, &which, &k, &rkm);
}

// ----------------------------------------------------------------------------
// Diagonal-cell integrals triang_*: dbsr_lib_dbs.f90:2979-3063 (pppp),
// 3151-3245 (pqpq), 3333-3427 (qpqp), 3512-3597 (qqqq), 3682-3767 (ppqq),
// 3852-3936 (pqqp).  One thread block per interval iv.  For each outer
// Gauss point r2 = gr(iv,m) the inner integral of B_j B_jp r^k over
// [t_iv, r2] uses ks Gauss points; B-splines at the inner points come from
// the same de Boor recursion as zbsplvd.
//   type 0 pppp, 1 qqqq: rkd = a + a^T, a(outer pair, inner pair)
//   type 2 pqpq: rkd(P pair, Q pair) = sum bp*INTQ + sum bq*INTP
//   type 3 qpqp: rkd(Q pair, P pair) = the same two sums
//   type 4 ppqq: rkd(inner (P,Q), outer (P,Q))
//   type 5 pqqp: rkd(inner (P,Q), outer (Q,P))
// Inner points of the diagonal cells of every interval iv: for outer point
// r2 = gr(iv,m) the inner Gauss points x = t_iv + (r2 - t_iv) gx(i) on
// [t_iv, r2], their weights (r2 - t_iv) gw(i) and the P and Q B-splines
// there (zbsplvd recursion); one thread per (iv, m, i).
__global__ void k_triang_points(int nv, int ks, int ksp, int ksq, const double *t,
                                const double *tp, const double *tq, const double *gx,
                                const double *gw, const double *gr, double *tri) {
  const int KS2 = ks * ks;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nv * KS2) return;
  const int iv = q / KS2, p = q % KS2, m = p / ks, i = p % ks;
  double *tb = tri + (size_t)iv * KS2 * (2 + ksp + ksq);
  const double xbase = t[iv + ks - 1];
  const double r2 = gr[IDX2(iv, m, nv)];
  const double d = __dsub_rn(r2, xbase);
  const double x = __dadd_rn(__dmul_rn(d, gx[i]), xbase);
  tb[p] = x;
  tb[KS2 + p] = __dmul_rn(d, gw[i]);
  double v[DBSRG_MAXK];
  bspline_values(tp, ksp, iv + ksp, x, v);
  for (int j = 0; j < ksp; j++) tb[2 * KS2 + (size_t)p * ksp + j] = v[j];
  bspline_values(tq, ksq, iv + ksq, x, v);
  for (int j = 0; j < ksq; j++) tb[2 * KS2 + (size_t)KS2 * ksp + (size_t)p * ksq + j] = v[j];
}

__global__ void k_triang(int nv, int ks, int ksp, int ksq, int type, int k, const double *tri,
                         const double *grm, const double *grw, const double *pbsp,
                         const double *qbsp, double *rkd) {
  extern __shared__ double sm[];
  const int iv = blockIdx.x;  // 0-based interval
  // this block's share of the interval's kk*kk output cells (blockIdx.y of
  // gridDim.y, launched with one block per interval: the inner integrals
  // would be repeated by every block of an interval)
  const int nq = ks * ks * ks * ks, part = (nq + gridDim.y - 1) / gridDim.y;
  const int q0 = blockIdx.y * part, q1 = min(nq, q0 + part);
  const int nw = nv + 1, kk = ks * ks;
  const int KS2 = ks * ks;
  const double *tb = tri + (size_t)iv * KS2 * (2 + ksp + ksq);  // x | w | BP | BQ
  double *wk = sm;                 // (m,i) inner weight * r^k       [ks*ks]
  double *BP = wk + KS2;           // (m,i,j) P values at inner pts  [ks*ks*ksp]
  double *BQ = BP + KS2 * ksp;     // (m,i,j) Q values               [ks*ks*ksq]
  double *INTP = BQ + KS2 * ksq;   // (j,jp,m) over P x P            [ksp*ksp*ks]
  double *INTQ = INTP + ksp * ksp * ks;  // Q x Q                    [ksq*ksq*ks]
  double *INTPQ = INTQ + ksq * ksq * ks; // P x Q                    [ksp*ksq*ks]
  double *gxo = INTPQ + ksp * ksq * ks;  // outer weights            [ks]
  double *A = gxo + ks;                  // a(ii,jj) for pppp/qqqq   [kk*kk]
  // outer products b1(m,i) b2(m,ip) gxo(m) per pair and outer point, formed
  // once per interval: OB1 for the first pair family, OB2 for the second
  double *OB1 = A + kk * kk;             //                          [kk*ks]
  double *OB2 = OB1 + kk * ks;           //                          [kk*ks]

  // phase 1: inner points, weights and B-spline values (k_triang_points)
  for (int q = threadIdx.x; q < KS2; q += blockDim.x)
    wk[q] = __dmul_rn(tb[KS2 + q], ipow_d(tb[q], k));
  for (int q = threadIdx.x; q < KS2 * (ksp + ksq); q += blockDim.x)
    BP[q] = tb[2 * KS2 + q];  // BQ follows BP in both layouts
  for (int m = threadIdx.x; m < ks; m += blockDim.x)
    gxo[m] = __dmul_rn(grw[IDX2(iv, m, nv)], ipow_d(grm[IDX2(iv, m, nv)], k + 1));
  __syncthreads();
  // phase 2: INT(j,jp,m) = sum_i (wk*Ba_j)*Bb_jp
  // (the weighted first factors wk*Ba are formed once per call in A, which
  // phase 3 fills only after the last call)
  auto inner = [&](const double *Ba, int ka, const double *Bb, int kb, double *INT) {
    double *WB = A;
    for (int q = threadIdx.x; q < KS2 * ka; q += blockDim.x) WB[q] = __dmul_rn(wk[q / ka], Ba[q]);
    __syncthreads();
    for (int q = threadIdx.x; q < ka * kb * ks; q += blockDim.x) {
      int j = q % ka, jp = (q / ka) % kb, m = q / (ka * kb);
      double s = 0.0;
      for (int i = 0; i < ks; i++) {
        int p = m * ks + i;
        s = fma(WB[(size_t)p * ka + j], Bb[(size_t)p * kb + jp], s);
      }
      INT[j + ka * (jp + kb * m)] = s;
    }
    __syncthreads();
  };
  if (type == 0) inner(BP, ksp, BP, ksp, INTP);
  if (type == 1) inner(BQ, ksq, BQ, ksq, INTQ);
  if (type == 2 || type == 3) {
    inner(BP, ksp, BP, ksp, INTP);
    inner(BQ, ksq, BQ, ksq, INTQ);
  }
  if (type == 4 || type == 5) inner(BP, ksp, BQ, ksq, INTPQ);
  __syncthreads();

  double *out = rkd + (size_t)kk * kk * iv;
  auto ob = [&](const double *b1, int i, const double *b2, int ip, int m) -> double {
    return __dmul_rn(__dmul_rn(b1[IDX3(iv, m, i, nw, ks)], b2[IDX3(iv, m, ip, nw, ks)]), gxo[m]);
  };
  auto pair_of = [](int ii, int kx, int *i, int *ip) {
    int r = ii, row = 0;
    while (r >= kx - row) {
      r -= kx - row;
      row++;
    }
    *i = row;
    *ip = row + r;
  };
  // triangular pairs (i <= ip) of one basis: OB[ii*ks + m]
  auto fill_tri = [&](const double *bs, int kx, double *OB) {
    const int ik = kx * (kx + 1) / 2;
    for (int q = threadIdx.x; q < ik * ks; q += blockDim.x) {
      const int ii = q / ks, m = q % ks;
      int i, ip;
      pair_of(ii, kx, &i, &ip);
      OB[q] = ob(bs, i, bs, ip, m);
    }
  };
  if (type == 0) fill_tri(pbsp, ksp, OB1);
  if (type == 1) fill_tri(qbsp, ksq, OB1);
  if (type == 2 || type == 3) {
    fill_tri(pbsp, ksp, OB1);
    fill_tri(qbsp, ksq, OB2);
  }
  if (type == 4 || type == 5) {  // outer (P,Q) pairs ii = i*ksq + ip, or (Q,P) ii = i*ksp + ip
    const int np = ksp * ksq;
    for (int q = threadIdx.x; q < np * ks; q += blockDim.x) {
      const int ii = q / ks, m = q % ks;
      OB1[q] = type == 4 ? ob(pbsp, ii / ksq, qbsp, ii % ksq, m)
                         : ob(qbsp, ii / ksp, pbsp, ii % ksp, m);
    }
  }
  __syncthreads();
  if (type == 0 || type == 1) {
    const int kx = type == 0 ? ksp : ksq;
    const double *INT = type == 0 ? INTP : INTQ;
    const int ik = kx * (kx + 1) / 2;
    for (int q = threadIdx.x; q < ik * ik; q += blockDim.x) {
      int ii = q % ik, jj = q / ik;
      int j, jp;
      pair_of(jj, kx, &j, &jp);
      const double *o = OB1 + ii * ks;
      double s = 0.0;
      for (int m = 0; m < ks; m++) s = fma(o[m], INT[j + kx * (jp + kx * m)], s);
      A[q] = s;
    }
    __syncthreads();
    for (int q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
      int ii = q % kk, jj = q / kk;
      out[q] = (ii < ik && jj < ik) ? __dadd_rn(A[ii + ik * jj], A[jj + ik * ii]) : 0.0;
    }
  } else if (type == 2 || type == 3) {
    const int ikp = ksp * (ksp + 1) / 2, ikq = ksq * (ksq + 1) / 2;
    for (int q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
      int r = q % kk, cc = q / kk;
      int pp_ = type == 2 ? r : cc, qq_ = type == 2 ? cc : r;  // P pair, Q pair
      double v = 0.0;
      if (pp_ < ikp && qq_ < ikq) {
        int i, ip, j, jp;
        pair_of(pp_, ksp, &i, &ip);
        pair_of(qq_, ksq, &j, &jp);
        const double *o1 = OB1 + pp_ * ks, *o2 = OB2 + qq_ * ks;
        double s1 = 0.0, s2 = 0.0;
        for (int m = 0; m < ks; m++) s1 = fma(o1[m], INTQ[j + ksq * (jp + ksq * m)], s1);
        for (int m = 0; m < ks; m++) s2 = fma(o2[m], INTP[i + ksp * (ip + ksp * m)], s2);
        v = __dadd_rn(s1, s2);
      }
      out[q] = v;
    }
  } else {
    const int np = ksp * ksq;
    for (int q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
      int jj = q % kk, ii = q / kk;  // rkd(jj,ii): jj inner (P,Q), ii outer
      double v = 0.0;
      if (jj < np && ii < np) {
        int j = jj / ksq, jp = jj % ksq;
        const double *o = OB1 + ii * ks;
        double s = 0.0;
        for (int m = 0; m < ks; m++) s = fma(o[m], INTPQ[j + ksp * (jp + ksq * m)], s);
        v = s;
      }
      out[q] = v;
    }
  }
}

static int build_triang_points(dbsrg_ctx *c) {
  DeviceGrid &g = c->g;
  const int KS2 = g.ks * g.ks;
  const size_t n = (size_t)g.nv * KS2 * (2 + g.ksp + g.ksq);
  DBSRG_TRY(c, cudaMalloc((void **)&g.tri, n * sizeof(double)));
  const int nq = g.nv * KS2;
  DBSRG_RUN(c, "k_triang_points",
            k_triang_points<<<(nq + 127) / 128, 128, 0, c->stream>>>(
                g.nv, g.ks, g.ksp, g.ksq, g.t, g.tp, g.tq, g.gx, g.gw, g.gr, g.tri));
  return DBSRG_OK;
}

int compute_diag_cells(dbsrg_ctx *c, int type, int k, double *rkd) {
  const DeviceGrid &g = c->g;
  const int ks = g.ks, kk = ks * ks;
  size_t nsm = (size_t)ks * ks + (size_t)ks * ks * g.ksp + (size_t)ks * ks * g.ksq +
               (size_t)g.ksp * g.ksp * ks + (size_t)g.ksq * g.ksq * ks +
               (size_t)g.ksp * g.ksq * ks + ks + (size_t)kk * kk + 2 * (size_t)kk * ks;
  size_t bytes = nsm * sizeof(double);
  int rc = raise_smem_limit(c, (const void *)k_triang, bytes);
  if (rc) return rc;
  DBSRG_RUN(c, "k_triang",
            k_triang<<<dim3(g.nv, 1), 256, bytes, c->stream>>>(g.nv, ks, g.ksp, g.ksq, type, k, g.tri,
                                                      g.grm, g.grw, g.pbsp, g.qbsp, rkd));
  return DBSRG_OK;
}

// ----------------------------------------------------------------------------
// R^k table fill: mrk_pppp/qqqq/pqpq/qpqp, dbsr_lib_dbs.f90:2898-2959,
// 3431-3492, 3067-3131, 3249-3313.  One thread per table element
// rkb(i,j,ip,jp); the element gathers its cell contributions in the
// reference's accumulation order (jv ascending, then iv ascending).
__device__ __forceinline__ int tri_index(int h, int hp, int kx) {  // 1-based
  return (h - 1) * kx - ((h - 1) * (h - 2)) / 2 + (hp - h + 1);
}

// band > 0: only the elements with |j - i| <= band, stored as
// rkb(i, j-i+band+1, ip, jp) of shape (ns, 2*band+1, ks, ks) -- all that the
// band part of the factored exchange reads.
__global__ void k_fill_r(int ns, int ks, int nv, int ka, int kb, const double *lowA,
                         const double *highA, const double *lowB, const double *highB,
                         const double *rkd, double *rkb, int band) {
  size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int nj = band > 0 ? 2 * band + 1 : ns;
  size_t total = (size_t)ns * nj * ks * ks;
  if (q >= total) return;
  const int kk = ks * ks;
  int i = (int)(q % ns) + 1;
  size_t r = q / ns;
  int j = (int)(r % nj) + 1;
  if (band > 0) j = i + (j - 1) - band;
  r /= nj;
  int ip = (int)(r % ks) + 1;
  int jp = (int)(r / ks) + 1;
  double acc = 0.0;
  if (ip <= ka && jp <= kb && j >= 1 && j <= ns) {
    const int ivlo = max(1, i - ka + ip), ivhi = min(nv, i);
    const int jvlo = max(1, j - kb + jp), jvhi = min(nv, j);
    // moment positions of the electron-1 pair in cell iv and the electron-2
    // pair in cell jv
    auto ia = [&](int iv) {
      const int ih = i - iv + 1;
      return (size_t)(tri_index(ih, ih + ip - 1, ka) - 1) + (size_t)kk * (iv - 1);
    };
    auto jb = [&](int jv) {
      const int jh = j - jv + 1;
      return (size_t)(tri_index(jh, jh + jp - 1, kb) - 1) + (size_t)kk * (jv - 1);
    };
    // the separable cells: iv < jv adds lowA(iv) times the sum of highB over
    // the cells jv > iv, iv > jv adds highA(iv) times the sum of lowB over
    // jv < iv.  Both sums are formed by additions only (the moments of
    // B-spline products are positive), suffix sums with iv descending and
    // prefix sums with iv ascending, so every element keeps full relative
    // precision with O(ka + kb) operations instead of O(ka kb).
    double suf = 0.0;
    for (int jv = jvhi; jv >= max(jvlo, ivhi + 1); jv--) suf += highB[jb(jv)];
    for (int iv = ivhi; iv >= ivlo; iv--) {
      acc = fma(lowA[ia(iv)], suf, acc);
      if (iv >= jvlo && iv <= jvhi) suf += highB[jb(iv)];
    }
    double pre = 0.0;
    for (int jv = jvlo; jv <= min(jvhi, ivlo - 1); jv++) pre += lowB[jb(jv)];
    for (int iv = ivlo; iv <= ivhi; iv++) {
      acc = fma(highA[ia(iv)], pre, acc);
      if (iv >= jvlo && iv <= jvhi) {  // the diagonal cell, then jv = iv joins the prefix
        const int ih = i - iv + 1, jh = j - iv + 1;
        const int ii = tri_index(ih, ih + ip - 1, ka), jj = tri_index(jh, jh + jp - 1, kb);
        acc += rkd[(ii - 1) + (size_t)kk * ((jj - 1) + (size_t)kk * (iv - 1))];
        pre += lowB[jb(iv)];
      }
    }
  }
  rkb[q] = acc;
}

// S^k table fill: msk_ppqq / msk_pqqp, dbsr_lib_dbs.f90:3601-3662,
// 3771-3833.  Only cells iv <= jv; band offsets ip = ihp-ih+ks.
__global__ void k_fill_s(int ns, int ks, int nv, int ksp, int ksq, int kj1, int kj2,
                         const double *r1, const double *r2, const double *rkd, double *rkb,
                         int band) {
  const int kb2 = 2 * ks - 1, kk = ks * ks;
  size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int nj = band > 0 ? 2 * band + 1 : ns;
  size_t total = (size_t)ns * nj * kb2 * kb2;
  if (q >= total) return;
  int i = (int)(q % ns) + 1;
  size_t r = q / ns;
  int j = (int)(r % nj) + 1;
  if (band > 0) j = i + (j - 1) - band;
  r /= nj;
  int ip = (int)(r % kb2) + 1;
  int jp = (int)(r / kb2) + 1;
  double acc = 0.0;
  if (j < 1 || j > ns) {
    rkb[q] = 0.0;
    return;
  }
  // electron 1: ih in [1,ksp], ihp = ip+ih-ks in [1,ksq], iv = i-ih+1
  const int ihlo = max(1, ks - ip + 1), ihhi = min(ksp, ks - ip + ksq);
  // electron 2: jh in [1,kj1], jhp = jp+jh-ks in [1,kj2], jv = j-jh+1
  const int jhlo = max(1, ks - jp + 1), jhhi = min(kj1, ks - jp + kj2);
  const int ivlo = max(1, i - ihhi + 1), ivhi = min(nv, i - ihlo + 1);
  const int jvlo = max(1, j - jhhi + 1), jvhi = min(nv, j - jhlo + 1);
  auto ia = [&](int iv) {  // (ii - 1) and the cell offset of electron 1
    const int ih = i - iv + 1;
    return (size_t)((ih - 1) * ksq + ip + ih - ks - 1);
  };
  auto jb = [&](int jv) {
    const int jh = j - jv + 1;
    return (size_t)((jh - 1) * kj2 + jp + jh - ks - 1);
  };
  // cells iv < jv: r1(iv) times the suffix sum of r2 over jv > iv (positive
  // moments, additions only, iv descending); the diagonal cells iv = jv
  double suf = 0.0;
  for (int jv = jvhi; jv >= max(jvlo, ivhi + 1); jv--) suf += r2[jb(jv) + (size_t)kk * (jv - 1)];
  for (int iv = ivhi; iv >= ivlo; iv--) {
    acc = fma(r1[ia(iv) + (size_t)kk * (iv - 1)], suf, acc);
    if (iv >= jvlo && iv <= jvhi) {
      acc += rkd[ia(iv) + (size_t)kk * (jb(iv) + (size_t)kk * (iv - 1))];
      suf += r2[jb(iv) + (size_t)kk * (iv - 1)];
    }
  }
  rkb[q] = acc;
}

static int ensure_slot(dbsrg_ctx *c, std::vector<double *> &v, size_t idx) {
  if (v.size() <= idx) v.resize(idx + 1, nullptr);
  return 0;
}

// Cell moments and diagonal-cell integrals of one table (family, type, k),
// kept resident: the table fill and the factored contraction both read
// them.  R: lo1/hi1 = moments of the electron-1 basis at r^k / r^-(k+1),
// lo2/hi2 the same for electron 2 (mrk_*: rkd1..rkd4).  S: lo1 =
// moments_pq(k) of electron 1, hi2 = moments_pq or moments_qp(-(k+1)) of
// electron 2 (msk_*: rkd1, rkd2); hi1 = lo2 = null (no r1 > r2 cells).
int get_celldata(dbsrg_ctx *c, int family, int type, int k, const CellData **out) {
  const DeviceGrid &g = c->g;
  std::vector<CellData> &v = family == 0 ? c->rcell : c->scell;
  size_t idx = (size_t)k * (family == 0 ? 4 : 2) + type;
  if (v.size() <= idx) v.resize(idx + 1);
  if (v[idx].rkd) {
    *out = &v[idx];
    return DBSRG_OK;
  }
  const int nv = g.nv, kk = g.ks * g.ks;
  size_t m = (size_t)kk * nv, d = (size_t)kk * kk * nv;
  double *base = nullptr;
  if (!(base = (double *)cache_alloc(c, (4 * m + d) * sizeof(double))))
    return set_err(c, DBSRG_ENOMEM, "cell data allocation failed");
  CellData cd;
  cd.lo1 = base;
  cd.hi1 = base + m;
  cd.lo2 = base + 2 * m;
  cd.hi2 = base + 3 * m;
  cd.rkd = base + 4 * m;
  int rc;
  if (family == 0) {
    int wa = (type == 0 || type == 2) ? 0 : 1, wb = (type == 0 || type == 3) ? 0 : 1;
    const int wh[4] = {wa, wa, wb, wb}, kp[4] = {k, -(k + 1), k, -(k + 1)};
    double *const out[4] = {cd.lo1, cd.hi1, cd.lo2, cd.hi2};
    if ((rc = compute_moment_set(c, 4, wh, kp, out))) return rc;
    if ((rc = compute_diag_cells(c, type, k, cd.rkd))) return rc;
  } else {
    const int wh[2] = {2, type == 0 ? 2 : 3}, kp[2] = {k, -(k + 1)};
    double *const out[2] = {cd.lo1, cd.hi2};
    if ((rc = compute_moment_set(c, 2, wh, kp, out))) return rc;
    if ((rc = compute_diag_cells(c, type == 0 ? 4 : 5, k, cd.rkd))) return rc;
    cd.hi1 = nullptr;
    cd.lo2 = nullptr;
  }
  v[idx] = cd;
  *out = &v[idx];
  return DBSRG_OK;
}

// full (band == 0) or band-limited table of (family, type, k), cached
static int get_table_any(dbsrg_ctx *c, int family, int type, int k, int band,
                         const double **out) {
  const DeviceGrid &g = c->g;
  std::vector<double *> &v = family == 0 ? (band ? c->rbtab : c->rtab) : (band ? c->sbtab : c->stab);
  size_t idx = (size_t)k * (family == 0 ? 4 : 2) + type;
  ensure_slot(c, v, idx);
  if (v[idx]) {
    *out = v[idx];
    return DBSRG_OK;
  }
  const int ns = g.ns, ks = g.ks, nv = g.nv, kb = family == 0 ? ks : 2 * ks - 1;
  const int nj = band ? 2 * band + 1 : ns;
  size_t nt = (size_t)ns * nj * kb * kb;
  const CellData *cd;
  int rc = get_celldata(c, family, type, k, &cd);
  if (rc) return rc;
  double *tab = nullptr;
  if (!(tab = (double *)cache_alloc(c, nt * sizeof(double))))
    return set_err(c, DBSRG_ENOMEM, "table allocation failed");
  unsigned nb = (unsigned)((nt + 255) / 256);
  if (family == 0) {
    int wa = (type == 0 || type == 2) ? 0 : 1, wb = (type == 0 || type == 3) ? 0 : 1;
    int ka = wa ? g.ksq : g.ksp, kbb = wb ? g.ksq : g.ksp;
    DBSRG_RUN(c, "k_fill_r",
              k_fill_r<<<nb, 256, 0, c->stream>>>(ns, ks, nv, ka, kbb, cd->lo1, cd->hi1, cd->lo2,
                                                  cd->hi2, cd->rkd, tab, band));
  } else {
    int kj1 = type == 0 ? g.ksp : g.ksq, kj2 = type == 0 ? g.ksq : g.ksp;
    DBSRG_RUN(c, "k_fill_s",
              k_fill_s<<<nb, 256, 0, c->stream>>>(ns, ks, nv, g.ksp, g.ksq, kj1, kj2, cd->lo1,
                                                  cd->hi2, cd->rkd, tab, band));
  }
  v[idx] = tab;
  *out = tab;
  return DBSRG_OK;
}

int get_rtable(dbsrg_ctx *c, int type, int k, const double **out) {
  return get_table_any(c, 0, type, k, 0, out);
}
int get_stable(dbsrg_ctx *c, int type, int k, const double **out) {
  return get_table_any(c, 1, type, k, 0, out);
}
int get_band_table(dbsrg_ctx *c, int family, int type, int k, const double **out) {
  return get_table_any(c, family, type, k, DBSRG_TABLE_BAND, out);
}

// ----------------------------------------------------------------------------
// <a|r^k|b> split by component for all orbital pairs: quadr
// (dbsr_lib_dbs.f90:3940-3976), used for the asymptotic coefficients
// (QUADR_PQ at R_data.f90:224, which selects the component by atype).
// First the banded matrix G(i,i+d) = sum over intervals and Gauss points of
// r^k w B_i B_{i+d} (d = 0..kx-1) per component, then quad(a,b,comp) =
// sum_{i,j} G(i,j) p_a(i) p_b(j) as W = G P per orbital and the products
// P^T W of all orbital pairs.
// blockIdx.y 0: the P basis (order kp, values bp, into Gp); 1: the Q basis
__global__ void k_rk_gram(int ns, int nv, int ks, int kp, int kq, int k, const double *bp,
                          const double *bq, const double *gr, const double *grw, double *Gp,
                          double *Gq) {
  const int kx = blockIdx.y ? kq : kp;
  const double *bs = blockIdx.y ? bq : bp;
  double *G = blockIdx.y ? Gq : Gp;
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ns * kx) return;
  int i = q % ns + 1, d = q / ns, j = i + d;  // 1-based i, j = i + d
  const int nw = nv + 1;
  double acc = 0.0;
  if (j <= ns) {
    int lo = max(1, j - kx + 1), hi = min(nv, i);
    for (int iv = lo; iv <= hi; iv++) {
      int ith = i - iv, jth = j - iv;
      double s = 0.0;
      for (int m = 0; m < ks; m++) {
        double wk = __dmul_rn(ipow_d(gr[IDX2(iv - 1, m, nv)], k), grw[IDX2(iv - 1, m, nv)]);
        s = __dadd_rn(s, __dmul_rn(bs[IDX3(iv - 1, m, jth, nw, ks)],
                                   __dmul_rn(wk, bs[IDX3(iv - 1, m, ith, nw, ks)])));
      }
      acc = __dadd_rn(acc, s);
    }
  }
  G[q] = acc;
}

// W(b, comp)(i) = sum_j G(i,j) p_b(j) over the symmetric band G (d = 0..kx-1
// stored as G(i, i+d))
__global__ void k_quad_w(int nbf, int ns, int ksp, int ksq, const double *pq, const double *GP,
                         const double *GQ, double *W) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= 2 * nbf * ns) return;
  const int i = q % ns, b = (q / ns) % nbf, comp = q / (ns * nbf);
  const int kx = comp == 0 ? ksp : ksq;
  const double *G = comp == 0 ? GP : GQ;
  const double *pb = pq + (size_t)ns * comp + (size_t)2 * ns * b;
  double s = G[i] * pb[i];
  for (int d = 1; d < kx; d++) {
    if (i + d < ns) s += G[(size_t)i + (size_t)ns * d] * pb[i + d];
    if (i - d >= 0) s += G[(size_t)(i - d) + (size_t)ns * d] * pb[i - d];
  }
  W[q] = s;
}

// quad(a, b, comp) = sum_i p_a(i) W(b, comp)(i): 32 x 32 tiles of (a, b)
__global__ void k_quad_dot(int nbf, int ns, const double *pq, const double *W, double *quad) {
  __shared__ double sa[32][33], sw[32][33];
  const int comp = blockIdx.z, a0 = blockIdx.x * 32, b0 = blockIdx.y * 32;
  const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;  // 256 threads: 8 rows
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i0 = 0; i0 < ns; i0 += 32) {
    for (int r = ty; r < 32; r += 8) {
      const int a = a0 + r, b = b0 + r, i = i0 + tx;
      sa[r][tx] = (a < nbf && i < ns) ? pq[(size_t)i + (size_t)ns * comp + (size_t)2 * ns * a] : 0.0;
      sw[r][tx] = (b < nbf && i < ns) ? W[(size_t)i + (size_t)ns * (b + (size_t)nbf * comp)] : 0.0;
    }
    __syncthreads();
    for (int k = 0; k < 4; k++) {
      const int ar = ty + 8 * k;
      double s = acc[k];
      for (int ii = 0; ii < 32; ii++) s += sa[ar][ii] * sw[tx][ii];
      acc[k] = s;
    }
    __syncthreads();
  }
  for (int k = 0; k < 4; k++) {
    const int a = a0 + ty + 8 * k, b = b0 + tx;
    if (a < nbf && b < nbf) quad[(size_t)a + (size_t)nbf * (b + (size_t)nbf * comp)] = acc[k];
  }
}

int get_quad(dbsrg_ctx *c, int k, const double **out) {
  if ((int)c->quad.size() <= k) c->quad.resize(k + 1, nullptr);
  if (c->quad[k]) {
    *out = c->quad[k];
    return DBSRG_OK;
  }
  const DeviceGrid &g = c->g;
  double *q = nullptr;
  size_t n = (size_t)c->nbf * c->nbf * 2;
  size_t gp = (size_t)g.ns * g.ksp, gq = (size_t)g.ns * g.ksq, nw = (size_t)2 * c->nbf * g.ns;
  if (!(q = (double *)cache_alloc(c, (n + gp + gq + nw) * sizeof(double))))
    return set_err(c, DBSRG_ENOMEM, "quad allocation failed");
  double *GP = q + n, *GQ = GP + gp, *W = GQ + gq;
  DBSRG_RUN(c, "k_rk_gram",
            k_rk_gram<<<dim3((unsigned)((std::max(gp, gq) + 63) / 64), 2), 64, 0, c->stream>>>(
                g.ns, g.nv, g.ks, g.ksp, g.ksq, k, g.pbsp, g.qbsp, g.gr, g.grw, GP, GQ));
  DBSRG_RUN(c, "k_quad_w", k_quad_w<<<(unsigned)((nw + 255) / 256), 256, 0, c->stream>>>(
                               c->nbf, g.ns, g.ksp, g.ksq, c->pq, GP, GQ, W));
  dim3 gd((unsigned)((c->nbf + 31) / 32), (unsigned)((c->nbf + 31) / 32), 2);
  DBSRG_RUN(c, "k_quad_dot", k_quad_dot<<<gd, 256, 0, c->stream>>>(c->nbf, g.ns, c->pq, W, q));
  c->quad[k] = q;
  *out = q;
  return DBSRG_OK;
}
