/*
 * dbsr_oracle.c -- CPU restatement (test infrastructure only) of the
 * DBSR_MAT3 Hamiltonian-block assembly path.  See dbsr_oracle.h for the
 * role of this file and how it is pinned.
 *
 * Layout: all arrays are Fortran column-major with the reference's own
 * dimensions; the macros below translate 1-based Fortran subscripts to
 * 0-based offsets so that every loop reads like the routine it follows.
 * Build with -ffp-contract=off so x86-64 and aarch64 hosts give the same
 * bits (no fused multiply-add contraction).
 */
#include "dbsr_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define A2(a, i, j, n1) (a)[((size_t)(i)-1) + (size_t)(n1) * ((size_t)(j)-1)]
#define A3(a, i, j, m, n1, n2)                                               \
  (a)[((size_t)(i)-1) +                                                      \
      (size_t)(n1) * (((size_t)(j)-1) + (size_t)(n2) * ((size_t)(m)-1))]
#define A4(a, i, j, k, l, n1, n2, n3)                                        \
  (a)[((size_t)(i)-1) +                                                      \
      (size_t)(n1) *                                                         \
          (((size_t)(j)-1) +                                                 \
           (size_t)(n2) * (((size_t)(k)-1) + (size_t)(n3) * ((size_t)(l)-1)))]

static int imax(int a, int b) { return a > b ? a : b; }
static int imin(int a, int b) { return a < b ? a : b; }

/* Integer power by binary exponentiation (the libgcc __powidf2 method
 * that gfortran uses for real**integer). */
static double ipow(double x, int m) {
  unsigned int n = m < 0 ? (unsigned)(-m) : (unsigned)m;
  double y = (n % 2) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2) y = y * x;
  }
  return m < 0 ? 1.0 / y : y;
}

/* ------------------------------------------------------------------ */
/* gauleg: dbsr_lib_zcom.f90:1990-2039 (Numerical-Recipes Newton).     */
void orc_gauleg(double x1, double x2, double *x, double *w, int n) {
  const double EPS = 1.0e-14;
  int m = (n + 1) / 2;
  double xm = 0.5 * (x2 + x1), xl = 0.5 * (x2 - x1);
  for (int i = 1; i <= m; i++) {
    double z = cos(3.141592654 * (i - 0.25) / (n + 0.5));
    double z1, pp, p1, p2, p3;
    do {
      p1 = 1.0;
      p2 = 0.0;
      for (int j = 1; j <= n; j++) {
        p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      z1 = z;
      z = z1 - p1 / pp;
    } while (fabs(z - z1) > EPS);
    x[i - 1] = xm - xl * z;
    x[n - i] = xm + xl * z;
    w[i - 1] = 2.0 * xl / ((1.0 - z * z) * pp * pp);
    w[n - i] = w[i - 1];
  }
}

/* ------------------------------------------------------------------ */
/* mkgrid_01: dbsr_lib_dbs.f90:724-783.  hs is the first step (hi/Z for a
 * point nucleus, 4 ln3 a_fermi * hi for a Fermi nucleus, :738-747).
 * Writes t(1:ns+ks) into t_out and returns ns (or -1 if max_t is too
 * small). */
int orc_mkgrid_01(int ks, int ml, double hs, double hi_unused, double he,
                  double hmax, double rmax, double *t_out, int max_t) {
  (void)hi_unused;
  double ti = hs * ml;
  int ns = ks + ml;
  double ht = 1.0 + he;
  int ne = ns;
  for (;;) {
    double tj = ti * ht;
    if (tj - ti > hmax) break;
    ns = ns + 1;
    ti = tj;
    ne = ns;
    if (ti > rmax) {
      ns = ns - 1;
      break;
    }
  }
  if (ti < rmax) {
    for (;;) {
      ti = ti + hmax;
      if (ti >= rmax) break;
      ns = ns + 1;
    }
  }
  if (ns + ks > max_t) return -1;
  double *t = t_out - 1; /* 1-based view */
  for (int i = 1; i <= ns + ks; i++) t[i] = 0.0;
  for (int i = ks + 1; i <= ks + ml; i++) t[i] = hs * (i - ks);
  for (int i = ks + ml + 1; i <= ne; i++) t[i] = t[i - 1] * ht;
  if (t[ne] < rmax)
    for (int i = ne + 1; i <= ns + 1; i++) t[i] = t[i - 1] + hmax;
  for (int i = ns + 2; i <= ns + ks; i++) t[i] = t[ns + 1];
  return ns;
}

/* ------------------------------------------------------------------ */
/* zbsplvd / zbsplvb: dbsr_lib_dbs.f90:4197-4468 (vector form of de
 * Boor's bsplvd/bsplvb).  dbiatx has the declared shape (nv,ks,ks). */
typedef struct {
  const double *t; /* 1-based view */
  int ks, nv, ni;
  double *deltar, *deltal; /* (ni,ks) */
  double *saved;           /* (ni) */
  int j;                   /* the SAVEd order counter of zbsplvb */
} bspl_ws;

static void zbsplvb(bspl_ws *s, int kg, const double *x, int jhigh, int index,
                    double *biatx) {
  const int ni = s->ni, nv = s->nv;
  const double *t = s->t;
  double *saved = s->saved, term;
  if (index == 1) {
    s->j = 1;
    for (int i = 1; i <= ni; i++) A2(biatx, i, 1, nv) = 1.0;
    if (s->j >= jhigh) return;
  }
  for (;;) {
    int j = s->j, jp1 = j + 1;
    for (int i = 1; i <= ni; i++) saved[i - 1] = 0.0;
    for (int i = 1; i <= ni; i++) {
      A2(s->deltar, i, j, ni) = t[i + kg - 1 + j] - x[i - 1];
      A2(s->deltal, i, j, ni) = x[i - 1] - t[i + kg - j];
    }
    for (int m = 1; m <= j; m++) {
      for (int i = 1; i <= ni; i++) {
        term = A2(biatx, i, m, nv) /
               (A2(s->deltar, i, m, ni) + A2(s->deltal, i, jp1 - m, ni));
        A2(biatx, i, m, nv) = saved[i - 1] + A2(s->deltar, i, m, ni) * term;
        saved[i - 1] = A2(s->deltal, i, jp1 - m, ni) * term;
      }
    }
    for (int i = 1; i <= ni; i++) A2(biatx, i, jp1, nv) = saved[i - 1];
    s->j = jp1;
    if (s->j >= jhigh) break;
  }
}

void orc_zbsplvd(int ns, int ks, int nv, const double *t, int kg, int ni,
                 const double *x, int nderiv, double *dbiatx) {
  (void)ns;
  /* per-point work arrays; ni is at most nv */
  double *deltar = (double *)calloc((size_t)ni * ks, sizeof(double));
  double *deltal = (double *)calloc((size_t)ni * ks, sizeof(double));
  double *savedv = (double *)calloc((size_t)ni, sizeof(double));
  bspl_ws s = {t - 1, ks, nv, ni, deltar, deltal, savedv, 1};
  int mhigh = imax(imin(nderiv, ks), 1);
  int kp1 = ks + 1;
  int jhigh = kp1 - mhigh;
  zbsplvb(&s, kg, x, jhigh, 1, dbiatx);
  if (mhigh == 1) {
    free(deltar);
    free(deltal);
    free(savedv);
    return;
  }
  int ideriv = mhigh;
  for (int m = 2; m <= mhigh; m++) {
    int jpimid = 1;
    for (int j = ideriv; j <= ks; j++) {
      for (int i = 1; i <= ni; i++)
        A3(dbiatx, i, j, ideriv, nv, ks) = A3(dbiatx, i, jpimid, 1, nv, ks);
      jpimid++;
    }
    ideriv--;
    jhigh = kp1 - ideriv;
    zbsplvb(&s, kg, x, jhigh, 2, dbiatx);
  }
  double *w31 = (double *)calloc((size_t)ni * ks * ks, sizeof(double));
  double *w1 = (double *)calloc((size_t)ni, sizeof(double));
  double *w2 = (double *)calloc((size_t)ni, sizeof(double));
  const double *tt = t - 1;
  int jlow = 1;
  for (int i = 1; i <= ks; i++) {
    for (int j = jlow; j <= ks; j++)
      for (int q = 1; q <= ni; q++) A3(w31, q, j, i, ni, ks) = 0.0;
    jlow = i;
    for (int q = 1; q <= ni; q++) A3(w31, q, i, i, ni, ks) = 1.0;
  }
  for (int m = 2; m <= mhigh; m++) {
    int kpimm = kp1 - m;
    double fkpimm = kpimm;
    int i = ks, il = 0;
    for (int ld = 1; ld <= kpimm; ld++) {
      for (int n = kg - il; n <= ni + kg - il - 1; n++)
        w1[n - kg + il] = fkpimm / (tt[n + kpimm] - tt[n]);
      for (int j = 1; j <= i; j++)
        for (int q = 1; q <= ni; q++)
          A3(w31, q, i, j, ni, ks) =
              (A3(w31, q, i, j, ni, ks) - A3(w31, q, i - 1, j, ni, ks)) *
              w1[q - 1];
      il++;
      i--;
    }
    for (int ii = 1; ii <= ks; ii++) {
      for (int q = 0; q < ni; q++) w2[q] = 0.0;
      int jl = imax(ii, m);
      for (int j = jl; j <= ks; j++)
        for (int q = 1; q <= ni; q++)
          w2[q - 1] = w2[q - 1] +
                      A3(w31, q, j, ii, ni, ks) * A3(dbiatx, q, j, m, nv, ks);
      for (int q = 1; q <= ni; q++) A3(dbiatx, q, ii, m, nv, ks) = w2[q - 1];
    }
  }
  free(w31);
  free(w1);
  free(w2);
  free(deltar);
  free(deltal);
  free(savedv);
}

/* ZINTYM: dbsr_lib_dbs.f90:4472-4497 */
static void zintym(int nv, int ks, int ks1, int ks2, const double *b1,
                   const double *b2, const double *ygr, int mm, double *ym) {
  memset(ym, 0, sizeof(double) * (size_t)mm * mm);
  for (int iv = 1; iv <= nv; iv++)
    for (int ith = 1; ith <= ks1; ith++) {
      int i = iv + ith - 1;
      for (int jth = 1; jth <= ks2; jth++) {
        int j = iv + jth - 1;
        double s = 0.0;
        for (int m = 1; m <= ks; m++)
          s += A2(ygr, iv, m, nv) * A3(b1, iv, m, ith, nv + 1, ks) *
               A3(b2, iv, m, jth, nv + 1, ks);
        A2(ym, i, j, mm) = A2(ym, i, j, mm) + s;
      }
    }
}

/* Def_pbsp / Def_qbsp: dbsr_lib_dbs.f90:987-1074 */
static void def_xbsp(orc_grid *g, int kx, double *tx, double *bsp,
                     double *bsd) {
  const int nv = g->nv, ks = g->ks, ns = g->ns;
  const int nsx = nv + kx - 1, nw = nv + 1;
  for (int i = 1; i <= kx; i++) tx[i - 1] = g->t[0];
  for (int i = kx + 1; i <= nsx; i++) tx[i - 1] = g->t[ks + (i - kx) - 1];
  for (int i = nsx + 1; i <= nsx + kx; i++)
    tx[i - 1] = g->t[ns + (i - nsx) - 1];
  double *dbi = (double *)calloc((size_t)nv * kx * kx, sizeof(double));
  for (int m = 1; m <= ks; m++) {
    orc_zbsplvd(nsx, kx, nv, tx, kx, nv, &A2(g->gr, 1, m, nv), 2, dbi);
    for (int ith = 1; ith <= kx; ith++)
      for (int i = 1; i <= nv; i++) {
        A3(bsp, i, m, ith, nw, ks) = A3(dbi, i, ith, 1, nv, kx);
        A3(bsd, i, m, ith, nw, ks) = A3(dbi, i, ith, 2, nv, kx);
      }
  }
  for (int m = 1; m <= ks; m++)
    for (int ith = 1; ith <= kx; ith++) {
      A3(bsp, nw, m, ith, nw, ks) = 0.0;
      A3(bsd, nw, m, ith, nw, ks) = 0.0;
    }
  orc_zbsplvd(nsx, kx, nv, tx, nsx, 1, &tx[nsx], 2, dbi);
  for (int ith = 1; ith <= kx; ith++) {
    A3(bsp, nw, 1, ith, nw, ks) = A3(dbi, 1, ith, 1, nv, kx);
    A3(bsd, nw, 1, ith, nw, ks) = A3(dbi, 1, ith, 2, nv, kx);
  }
  free(dbi);
}

/* alloc_DBS_gauss + Def_pbsp + Def_qbsp + Def_pq_arrays:
 * dbsr_lib_dbs.f90:911-983, 987-1102 (order-ks bsp arrays are not built:
 * nothing on the assembly path reads them). */
orc_grid *orc_grid_new(int ns, int ks, int ksp, int ksq, const double *t) {
  orc_grid *g = (orc_grid *)calloc(1, sizeof(orc_grid));
  g->ns = ns;
  g->ks = ks;
  g->ksp = ksp;
  g->ksq = ksq;
  g->nv = ns - ks + 1;
  g->nsp = g->nv + ksp - 1;
  g->nsq = g->nv + ksq - 1;
  g->ms = 2 * ns;
  const int nv = g->nv, nw = nv + 1, ms = g->ms;
  g->t = (double *)malloc(sizeof(double) * (ns + ks));
  memcpy(g->t, t, sizeof(double) * (ns + ks));
  g->tp = (double *)calloc(g->nsp + ksp, sizeof(double));
  g->tq = (double *)calloc(g->nsq + ksq, sizeof(double));
  g->gx = (double *)calloc(ks, sizeof(double));
  g->gw = (double *)calloc(ks, sizeof(double));
  g->gr = (double *)calloc((size_t)nv * ks, sizeof(double));
  g->grw = (double *)calloc((size_t)nv * ks, sizeof(double));
  g->grm = (double *)calloc((size_t)nv * ks, sizeof(double));
  g->pbsp = (double *)calloc((size_t)nw * ks * ksp, sizeof(double));
  g->pbsd = (double *)calloc((size_t)nw * ks * ksp, sizeof(double));
  g->qbsp = (double *)calloc((size_t)nw * ks * ksq, sizeof(double));
  g->qbsd = (double *)calloc((size_t)nw * ks * ksq, sizeof(double));
  size_t nn = (size_t)ns * ns;
  g->fpbs = (double *)calloc(nn, sizeof(double));
  g->fqbs = (double *)calloc(nn, sizeof(double));
  g->fpqbs = (double *)calloc(nn, sizeof(double));
  g->fqpbs = (double *)calloc(nn, sizeof(double));
  g->fpqbsd = (double *)calloc(nn, sizeof(double));
  g->fqpbsd = (double *)calloc(nn, sizeof(double));
  g->fppqq = (double *)calloc((size_t)ms * ms, sizeof(double));

  orc_gauleg(0.0, 1.0, g->gx, g->gw, ks);
  const double *tt = g->t - 1;
  for (int m = 1; m <= ks; m++)
    for (int i = 1; i <= nv; i++) {
      double h = tt[ks + i] - tt[ks + i - 1];
      A2(g->gr, i, m, nv) = h * g->gx[m - 1] + tt[ks + i - 1];
      A2(g->grm, i, m, nv) = 1.0 / A2(g->gr, i, m, nv);
      A2(g->grw, i, m, nv) = h * g->gw[m - 1];
    }
  def_xbsp(g, ksp, g->tp, g->pbsp, g->pbsd);
  zintym(nv, ks, ksp, ksp, g->pbsp, g->pbsp, g->grw, ns, g->fpbs);
  def_xbsp(g, ksq, g->tq, g->qbsp, g->qbsd);
  zintym(nv, ks, ksq, ksq, g->qbsp, g->qbsp, g->grw, ns, g->fqbs);
  double *ygw = (double *)calloc((size_t)nv * ks, sizeof(double));
  for (size_t q = 0; q < (size_t)nv * ks; q++) ygw[q] = g->grm[q] * g->grw[q];
  zintym(nv, ks, ksp, ksq, g->pbsp, g->qbsp, ygw, ns, g->fpqbs);
  zintym(nv, ks, ksq, ksp, g->qbsp, g->pbsp, ygw, ns, g->fqpbs);
  zintym(nv, ks, ksp, ksq, g->pbsp, g->qbsd, g->grw, ns, g->fpqbsd);
  zintym(nv, ks, ksq, ksp, g->qbsp, g->pbsd, g->grw, ns, g->fqpbsd);
  free(ygw);
  for (int j = 1; j <= ns; j++)
    for (int i = 1; i <= ns; i++) {
      A2(g->fppqq, i, j, ms) = A2(g->fpbs, i, j, ns);
      A2(g->fppqq, ns + i, ns + j, ms) = A2(g->fqbs, i, j, ns);
    }
  return g;
}

void orc_grid_free(orc_grid *g) {
  if (!g) return;
  free(g->t); free(g->tp); free(g->tq); free(g->gx); free(g->gw);
  free(g->gr); free(g->grw); free(g->grm); free(g->pbsp); free(g->pbsd);
  free(g->qbsp); free(g->qbsd); free(g->fpbs); free(g->fqbs);
  free(g->fpqbs); free(g->fqpbs); free(g->fpqbsd); free(g->fqpbsd);
  free(g->fppqq);
  free(g);
}

/* ------------------------------------------------------------------ */
/* moment_pp/qq/pq/qp: dbsr_lib_dbs.f90:1401-1564.  rkm(ks*ks,nv);
 * pp/qq are packed upper-triangular (i<=j), pq/qp full (i outer). */
void orc_moments(const orc_grid *g, int which, int k, double *rkm) {
  const int nv = g->nv, ks = g->ks, kk = ks * ks, nw = nv + 1;
  const double *b1s, *b2s;
  int k1, k2, sym;
  switch (which) {
    case 0: b1s = g->pbsp; b2s = g->pbsp; k1 = g->ksp; k2 = g->ksp; sym = 1; break;
    case 1: b1s = g->qbsp; b2s = g->qbsp; k1 = g->ksq; k2 = g->ksq; sym = 1; break;
    case 2: b1s = g->pbsp; b2s = g->qbsp; k1 = g->ksp; k2 = g->ksq; sym = 0; break;
    default: b1s = g->qbsp; b2s = g->pbsp; k1 = g->ksq; k2 = g->ksp; sym = 0; break;
  }
  memset(rkm, 0, sizeof(double) * (size_t)kk * nv);
  double gwv[64], b2[64 * 16];
  for (int iv = 1; iv <= nv; iv++) {
    for (int m = 1; m <= ks; m++) {
      double w = A2(g->grw, iv, m, nv);
      if (k > 0) w = A2(g->grw, iv, m, nv) * ipow(A2(g->gr, iv, m, nv), k);
      if (k < 0) w = A2(g->grw, iv, m, nv) * ipow(A2(g->grm, iv, m, nv), -k);
      gwv[m - 1] = w;
    }
    for (int j = 1; j <= k2; j++)
      for (int m = 1; m <= ks; m++)
        b2[(m - 1) + ks * (j - 1)] = A3(b2s, iv, m, j, nw, ks) * gwv[m - 1];
    int ii = 0;
    for (int i = 1; i <= k1; i++) {
      int j0 = sym ? i : 1;
      for (int j = j0; j <= k2; j++) {
        ii++;
        double s = 0.0;
        for (int m = 1; m <= ks; m++)
          s += A3(b1s, iv, m, i, nw, ks) * b2[(m - 1) + ks * (j - 1)];
        A2(rkm, ii, iv, kk) = s;
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* Diagonal-cell integrals triang_*: dbsr_lib_dbs.f90:2979-3063 (pppp),
 * 3151-3245 (pqpq), 3333-3427 (qpqp), 3512-3597 (qqqq), 3682-3767 (ppqq),
 * 3852-3936 (pqqp).  Inner integral over [t_iv, r] with ks Gauss points,
 * B-splines at the inner points from zbsplvd (order ksp or ksq). */

/* values of the kx B-splines nonzero on interval iv at point x */
static void bvals(const orc_grid *g, int kx, int iv, double x, double *out) {
  const double *tx = (kx == g->ksp) ? g->tp : g->tq;
  int nsx = g->nv + kx - 1;
  /* with ni=1 only dbiatx(1,:,1) is touched, so a leading dimension of 1
   * addresses the same elements as the reference's (nv,kx,kx) array */
  double buf[32 * 32];
  orc_zbsplvd(nsx, kx, 1, tx, iv + kx - 1, 1, &x, 1, buf);
  for (int j = 1; j <= kx; j++) out[j - 1] = buf[j - 1];
}

/* INT(j,jp,m) tables for one interval: for each outer point m, the inner
 * quadrature of B_j B_jp r^k over [t_iv, gr(iv,m)].  full=1 gives all
 * (j,jp) pairs of bases (ka,kb), full=0 only jp>=j (same basis). */
static void inner_table(const orc_grid *g, int iv, int k, int ka, int kb,
                        int full, double *INT /* (ka,kb,ks) */) {
  const int ks = g->ks, nv = g->nv;
  double x[32], w[32], gxl[32], gwl[32], ba[32 * 32], bb[32 * 32], v[32];
  orc_gauleg(0.0, 1.0, x, w, ks);
  double xbase = g->t[(iv + ks - 1) - 1];
  for (int m = 1; m <= ks; m++) {
    double r2 = A2(g->gr, iv, m, nv);
    for (int i = 0; i < ks; i++) gxl[i] = (r2 - xbase) * x[i] + xbase;
    for (int i = 0; i < ks; i++) {
      bvals(g, ka, iv, gxl[i], v);
      for (int j = 0; j < ka; j++) ba[i + ks * j] = v[j];
      bvals(g, kb, iv, gxl[i], v);
      for (int j = 0; j < kb; j++) bb[i + ks * j] = v[j];
    }
    for (int i = 0; i < ks; i++) gwl[i] = (r2 - xbase) * w[i];
    for (int i = 0; i < ks; i++) gxl[i] = gwl[i] * ipow(gxl[i], k);
    for (int j = 1; j <= ka; j++) {
      for (int i = 0; i < ks; i++) gwl[i] = gxl[i] * ba[i + ks * (j - 1)];
      int jp0 = full ? 1 : j;
      for (int jp = jp0; jp <= kb; jp++) {
        double s = 0.0;
        for (int i = 0; i < ks; i++) s += gwl[i] * bb[i + ks * (jp - 1)];
        A3(INT, j, jp, m, ka, kb) = s;
      }
    }
  }
}

void orc_triang(const orc_grid *g, int type, int k, double *rkd) {
  const int ks = g->ks, nv = g->nv, kk = ks * ks, nw = nv + 1;
  const int ksp = g->ksp, ksq = g->ksq;
  memset(rkd, 0, sizeof(double) * (size_t)kk * kk * nv);
  double *INTA = (double *)calloc((size_t)ks * ks * ks, sizeof(double));
  double *INTB = (double *)calloc((size_t)ks * ks * ks, sizeof(double));
  double *a = (double *)calloc((size_t)kk * kk, sizeof(double));
  double gxo[32], bi[32];
  for (int iv = 1; iv <= nv; iv++) {
    for (int m = 1; m <= ks; m++)
      gxo[m - 1] = A2(g->grw, iv, m, nv) * ipow(A2(g->grm, iv, m, nv), k + 1);
    if (type == 0 || type == 1) { /* pppp / qqqq: a + a^T */
      int kx = type == 0 ? ksp : ksq;
      const double *bs = type == 0 ? g->pbsp : g->qbsp;
      inner_table(g, iv, k, kx, kx, 0, INTA);
      int ik = kx * (kx + 1) / 2;
      int ii = 0;
      for (int i = 1; i <= kx; i++)
        for (int ip = i; ip <= kx; ip++) {
          ii++;
          for (int m = 1; m <= ks; m++)
            bi[m - 1] = A3(bs, iv, m, i, nw, ks) * A3(bs, iv, m, ip, nw, ks) *
                        gxo[m - 1];
          int jj = 0;
          for (int j = 1; j <= kx; j++)
            for (int jp = j; jp <= kx; jp++) {
              jj++;
              double s = 0.0;
              for (int m = 1; m <= ks; m++)
                s += bi[m - 1] * A3(INTA, j, jp, m, kx, kx);
              A2(a, ii, jj, ik) = s;
            }
        }
      for (int jj = 1; jj <= ik; jj++)
        for (int ii2 = 1; ii2 <= ik; ii2++)
          A3(rkd, ii2, jj, iv, kk, kk) = A2(a, ii2, jj, ik) + A2(a, jj, ii2, ik);
    } else if (type == 2 || type == 3) { /* pqpq / qpqp */
      inner_table(g, iv, k, ksp, ksp, 0, INTA); /* INTP */
      inner_table(g, iv, k, ksq, ksq, 0, INTB); /* INTQ */
      int ii = 0;
      for (int i = 1; i <= ksp; i++)
        for (int ip = i; ip <= ksp; ip++) {
          ii++;
          for (int m = 1; m <= ks; m++)
            bi[m - 1] = A3(g->pbsp, iv, m, i, nw, ks) *
                        A3(g->pbsp, iv, m, ip, nw, ks) * gxo[m - 1];
          int jj = 0;
          for (int j = 1; j <= ksq; j++)
            for (int jp = j; jp <= ksq; jp++) {
              jj++;
              double s = 0.0;
              for (int m = 1; m <= ks; m++)
                s += bi[m - 1] * A3(INTB, j, jp, m, ksq, ksq);
              if (type == 2)
                A3(rkd, ii, jj, iv, kk, kk) = A3(rkd, ii, jj, iv, kk, kk) + s;
              else
                A3(rkd, jj, ii, iv, kk, kk) = A3(rkd, jj, ii, iv, kk, kk) + s;
            }
        }
      ii = 0;
      for (int i = 1; i <= ksq; i++)
        for (int ip = i; ip <= ksq; ip++) {
          ii++;
          for (int m = 1; m <= ks; m++)
            bi[m - 1] = A3(g->qbsp, iv, m, i, nw, ks) *
                        A3(g->qbsp, iv, m, ip, nw, ks) * gxo[m - 1];
          int jj = 0;
          for (int j = 1; j <= ksp; j++)
            for (int jp = j; jp <= ksp; jp++) {
              jj++;
              double s = 0.0;
              for (int m = 1; m <= ks; m++)
                s += bi[m - 1] * A3(INTA, j, jp, m, ksp, ksp);
              if (type == 2)
                A3(rkd, jj, ii, iv, kk, kk) = A3(rkd, jj, ii, iv, kk, kk) + s;
              else
                A3(rkd, ii, jj, iv, kk, kk) = A3(rkd, ii, jj, iv, kk, kk) + s;
            }
        }
    } else { /* 4 ppqq: outer (P_i,Q_ip), inner (P_j,Q_jp);
                5 pqqp: outer (Q_i,P_ip), inner (P_j,Q_jp) */
      inner_table(g, iv, k, ksp, ksq, 1, INTA); /* INTPQ */
      const double *b1 = type == 4 ? g->pbsp : g->qbsp;
      const double *b2 = type == 4 ? g->qbsp : g->pbsp;
      int k1 = type == 4 ? ksp : ksq, k2 = type == 4 ? ksq : ksp;
      int ii = 0;
      for (int i = 1; i <= k1; i++)
        for (int ip = 1; ip <= k2; ip++) {
          ii++;
          for (int m = 1; m <= ks; m++)
            bi[m - 1] = A3(b1, iv, m, i, nw, ks) * A3(b2, iv, m, ip, nw, ks) *
                        gxo[m - 1];
          int jj = 0;
          for (int j = 1; j <= ksp; j++)
            for (int jp = 1; jp <= ksq; jp++) {
              jj++;
              double s = 0.0;
              for (int m = 1; m <= ks; m++)
                s += bi[m - 1] * A3(INTA, j, jp, m, ksp, ksq);
              A3(rkd, jj, ii, iv, kk, kk) = s;
            }
        }
    }
  }
  free(INTA);
  free(INTB);
  free(a);
}

/* ------------------------------------------------------------------ */
/* R^k table fill: mrk_pppp/qqqq/pqpq/qpqp, dbsr_lib_dbs.f90:2898-2959,
 * 3431-3492, 3067-3131, 3249-3313.  Electron 1 (i,i') in basis A, electron
 * 2 (j,j') in basis B; off-diagonal cells are products of the 1-D moments,
 * diagonal cells come from triang_*. */
void orc_mrk(const orc_grid *g, int type, int k, double *rkb) {
  const int ns = g->ns, ks = g->ks, nv = g->nv, kk = ks * ks;
  int wa = (type == 0 || type == 2) ? 0 : 1; /* 0 = P, 1 = Q */
  int wb = (type == 0 || type == 3) ? 0 : 1;
  int ka = wa ? g->ksq : g->ksp, kb = wb ? g->ksq : g->ksp;
  double *lowA = (double *)malloc(sizeof(double) * kk * nv);
  double *highA = (double *)malloc(sizeof(double) * kk * nv);
  double *lowB = (double *)malloc(sizeof(double) * kk * nv);
  double *highB = (double *)malloc(sizeof(double) * kk * nv);
  double *rkd = (double *)malloc(sizeof(double) * (size_t)kk * kk * nv);
  orc_moments(g, wa, k, lowA);
  orc_moments(g, wa, -(k + 1), highA);
  orc_moments(g, wb, k, lowB);
  orc_moments(g, wb, -(k + 1), highB);
  orc_triang(g, type, k, rkd);
  memset(rkb, 0, sizeof(double) * (size_t)ns * ns * ks * ks);
  for (int jv = 1; jv <= nv; jv++) {
    int jj = 0;
    for (int jh = 1; jh <= kb; jh++) {
      int j = jv + jh - 1;
      for (int jhp = jh; jhp <= kb; jhp++) {
        int jp = jhp - jh + 1;
        jj++;
        for (int iv = 1; iv <= nv; iv++) {
          int ii = 0;
          for (int ih = 1; ih <= ka; ih++) {
            int i = iv + ih - 1;
            for (int ihp = ih; ihp <= ka; ihp++) {
              int ip = ihp - ih + 1;
              ii++;
              double c;
              if (iv < jv)
                c = A2(lowA, ii, iv, kk) * A2(highB, jj, jv, kk);
              else if (iv > jv)
                c = A2(lowB, jj, jv, kk) * A2(highA, ii, iv, kk);
              else
                c = A3(rkd, ii, jj, iv, kk, kk);
              A4(rkb, i, j, ip, jp, ns, ns, ks) =
                  A4(rkb, i, j, ip, jp, ns, ns, ks) + c;
            }
          }
        }
      }
    }
  }
  free(lowA); free(highA); free(lowB); free(highB); free(rkd);
}

/* S^k table fill: msk_ppqq / msk_pqqp, dbsr_lib_dbs.f90:3601-3662,
 * 3771-3833.  Only cells iv<=jv; band offsets ip = ihp-ih+ks. */
void orc_msk(const orc_grid *g, int type, int k, double *rkb) {
  const int ns = g->ns, ks = g->ks, nv = g->nv, kk = ks * ks, kb2 = 2 * ks - 1;
  const int ksp = g->ksp, ksq = g->ksq;
  double *r1 = (double *)malloc(sizeof(double) * kk * nv);
  double *r2 = (double *)malloc(sizeof(double) * kk * nv);
  double *rkd = (double *)malloc(sizeof(double) * (size_t)kk * kk * nv);
  orc_moments(g, 2, k, r1);                       /* pq(k)      */
  orc_moments(g, type == 0 ? 2 : 3, -(k + 1), r2); /* pq or qp   */
  orc_triang(g, type == 0 ? 4 : 5, k, rkd);
  memset(rkb, 0, sizeof(double) * (size_t)ns * ns * kb2 * kb2);
  int kj1 = type == 0 ? ksp : ksq, kj2 = type == 0 ? ksq : ksp;
  for (int jv = 1; jv <= nv; jv++) {
    int jj = 0;
    for (int jh = 1; jh <= kj1; jh++) {
      int j = jv + jh - 1;
      for (int jhp = 1; jhp <= kj2; jhp++) {
        int jp = jhp - jh + ks;
        jj++;
        for (int iv = 1; iv <= jv; iv++) {
          int ii = 0;
          for (int ih = 1; ih <= ksp; ih++) {
            int i = iv + ih - 1;
            for (int ihp = 1; ihp <= ksq; ihp++) {
              int ip = ihp - ih + ks;
              ii++;
              double c;
              if (iv == jv)
                c = A3(rkd, ii, jj, iv, kk, kk);
              else
                c = A2(r1, ii, iv, kk) * A2(r2, jj, jv, kk);
              A4(rkb, i, j, ip, jp, ns, ns, kb2) =
                  A4(rkb, i, j, ip, jp, ns, ns, kb2) + c;
            }
          }
        }
      }
    }
  }
  free(r1); free(r2); free(rkd);
}

/* ------------------------------------------------------------------ */
/* density: dbsr_lib_dbs.f90:2834-2891 */
void orc_density(int ns, int ks, double *d, const double *p1,
                 const double *p2, char type) {
  const double *P1 = p1 - 1, *P2 = p2 - 1;
  if (type == 's' || type == 'u') {
    for (int j = 1; j <= ks; j++)
      for (int i = 1; i <= ns; i++) A2(d, i, j, ns) = 0.0;
    for (int i = 1; i <= ns; i++) A2(d, i, 1, ns) = P1[i] * P2[i];
    for (int j = 2; j <= ks; j++)
      for (int i = 1; i <= ns - j + 1; i++)
        A2(d, i, j, ns) = P1[i] * P2[i + j - 1] + P1[i + j - 1] * P2[i];
  } else if (type == 'l') {
    for (int j = 1; j <= ks; j++)
      for (int i = 1; i <= ns; i++) A2(d, i, j, ns) = 0.0;
    for (int i = 1; i <= ns; i++) A2(d, i, ks, ns) = P1[i] * P2[i];
    for (int j = 1; j <= ks - 1; j++)
      for (int i = ks + 1 - j; i <= ns; i++)
        A2(d, i, j, ns) = P1[i] * P2[i + j - ks] + P1[i + j - ks] * P2[i];
  } else if (type == 'n') {
    for (int j = 1; j <= 2 * ks - 1; j++)
      for (int i = 1; i <= ns; i++) A2(d, i, j, ns) = 0.0;
    for (int j = 1; j <= 2 * ks - 1; j++) {
      int i0 = imax(1, 1 + ks - j), i1 = imin(ns, ns + ks - j);
      for (int i = i0; i <= i1; i++) A2(d, i, j, ns) = P1[i] * P2[i + j - ks];
    }
  } else {
    for (int j = 1; j <= ns; j++)
      for (int i = 1; i <= ns; i++) A2(d, i, j, ns) = P1[i] * P2[j];
  }
}

/* ------------------------------------------------------------------ */
/* convol / convol_sk: dbsr_lib_dbs.f90:2208-2478, 2482-2752.  The table
 * is passed explicitly; kb is its declared band extent (ks or 2ks-1). */
#define RKB(i, j, ip, jp) A4(rkb, i, j, ip, jp, ns, ns, kb)
#define AA(i, j) A2(a, i, j, ns)
#define DD(i, j) A2(d, i, j, ns)
void orc_convol(int ns, int ks, int kb, const double *rkb, double *a,
                const double *d, int icase, char sym_i, char sym_j) {
  int ii, jj;
  double c;
  if (icase <= 2)
    for (int j = 1; j <= ks; j++)
      for (int i = 1; i <= ns; i++) AA(i, j) = 0.0;
  if (icase > 2)
    for (int j = 1; j <= ns; j++)
      for (int i = 1; i <= ns; i++) AA(i, j) = 0.0;
  const int k2 = ks + ks - 1;
  switch (icase) {
    case 1:
      if (sym_i == 's' && sym_j == 's') {
        for (int ip = 1; ip <= ks; ip++)
          for (int i = 1; i <= ns - ip + 1; i++) {
            c = 0.0;
            for (int jp = 1; jp <= ks; jp++)
              for (int j = 1; j <= ns - jp + 1; j++) c = c + DD(j, jp) * RKB(i, j, ip, jp);
            AA(i, ip) = c;
          }
      } else if (sym_i == 'n' && sym_j == 'n') {
        for (int ip = 1; ip <= k2; ip++) {
          int i0 = imax(1, 1 + ks - ip), i1 = imin(ns, ns + ks - ip);
          for (int i = i0; i <= i1; i++) {
            c = 0.0;
            for (int jp = 1; jp <= k2; jp++) {
              int j0 = imax(1, 1 + ks - jp), j1 = imin(ns, ns + ks - jp);
              for (int j = j0; j <= j1; j++) c = c + DD(j, jp) * RKB(i, j, ip, jp);
            }
            AA(i, ip) = c;
          }
        }
      } else if (sym_i == 'l' && sym_j == 'l') {
        for (int ip = 1; ip <= ks; ip++)
          for (int i = ks + 1 - ip; i <= ns; i++) {
            c = 0.0;
            for (int jp = 1; jp <= ks; jp++)
              for (int j = ks + 1 - jp; j <= ns; j++) c = c + DD(j, jp) * RKB(i, j, ip, jp);
            AA(i, ip) = c;
          }
      } else if (sym_i == 'l' && sym_j == 'n') {
        for (int ip = 1; ip <= ks; ip++)
          for (int i = ks + 1 - ip; i <= ns; i++) {
            c = 0.0;
            for (int jp = 1; jp <= k2; jp++) {
              int j0 = imax(1, 1 + ks - jp), j1 = imin(ns, ns + ks - jp);
              for (int j = j0; j <= j1; j++) c = c + DD(j, jp) * RKB(i, j, ip, jp);
            }
            AA(i, ip) = c;
          }
      } else if (sym_i == 'n' && sym_j == 'l') {
        for (int ip = 1; ip <= k2; ip++) {
          int i0 = imax(1, 1 + ks - ip), i1 = imin(ns, ns + ks - ip);
          for (int i = i0; i <= i1; i++) {
            c = 0.0;
            for (int jp = 1; jp <= ks; jp++)
              for (int j = ks + 1 - jp; j <= ns; j++) c = c + DD(j, jp) * RKB(i, j, ip, jp);
            AA(i, ip) = c;
          }
        }
      }
      break;
    case 2:
      if (sym_i == 's' && sym_j == 's') {
        for (int jp = 1; jp <= ks; jp++)
          for (int j = 1; j <= ns - jp + 1; j++) {
            c = 0.0;
            for (int ip = 1; ip <= ks; ip++)
              for (int i = 1; i <= ns - ip + 1; i++) c = c + DD(i, ip) * RKB(i, j, ip, jp);
            AA(j, jp) = c;
          }
      } else if (sym_i == 'n' && sym_j == 'n') {
        for (int jp = 1; jp <= k2; jp++) {
          int j0 = imax(1, 1 + ks - jp), j1 = imin(ns, ns + ks - jp);
          for (int j = j0; j <= j1; j++) {
            c = 0.0;
            for (int ip = 1; ip <= k2; ip++) {
              int i0 = imax(1, 1 + ks - ip), i1 = imin(ns, ns + ks - ip);
              for (int i = i0; i <= i1; i++) c = c + DD(i, ip) * RKB(i, j, ip, jp);
            }
            AA(j, jp) = c;
          }
        }
      } else if (sym_i == 'l' && sym_j == 'l') {
        for (int jp = 1; jp <= ks; jp++)
          for (int j = ks + 1 - jp; j <= ns; j++) {
            c = 0.0;
            for (int ip = 1; ip <= ks; ip++)
              for (int i = ks + 1 - ip; i <= ns; i++) c = c + DD(i, ip) * RKB(i, j, ip, jp);
            AA(j, jp) = c;
          }
      } else if (sym_i == 'l' && sym_j == 'n') {
        for (int jp = 1; jp <= k2; jp++) {
          int j0 = imax(1, 1 + ks - jp), j1 = imin(ns, ns + ks - jp);
          for (int j = j0; j <= j1; j++) {
            c = 0.0;
            for (int ip = 1; ip <= ks; ip++)
              for (int i = ks + 1 - ip; i <= ns; i++) c = c + DD(i, ip) * RKB(i, j, ip, jp);
            AA(j, jp) = c;
          }
        }
      } else if (sym_i == 'n' && sym_j == 'l') {
        for (int jp = 1; jp <= ks; jp++)
          for (int j = ks + 1 - jp; j <= ns; j++) {
            c = 0.0;
            for (int ip = 1; ip <= k2; ip++) {
              int i0 = imax(1, 1 + ks - ip), i1 = imin(ns, ns + ks - ip);
              for (int i = i0; i <= i1; i++) c = c + DD(i, ip) * RKB(i, j, ip, jp);
            }
            AA(j, jp) = c;
          }
      }
      break;
    case 3:
      if (sym_i == 's' && sym_j == 's') {
        for (int jp = 1; jp <= ks; jp++)
          for (int j = 1; j <= ns - jp + 1; j++) {
            jj = j + jp - 1;
            for (int ip = 1; ip <= ks; ip++)
              for (int i = 1; i <= ns - ip + 1; i++) {
                ii = i + ip - 1;
                c = RKB(i, j, ip, jp);
                AA(i, jj) = AA(i, jj) + c * DD(ii, j);
                if (ip > 1) AA(ii, jj) = AA(ii, jj) + c * DD(i, j);
                if (jp > 1) AA(i, j) = AA(i, j) + c * DD(ii, jj);
                if (ip > 1 && jp > 1) AA(ii, j) = AA(ii, j) + c * DD(i, jj);
              }
          }
      } else if (sym_i == 'l' && sym_j == 'l') {
        for (int jp = 1; jp <= ks; jp++)
          for (int j = ks + 1 - jp; j <= ns; j++) {
            jj = j + jp - ks;
            for (int ip = 1; ip <= ks; ip++)
              for (int i = ks + 1 - ip; i <= ns; i++) {
                ii = i + ip - ks;
                c = RKB(i, j, ip, jp);
                AA(i, jj) = AA(i, jj) + c * DD(ii, j);
                if (ip != ks) AA(ii, jj) = AA(ii, jj) + c * DD(i, j);
                if (jp != ks) AA(i, j) = AA(i, j) + c * DD(ii, jj);
                if (ip != ks && jp != ks) AA(ii, j) = AA(ii, j) + c * DD(i, jj);
              }
          }
      } else if (sym_i == 'n' && sym_j == 'n') {
        for (int jp = 1; jp <= k2; jp++) {
          int j0 = imax(1, 1 + ks - jp), j1 = imin(ns, ns + ks - jp);
          for (int j = j0; j <= j1; j++) {
            jj = j + jp - ks;
            for (int ip = 1; ip <= k2; ip++) {
              int i0 = imax(1, 1 + ks - ip), i1 = imin(ns, ns + ks - ip);
              for (int i = i0; i <= i1; i++) {
                ii = i + ip - ks;
                c = RKB(i, j, ip, jp);
                AA(i, jj) = AA(i, jj) + c * DD(ii, j);
              }
            }
          }
        }
      } else if (sym_i == 'n' && sym_j == 'l') {
        for (int jp = 1; jp <= ks; jp++)
          for (int j = ks + 1 - jp; j <= ns; j++) {
            jj = j + jp - ks;
            for (int ip = 1; ip <= k2; ip++) {
              int i0 = imax(1, 1 + ks - ip), i1 = imin(ns, ns + ks - ip);
              for (int i = i0; i <= i1; i++) {
                ii = i + ip - ks;
                c = RKB(i, j, ip, jp);
                AA(i, jj) = AA(i, jj) + c * DD(ii, j);
                if (jp != ks) AA(i, j) = AA(i, j) + c * DD(ii, jj);
              }
            }
          }
      } else if (sym_i == 'l' && sym_j == 'n') {
        for (int jp = 1; jp <= k2; jp++) {
          int j0 = imax(1, 1 + ks - jp), j1 = imin(ns, ns + ks - jp);
          for (int j = j0; j <= j1; j++) {
            jj = j + jp - ks;
            for (int ip = 1; ip <= ks; ip++)
              for (int i = ks + 1 - ip; i <= ns; i++) {
                ii = i + ip - ks;
                c = RKB(i, j, ip, jp);
                AA(i, jj) = AA(i, jj) + c * DD(ii, j);
                if (ip != ks) AA(ii, jj) = AA(ii, jj) + c * DD(i, j);
              }
          }
        }
      }
      break;
    case 4:
      if (sym_i == 's' && sym_j == 's') {
        for (int jp = 1; jp <= ks; jp++)
          for (int j = 1; j <= ns - jp + 1; j++) {
            jj = j + jp - 1;
            for (int ip = 1; ip <= ks; ip++)
              for (int i = 1; i <= ns - ip + 1; i++) {
                ii = i + ip - 1;
                c = RKB(i, j, ip, jp);
                AA(ii, j) = AA(ii, j) + c * DD(i, jj);
                if (ip > 1) AA(i, j) = AA(i, j) + c * DD(ii, jj);
                if (jp > 1) AA(ii, jj) = AA(ii, jj) + c * DD(i, j);
                if (ip > 1 && jp > 1) AA(i, jj) = AA(i, jj) + c * DD(ii, j);
              }
          }
      } else if (sym_i == 'n' && sym_j == 'n') {
        for (int jp = 1; jp <= k2; jp++) {
          int j0 = imax(1, 1 + ks - jp), j1 = imin(ns, ns + ks - jp);
          for (int j = j0; j <= j1; j++) {
            jj = j + jp - ks;
            for (int ip = 1; ip <= k2; ip++) {
              int i0 = imax(1, 1 + ks - ip), i1 = imin(ns, ns + ks - ip);
              for (int i = i0; i <= i1; i++) {
                ii = i + ip - ks;
                c = RKB(i, j, ip, jp);
                AA(ii, j) = AA(ii, j) + c * DD(i, jj);
              }
            }
          }
        }
      } else if (sym_i == 'l' && sym_j == 'l') {
        for (int jp = 1; jp <= ks; jp++)
          for (int j = ks + 1 - jp; j <= ns; j++) {
            jj = j + jp - ks;
            for (int ip = 1; ip <= ks; ip++)
              for (int i = ks + 1 - ip; i <= ns; i++) {
                ii = i + ip - ks;
                c = RKB(i, j, ip, jp);
                AA(ii, j) = AA(ii, j) + c * DD(i, jj);
                if (ip != ks) AA(i, j) = AA(i, j) + c * DD(ii, jj);
                if (jp != ks) AA(ii, jj) = AA(ii, jj) + c * DD(i, j);
                if (ip != ks && jp != ks) AA(i, jj) = AA(i, jj) + c * DD(ii, j);
              }
          }
      } else if (sym_i == 'n' && sym_j == 'l') {
        for (int jp = 1; jp <= ks; jp++)
          for (int j = ks + 1 - jp; j <= ns; j++) {
            jj = j + jp - ks;
            for (int ip = 1; ip <= k2; ip++) {
              int i0 = imax(1, 1 + ks - ip), i1 = imin(ns, ns + ks - ip);
              for (int i = i0; i <= i1; i++) {
                ii = i + ip - ks;
                c = RKB(i, j, ip, jp);
                AA(ii, j) = AA(ii, j) + c * DD(i, jj);
                if (jp != ks) AA(ii, jj) = AA(ii, jj) + c * DD(i, j);
              }
            }
          }
      } else if (sym_i == 'l' && sym_j == 'n') {
        for (int jp = 1; jp <= k2; jp++) {
          int j0 = imax(1, 1 + ks - jp), j1 = imin(ns, ns + ks - jp);
          for (int j = j0; j <= j1; j++) {
            jj = j + jp - ks;
            for (int ip = 1; ip <= ks; ip++)
              for (int i = ks + 1 - ip; i <= ns; i++) {
                ii = i + ip - ks;
                c = RKB(i, j, ip, jp);
                AA(ii, j) = AA(ii, j) + c * DD(i, jj);
                if (ip != ks) AA(i, j) = AA(i, j) + c * DD(ii, jj);
              }
          }
        }
      }
      break;
    default:
      break;
  }
}
#undef RKB
#undef AA
#undef DD

/* SUM_AmB: dbsr_lib_dbs.f90:4027-4080 */
double orc_sum_amb(int ns, int ks, const double *a, const double *b,
                   char sym) {
  double x = 0.0;
  if (sym == 'x') {
    for (int i = 1; i <= ns; i++)
      for (int j = 1; j <= ns; j++) x = x + A2(a, i, j, ns) * A2(b, i, j, ns);
  } else if (sym == 's') {
    for (int j = 1; j <= ks; j++)
      for (int i = 1; i <= ns - j + 1; i++) x = x + A2(a, i, j, ns) * A2(b, i, j, ns);
  } else if (sym == 'l') {
    for (int j = 1; j <= ks; j++)
      for (int i = ks + 1 - j; i <= ns; i++) x = x + A2(a, i, j, ns) * A2(b, i, j, ns);
  } else if (sym == 'n') {
    for (int j = 1; j <= 2 * ks - 1; j++) {
      int i0 = imax(1, 1 + ks - j), i1 = imin(ns, ns + ks - j);
      for (int i = i0; i <= i1; i++) x = x + A2(a, i, j, ns) * A2(b, i, j, ns);
    }
  }
  return x;
}

/* quadr: dbsr_lib_dbs.f90:3940-3976; fi,fj are (ns,2) */
static double quadr_part(const orc_grid *g, const double *fi, const double *fj,
                         int m, int comp) {
  const int nv = g->nv, ks = g->ks, ns = g->ns, nw = nv + 1;
  const int kx = comp == 0 ? g->ksp : g->ksq;
  const double *bs = comp == 0 ? g->pbsp : g->qbsp;
  const double *Fi = fi + (size_t)ns * comp - 1, *Fj = fj + (size_t)ns * comp - 1;
  double q = 0.0, gxl[64], gwl[64];
  for (int iv = 1; iv <= nv; iv++) {
    for (int mm = 1; mm <= ks; mm++)
      gxl[mm - 1] = ipow(A2(g->gr, iv, mm, nv), m) * A2(g->grw, iv, mm, nv);
    for (int ith = 1; ith <= kx; ith++) {
      int i = iv + ith - 1;
      double pi = Fi[i];
      for (int mm = 1; mm <= ks; mm++)
        gwl[mm - 1] = gxl[mm - 1] * A3(bs, iv, mm, ith, nw, ks);
      for (int jth = 1; jth <= kx; jth++) {
        int j = iv + jth - 1;
        double pj = Fj[j], s = 0.0;
        for (int mm = 1; mm <= ks; mm++) s += A3(bs, iv, mm, jth, nw, ks) * gwl[mm - 1];
        q = q + s * pi * pj;
      }
    }
  }
  return q;
}

double orc_quadr(const orc_grid *g, const double *fi, const double *fj,
                 int m) {
  /* the reference accumulates the Q part onto the running P sum */
  const int nv = g->nv, ks = g->ks, ns = g->ns, nw = nv + 1;
  double q = quadr_part(g, fi, fj, m, 0);
  const double *Fi = fi + ns - 1, *Fj = fj + ns - 1;
  double gxl[64], gwl[64];
  for (int iv = 1; iv <= nv; iv++) {
    for (int mm = 1; mm <= ks; mm++)
      gxl[mm - 1] = ipow(A2(g->gr, iv, mm, nv), m) * A2(g->grw, iv, mm, nv);
    for (int ith = 1; ith <= g->ksq; ith++) {
      int i = iv + ith - 1;
      double qi = Fi[i];
      for (int mm = 1; mm <= ks; mm++)
        gwl[mm - 1] = gxl[mm - 1] * A3(g->qbsp, iv, mm, ith, nw, ks);
      for (int jth = 1; jth <= g->ksq; jth++) {
        int j = iv + jth - 1;
        double qj = Fj[j], s = 0.0;
        for (int mm = 1; mm <= ks; mm++)
          s += A3(g->qbsp, iv, mm, jth, nw, ks) * gwl[mm - 1];
        q = q + s * qi * qj;
      }
    }
  }
  return q;
}

/* rk: dbsr_lib_dbs.f90:3981-4022 */
double orc_rk(const orc_grid *g, const double *f1, const double *f2,
              const double *f3, const double *f4, int k) {
  const int ns = g->ns, ks = g->ks;
  size_t nb = (size_t)ns * ks;
  double *d1 = (double *)malloc(sizeof(double) * nb);
  double *d2 = (double *)malloc(sizeof(double) * nb);
  double *d3 = (double *)malloc(sizeof(double) * nb);
  double *d4 = (double *)malloc(sizeof(double) * nb);
  double *cv = (double *)malloc(sizeof(double) * nb);
  double *rkb = (double *)malloc(sizeof(double) * (size_t)ns * ns * ks * ks);
  orc_density(ns, ks, d1, f1, f3, 's');
  orc_density(ns, ks, d2, f2, f4, 's');
  orc_density(ns, ks, d3, f1 + ns, f3 + ns, 's');
  orc_density(ns, ks, d4, f2 + ns, f4 + ns, 's');
  double r = 0.0;
  orc_mrk(g, 0, k, rkb);
  orc_convol(ns, ks, ks, rkb, cv, d1, 2, 's', 's');
  r = r + orc_sum_amb(ns, ks, cv, d2, 's');
  orc_mrk(g, 1, k, rkb);
  orc_convol(ns, ks, ks, rkb, cv, d3, 2, 's', 's');
  r = r + orc_sum_amb(ns, ks, cv, d4, 's');
  orc_mrk(g, 3, k, rkb);
  orc_convol(ns, ks, ks, rkb, cv, d3, 2, 's', 's');
  r = r + orc_sum_amb(ns, ks, cv, d2, 's');
  orc_mrk(g, 2, k, rkb);
  orc_convol(ns, ks, ks, rkb, cv, d1, 2, 's', 's');
  r = r + orc_sum_amb(ns, ks, cv, d4, 's');
  free(d1); free(d2); free(d3); free(d4); free(cv); free(rkb);
  return r;
}

/* Symmetric band matrix in 's' storage (a(i,ip) holds A(i,i+ip-1)) times a
   vector, accumulated: out(m) += s * sum_j A(m,j) f(j) -- the BAV product
   (used by R_data.f90:181, S_data.f90:205) for the symmetric storage. */
static void band_sym_mv(int ns, int ks, const double *a, const double *f, double s,
                        double *out) {
  for (int m = 1; m <= ns; m++) {
    double acc = 0.0;
    for (int j = imax(1, m - ks + 1); j <= imin(ns, m + ks - 1); j++) {
      int lo = imin(m, j), ip = (m > j ? m - j : j - m) + 1;
      acc = acc + A2(a, lo, ip, ns) * f[j - 1];
    }
    out[m - 1] = out[m - 1] + s * acc;
  }
}

/* E = sum_e coef[e] R^k[e](i1,i2;i3,i4), R^k as in rk (dbsr_lib_dbs.f90:
   3981-4022), and dE/d pq(ns,2,nbf).  R^k is bilinear in the pair densities
   of the two electrons, so its derivative with respect to a function of one
   electron is the potential of the other electron's pair density (convol
   case 1 for electron 1, case 2 for electron 2) applied to the partner
   function: the direct potentials DBSR_HF builds (hf_matrix.f90:2-163).
   Orbitals are 1-based indices into pq; R tables are built once per (k,type). */
double orc_rk_energy_grad(const orc_grid *g, int n, const int *kk, const int *i1,
                          const int *i2, const int *i3, const int *i4, const double *coef,
                          const double *pq, int nbf, double *grad) {
  const int ns = g->ns, ks = g->ks;
  const size_t nb = (size_t)ns * ks, nt = (size_t)ns * ns * ks * ks;
  int kmax = 0;
  for (int e = 0; e < n; e++) kmax = imax(kmax, kk[e]);
  double **tab = (double **)calloc((size_t)(kmax + 1) * 4, sizeof(double *));
  double *d1 = (double *)malloc(sizeof(double) * nb), *d2 = (double *)malloc(sizeof(double) * nb);
  double *a1 = (double *)malloc(sizeof(double) * (size_t)ns * ns);
  double *a2 = (double *)malloc(sizeof(double) * (size_t)ns * ns);
  if (grad) memset(grad, 0, sizeof(double) * (size_t)ns * 2 * nbf);
  /* types in rk's order with the bases of electron 1 (A) and 2 (B): 1 P, 2 Q */
  static const int types[4] = {0, 1, 3, 2}, ca[4] = {1, 2, 2, 1}, cb[4] = {1, 2, 1, 2};
  double E = 0.0;
  for (int e = 0; e < n; e++) {
    const int k = kk[e];
    const double *f1 = pq + (size_t)2 * ns * (i1[e] - 1), *f2 = pq + (size_t)2 * ns * (i2[e] - 1);
    const double *f3 = pq + (size_t)2 * ns * (i3[e] - 1), *f4 = pq + (size_t)2 * ns * (i4[e] - 1);
    double r = 0.0;
    for (int q = 0; q < 4; q++) {
      const int t = types[q], A = ca[q] - 1, B = cb[q] - 1;
      double **tp = &tab[(size_t)k * 4 + t];
      if (!*tp) {
        *tp = (double *)malloc(sizeof(double) * nt);
        orc_mrk(g, t, k, *tp);
      }
      orc_density(ns, ks, d1, f1 + (size_t)ns * A, f3 + (size_t)ns * A, 's');
      orc_density(ns, ks, d2, f2 + (size_t)ns * B, f4 + (size_t)ns * B, 's');
      orc_convol(ns, ks, ks, *tp, a2, d1, 2, 's', 's');
      r = r + orc_sum_amb(ns, ks, a2, d2, 's');
      if (!grad) continue;
      orc_convol(ns, ks, ks, *tp, a1, d2, 1, 's', 's');
      const double c = coef[e];
      band_sym_mv(ns, ks, a1, f3 + (size_t)ns * A, c, grad + (size_t)2 * ns * (i1[e] - 1) + (size_t)ns * A);
      band_sym_mv(ns, ks, a1, f1 + (size_t)ns * A, c, grad + (size_t)2 * ns * (i3[e] - 1) + (size_t)ns * A);
      band_sym_mv(ns, ks, a2, f4 + (size_t)ns * B, c, grad + (size_t)2 * ns * (i2[e] - 1) + (size_t)ns * B);
      band_sym_mv(ns, ks, a2, f2 + (size_t)ns * B, c, grad + (size_t)2 * ns * (i4[e] - 1) + (size_t)ns * B);
    }
    E = E + coef[e] * r;
  }
  for (int i = 0; i < (kmax + 1) * 4; i++) free(tab[i]);
  free(tab); free(d1); free(d2); free(a1); free(a2);
  return E;
}

/* ------------------------------------------------------------------ */
/* DBSR_MAT3 matrix structures */
orc_mat *orc_mat_new(const orc_grid *g, int nbf, const double *pq,
                     const int *ipbs, int nch, const int *icc, int iicc,
                     double *hch, int mk, double *acf) {
  orc_mat *m = (orc_mat *)calloc(1, sizeof(orc_mat));
  m->g = g;
  m->nbf = nbf;
  m->pq = pq;
  m->ipbs = ipbs;
  m->nch = nch;
  m->icc = icc;
  m->iicc = iicc;
  m->hch = hch;
  m->mk = mk;
  m->acf = acf;
  m->kmax_cache = mk + 2;
  m->rcache = (double **)calloc((size_t)(m->kmax_cache + 1) * 4, sizeof(double *));
  m->scache = (double **)calloc((size_t)(m->kmax_cache + 1) * 2, sizeof(double *));
  m->eps_c = 1.0e-10;
  m->check_target = 1;
  return m;
}

void orc_mat_set_perturbers(orc_mat *m, int npert, const int *icb, int iicb,
                            const int *ibb, int iibb, double *hcp, double *hp) {
  m->npert = npert;
  m->icb = icb;
  m->iicb = iicb;
  m->ibb = ibb;
  m->iibb = iibb;
  m->hcp = hcp;
  m->hp = hp;
}

void orc_mat_set_targets(orc_mat *m, int ntarg, const int *iptar, double *htarg,
                         double *otarg, int iitar, int check_target) {
  m->ntarg = ntarg;
  m->iptar = iptar;
  m->htarg = htarg;
  m->otarg = otarg;
  m->iitar = iitar;
  m->check_target = check_target;
}

void orc_mat_set_dhl(orc_mat *m, int nkap, const int *kap_list, const double *hd,
                     const int *kbs) {
  m->nkap = nkap;
  m->kap_list = kap_list;
  m->hd = hd;
  m->kbs = kbs;
}

void orc_mat_set_eps_c(orc_mat *m, double eps_c) { m->eps_c = eps_c; }

void orc_mat_free(orc_mat *m) {
  if (!m) return;
  for (int i = 0; i < (m->kmax_cache + 1) * 4; i++) free(m->rcache[i]);
  for (int i = 0; i < (m->kmax_cache + 1) * 2; i++) free(m->scache[i]);
  free(m->rcache);
  free(m->scache);
  free(m);
}

/* cached table lookup (the irka flag, dbsr_lib_dbs.f90:2919-2925) */
static const double *rtable(orc_mat *m, int type, int k) {
  double **slot = &m->rcache[k * 4 + type];
  if (!*slot) {
    const orc_grid *g = m->g;
    *slot = (double *)malloc(sizeof(double) * (size_t)g->ns * g->ns * g->ks * g->ks);
    orc_mrk(g, type, k, *slot);
  }
  return *slot;
}
static const double *stable(orc_mat *m, int type, int k) {
  double **slot = &m->scache[k * 2 + type];
  if (!*slot) {
    const orc_grid *g = m->g;
    size_t kb = 2 * g->ks - 1;
    *slot = (double *)malloc(sizeof(double) * (size_t)g->ns * g->ns * kb * kb);
    orc_msk(g, type, k, *slot);
  }
  return *slot;
}

#define ICC(i, j) A2(m->icc, i, j, m->nch)
#define HCH(i, j, b) A3(m->hch, i, j, b, ms, ms)

/* UPDATE_HS: DBSR_MAT3/updates.f90:110-179 */
void orc_update_hs(orc_mat *m, int ich, int jch, const double *d, char sym,
                   int ii, int jj) {
  const int ns = m->g->ns, ks = m->g->ks, ms = m->g->ms;
  double *y = (double *)calloc((size_t)ns * ns, sizeof(double));
  if (sym == 's') {
    for (int jp = 1; jp <= ks; jp++)
      for (int i = 1; i <= ns - jp + 1; i++) {
        int j = i + jp - 1;
        A2(y, i, j, ns) = A2(d, i, jp, ns);
        A2(y, j, i, ns) = A2(d, i, jp, ns);
      }
  } else if (sym == 'n') {
    for (int jp = 1; jp <= ks + ks - 1; jp++) {
      int i0 = imax(1, 1 + ks - jp), i1 = imin(ns, ns + ks - jp);
      for (int i = i0; i <= i1; i++) A2(y, i, i + jp - ks, ns) = A2(d, i, jp, ns);
    }
  } else {
    memcpy(y, d, sizeof(double) * (size_t)ns * ns);
  }
  int b = ICC(ich, jch);
  int i1 = 1 + (ii - 1) * ns, j1 = 1 + (jj - 1) * ns;
  if (ich > jch) {
    for (int j = 1; j <= ns; j++)
      for (int i = 1; i <= ns; i++)
        HCH(i1 + i - 1, j1 + j - 1, b) = HCH(i1 + i - 1, j1 + j - 1, b) + A2(y, i, j, ns);
  } else if (jch > ich) {
    for (int j = 1; j <= ns; j++)
      for (int i = 1; i <= ns; i++)
        HCH(i1 + i - 1, j1 + j - 1, b) = HCH(i1 + i - 1, j1 + j - 1, b) + A2(y, j, i, ns);
  } else {
    for (size_t q = 0; q < (size_t)ns * ns; q++) y[q] = y[q] / 2.0;
    for (int j = 1; j <= ns; j++)
      for (int i = 1; i <= ns; i++)
        HCH(i1 + i - 1, j1 + j - 1, b) = HCH(i1 + i - 1, j1 + j - 1, b) + A2(y, i, j, ns);
    for (int j = 1; j <= ns; j++)
      for (int i = 1; i <= ns; i++)
        HCH(j1 + i - 1, i1 + j - 1, b) = HCH(j1 + i - 1, i1 + j - 1, b) + A2(y, j, i, ns);
  }
  free(y);
}

/* UPDATE_HX: updates.f90:79-106 */
void orc_update_hx(orc_mat *m, int ich, int jch, const double *d, double c) {
  const int ms = m->g->ms;
  int b = ICC(ich, jch);
  for (int j = 1; j <= ms; j++)
    for (int i = 1; i <= ms; i++) {
      double x = ich >= jch ? c * A2(d, i, j, ms) : c * A2(d, j, i, ms);
      HCH(i, j, b) = HCH(i, j, b) + x;
    }
}

/* hf_matrix: DBSR_HF/hf_matrix.f90:2-70 without the Breit part (mbreit = 2,
 * :91-163).  The potential matrix of orbital iorb (1-based):
 *   hfm = (qsum dhl + sum_{ii,jj = 1,2} sum_k [direct + exchange]) / qsum,
 * direct: convol case 1 ('s','s') of table mrk_aaaa(k,ii,jj) with
 *   dd = sum_j c_j density_s(p(:,jj,j), p(:,jj,j)), c_j = a(j,k), doubled
 *   for j = iorb, into quadrant (ii,ii);
 * exchange: convol case 4 of xx = sum_j b(j,k) density_x(p(:,ii,j),
 *   p(:,jj,j)) into quadrant (ii,jj);
 * both through the HF library's Update_hs (dbsr_lib_dbs.f90:4137-4193:
 * y/2 into (ii,jj), its transpose /2 into (jj,ii)).  a, b: (nbf, 0:kmax),
 * the values of a(iorb,j,k) and b(iorb,j,k) (hf_MOD_energy.f90:20-57);
 * dhl: the one-electron matrix (ms x ms) of MAT_dhl_pq, or NULL. */
static void hf_update(int ns, int ks, int ms, double *hm, int ii, int jj, const double *d,
                      char sym) {
  double *y = (double *)calloc((size_t)ns * ns, sizeof(double));
  if (sym == 's') {
    for (int jp = 1; jp <= ks; jp++)
      for (int i = 1; i <= ns - jp + 1; i++) {
        const int j = i + jp - 1;
        A2(y, i, j, ns) = A2(d, i, jp, ns);
        A2(y, j, i, ns) = A2(d, i, jp, ns);
      }
  } else if (sym == 'n') {
    for (int jp = 1; jp <= ks + ks - 1; jp++) {
      const int i0 = imax(1, 1 + ks - jp), i1 = imin(ns, ns + ks - jp);
      for (int i = i0; i <= i1; i++) A2(y, i, i + jp - ks, ns) = A2(d, i, jp, ns);
    }
  } else {
    memcpy(y, d, sizeof(double) * (size_t)ns * ns);
  }
  const int i1 = 1 + (ii - 1) * ns, j1 = 1 + (jj - 1) * ns;
  for (size_t q = 0; q < (size_t)ns * ns; q++) y[q] = y[q] / 2.0;
  for (int j = 1; j <= ns; j++)
    for (int i = 1; i <= ns; i++)
      A2(hm, i1 + i - 1, j1 + j - 1, ms) = A2(hm, i1 + i - 1, j1 + j - 1, ms) + A2(y, i, j, ns);
  for (int j = 1; j <= ns; j++)
    for (int i = 1; i <= ns; i++)
      A2(hm, j1 + i - 1, i1 + j - 1, ms) = A2(hm, j1 + i - 1, i1 + j - 1, ms) + A2(y, j, i, ns);
  free(y);
}

void orc_hf_matrix(const orc_grid *g, int nbf, const double *pq, int iorb, int kmax,
                   const double *a, const double *b, double qsum, const double *dhl,
                   double *hfm) {
  const int ns = g->ns, ks = g->ks, ms = g->ms;
  /* table of mrk_aaaa(k,ii,jj): 11 pppp, 12 pqpq, 21 qpqp, 22 qqqq */
  static const int ttype[2][2] = {{0, 2}, {3, 1}};
  double *rkb = (double *)malloc(sizeof(double) * (size_t)ns * ns * ks * ks);
  double *d = (double *)malloc(sizeof(double) * (size_t)ns * ns);
  double *dd = (double *)malloc(sizeof(double) * (size_t)ns * ns);
  double *x = (double *)malloc(sizeof(double) * (size_t)ns * ns);
  double *xx = (double *)malloc(sizeof(double) * (size_t)ns * ns);
  for (size_t q = 0; q < (size_t)ms * ms; q++) hfm[q] = dhl ? qsum * dhl[q] : 0.0;
  for (int ii = 1; ii <= 2; ii++)
    for (int jj = 1; jj <= 2; jj++)
      for (int k = 0; k <= kmax; k++) {
        orc_mrk(g, ttype[ii - 1][jj - 1], k, rkb);
        /* direct */
        int met = 0;
        memset(dd, 0, sizeof(double) * (size_t)ns * ks);
        for (int j = 1; j <= nbf; j++) {
          double c = a[(j - 1) + (size_t)nbf * k];
          if (c == 0.0) continue;
          if (j == iorb) c = c + c;
          const double *pj = pq + (size_t)2 * ns * (j - 1) + (size_t)ns * (jj - 1);
          orc_density(ns, ks, d, pj, pj, 's');
          for (size_t q = 0; q < (size_t)ns * ks; q++) dd[q] = dd[q] + c * d[q];
          met++;
        }
        if (met > 0) {
          orc_convol(ns, ks, ks, rkb, d, dd, 1, 's', 's');
          hf_update(ns, ks, ms, hfm, ii, ii, d, 's');
        }
        /* exchange */
        met = 0;
        memset(xx, 0, sizeof(double) * (size_t)ns * ns);
        for (int j = 1; j <= nbf; j++) {
          const double c = b[(j - 1) + (size_t)nbf * k];
          if (c == 0.0) continue;
          const double *p1 = pq + (size_t)2 * ns * (j - 1) + (size_t)ns * (ii - 1);
          const double *p2 = pq + (size_t)2 * ns * (j - 1) + (size_t)ns * (jj - 1);
          orc_density(ns, ks, x, p1, p2, 'x');
          for (size_t q = 0; q < (size_t)ns * ns; q++) xx[q] = xx[q] + x[q] * c;
          met++;
        }
        if (met > 0) {
          orc_convol(ns, ks, ks, rkb, x, xx, 4, 's', 's');
          hf_update(ns, ks, ms, hfm, ii, jj, x, 'x');
        }
      }
  for (size_t q = 0; q < (size_t)ms * ms; q++) hfm[q] = hfm[q] / qsum;
  free(rkb);
  free(d);
  free(dd);
  free(x);
  free(xx);
}

/* DBS_ORTH: DBSR_MAT3/dbs_orth.f90:28-84 (channel-channel blocks; the
 * perturber part needs hcp, which is not held).  For each channel ich with
 * orbitals j selected by iort(j,ich) (the reference's ipbs(j) = 0,
 * kbs(j) = kbs(i), IBORT(i,j) = 0 filter, :39-43), aa = sum_j w_j v_j^T and
 * bb = aa^T with v_j = Get_pv = (P_j; Q_j) and w_j = Get_qv = (fpbs P_j;
 * fqbs Q_j) (bpq, read_data.f90:144-145); then every block of the channel's
 * row: x - aa x (ich > jch), x - aa x then - x bb (ich = jch), x - x bb
 * (ich < jch), as full ms x ms products in the order of matmul. */
void orc_dbs_orth(orc_mat *m, const int *iort) {
  const orc_grid *g = m->g;
  const int ns = g->ns, ms = g->ms, nch = m->nch, nbf = m->nbf;
  double *aa = (double *)malloc(sizeof(double) * (size_t)ms * ms);
  double *bb = (double *)malloc(sizeof(double) * (size_t)ms * ms);
  double *cc = (double *)malloc(sizeof(double) * (size_t)ms * ms);
  double *vv = (double *)malloc(sizeof(double) * ms);
  double *ww = (double *)malloc(sizeof(double) * ms);
  for (int ich = 1; ich <= nch; ich++) {
    int nort = 0;
    memset(aa, 0, sizeof(double) * (size_t)ms * ms);
    memset(bb, 0, sizeof(double) * (size_t)ms * ms);
    for (int j = 1; j <= nbf; j++) {
      if (!iort[(j - 1) + (size_t)nbf * (ich - 1)]) continue;
      if (m->ipbs[j - 1] > 0) continue;
      nort++;
      const double *p = m->pq + (size_t)2 * ns * (j - 1), *q = p + ns;
      for (int i = 1; i <= ns; i++) {
        vv[i - 1] = p[i - 1];
        vv[ns + i - 1] = q[i - 1];
      }
      for (int i = 1; i <= ns; i++) {
        double sp = 0.0, sq = 0.0;
        for (int k = 1; k <= ns; k++) {
          sp = sp + A2(g->fpbs, i, k, ns) * p[k - 1];
          sq = sq + A2(g->fqbs, i, k, ns) * q[k - 1];
        }
        ww[i - 1] = sp;
        ww[ns + i - 1] = sq;
      }
      for (int jj = 1; jj <= ms; jj++)
        for (int ii = 1; ii <= ms; ii++) {
          const double S = ww[ii - 1] * vv[jj - 1];
          A2(aa, ii, jj, ms) = A2(aa, ii, jj, ms) + S;
          A2(bb, jj, ii, ms) = A2(bb, jj, ii, ms) + S;
        }
    }
    if (nort == 0) continue;
    for (int jch = 1; jch <= nch; jch++) {
      const int b = ICC(ich, jch);
      if (b == 0) continue;
      for (int pass = 0; pass < 2; pass++) {
        /* pass 0: x - aa x (ich >= jch); pass 1: x - x bb (ich <= jch) */
        if (pass == 0 && ich < jch) continue;
        if (pass == 1 && ich > jch) continue;
        for (int j = 1; j <= ms; j++)
          for (int i = 1; i <= ms; i++) {
            double s = 0.0;
            if (pass == 0)
              for (int k = 1; k <= ms; k++) s = s + A2(aa, i, k, ms) * HCH(k, j, b);
            else
              for (int k = 1; k <= ms; k++) s = s + HCH(i, k, b) * A2(bb, k, j, ms);
            A2(cc, i, j, ms) = s;
          }
        for (int j = 1; j <= ms; j++)
          for (int i = 1; i <= ms; i++) HCH(i, j, b) = HCH(i, j, b) - A2(cc, i, j, ms);
      }
    }
  }
  free(aa);
  free(bb);
  free(cc);
  free(vv);
  free(ww);
}

/* UPDATE_HW: updates.f90:183-216 */
void orc_update_hw(orc_mat *m, int ich, int jch, const double *v,
                   const double *w, double c) {
  const int ms = m->g->ms;
  int b = ICC(ich, jch);
  for (int j = 1; j <= ms; j++)
    for (int i = 1; i <= ms; i++) {
      double xx;
      if (ich > jch)
        xx = c * (v[i - 1] * w[j - 1]);
      else if (jch > ich)
        xx = c * (v[j - 1] * w[i - 1]);
      else
        xx = (c / 2.0) * (v[i - 1] * w[j - 1] + v[j - 1] * w[i - 1]);
      HCH(i, j, b) = HCH(i, j, b) + xx;
    }
}

/* UPDATE_ACF: updates.f90:268-292 */
static void update_acf(orc_mat *m, int k, int ich, int jch, double c) {
  int b = ICC(ich, jch);
  A2(m->acf, b, k + 1, m->iicc) = A2(m->acf, b, k + 1, m->iicc) + c;
}

/* V_ch restatement (Get_v_ch is not in the reference snapshot): the
 * B-spline overlap vector of a bound orbital, <B_i|P_b> and <B_i|Q_b>. */
void orc_v_ch(const orc_grid *g, const double *pq_b, double *v) {
  const int ns = g->ns;
  for (int i = 1; i <= ns; i++) {
    double sp = 0.0, sq = 0.0;
    for (int j = 1; j <= ns; j++) {
      sp += A2(g->fpbs, i, j, ns) * pq_b[j - 1];
      sq += A2(g->fqbs, i, j, ns) * pq_b[ns + j - 1];
    }
    v[i - 1] = sp;
    v[ns + i - 1] = sq;
  }
}

#define PQ(orb, comp) (m->pq + (size_t)ns * ((comp)-1) + (size_t)2 * ns * ((orb)-1))

/* KBORT restatement (not in the reference snapshot): the index of the
 * overlap vector V_ch of channel orbital io1 with bound orbital io2 is io2
 * (V_ch is the overlap vector of io2, orc_v_ch); 0 when io1 is not a
 * channel orbital or an index is out of range. */
static int kbort(const orc_mat *m, int io1, int io2) {
  if (io1 < 1 || io1 > m->nbf || io2 < 1 || io2 > m->nbf) return 0;
  const int ich = m->ipbs[io1 - 1];
  if (ich < 1 || ich > m->nch) return 0;
  return io2;
}

/* the UPDATE_* bound checks (updates.f90:91-94,153-159,196-199): -4 */
static int block_of(const orc_mat *m, int ich, int jch) {
  if (ich < 1 || jch < 1 || ich > m->nch || jch > m->nch) return 0;
  int b = ICC(ich, jch);
  return (b >= 1 && b <= m->iicc) ? b : 0;
}
static int update_hw_checked(orc_mat *m, int ich, int jch, const double *v,
                             const double *w, double c) {
  if (!block_of(m, ich, jch)) return -4;
  orc_update_hw(m, ich, jch, v, w, c);
  return 0;
}
static int update_hx_checked(orc_mat *m, int ich, int jch, const double *d, double c) {
  if (!block_of(m, ich, jch)) return -4;
  orc_update_hx(m, ich, jch, d, c);
  return 0;
}

/* UPDATE_HV: updates.f90:220-242 */
int orc_update_hv(orc_mat *m, int ich, int ip, const double *v, double c) {
  const int ms = m->g->ms;
  if (ich < 1 || ich > m->nch || ip < 1 || ip > m->npert) return -4;
  int i = A2(m->icb, ich, ip, m->nch);
  if (i < 1 || i > m->iicb) return -4;
  for (int r = 1; r <= ms; r++) A2(m->hcp, r, i, ms) = A2(m->hcp, r, i, ms) + c * v[r - 1];
  return 0;
}

/* UPDATE_HB: updates.f90:245-264 */
int orc_update_hb(orc_mat *m, int ic, int jc, double c) {
  if (ic > m->npert || jc > m->npert || ic <= 0 || jc <= 0) return -4;
  int i = A2(m->ibb, ic, jc, m->npert);
  if (i < 1 || i > m->iibb) return -4;
  m->hp[i - 1] = m->hp[i - 1] + c;
  return 0;
}

/* Target_h: target_subs.f90:2-31 (nothing when no targets are given) */
static int target_h(orc_mat *m, int ich, int jch, double c, double cc) {
  if (m->ntarg <= 0) return 0;
  if (ich < 0 || jch < 0 || ich > m->nch || jch > m->nch) return -4;
  if (ich < 1 || jch < 1 || ICC(ich, jch) == 0) return 0;
  int it = m->iptar[ich - 1], jt = m->iptar[jch - 1];
  int i = it > jt ? it : jt, j = it > jt ? jt : it;
  if (j < 1 || i > m->ntarg) return -4;
  int ij = (i - 1) * i / 2 + j;
  m->htarg[ij - 1] = m->htarg[ij - 1] + c;
  m->otarg[ij - 1] = m->otarg[ij - 1] + cc;
  return 0;
}

/* BAV restatement: band matrix (storage sym) times vector, from the right
 * (dir 'r': v = A b) or the left ('l': v = A^T b); the band entries are
 * visited column of the band by column (jp outer), rows inner. */
void orc_bav(int ns, int ks, const double *a, const double *b, double *v,
             char sym, char dir) {
  for (int i = 1; i <= ns; i++) v[i - 1] = 0.0;
  if (sym == 's') {
    for (int jp = 1; jp <= ks; jp++)
      for (int i = 1; i <= ns - jp + 1; i++) {
        int j = i + jp - 1;
        double x = A2(a, i, jp, ns);
        v[i - 1] = v[i - 1] + x * b[j - 1];
        if (jp > 1) v[j - 1] = v[j - 1] + x * b[i - 1];
      }
  } else {
    for (int jp = 1; jp <= 2 * ks - 1; jp++) {
      int i0 = imax(1, 1 + ks - jp), i1 = imin(ns, ns + ks - jp);
      for (int i = i0; i <= i1; i++) {
        int j = i + jp - ks;
        double x = A2(a, i, jp, ns);
        if (dir == 'l')
          v[j - 1] = v[j - 1] + x * b[i - 1];
        else
          v[i - 1] = v[i - 1] + x * b[j - 1];
      }
    }
  }
}

/* Structures 1.x (bound-bound integral times overlap factors) of R_data
 * (R_data.f90:92-163) and S_data (S_data.f90:115-187): the routing of
 * C = S * cdata by the signs of ic = -k3, jc = -k4. */
static int route_bound(orc_mat *m, int k3, int k4, double C, double *vv, double *ww) {
  const orc_grid *g = m->g;
  const int ns = g->ns;
  int ic = -k3, jc = -k4, io = -ic, jo = -jc;
  if (ic > 0 && jc > 0) return orc_update_hb(m, ic, jc, C);
  if (ic < 0 && jc > 0) {
    int o1 = io / ORC_IBO, o2 = io % ORC_IBO;
    if (!kbort(m, o1, o2)) return -4;
    orc_v_ch(g, PQ(o2, 1), vv);
    return orc_update_hv(m, m->ipbs[o1 - 1], jc, vv, C);
  }
  if (ic < 0 && jc < 0) {
    int o1 = io / ORC_IBO, o2 = io % ORC_IBO, p1 = jo / ORC_IBO, p2 = jo % ORC_IBO;
    if (!kbort(m, o1, o2) || !kbort(m, p1, p2)) return -4;
    orc_v_ch(g, PQ(o2, 1), vv);
    orc_v_ch(g, PQ(p2, 1), ww);
    return update_hw_checked(m, m->ipbs[o1 - 1], m->ipbs[p1 - 1], vv, ww, C);
  }
  if (ic < 0 && jc == 0) {
    int o1 = io / ORC_IBO, o2 = io % ORC_IBO;
    if (o1 < 1 || o1 > m->nbf || o2 < 1 || o2 > m->nbf) return -4;
    int ich = m->ipbs[o1 - 1], jch = m->ipbs[o2 - 1];
    int rc = target_h(m, ich, jch, C, 0.0);
    if (rc) return rc;
    if (m->iitar > 0 && ich != jch) return update_hx_checked(m, ich, jch, g->fppqq, C);
    return 0;
  }
  return -1;
}

/* Structures 2.x (channel orbital in one position of the integral) of
 * R_data (R_data.f90:167-211) and S_data (S_data.f90:191-236): vv carries
 * the potential-times-orbital vector in its P or Q half; io = k4 > 0 gives
 * UPDATE_HW with V_ch, io < 0 UPDATE_HV. */
static int route_channel(orc_mat *m, int ich, int io, double C, const double *vv, double *ww) {
  const orc_grid *g = m->g;
  const int ns = g->ns;
  if (io > 0) {
    int o1 = io / ORC_IBO, o2 = io % ORC_IBO;
    if (!kbort(m, o1, o2)) return -4;
    orc_v_ch(g, PQ(o2, 1), ww);
    return update_hw_checked(m, ich, m->ipbs[o1 - 1], vv, ww, C);
  }
  if (io < 0) return orc_update_hv(m, ich, -io, vv, C);
  return -1;
}

/* itypes 1 and 2 of one table (R or S): density/convol of the bound pair
 * K1, then SUM_AmB with the density of K2 (itype 1) or BAV with orbital K2
 * (itype 2, placed into the half of component ipv). */
static int bound_structures(orc_mat *m, int itype, const double *rkb, int kb, char sym,
                            int in, int ip1, int ip2, int jp1, int jp2, int ipo, int ipv,
                            char sym_v, int ncdata, const int *ipt, const int *k1,
                            const int *k2, const int *k3, const int *k4,
                            const double *cdata) {
  const orc_grid *g = m->g;
  const int ns = g->ns, ks = g->ks, ms = g->ms;
  size_t nn = (size_t)ns * ns;
  double *d = (double *)calloc(nn, sizeof(double));
  double *xx = (double *)calloc(nn, sizeof(double));
  double *dd = (double *)calloc(nn, sizeof(double));
  double *v = (double *)calloc(ns, sizeof(double));
  double *vv = (double *)calloc(ms, sizeof(double));
  double *ww = (double *)calloc(ms, sizeof(double));
  int rc = 0, iii = 0, jjj = 0;
  double S = 0.0;
  for (int j = 1; j <= ncdata && !rc; j++) {
    int i = ipt[j - 1];
    if (itype == 1) {
      int K1 = k1[i - 1], K2 = k2[i - 1];
      int i1 = K1 / ORC_IBO, i2 = K1 % ORC_IBO, j1 = K2 / ORC_IBO, j2 = K2 % ORC_IBO;
      if (i1 < 1 || i1 > m->nbf || i2 < 1 || i2 > m->nbf || j1 < 1 || j1 > m->nbf ||
          j2 < 1 || j2 > m->nbf) { rc = -4; break; }
      if (K1 != iii) {
        orc_density(ns, ks, d, PQ(i1, ip1), PQ(i2, ip2), sym);
        orc_convol(ns, ks, kb, rkb, xx, d, in, sym, sym);
      }
      if (K2 != jjj) orc_density(ns, ks, dd, PQ(j1, jp1), PQ(j2, jp2), sym);
      if (K1 != iii || K2 != jjj) S = orc_sum_amb(ns, ks, xx, dd, sym);
      iii = K1;
      jjj = K2;
      rc = route_bound(m, k3[i - 1], k4[i - 1], S * cdata[i - 1], vv, ww);
    } else {
      int jj = k1[i - 1], ii = k2[i - 1], ich = k3[i - 1], io = k4[i - 1];
      int j1 = jj / ORC_IBO, j2 = jj % ORC_IBO;
      if (j1 < 1 || j1 > m->nbf || j2 < 1 || j2 > m->nbf || ii < 1 || ii > m->nbf) {
        rc = -4;
        break;
      }
      if (jj != jjj || ii != iii) {
        if (jj != jjj) {
          orc_density(ns, ks, dd, PQ(j1, jp1), PQ(j2, jp2), sym);
          orc_convol(ns, ks, kb, rkb, xx, dd, in, sym, sym);
          jjj = jj;
        }
        orc_bav(ns, ks, xx, PQ(ii, ipo), v, sym, sym_v);
        iii = ii;
      }
      for (int r = 0; r < ms; r++) vv[r] = 0.0;
      for (int r = 0; r < ns; r++) vv[(size_t)ns * (ipv - 1) + r] = v[r];
      rc = route_channel(m, ich, io, cdata[i - 1], vv, ww);
    }
  }
  free(d); free(xx); free(dd); free(v); free(vv); free(ww);
  return rc;
}

/* R_data itype 3 (direct) and 4 (exchange): DBSR_MAT3/R_data.f90:56-86,
 * 214-277.  QUADR_PQ (not in the reference snapshot) is restated as the
 * component of quadr selected by atype (P for atype 0, Q for atype 1). */
static int r_data(orc_mat *m, int itype, int kpol, int btype, int ncdata,
                  const int *ipt, const int *k1, const int *k2, const int *k3,
                  const int *k4, const double *cdata) {
  const orc_grid *g = m->g;
  const int ns = g->ns, ks = g->ks;
  int ip1, ip2, jp1, jp2, in;
  char sym_d, sym_r;
  if (itype == 3) { in = 1; sym_d = 's'; sym_r = 's'; }
  else if (itype == 4) { in = 3; sym_d = 'x'; sym_r = 'x'; }
  else if (itype == 1 || itype == 2) { in = 3 - itype; sym_d = 's'; sym_r = 's'; }
  else return -2;
  int atype = btype;
  switch (atype) {
    case 0: ip1 = 1; ip2 = 1; jp1 = 1; jp2 = 1; break;
    case 1: ip1 = 2; ip2 = 2; jp1 = 2; jp2 = 2; break;
    case 2: ip1 = 1; ip2 = 1; jp1 = 2; jp2 = 2;
      if (itype == 4) { ip1 = 1; ip2 = 2; jp1 = 1; jp2 = 2; }
      break;
    default: ip1 = 2; ip2 = 2; jp1 = 1; jp2 = 1;
      if (itype == 4) { ip1 = 2; ip2 = 1; jp1 = 2; jp2 = 1; }
      break;
  }
  const double *rkb = rtable(m, atype, kpol);
  if (itype <= 2)  /* R_data.f90:92-211; BAV with orbital K2 on ip1, into half ip2 */
    return bound_structures(m, itype, rkb, ks, 's', in, ip1, ip2, jp1, jp2, ip1, ip2, 'r',
                            ncdata, ipt, k1, k2, k3, k4, cdata);
  (void)sym_r;
  size_t nn = (size_t)ns * ns;
  double *xx = (double *)calloc(nn, sizeof(double));
  double *dd = (double *)calloc(nn, sizeof(double));
  double CA = 0.0;
  for (int j = 1; j <= ncdata; j++) {
    int i = ipt[j - 1];
    int j1 = k2[i - 1], j2 = k3[i - 1];
    orc_density(ns, ks, dd, PQ(j1, jp1), PQ(j2, jp2), sym_d);
    int ncol = sym_d == 's' ? ks : ns;
    for (size_t q = 0; q < (size_t)ns * ncol; q++) xx[q] = xx[q] + cdata[i - 1] * dd[q];
    if (itype == 3 && atype <= 1) {
      double S = quadr_part(g, PQ(j1, 1), PQ(j2, 1), kpol, atype);
      CA = CA + cdata[i - 1] * S;
    }
    int last = 1;
    if (j < ncdata && k1[i - 1] == k1[ipt[j] - 1]) last = 0;
    if (!last) continue;
    orc_convol(ns, ks, ks, rkb, dd, xx, in, 's', 's');
    int ich = k1[i - 1] / ORC_IBO, jch = k1[i - 1] % ORC_IBO;
    orc_update_hs(m, ich, jch, dd, sym_r, ip1, ip2);
    if (itype == 3 && atype <= 1) update_acf(m, kpol, ich, jch, CA);
    memset(xx, 0, nn * sizeof(double));
    CA = 0.0;
  }
  free(xx);
  free(dd);
  return 0;
}

/* S_data itypes 6-9: DBSR_MAT3/S_data.f90:67-113, 240-274, with the
 * contraction taken with convol_sk semantics (the S^k table). */
static int s_data(orc_mat *m, int ktype, int kpol, int ncdata, const int *ipt,
                  const int *k1, const int *k2, const int *k3, const int *k4,
                  const double *cdata) {
  const orc_grid *g = m->g;
  const int ns = g->ns, ks = g->ks;
  int atype = ktype / 10, itype = ktype % 10;
  int ip1, ip2, jp1, jp2, in;
  if (itype < 1 || itype > 9 || atype < 0 || atype > 1) return -2;
  if (itype <= 5) {  /* S_data.f90:74-97 (itypes 1-5), 115-236 */
    char sym_v = 'r';
    if (atype == 0) {
      switch (itype) {
        case 1: ip1 = 1; ip2 = 2; jp1 = 1; jp2 = 2; in = 2; break;
        case 2: ip1 = 1; ip2 = 2; jp1 = 1; jp2 = 2; in = 1; sym_v = 'r'; break;
        case 3: ip1 = 1; ip2 = 2; jp1 = 1; jp2 = 2; in = 2; sym_v = 'r'; break;
        case 4: ip1 = 2; ip2 = 1; jp1 = 1; jp2 = 2; in = 1; sym_v = 'l'; break;
        default: ip1 = 2; ip2 = 1; jp1 = 1; jp2 = 2; in = 2; sym_v = 'l'; break;
      }
    } else {
      switch (itype) {
        case 1: ip1 = 1; ip2 = 2; jp1 = 2; jp2 = 1; in = 2; break;
        case 2: ip1 = 1; ip2 = 2; jp1 = 2; jp2 = 1; in = 1; sym_v = 'r'; break;
        case 3: ip1 = 2; ip2 = 1; jp1 = 1; jp2 = 2; in = 2; sym_v = 'r'; break;
        case 4: ip1 = 2; ip2 = 1; jp1 = 2; jp2 = 1; in = 1; sym_v = 'l'; break;
        default: ip1 = 1; ip2 = 2; jp1 = 1; jp2 = 2; in = 2; sym_v = 'l'; break;
      }
    }
    const double *rkb = stable(m, atype, kpol);
    /* BAV with orbital K2 on component ip2, into half ip2 (S_data.f90:205-211) */
    return bound_structures(m, itype == 1 ? 1 : 2, rkb, 2 * ks - 1, 'n', in, ip1, ip2, jp1,
                            jp2, ip2, ip2, sym_v, ncdata, ipt, k1, k2, k3, k4, cdata);
  }
  if (atype == 0) {
    switch (itype) {
      case 6: ip1 = 1; ip2 = 2; jp1 = 1; jp2 = 2; in = 1; break;
      case 7: ip1 = 1; ip2 = 2; jp1 = 1; jp2 = 2; in = 2; break;
      case 8: ip1 = 1; ip2 = 2; jp1 = 2; jp2 = 1; in = 3; break;
      default: ip1 = 2; ip2 = 1; jp1 = 1; jp2 = 2; in = 4; break;
    }
  } else {
    switch (itype) {
      case 6: ip1 = 1; ip2 = 2; jp1 = 2; jp2 = 1; in = 1; break;
      case 7: ip1 = 2; ip2 = 1; jp1 = 1; jp2 = 2; in = 2; break;
      case 8: ip1 = 1; ip2 = 1; jp1 = 2; jp2 = 2; in = 3; break;
      default: ip1 = 2; ip2 = 2; jp1 = 1; jp2 = 1; in = 4; break;
    }
  }
  char sym_d = in <= 2 ? 'n' : 'x', sym_r = sym_d;
  const double *rkb = stable(m, atype, kpol);
  size_t nn = (size_t)ns * ns;
  double *xx = (double *)calloc(nn, sizeof(double));
  double *dd = (double *)calloc(nn, sizeof(double));
  for (int j = 1; j <= ncdata; j++) {
    int i = ipt[j - 1];
    int i1 = k2[i - 1], j1 = k3[i - 1];
    orc_density(ns, ks, dd, PQ(i1, jp1), PQ(j1, jp2), sym_d);
    int ncol = sym_d == 'n' ? 2 * ks - 1 : ns;
    for (size_t q = 0; q < (size_t)ns * ncol; q++) xx[q] = xx[q] + cdata[i - 1] * dd[q];
    int last = 1;
    if (j < ncdata && k1[i - 1] == k1[ipt[j] - 1]) last = 0;
    if (!last) continue;
    orc_convol(ns, ks, 2 * ks - 1, rkb, dd, xx, in, 'n', 'n');
    int ich = k1[i - 1] / ORC_IBO, jch = k1[i - 1] % ORC_IBO;
    orc_update_hs(m, ich, jch, dd, sym_r, ip1, ip2);
    memset(xx, 0, nn * sizeof(double));
  }
  free(xx);
  free(dd);
  return 0;
}

/* O_data: DBSR_MAT3/O_data.f90:2-90.  itype 1 <ic|jc> (UPDATE_HB), 2
 * <i|.> jc (UPDATE_HV), 3 <i|.><.|j> (UPDATE_HW), 4 <i|j> (Target_h, and
 * UPDATE_HX with fppqq for iitar > 1 and ich != jch); coefficients below
 * eps_c are skipped. */
static int o_data(orc_mat *m, int itype, int ncdata, const int *ipt,
                  const int *k1, const int *k2, const double *cdata) {
  const orc_grid *g = m->g;
  const int ns = g->ns, ms = g->ms;
  if (itype < 1 || itype > 4) return -2;
  double *v = (double *)malloc(sizeof(double) * ms);
  double *w = (double *)malloc(sizeof(double) * ms);
  int rc = 0;
  for (int j = 1; j <= ncdata && !rc; j++) {
    int i = ipt[j - 1];
    double C = cdata[i - 1];
    if (fabs(C) < m->eps_c) continue;
    if (itype == 1) {
      rc = orc_update_hb(m, k1[i - 1], k2[i - 1], C);
    } else if (itype == 2) {
      int io = k1[i - 1], jc = k2[i - 1];
      int i1 = io / ORC_IBO, i2 = io % ORC_IBO;
      if (!kbort(m, i1, i2)) { rc = -4; break; }
      orc_v_ch(g, PQ(i2, 1), v);
      rc = orc_update_hv(m, m->ipbs[i1 - 1], jc, v, C);
    } else if (itype == 3) {
      int io = k1[i - 1], jo = k2[i - 1];
      int i1 = io / ORC_IBO, i2 = io % ORC_IBO;
      int j1 = jo / ORC_IBO, j2 = jo % ORC_IBO;
      if (!kbort(m, i1, i2) || !kbort(m, j1, j2)) { rc = -4; break; }
      orc_v_ch(g, PQ(i2, 1), v);
      orc_v_ch(g, PQ(j2, 1), w);
      rc = update_hw_checked(m, m->ipbs[i1 - 1], m->ipbs[j1 - 1], v, w, C);
    } else {
      int io = k1[i - 1], i1 = io / ORC_IBO, i2 = io % ORC_IBO;
      if (i1 < 1 || i1 > m->nbf || i2 < 1 || i2 > m->nbf) { rc = -4; break; }
      int ich = m->ipbs[i1 - 1], jch = m->ipbs[i2 - 1];
      if ((rc = target_h(m, ich, jch, 0.0, C))) break;
      if (m->iitar > 1 && ich != jch) rc = update_hx_checked(m, ich, jch, g->fppqq, C);
    }
  }
  free(v);
  free(w);
  (void)ns;
  return rc;
}

/* L_data: DBSR_MAT3/L_data.f90:2-145.  Lval and Gen_Lvec (module dhl_core,
 * not in the reference snapshot) are restated with the caller's one-electron
 * matrices: Lval(i,j) = p_i^T hd(kappa_i) p_j and Gen_Lvec(i) = hd(kappa_i)
 * p_i with p = (P; Q) of length ms.  Coefficients below eps_c are skipped. */
static int kap_index(const orc_mat *m, int kappa) {
  for (int k = 1; k <= m->nkap; k++)
    if (m->kap_list[k - 1] == kappa) return k;
  return 0;
}
static const double *hd_of(const orc_mat *m, int orb) {
  if (!m->hd || !m->kbs || orb < 1 || orb > m->nbf) return NULL;
  int k = kap_index(m, m->kbs[orb - 1]);
  if (!k) return NULL;
  const int ms = m->g->ms;
  return m->hd + (size_t)ms * ms * (k - 1);
}
static void gen_lvec(const orc_mat *m, const double *hd, int orb, double *v) {
  const int ns = m->g->ns, ms = m->g->ms;
  const double *p = PQ(orb, 1);  /* P then Q: the ms-vector (P; Q) */
  for (int i = 1; i <= ms; i++) {
    double s = 0.0;
    for (int k = 1; k <= ms; k++) s = s + A2(hd, i, k, ms) * p[k - 1];
    v[i - 1] = s;
  }
}
static int l_data(orc_mat *m, int itype, int ncdata, const int *ipt, const int *k1,
                  const int *k2, const int *k3, const int *k4, const double *cdata) {
  const orc_grid *g = m->g;
  const int ns = g->ns, ms = g->ms;
  if (itype < 1 || itype > 3) return -2;
  double *v = (double *)malloc(sizeof(double) * ms);
  double *w = (double *)malloc(sizeof(double) * ms);
  int rc = 0;
  for (int j = 1; j <= ncdata && !rc; j++) {
    int i = ipt[j - 1];
    double C = cdata[i - 1];
    if (fabs(C) < m->eps_c) continue;
    if (itype == 1) {
      int i1 = k1[i - 1], i2 = k2[i - 1];
      const double *hd = hd_of(m, i1);
      if (!hd || i2 < 1 || i2 > m->nbf) { rc = -4; break; }
      gen_lvec(m, hd, i2, v);
      const double *p = PQ(i1, 1);
      double S = 0.0;
      for (int k = 1; k <= ms; k++) S = S + p[k - 1] * v[k - 1];
      C = C * S;
      int ic = k3[i - 1], jc = k4[i - 1];
      if (ic > 0 && jc > 0) {
        rc = orc_update_hb(m, ic, jc, C);
      } else if (ic < 0 && jc > 0) {
        int io = -ic, o1 = io / ORC_IBO, o2 = io % ORC_IBO;
        if (!kbort(m, o1, o2)) { rc = -4; break; }
        orc_v_ch(g, PQ(o2, 1), v);
        rc = orc_update_hv(m, m->ipbs[o1 - 1], jc, v, C);
      } else if (ic < 0 && jc < 0) {
        int io = -ic, o1 = io / ORC_IBO, o2 = io % ORC_IBO;
        int jo = -jc, p1 = jo / ORC_IBO, p2 = jo % ORC_IBO;
        if (!kbort(m, o1, o2) || !kbort(m, p1, p2)) { rc = -4; break; }
        orc_v_ch(g, PQ(o2, 1), v);
        orc_v_ch(g, PQ(p2, 1), w);
        rc = update_hw_checked(m, m->ipbs[o1 - 1], m->ipbs[p1 - 1], v, w, C);
      } else if (ic < 0 && jc == 0) {
        int io = -ic, o1 = io / ORC_IBO, o2 = io % ORC_IBO;
        if (o1 < 1 || o1 > m->nbf || o2 < 1 || o2 > m->nbf) { rc = -4; break; }
        int ich = m->ipbs[o1 - 1], jch = m->ipbs[o2 - 1];
        if (m->iitar > 0 && ich != jch && (rc = update_hx_checked(m, ich, jch, g->fppqq, C)))
          break;
        rc = target_h(m, ich, jch, C, 0.0);
      } else {
        rc = -1;
      }
    } else if (itype == 2) {
      int i1 = k1[i - 1], ich = k2[i - 1], jc = k3[i - 1];
      const double *hd = hd_of(m, i1);
      if (!hd) { rc = -4; break; }
      gen_lvec(m, hd, i1, v);
      if (jc > 0) {
        rc = orc_update_hv(m, ich, jc, v, C);
      } else if (jc < 0) {
        int jo = -jc, p1 = jo / ORC_IBO, p2 = jo % ORC_IBO;
        if (!kbort(m, p1, p2)) { rc = -4; break; }
        orc_v_ch(g, PQ(p2, 1), w);
        rc = update_hw_checked(m, ich, m->ipbs[p1 - 1], v, w, C);
      } else {
        rc = -1;
      }
    } else {
      int i1 = k1[i - 1], j1 = k2[i - 1];
      if (i1 < 1 || i1 > m->nbf || j1 < 1 || j1 > m->nbf || !m->kbs) { rc = -4; break; }
      int ich = m->ipbs[i1 - 1], jch = m->ipbs[j1 - 1];
      if (m->kbs[i1 - 1] != m->kbs[j1 - 1]) { rc = -1; break; }
      const double *hd = hd_of(m, i1);
      if (!hd) { rc = -4; break; }
      if (ich == jch || m->iitar > 1)
        rc = update_hx_checked(m, ich, jch, hd, C);
      else if (m->check_target == 1)
        rc = target_h(m, ich, jch, 0.0, C);
    }
  }
  free(v);
  free(w);
  (void)ns;
  return rc;
}

/* Gen_matrix: DBSR_MAT3/gen_matrix.f90:2-17 */
int orc_gen_matrix(orc_mat *m, int icase, int itype, int kpol, int ncdata,
                   const int *ipt, const int *k1, const int *k2,
                   const int *k3, const int *k4, const double *cdata) {
  if (ncdata == 0) return 0;
  if (kpol < 0 || kpol > m->kmax_cache) return -3;
  switch (icase) {
    case 0:
      return o_data(m, itype, ncdata, ipt, k1, k2, cdata);
    case 1:
      return l_data(m, itype, ncdata, ipt, k1, k2, k3, k4, cdata);
    case 2:
      for (int bt = 0; bt <= 3; bt++) {
        int rc = r_data(m, itype, kpol, bt, ncdata, ipt, k1, k2, k3, k4, cdata);
        if (rc) return rc;
      }
      return 0;
    case 3:
      return s_data(m, itype, kpol, ncdata, ipt, k1, k2, k3, k4, cdata);
    default:
      return -1;
  }
}

/* ------------------------------------------------------------------ */
/* Add_cdata semantics (MOD_c_data.f90:177-236) for a whole raw list:
 * entries are ordered by (K1,K2,K3,K4) and equal keys are summed in the
 * order they arrive.  A stable merge sort keeps arrival order among equal
 * keys, so the sequential sum below adds the coefficients exactly as the
 * insertion routine does. */
typedef struct {
  int k1, k2, k3, k4, pos;
} key5;
static int keycmp(const key5 *a, const key5 *b) {
  if (a->k1 != b->k1) return a->k1 < b->k1 ? -1 : 1;
  if (a->k2 != b->k2) return a->k2 < b->k2 ? -1 : 1;
  if (a->k3 != b->k3) return a->k3 < b->k3 ? -1 : 1;
  if (a->k4 != b->k4) return a->k4 < b->k4 ? -1 : 1;
  return 0;
}
static void msort(key5 *a, key5 *tmp, int n) {
  if (n < 2) return;
  int h = n / 2;
  msort(a, tmp, h);
  msort(a + h, tmp, n - h);
  int i = 0, j = h, o = 0;
  while (i < h && j < n) tmp[o++] = (keycmp(&a[j], &a[i]) < 0) ? a[j++] : a[i++];
  while (i < h) tmp[o++] = a[i++];
  while (j < n) tmp[o++] = a[j++];
  memcpy(a, tmp, sizeof(key5) * n);
}
int orc_sort_merge(int n, const int *k1, const int *k2, const int *k3,
                   const int *k4, const double *c, int *o1, int *o2,
                   int *o3, int *o4, double *oc) {
  key5 *a = (key5 *)malloc(sizeof(key5) * (n > 0 ? n : 1));
  key5 *tmp = (key5 *)malloc(sizeof(key5) * (n > 0 ? n : 1));
  for (int i = 0; i < n; i++) {
    a[i].k1 = k1[i]; a[i].k2 = k2[i]; a[i].k3 = k3[i]; a[i].k4 = k4[i];
    a[i].pos = i;
  }
  msort(a, tmp, n);
  int u = -1;
  for (int i = 0; i < n; i++) {
    if (u >= 0 && a[i].k1 == o1[u] && a[i].k2 == o2[u] && a[i].k3 == o3[u] &&
        a[i].k4 == o4[u]) {
      oc[u] = oc[u] + c[a[i].pos];
    } else {
      u++;
      o1[u] = a[i].k1; o2[u] = a[i].k2; o3[u] = a[i].k3; o4[u] = a[i].k4;
      oc[u] = c[a[i].pos];
    }
  }
  free(a);
  free(tmp);
  return u + 1;
}


/* hf_matrix_breit: DBSR_HF/hf_matrix.f90:91-163, the Breit part of the
 * potential matrix of orbital iorb, added into hfm (hf_matrix adds it
 * before the division by qsum, :64-66).  For itype 0 (S^k ppqq) and 1
 * (pqqp), k = 0..kmax and int = 1..4 (storage 'n','n','x','x'):
 *   xx = sum over the rk4 entries ik with kr1 = k + 1000 itype and
 *        i = kr3 (jnt = kr2, j = kr4) or i = kr4 (jnt = kint(kr2), j = kr3,
 *        kint = 2,1,4,3), jnt = int, of crk(ik) density(p(jp1,j), p(jp2,j))
 *   convol_sk case int of xx with the S^k table, into quadrant (ip1,ip2)
 *   through the HF library's Update_hs (half and half transposed),
 * with ip1,ip2,jp1,jp2 of :123-138. */
void orc_hf_matrix_breit(const orc_grid *g, int nbf, const double *pq, int iorb, int kmax,
                         int nrk, const int *kr1, const int *kr2, const int *kr3,
                         const int *kr4, const double *crk, double *hfm) {
  const int ns = g->ns, ks = g->ks, ms = g->ms, kb = 2 * ks - 1;
  static const char sym_int[4] = {'n', 'n', 'x', 'x'};
  static const int kint[4] = {2, 1, 4, 3};
  static const int ipt[2][4][4] = {
      {{1, 2, 1, 2}, {1, 2, 1, 2}, {1, 2, 2, 1}, {2, 1, 1, 2}},
      {{1, 2, 2, 1}, {2, 1, 1, 2}, {1, 1, 2, 2}, {2, 2, 1, 1}}};
  double *rkb = (double *)malloc(sizeof(double) * (size_t)ns * ns * kb * kb);
  double *x = (double *)calloc((size_t)ns * ns, sizeof(double));
  double *xx = (double *)calloc((size_t)ns * ns, sizeof(double));
  (void)nbf;
  for (int itype = 0; itype <= 1; itype++)
    for (int k = 0; k <= kmax; k++) {
      const int kk = k + 1000 * itype;
      orc_msk(g, itype, k, rkb);
      for (int in = 1; in <= 4; in++) {
        const char sym = sym_int[in - 1];
        const int ip1 = ipt[itype][in - 1][0], ip2 = ipt[itype][in - 1][1];
        const int jp1 = ipt[itype][in - 1][2], jp2 = ipt[itype][in - 1][3];
        memset(xx, 0, sizeof(double) * (size_t)ns * ns);
        int met = 0;
        for (int ik = 0; ik < nrk; ik++) {
          if (kk != kr1[ik]) continue;
          int jnt, j;
          if (iorb == kr3[ik]) {
            jnt = kr2[ik];
            j = kr4[ik];
          } else if (iorb == kr4[ik]) {
            jnt = kint[kr2[ik] - 1];
            j = kr3[ik];
          } else {
            continue;
          }
          if (jnt != in) continue;
          const double *p1 = pq + (size_t)2 * ns * (j - 1) + (size_t)ns * (jp1 - 1);
          const double *p2 = pq + (size_t)2 * ns * (j - 1) + (size_t)ns * (jp2 - 1);
          orc_density(ns, ks, x, p1, p2, sym);
          const size_t nn = (size_t)ns * (sym == 'n' ? kb : ns);
          for (size_t q = 0; q < nn; q++) xx[q] = xx[q] + crk[ik] * x[q];
          met++;
        }
        if (met > 0) {
          orc_convol(ns, ks, kb, rkb, x, xx, in, sym, sym);
          hf_update(ns, ks, ms, hfm, ip1, ip2, x, sym);
        }
      }
    }
  free(rkb);
  free(x);
  free(xx);
}

/* ======================================================================
 * Write-out of DBSR_MAT3: Diag_channels (diag.f90:2-81) and the block
 * transformation of Record_matrix (record_matrix.f90:14-26).
 *
 * Diag_channels solves, per channel with a diagonal block, H c = E B c on
 * the B-splines the zero conditions keep (iprm != 0) with LAPACK DSYGV
 * (itype 1, 'V', 'L').  LAPACK is a third-party library absent from the
 * reference tree; its published algorithm is restated here: the Cholesky
 * factor B = L L^T of the lower triangle, the standard problem
 * C = L^-1 A L^-T (A from its lower triangle), C y = E y by the cyclic
 * Jacobi method (rotations that zero one off-diagonal element at a time,
 * sweeps until the off-diagonal part vanishes to rounding), x = L^-T y
 * (so x^T B x = 1), eigenvalues ascending.  The eigenvectors agree with
 * LAPACK's up to sign for distinct eigenvalues; the reference fixes the
 * sign (largest component positive), so the comparison is sign-free.
 * Parity unpinned: the reference ships no dbsr_mat.nnn.
 * ====================================================================== */

/* lower Cholesky factor in place (a: n x n, leading dimension lda);
 * returns 0, or the order of the first non-positive pivot */
static int chol_lower(int n, double *a, int lda) {
  for (int j = 0; j < n; j++) {
    double d = a[j + (size_t)lda * j];
    for (int k = 0; k < j; k++) d -= a[j + (size_t)lda * k] * a[j + (size_t)lda * k];
    if (!(d > 0.0)) return j + 1;
    d = sqrt(d);
    a[j + (size_t)lda * j] = d;
    for (int i = j + 1; i < n; i++) {
      double s = a[i + (size_t)lda * j];
      for (int k = 0; k < j; k++) s -= a[i + (size_t)lda * k] * a[j + (size_t)lda * k];
      a[i + (size_t)lda * j] = s / d;
    }
  }
  return 0;
}

/* cyclic Jacobi: symmetric c (n x n, full storage) -> eigenvalues w and
 * eigenvectors v (columns), ascending */
static void jacobi_eig(int n, double *c, double *w, double *v) {
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) v[i + (size_t)n * j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        const double x = c[i + (size_t)n * j] * c[i + (size_t)n * j];
        tot += x;
        if (i != j) off += x;
      }
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; p++)
      for (int q = p + 1; q < n; q++) {
        const double apq = c[p + (size_t)n * q];
        if (apq == 0.0) continue;
        const double app = c[p + (size_t)n * p], aqq = c[q + (size_t)n * q];
        /* rotation angle: t = tan(phi) of the smaller root (Rutishauser) */
        const double th = (aqq - app) / (2.0 * apq);
        const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 0; k < n; k++) { /* columns p, q */
          const double akp = c[k + (size_t)n * p], akq = c[k + (size_t)n * q];
          c[k + (size_t)n * p] = cs * akp - sn * akq;
          c[k + (size_t)n * q] = sn * akp + cs * akq;
        }
        for (int k = 0; k < n; k++) { /* rows p, q */
          const double apk = c[p + (size_t)n * k], aqk = c[q + (size_t)n * k];
          c[p + (size_t)n * k] = cs * apk - sn * aqk;
          c[q + (size_t)n * k] = sn * apk + cs * aqk;
        }
        for (int k = 0; k < n; k++) {
          const double vkp = v[k + (size_t)n * p], vkq = v[k + (size_t)n * q];
          v[k + (size_t)n * p] = cs * vkp - sn * vkq;
          v[k + (size_t)n * q] = sn * vkp + cs * vkq;
        }
      }
  }
  for (int i = 0; i < n; i++) w[i] = c[i + (size_t)n * i];
  /* ascending order (selection sort of eigenpairs) */
  for (int i = 0; i < n - 1; i++) {
    int m = i;
    for (int j = i + 1; j < n; j++)
      if (w[j] < w[m]) m = j;
    if (m == i) continue;
    const double t = w[i];
    w[i] = w[m];
    w[m] = t;
    for (int k = 0; k < n; k++) {
      const double x = v[k + (size_t)n * i];
      v[k + (size_t)n * i] = v[k + (size_t)n * m];
      v[k + (size_t)n * m] = x;
    }
  }
}

/* Generalised symmetric-definite problem A x = E B x on the lower
 * triangles of a and b (n x n, lda); eigenvalues w ascending, eigenvectors
 * in the columns of x (n x n) with x^T B x = 1.  Returns 0 or the order of
 * the failed Cholesky pivot. */
int orc_sygv(int n, const double *a, const double *b, int lda, double *w, double *x) {
  double *L = (double *)malloc(sizeof(double) * (size_t)n * n);
  double *C = (double *)malloc(sizeof(double) * (size_t)n * n);
  double *Y = (double *)malloc(sizeof(double) * (size_t)n * n);
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) L[i + (size_t)n * j] = i >= j ? b[i + (size_t)lda * j] : 0.0;
  int rc = chol_lower(n, L, n);
  if (rc == 0) {
    /* C = L^-1 A L^-T with A symmetric from its lower triangle: first
     * Y = L^-1 A (forward substitution per column), then C = L^-1 Y^T */
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++)
        Y[i + (size_t)n * j] = i >= j ? a[i + (size_t)lda * j] : a[j + (size_t)lda * i];
    for (int pass = 0; pass < 2; pass++) {
      for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
          double s = Y[i + (size_t)n * j];
          for (int k = 0; k < i; k++) s -= L[i + (size_t)n * k] * Y[k + (size_t)n * j];
          Y[i + (size_t)n * j] = s / L[i + (size_t)n * i];
        }
      /* transpose: pass 0 leaves L^-1 A, its transpose is A L^-T */
      for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) C[i + (size_t)n * j] = Y[j + (size_t)n * i];
      memcpy(Y, C, sizeof(double) * (size_t)n * n);
    }
    /* symmetrise against rounding, then the standard problem */
    for (int j = 0; j < n; j++)
      for (int i = j + 1; i < n; i++) {
        const double s = 0.5 * (C[i + (size_t)n * j] + C[j + (size_t)n * i]);
        C[i + (size_t)n * j] = C[j + (size_t)n * i] = s;
      }
    jacobi_eig(n, C, w, Y);
    /* x = L^-T y (back substitution per column) */
    for (int j = 0; j < n; j++)
      for (int i = n - 1; i >= 0; i--) {
        double s = Y[i + (size_t)n * j];
        for (int k = i + 1; k < n; k++) s -= L[k + (size_t)n * i] * x[k + (size_t)n * j];
        x[i + (size_t)n * j] = s / L[i + (size_t)n * i];
      }
  }
  free(L);
  free(C);
  free(Y);
  return rc;
}

/* Diag_channels (diag.f90:2-81) without its printing: for every channel
 * ich with a diagonal block k = icc(ich,ich), the kept B-splines
 * (iprm(j,ich) != 0, j = 1..ms), the problem hch(:,:,k) c = E bdiag(:,:,ich)
 * c on them, the solutions with emin <= E <= emax and |E| >= egap in
 * ascending order, restored to the full net (zeros on the dropped
 * B-splines) with their largest component positive (maxloc: the first of
 * equal maxima), into sol(:,ksol,ich) (ms x ms x nch), their energies into
 * eval(ksol,ich) (ms x nch) and their count into nsol(ich).  Returns 0 or
 * -(ich) of a channel whose overlap block is not positive definite
 * ('channel diagonalization failed'). */
int orc_diag_channels(orc_mat *m, const double *bdiag, const int *iprm, double emin, double emax,
                      double egap, double *sol, double *eval, int *nsol) {
  const int ms = m->g->ms, nch = m->nch;
  double *a = (double *)malloc(sizeof(double) * (size_t)ms * ms);
  double *b = (double *)malloc(sizeof(double) * (size_t)ms * ms);
  double *x = (double *)malloc(sizeof(double) * (size_t)ms * ms);
  double *w = (double *)malloc(sizeof(double) * ms);
  double *v = (double *)malloc(sizeof(double) * ms);
  int rc = 0;
  memset(sol, 0, sizeof(double) * (size_t)ms * ms * nch);
  memset(eval, 0, sizeof(double) * (size_t)ms * nch);
  for (int ich = 1; ich <= nch && rc == 0; ich++) {
    nsol[ich - 1] = 0;
    const int k = ICC(ich, ich);
    if (k == 0) continue;
    const int *ip = iprm + (size_t)ms * (ich - 1);
    const double *bc = bdiag + (size_t)ms * ms * (ich - 1);
    int jj = 0, ii = 0;
    for (int j = 1; j <= ms; j++) {
      if (ip[j - 1] == 0) continue;
      jj++;
      ii = 0;
      for (int i = 1; i <= ms; i++) {
        if (ip[i - 1] == 0) continue;
        ii++;
        a[(ii - 1) + (size_t)ms * (jj - 1)] = HCH(i, j, k);
        b[(ii - 1) + (size_t)ms * (jj - 1)] = bc[(i - 1) + (size_t)ms * (j - 1)];
      }
    }
    if (orc_sygv(ii, a, b, ms, w, x)) {
      rc = -ich;
      break;
    }
    int ksol = 0;
    for (int i = 1; i <= ii; i++) {
      const double e = w[i - 1];
      if (e < emin || e > emax || fabs(e) < egap) continue;
      ksol++;
      int q = 0;
      for (int j = 1; j <= ms; j++) {
        v[j - 1] = 0.0;
        if (ip[j - 1] == 0) continue;
        q++;
        v[j - 1] = x[(q - 1) + (size_t)ii * (i - 1)];
      }
      int pos = 0;
      for (int j = 1; j < ms; j++)
        if (fabs(v[j]) > fabs(v[pos])) pos = j;
      const double sg = v[pos] < 0.0 ? -1.0 : 1.0;
      for (int j = 0; j < ms; j++) sol[j + (size_t)ms * (ksol - 1) + (size_t)ms * ms * (ich - 1)] = sg * v[j];
      eval[(ksol - 1) + (size_t)ms * (ich - 1)] = e;
    }
    nsol[ich - 1] = ksol;
  }
  free(a);
  free(b);
  free(x);
  free(w);
  free(v);
  return rc;
}

/* The block transformation of Record_matrix (record_matrix.f90:14-26) for
 * one block: c(i,j) = sum_l w(l) dj(l,j) with w(l) = sum_m di(m,i) h(m,l),
 * i = 1..ni, j = 1..nj (h ms x ms, di/dj ms x ni/nj, c ni x nj). */
void orc_record_block(int ms, const double *h, const double *di, int ni, const double *dj,
                      int nj, double *c) {
  double *w = (double *)malloc(sizeof(double) * ms);
  for (int i = 1; i <= ni; i++) {
    for (int l = 1; l <= ms; l++) {
      double s = 0.0;
      for (int mm = 1; mm <= ms; mm++)
        s = s + di[(mm - 1) + (size_t)ms * (i - 1)] * h[(mm - 1) + (size_t)ms * (l - 1)];
      w[l - 1] = s;
    }
    for (int j = 1; j <= nj; j++) {
      double s = 0.0;
      for (int l = 1; l <= ms; l++) s = s + w[l - 1] * dj[(l - 1) + (size_t)ms * (j - 1)];
      c[(i - 1) + (size_t)ni * (j - 1)] = s;
    }
  }
  free(w);
}

/* ======================================================================
 * DBSR_MCHF's SCF potential matrices (mchf_matrix.f90).
 *
 * orc_mchf_matrix restates mchf_matrix (mchf_matrix.f90:2-251) for an
 * orbital outside the core.  The caller passes the expansion-weighted
 * coefficients that mchf_matrix forms with WW (mchf_matrix.f90:65, 95):
 * L entries (li1, li2, lc = WW L_coef) and R^k entries (rk, ri1..ri4,
 * rc = WW Rk_coef) in the order of the integral lists (k ascending), the
 * one-electron matrix dhl of Get_hd_core (ms x ms), and the flags irhs and
 * newton.  Add_id4_data (module id4_data, absent from the reference tree)
 * is restated as appending (k, id2, id3, id4, C) to the list of its k.
 * The loop over id4 entries of the newton term convolves the density left
 * in x by the last entry it visits, unweighted (mchf_matrix.f90:211-216:
 * Convol(ns,ks,xx,x,4,...) writes its result over the weighted sum xx), and
 * this restatement does the same.  Outputs: hfm, rhs, hx (ms x ms, ms,
 * ms x ms), the energy e(i) and qsum(i).
 *
 * orc_mchf_core restates core_matrix (mchf_matrix.f90:255-346) with the
 * angular coefficients a(i,j,k), b(i,j,k) given as arrays (nbf, kmax+1),
 * qsum(nbf) and the one-electron matrix hd of Get_hd (ms x ms).
 * Parity unpinned (the reference ships no potential matrices).
 * ====================================================================== */

typedef struct {
  int id2, id3, id4;
  double c;
} id4_entry;

static void id4_add(id4_entry **v, int *n, int *cap, int id2, int id3, int id4, double c) {
  if (*n == *cap) {
    *cap = *cap ? 2 * *cap : 64;
    *v = (id4_entry *)realloc(*v, sizeof(id4_entry) * (size_t)*cap);
  }
  (*v)[*n].id2 = id2;
  (*v)[*n].id3 = id3;
  (*v)[*n].id4 = id4;
  (*v)[*n].c = c;
  (*n)++;
}

void orc_mchf_matrix(const orc_grid *g, int nbf, const double *pq, int iorb, int kmax, int nl,
                     const int *li1, const int *li2, const double *lc, int nr, const int *rk,
                     const int *ri1, const int *ri2, const int *ri3, const int *ri4,
                     const double *rc, const double *dhl, int irhs, int newton, double eps_c,
                     double *hfm, double *rhs, double *hx, double *e_out, double *qsum_out) {
  const int ns = g->ns, ks = g->ks, ms = g->ms, i = iorb;
  static const int ttype[2][2] = {{0, 2}, {3, 1}};
  const double qsum_min = 1e-8; /* MOD_dbsr_mchf.f90:55 */
  double *rkb = (double *)malloc(sizeof(double) * (size_t)ns * ns * ks * ks);
  double *d = (double *)malloc(sizeof(double) * (size_t)ns * ns);
  double *dd = (double *)malloc(sizeof(double) * (size_t)ns * ns);
  double *x = (double *)malloc(sizeof(double) * (size_t)ns * ns);
  double *xx = (double *)malloc(sizeof(double) * (size_t)ns * ns);
  double *aa = (double *)malloc(sizeof(double) * (size_t)ns * ks * nbf);
  int *iaa = (int *)malloc(sizeof(int) * nbf);
  double *v = (double *)malloc(sizeof(double) * ms);
  double *vv = (double *)malloc(sizeof(double) * ms);
  double *v1 = (double *)malloc(sizeof(double) * ns);
  double *CI = (double *)calloc(nbf, sizeof(double));
  id4_entry *ent = NULL;
  int cap = 0;
#define GETPV(io, vec)                                                     \
  do {                                                                     \
    const double *pp_ = pq + (size_t)2 * ns * ((io) - 1);                  \
    for (int q_ = 0; q_ < ns; q_++) {                                      \
      (vec)[q_] = pp_[q_];                                                 \
      (vec)[ns + q_] = pp_[ns + q_];                                       \
    }                                                                      \
  } while (0)
  for (size_t q = 0; q < (size_t)ms * ms; q++) hfm[q] = hx[q] = 0.0;
  for (int q = 0; q < ms; q++) rhs[q] = 0.0;
  /* one-electron integrals (:59-84) */
  double S = 0.0;
  for (int m = 0; m < nl; m++) {
    const int i1 = li1[m], i2 = li2[m];
    const double C = lc[m];
    if (i1 == i && i2 == i)
      S = S + C;
    else if (i1 == i && i2 != i)
      CI[i2 - 1] = CI[i2 - 1] + C;
    else if (i1 != i && i2 == i)
      CI[i1 - 1] = CI[i1 - 1] + C;
  }
  if (fabs(S) < qsum_min) S = qsum_min;
  *qsum_out = S;
  double sci = 0.0;
  for (int io = 0; io < nbf; io++) sci += fabs(CI[io]);
  if (sci != 0.0) {
    for (int q = 0; q < ms; q++) vv[q] = 0.0;
    for (int io = 1; io <= nbf; io++) {
      if (CI[io - 1] == 0.0) continue;
      GETPV(io, v);
      for (int q = 0; q < ms; q++) vv[q] = vv[q] + v[q] * CI[io - 1] / S / 2.0;
    }
    for (int r = 1; r <= ms; r++) { /* rhs + matmul(dhl, vv) */
      double s = 0.0;
      for (int q = 1; q <= ms; q++) s = s + A2(dhl, r, q, ms) * vv[q - 1];
      rhs[r - 1] = rhs[r - 1] + s;
    }
  }
  for (int k = 0; k <= kmax; k++) {
    int nid = 0;
    for (int m = 0; m < nr; m++) {
      if (rk[m] != k) continue;
      const int i1 = ri1[m], i2 = ri2[m], i3 = ri3[m], i4 = ri4[m];
      const double C = rc[m] / S;
      if (fabs(C) < eps_c) continue;
      const int ii = (i == i1) * 1000 + (i == i2) * 100 + (i == i3) * 10 + (i == i4);
      switch (ii) {
        case 1111: id4_add(&ent, &nid, &cap, -1, i1, i3, 2 * C);
                   id4_add(&ent, &nid, &cap, -3, i1, i3, 4 * C); break;
        case 1010: id4_add(&ent, &nid, &cap, -1, i2, i4, C); break;
        case 101:  id4_add(&ent, &nid, &cap, -1, i1, i3, C); break;
        case 1001: id4_add(&ent, &nid, &cap, -2, i2, i3, C); break;
        case 1100: id4_add(&ent, &nid, &cap, -2, i3, i4, C); break;
        case 110:  id4_add(&ent, &nid, &cap, -2, i1, i4, C); break;
        case 11:   id4_add(&ent, &nid, &cap, -2, i1, i2, C); break;
        case 111:  id4_add(&ent, &nid, &cap, -1, i1, i3, C);
                   id4_add(&ent, &nid, &cap, -2, i1, i3, C / 2);
                   id4_add(&ent, &nid, &cap, -3, i1, i3, 3 * C / 2); break;
        case 1011: id4_add(&ent, &nid, &cap, -1, i2, i4, C);
                   id4_add(&ent, &nid, &cap, -2, i2, i4, C / 2);
                   id4_add(&ent, &nid, &cap, -3, i2, i4, 3 * C / 2); break;
        case 1101: id4_add(&ent, &nid, &cap, -1, i1, i3, C);
                   id4_add(&ent, &nid, &cap, -2, i1, i3, C / 2);
                   id4_add(&ent, &nid, &cap, -3, i1, i3, 3 * C / 2); break;
        case 1110: id4_add(&ent, &nid, &cap, -1, i2, i4, C);
                   id4_add(&ent, &nid, &cap, -2, i2, i4, C / 2);
                   id4_add(&ent, &nid, &cap, -3, i2, i4, 3 * C / 2); break;
        case 1000: id4_add(&ent, &nid, &cap, i3, i2, i4, C / 2); break;
        case 100:  id4_add(&ent, &nid, &cap, i4, i1, i3, C / 2); break;
        case 10:   id4_add(&ent, &nid, &cap, i1, i2, i4, C / 2); break;
        case 1:    id4_add(&ent, &nid, &cap, i2, i1, i3, C / 2); break;
        default: break;
      }
    }
    if (nid == 0) continue;
    for (int ii = 1; ii <= 2; ii++)
      for (int jj = 1; jj <= 2; jj++) {
        orc_mrk(g, ttype[ii - 1][jj - 1], k, rkb);
#define PCOMP(io, comp) (pq + (size_t)2 * ns * ((io) - 1) + (size_t)ns * ((comp) - 1))
        /* direct (:155-169) */
        int met = 0;
        memset(dd, 0, sizeof(double) * (size_t)ns * ks);
        for (int j = 0; j < nid; j++) {
          if (ent[j].id2 != -1 || ent[j].c == 0.0) continue;
          orc_density(ns, ks, d, PCOMP(ent[j].id3, jj), PCOMP(ent[j].id4, jj), 's');
          for (size_t q = 0; q < (size_t)ns * ks; q++) dd[q] = dd[q] + ent[j].c * d[q];
          met = 1;
        }
        if (met) {
          orc_convol(ns, ks, ks, rkb, d, dd, 1, 's', 's');
          hf_update(ns, ks, ms, hfm, ii, ii, d, 's');
        }
        /* exchange (:171-185) */
        met = 0;
        memset(xx, 0, sizeof(double) * (size_t)ns * ns);
        for (int j = 0; j < nid; j++) {
          if (ent[j].id2 != -2 || ent[j].c == 0.0) continue;
          orc_density(ns, ks, x, PCOMP(ent[j].id3, ii), PCOMP(ent[j].id4, jj), 'x');
          for (size_t q = 0; q < (size_t)ns * ns; q++) xx[q] = xx[q] + ent[j].c * x[q];
          met = 1;
        }
        if (met) {
          orc_convol(ns, ks, ks, rkb, x, xx, 4, 's', 's');
          hf_update(ns, ks, ms, hfm, ii, jj, x, 'x');
        }
        /* rhs (:187-205) */
        memset(aa, 0, sizeof(double) * (size_t)ns * ks * nbf);
        memset(iaa, 0, sizeof(int) * nbf);
        for (int j = 0; j < nid; j++) {
          if (ent[j].id2 <= 0) continue;
          orc_density(ns, ks, d, PCOMP(ent[j].id3, jj), PCOMP(ent[j].id4, jj), 's');
          double *a_ = aa + (size_t)ns * ks * (ent[j].id2 - 1);
          for (size_t q = 0; q < (size_t)ns * ks; q++) a_[q] = a_[q] + d[q] * ent[j].c;
          iaa[ent[j].id2 - 1]++;
        }
        for (int j = 1; j <= nbf; j++) {
          if (iaa[j - 1] == 0) continue;
          memcpy(d, aa + (size_t)ns * ks * (j - 1), sizeof(double) * (size_t)ns * ks);
          orc_convol(ns, ks, ks, rkb, dd, d, 1, 's', 's');
          /* Full_mat_sym 's' (dbsr_lib_zcom.f90:1263-1268) into xx */
          memset(xx, 0, sizeof(double) * (size_t)ns * ns);
          for (int jp = 1; jp <= ks; jp++)
            for (int r = 1; r <= ns - jp + 1; r++) {
              const int cidx = r + jp - 1;
              A2(xx, r, cidx, ns) = A2(dd, r, jp, ns);
              A2(xx, cidx, r, ns) = A2(dd, r, jp, ns);
            }
          const double *pj = PCOMP(j, ii);
          for (int r = 1; r <= ns; r++) {
            double s = 0.0;
            for (int q = 1; q <= ns; q++) s = s + A2(xx, r, q, ns) * pj[q - 1];
            v1[r - 1] = s;
          }
          for (int r = 0; r < ns; r++) rhs[(ii - 1) * ns + r] = rhs[(ii - 1) * ns + r] + v1[r];
        }
        /* hx for the Newton-Raphson method (:209-221) */
        if (newton != 0) {
          met = 0;
          memset(xx, 0, sizeof(double) * (size_t)ns * ns);
          for (int j = 0; j < nid; j++) {
            if (ent[j].id2 != -3 || ent[j].c == 0.0) continue;
            orc_density(ns, ks, x, PCOMP(ent[j].id3, jj), PCOMP(ent[j].id4, jj), 'x');
            for (size_t q = 0; q < (size_t)ns * ns; q++) xx[q] = xx[q] + ent[j].c * x[q];
            met = 1;
          }
          if (met) {
            orc_convol(ns, ks, ks, rkb, xx, x, 4, 's', 's');
            hf_update(ns, ks, ms, hx, ii, jj, xx, 'x');
          }
        }
#undef PCOMP
      }
  }
  /* rhs into hfm (:223-241) */
  double srhs = 0.0;
  for (int q = 0; q < ms; q++) srhs += fabs(rhs[q]);
  if (srhs < 1e-8) {
    for (int q = 0; q < ms; q++) rhs[q] = 0.0;
    srhs = 0.0;
  }
  if (irhs > 0 && srhs > 0.0) {
    GETPV(i, v);
    double SS = 0.0;
    for (int q = 0; q < ms; q++) SS += rhs[q] * v[q];
    SS = -SS;
    for (size_t q = 0; q < (size_t)ms * ms; q++) hfm[q] = hfm[q] + SS * g->fppqq[q];
    for (int r = 1; r <= ms; r++) {
      double s = 0.0;
      for (int q = 1; q <= ms; q++) s = s + A2(g->fppqq, r, q, ms) * v[q - 1];
      vv[r - 1] = s;
    }
    for (int a_ = 1; a_ <= ms; a_++)
      for (int b_ = 1; b_ <= ms; b_++)
        A2(hfm, a_, b_, ms) = A2(hfm, a_, b_, ms) + rhs[a_ - 1] * vv[b_ - 1] + rhs[b_ - 1] * vv[a_ - 1];
    for (int q = 0; q < ms; q++) rhs[q] = 0.0;
  }
  /* final matrix and energy (:243-249) */
  for (size_t q = 0; q < (size_t)ms * ms; q++) hfm[q] = dhl[q] + hfm[q];
  for (int q = 0; q < ms; q++) rhs[q] = -rhs[q];
  GETPV(i, v);
  double e = 0.0;
  for (int r = 1; r <= ms; r++) {
    double s = 0.0;
    for (int q = 1; q <= ms; q++) s = s + A2(hfm, r, q, ms) * v[q - 1];
    e += v[r - 1] * (s - rhs[r - 1]);
  }
  *e_out = e;
#undef GETPV
  free(ent);
  free(rkb); free(d); free(dd); free(x); free(xx); free(aa); free(iaa);
  free(v); free(vv); free(v1); free(CI);
}

void orc_mchf_core(const orc_grid *g, int nbf, const double *pq, int iorb, int kmax,
                   const double *a, const double *b, const double *qsum, const double *hd,
                   int newton, double *hfm, double *hx) {
  const int ns = g->ns, ks = g->ks, ms = g->ms, i = iorb;
  static const int ttype[2][2] = {{0, 2}, {3, 1}};
  double *rkb = (double *)malloc(sizeof(double) * (size_t)ns * ns * ks * ks);
  double *d = (double *)malloc(sizeof(double) * (size_t)ns * ns);
  double *dd = (double *)malloc(sizeof(double) * (size_t)ns * ns);
  double *x = (double *)malloc(sizeof(double) * (size_t)ns * ns);
  double *xx = (double *)malloc(sizeof(double) * (size_t)ns * ns);
  const double qi = qsum[i - 1];
  for (size_t q = 0; q < (size_t)ms * ms; q++) {
    hfm[q] = qi * hd[q];
    hx[q] = 0.0;
  }
#define PCOMP(io, comp) (pq + (size_t)2 * ns * ((io) - 1) + (size_t)ns * ((comp) - 1))
  for (int ii = 1; ii <= 2; ii++)
    for (int jj = 1; jj <= 2; jj++)
      for (int k = 0; k <= kmax; k++) {
        orc_mrk(g, ttype[ii - 1][jj - 1], k, rkb);
        int met = 0;
        memset(dd, 0, sizeof(double) * (size_t)ns * ks);
        for (int j = 1; j <= nbf; j++) {
          double c = a[(j - 1) + (size_t)nbf * k];
          if (i != j) c = c * qi * qsum[j - 1];
          if (i == j) c = c * qi * (qi - 1);
          if (c == 0.0) continue;
          orc_density(ns, ks, d, PCOMP(j, jj), PCOMP(j, jj), 's');
          for (size_t q = 0; q < (size_t)ns * ks; q++) dd[q] = dd[q] + c * d[q];
          met = 1;
        }
        if (met) {
          orc_convol(ns, ks, ks, rkb, d, dd, 1, 's', 's');
          hf_update(ns, ks, ms, hfm, ii, ii, d, 's');
        }
        met = 0;
        memset(xx, 0, sizeof(double) * (size_t)ns * ns);
        for (int j = 1; j <= nbf; j++) {
          double c = b[(j - 1) + (size_t)nbf * k];
          if (i != j) c = c * qi * qsum[j - 1];
          if (i == j) c = c * qi * (qi - 1);
          if (c == 0.0) continue;
          orc_density(ns, ks, x, PCOMP(j, ii), PCOMP(j, jj), 'x');
          for (size_t q = 0; q < (size_t)ns * ns; q++) xx[q] = xx[q] + x[q] * c;
          met = 1;
        }
        if (met) {
          orc_convol(ns, ks, ks, rkb, x, xx, 4, 's', 's');
          hf_update(ns, ks, ms, hfm, ii, jj, x, 'x');
        }
        if (newton != 0) {
          double c = 2.0 * a[(i - 1) + (size_t)nbf * k];
          if (c == 0.0) continue;
          c = c * qi * (qi - 1);
          orc_density(ns, ks, x, PCOMP(i, ii), PCOMP(i, jj), 'x');
          for (size_t q = 0; q < (size_t)ns * ns; q++) xx[q] = c * x[q];
          orc_convol(ns, ks, ks, rkb, x, xx, 4, 's', 's');
          hf_update(ns, ks, ms, hx, ii, jj, x, 'x');
        }
      }
#undef PCOMP
  for (size_t q = 0; q < (size_t)ms * ms; q++) {
    hfm[q] = hfm[q] / qi;
    hx[q] = hx[q] / qi;
  }
  free(rkb); free(d); free(dd); free(x); free(xx);
}
