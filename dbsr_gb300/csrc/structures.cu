// structures.cu -- the coefficient-list structures whose terms are not
// channel-pair contractions, and the matrix parts they update:
//   R_data itype 1 (bound-bound integral times overlap factors) and 2 (a
//     channel orbital in one position)          DBSR_MAT3/R_data.f90:92-211
//   S_data itypes 1-5                           DBSR_MAT3/S_data.f90:74-236
//   L_data itypes 1-3                           DBSR_MAT3/L_data.f90:2-145
//   O_data itypes 1, 2, 4                       DBSR_MAT3/O_data.f90:33-78
//   UPDATE_HW/HV/HB/HX, Target_h                updates.f90:79-264,
//                                               target_subs.f90:2-31
// and the matrix parts beside hch: the perturber vectors hcp and scalars hp
// (Alloc_dbsr_matrix, updates.f90:47-72) and the target matrices htarg and
// otarg.
//
// A list is planned once on the host: every entry is classified exactly as
// the reference routes it (the same bound checks, returned as status codes
// where the reference stops), and each update becomes a term that names a
// coefficient slot and one or two vectors.  The terms are grouped, in the
// reference's order (atype by atype, entries in IPT order), by the block,
// perturber column or scalar they update.  Execution computes on the device
// what the terms read -- the potentials of the bound pairs (density and
// convol on the full tables, FP64), the per-entry integrals (SUM_AmB), the
// potential-times-orbital vectors (BAV), the one-electron values and
// vectors, the overlap vectors V_ch and the coefficient slots -- then
// applies the terms: one thread per row of 32 columns of a block walks that
// block's terms in order (no atomics), likewise per perturber column and
// per scalar.  The work is small beside the channel-pair contraction and
// stays FP64 in every precision form.
//
// Routines that live only in the unvendored Libraries_03 are restated:
//   V_ch / KBORT: the B-spline overlap vector (fpbs P; fqbs Q) of the bound
//     orbital io2 of an overlap code io = io1*ibo + io2 (io1 a channel
//     orbital), as for O_data itype 3;
//   BAV: band matrix times vector, 's' symmetric (ns,ks) or 'n' (ns,2ks-1)
//     with A(i,i+jp-ks) = a(i,jp), from the right ('r': A b) or the left
//     ('l': A^T b);
//   Lval(i,j) = p_i^T hd(kappa_i) p_j and Gen_Lvec(i) = hd(kappa_i) p_i,
//     with p = (P; Q) and the caller's one-electron matrices hd.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <vector>

#include "internal.cuh"

namespace {

// a term: kind 0-2 a rank-1 UPDATE_HW (ich > jch, ich < jch, ich = jch),
// 3-4 an UPDATE_HX (ich >= jch, ich < jch; a = 0 fppqq, 1+k hd(:,:,k+1)),
// for perturber columns a = the vector, for scalars a = the array (0 hp,
// 1 htarg, 2 otarg) and b its 0-based index; cidx the coefficient slot
struct StTerm {
  int kind, cidx, a, b;
};
static_assert(sizeof(StTerm) == 16, "StTerm is 16 bytes");

size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

// ---------------------------------------------------------------------------
// densities of bound pairs (density, dbsr_lib_dbs.f90:2834-2891): X[q] of
// pair (a, b) with components c1, c2, 's' (ns,ks) or 'n' (ns,2ks-1) storage
__global__ void k_st_density(int ns, int ks, char sym, int kb, int npot, const int2 *pots,
                             int c1, int c2, const double *pq, double *X) {
  const size_t per = (size_t)ns * kb;
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= per) return;
  const int pi = blockIdx.y;
  const int i = (int)(q % ns) + 1, j = (int)(q / ns) + 1;
  const int2 pr = pots[pi];
  const double *p1 = pq + (size_t)ns * (c1 - 1) + (size_t)2 * ns * (pr.x - 1) - 1;
  const double *p2 = pq + (size_t)ns * (c2 - 1) + (size_t)2 * ns * (pr.y - 1) - 1;
  double d = 0.0;
  if (sym == 's') {
    if (j == 1)
      d = p1[i] * p2[i];
    else if (i <= ns - j + 1)
      d = p1[i] * p2[i + j - 1] + p1[i + j - 1] * p2[i];
  } else {
    const int i0 = max(1, 1 + ks - j), i1 = min(ns, ns + ks - j);
    if (i >= i0 && i <= i1) d = p1[i] * p2[i + j - ks];
  }
  X[(size_t)pi * per + q] = d;
}

// SUM_AmB (dbsr_lib_dbs.f90:4027-4080) of a pair potential with the density
// of the entry's K2 pair, one warp per entry: Ce = S * cdata
__global__ void k_st_sumamb(int ns, int ks, char sym, int kb, int n, const int *epot,
                            const int *ej1, const int *ej2, int c1, int c2, const double *pq,
                            const double *Y, const double *cd, double *Ce) {
  const int e = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x % 32;
  if (e >= n || epot[e] < 0) return;
  const double *y = Y + (size_t)epot[e] * ns * kb;
  const double *p1 = pq + (size_t)ns * (c1 - 1) + (size_t)2 * ns * (ej1[e] - 1) - 1;
  const double *p2 = pq + (size_t)ns * (c2 - 1) + (size_t)2 * ns * (ej2[e] - 1) - 1;
  double acc = 0.0;
  for (int jp = 1; jp <= kb; jp++) {
    int i0, i1;
    if (sym == 's') {
      i0 = 1;
      i1 = ns - jp + 1;
    } else {
      i0 = max(1, 1 + ks - jp);
      i1 = min(ns, ns + ks - jp);
    }
    for (int i = i0 + lane; i <= i1; i += 32) {
      double d;
      if (sym == 's')
        d = jp == 1 ? p1[i] * p2[i] : p1[i] * p2[i + jp - 1] + p1[i + jp - 1] * p2[i];
      else
        d = p1[i] * p2[i + jp - ks];
      acc = fma(y[(i - 1) + (size_t)ns * (jp - 1)], d, acc);
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) Ce[e] = acc * cd[e];
}

// BAV: the potential of pair pot times orbital b (component ipo), into half
// ipv of an ms-vector of the pool (the other half zero); one thread per row
__global__ void k_st_bav(int ns, int ks, char sym, char dir, int kb, int nvj, const int2 *vj,
                         int ipo, int ipv, const double *pq, const double *Y, double *pool) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int q = blockIdx.y;
  if (i > ns || q >= nvj) return;
  const int2 job = vj[q];  // (potential, orbital)
  const double *a = Y + (size_t)job.x * ns * kb;
  const double *b = pq + (size_t)ns * (ipo - 1) + (size_t)2 * ns * (job.y - 1) - 1;
  auto A = [&](int r, int c) { return a[(r - 1) + (size_t)ns * (c - 1)]; };
  double v = 0.0;
  if (sym == 's') {
    for (int jp = 1; jp <= ks; jp++)
      if (i + jp - 1 <= ns) v = fma(A(i, jp), b[i + jp - 1], v);
    for (int jp = 2; jp <= ks; jp++)
      if (i - jp + 1 >= 1) v = fma(A(i - jp + 1, jp), b[i - jp + 1], v);
  } else {
    for (int jp = 1; jp <= 2 * ks - 1; jp++) {
      const int i0 = max(1, 1 + ks - jp), i1 = min(ns, ns + ks - jp);
      if (dir == 'l') {
        const int r = i - jp + ks;  // row whose band element lands in column i
        if (r >= i0 && r <= i1) v = fma(A(r, jp), b[r], v);
      } else if (i >= i0 && i <= i1) {
        v = fma(A(i, jp), b[i + jp - ks], v);
      }
    }
  }
  double *out = pool + (size_t)q * 2 * ns;
  out[(size_t)ns * (ipv - 1) + i - 1] = v;
  out[(size_t)ns * (2 - ipv) + i - 1] = 0.0;
}

// V_ch restatement: (fpbs P_b; fqbs Q_b) for every orbital b
__global__ void k_st_vch(int ns, int nbf, const double *fpbs, const double *fqbs,
                         const double *pq, double *vch) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= 2 * ns * nbf) return;
  const int i = q % (2 * ns), b = q / (2 * ns);
  const int comp = i / ns, ii = i % ns;
  const double *F = comp == 0 ? fpbs : fqbs;
  const double *p = pq + (size_t)2 * ns * b + (size_t)ns * comp;
  double s = 0.0;
  for (int j = 0; j < ns; j++) s += F[(size_t)ii + (size_t)ns * j] * p[j];
  vch[q] = s;
}

// Gen_Lvec restatement: hd(:,:,k) (P; Q)_orbital for each (orbital, k)
__global__ void k_st_lvec(int ms, int nlv, const int2 *lv, const double *hd, const double *pq,
                          double *pool) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int l = blockIdx.y;
  if (r >= ms || l >= nlv) return;
  const int2 job = lv[l];  // (orbital, kappa slot)
  const double *h = hd + (size_t)ms * ms * job.y;
  const double *p = pq + (size_t)ms * (job.x - 1);
  double s = 0.0;
  for (int k = 0; k < ms; k++) s = s + h[r + (size_t)ms * k] * p[k];
  pool[(size_t)l * ms + r] = s;
}

// Lval restatement: p_i1 . Gen_Lvec(i2) per entry, Ce = cdata * Lval
__global__ void k_st_lval(int ms, int n, const int *ej1, const int *elv, const double *pq,
                          const double *lpool, const double *cd, double *Ce) {
  const int e = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x % 32;
  if (e >= n || elv[e] < 0) return;
  const double *p = pq + (size_t)ms * (ej1[e] - 1);
  const double *v = lpool + (size_t)ms * elv[e];
  double s = 0.0;
  for (int k = lane; k < ms; k += 32) s = fma(p[k], v[k], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) Ce[e] = cd[e] * s;
}

// the coefficient slots of the structures whose factor is the coefficient
__global__ void k_st_copyc(int n, int na, const double *cd, double *Ce) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n * na) return;
  Ce[q] = cd[q % n];
}

// UPDATE_HW / UPDATE_HX terms of the window's blocks: one thread per row r
// and 32 consecutive columns of block tlist[z], its terms in list order
__global__ void k_st_block_terms(int ms, const int *tlist, const int *bstart,
                                 const StTerm *terms, const double *Ce, const double *pool,
                                 const double *fppqq, const double *hd, double *hch) {
  constexpr int NC = 32;
  const int bi = blockIdx.z;
  const int b = tlist[bi];
  const int t0 = bstart[bi], t1 = bstart[bi + 1];
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c0 = blockIdx.y * NC;
  if (r >= ms) return;
  const int ncol = min(NC, ms - c0);
  double *h = hch + (size_t)(b - 1) * ms * ms + r + (size_t)ms * c0;
  double val[NC];
#pragma unroll
  for (int j = 0; j < NC; j++) val[j] = j < ncol ? h[(size_t)ms * j] : 0.0;
  for (int t = t0; t < t1; t++) {
    const StTerm T = terms[t];
    const double C = Ce[T.cidx];
    if (T.kind <= 2) {
      const double *v = pool + (size_t)ms * T.a, *w = pool + (size_t)ms * T.b;
      if (T.kind == 0) {  // C * (v(r) w(c))
        const double vr = v[r];
#pragma unroll
        for (int j = 0; j < NC; j++)
          if (j < ncol) val[j] = __dadd_rn(val[j], __dmul_rn(C, __dmul_rn(vr, w[c0 + j])));
      } else if (T.kind == 1) {  // C * (v(c) w(r))
        const double wr = w[r];
#pragma unroll
        for (int j = 0; j < NC; j++)
          if (j < ncol) val[j] = __dadd_rn(val[j], __dmul_rn(C, __dmul_rn(v[c0 + j], wr)));
      } else {  // (C/2) * (v(r) w(c) + v(c) w(r))
        const double h2 = C / 2.0, vr = v[r], wr = w[r];
#pragma unroll
        for (int j = 0; j < NC; j++)
          if (j < ncol)
            val[j] = __dadd_rn(val[j], __dmul_rn(h2, __dadd_rn(__dmul_rn(vr, w[c0 + j]),
                                                                __dmul_rn(v[c0 + j], wr))));
      }
    } else {
      const double *d = T.a == 0 ? fppqq : hd + (size_t)ms * ms * (T.a - 1);
#pragma unroll
      for (int j = 0; j < NC; j++)
        if (j < ncol) {
          const double x = T.kind == 3 ? d[r + (size_t)ms * (c0 + j)] : d[(c0 + j) + (size_t)ms * r];
          val[j] = __dadd_rn(val[j], __dmul_rn(C, x));
        }
    }
  }
#pragma unroll
  for (int j = 0; j < NC; j++)
    if (j < ncol) h[(size_t)ms * j] = val[j];
}

// UPDATE_HV terms: one thread per row of a perturber column, terms in order
__global__ void k_st_hv_terms(int ms, const int *cols, const int *cstart, const StTerm *terms,
                              const double *Ce, const double *pool, double *hcp) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int ci = blockIdx.y;
  if (r >= ms) return;
  double *h = hcp + (size_t)ms * (cols[ci] - 1) + r;
  double val = *h;
  for (int t = cstart[ci]; t < cstart[ci + 1]; t++) {
    const StTerm T = terms[t];
    val = __dadd_rn(val, __dmul_rn(Ce[T.cidx], pool[(size_t)ms * T.a + r]));
  }
  *h = val;
}

// UPDATE_HB and Target_h terms: one thread per scalar, terms in order
__global__ void k_st_scalar_terms(int ng, const int *gstart, const StTerm *terms,
                                  const double *Ce, double *hp, double *htarg, double *otarg) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  const int t0 = gstart[g], t1 = gstart[g + 1];
  if (t0 == t1) return;
  const StTerm F = terms[t0];
  double *dst = (F.a == 0 ? hp : F.a == 1 ? htarg : otarg) + F.b;
  double val = *dst;
  for (int t = t0; t < t1; t++) val = __dadd_rn(val, Ce[terms[t].cidx]);
  *dst = val;
}

// single-term updates of the C ABI
__global__ void k_st_hw1(int ms, int kind, double C, const double *v, const double *w,
                         double *blk) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (size_t)ms * ms) return;
  const int r = (int)(q % ms), c = (int)(q / ms);
  double x;
  if (kind == 0)
    x = __dmul_rn(C, __dmul_rn(v[r], w[c]));
  else if (kind == 1)
    x = __dmul_rn(C, __dmul_rn(v[c], w[r]));
  else
    x = __dmul_rn(C / 2.0, __dadd_rn(__dmul_rn(v[r], w[c]), __dmul_rn(v[c], w[r])));
  blk[q] = __dadd_rn(blk[q], x);
}
__global__ void k_st_hv1(int ms, double C, const double *v, double *col) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < ms) col[r] = __dadd_rn(col[r], __dmul_rn(C, v[r]));
}
__global__ void k_st_hb1(double C, double *dst) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *dst = __dadd_rn(*dst, C);
}
__global__ void k_st_scale(size_t n, double s, double *x) {
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += (size_t)gridDim.x * blockDim.x)
    x[q] = __dmul_rn(x[q], s);
}

}  // namespace

// ---------------------------------------------------------------------------
struct StructPlan {
  int icase = 0, itype = 0, kpol = 0, n = 0;
  int na = 1, family = -1, kb = 0;
  char sym = 's', dir = 'r';
  int icv = 1, ttype[4] = {0, 0, 0, 0};
  int dc1[4] = {1, 1, 1, 1}, dc2[4] = {1, 1, 1, 1};  // components of the K1 density
  int ec1[4] = {1, 1, 1, 1}, ec2[4] = {1, 1, 1, 1};  // components of the K2 density
  int ipo[4] = {1, 1, 1, 1}, ipv[4] = {1, 1, 1, 1};  // BAV orbital component, vector half
  bool sum_amb = false, bav = false, lval = false, lvec = false, copyc = false;
  int npot = 0, npv = 0, nlv = 0, nbf = 0;
  int2 *pots = nullptr, *vjobs = nullptr, *ljobs = nullptr;
  int *epot = nullptr, *ej1 = nullptr, *ej2 = nullptr, *elv = nullptr;
  double *Ce = nullptr, *lcd = nullptr;
  StTerm *terms = nullptr;
  // block terms: window w holds groups [wb[w], wb[w+1]) of blist/bstart
  std::vector<int> wb;
  int *blist = nullptr, *bstart = nullptr;
  // perturber-column and scalar terms, applied in window wfirst
  int wfirst = -1, nhv = 0, nsc = 0;
  int *hvcol = nullptr, *hvstart = nullptr, *scstart = nullptr;
  StTerm *hvterms = nullptr, *scterms = nullptr;
  bool any_block = false;
};

bool is_structure_list(int icase, int itype) {
  switch (icase) {
    case 0: return itype == 1 || itype == 2 || itype == 4;
    case 1: return itype >= 1 && itype <= 3;
    case 2: return itype == 1 || itype == 2;
    case 3: {
      const int at = itype / 10, it = itype % 10;
      return at >= 0 && at <= 1 && it >= 1 && it <= 5;
    }
    default: return false;
  }
}

// device bytes of a structure list's plan (upper bounds by entry count)
size_t structure_plan_bytes(const dbsrg_ctx *c, int icase, int itype, int n) {
  (void)itype;
  const size_t na = icase == 2 ? 4 : 1;
  const size_t N = (size_t)n + 1;
  size_t t = 0;
  t += al256(sizeof(double) * N);                      // coefficients in IPT order
  t += al256(sizeof(double) * N * na);                 // coefficient slots
  t += 3 * al256(sizeof(int2) * N);                    // potentials, BAV and L vector jobs
  t += 4 * al256(sizeof(int) * N);                     // per-entry jobs
  t += 3 * al256(sizeof(StTerm) * 2 * N * na);         // block, column and scalar terms
  t += 2 * al256(sizeof(int) * (2 * N * na + 2));      // block and column groups
  t += al256(sizeof(int) * (2 * N * na + 2));          // scalar groups
  (void)c;
  return t;
}

void free_structure_plan(StructPlan *P) { delete P; }

namespace {

struct Builder {
  dbsrg_ctx *c;
  int blo0, nwin, nw;
  const int *wstart;  // explicit window starts (nw + 1), or null
  std::vector<std::pair<int, StTerm>> bterms;  // (block, term)
  std::vector<std::pair<int, StTerm>> hvterms; // (hcp column, term)
  std::vector<std::pair<long long, StTerm>> scterms;  // (array*2^40 + index, term)
  int wof(int b) const {
    if (wstart) {
      if (b < wstart[0] || b >= wstart[nw]) return -1;
      return (int)(std::upper_bound(wstart, wstart + nw + 1, b) - wstart) - 1;
    }
    if (b < blo0) return -1;
    const int w = (b - blo0) / nwin;
    return w < nw ? w : -1;
  }
  int block(int ich, int jch, int *b) {
    if (ich < 1 || jch < 1 || ich > c->nch || jch > c->nch)
      return set_err(c, DBSRG_ERANGE, "UPDATE_*: channel index out of range");
    *b = c->h_icc[(ich - 1) + (size_t)c->nch * (jch - 1)];
    if (*b < 1 || *b > c->iicc) return set_err(c, DBSRG_ERANGE, "UPDATE_*: block out of range");
    return DBSRG_OK;
  }
  // UPDATE_HW(ich, jch, v, w, C): pool vectors vi, wi, slot cidx
  int hw(int ich, int jch, int vi, int wi, int cidx) {
    int b, rc;
    if ((rc = block(ich, jch, &b))) return rc;
    if (wof(b) < 0) return DBSRG_OK;
    const int kind = ich > jch ? 0 : (ich < jch ? 1 : 2);
    bterms.push_back({b, StTerm{kind, cidx, vi, wi}});
    return DBSRG_OK;
  }
  // UPDATE_HX(ich, jch, d, C): d = fppqq (mat 0) or hd(:,:,mat)
  int hx(int ich, int jch, int mat, int cidx) {
    int b, rc;
    if ((rc = block(ich, jch, &b))) return rc;
    if (wof(b) < 0) return DBSRG_OK;
    bterms.push_back({b, StTerm{ich >= jch ? 3 : 4, cidx, mat, 0}});
    return DBSRG_OK;
  }
  int hv(int ich, int ip, int vi, int cidx) {
    if (ich < 1 || ich > c->nch) return set_err(c, DBSRG_ERANGE, "UPDATE_HV: channel out of range");
    if (ip < 1 || ip > c->npert)
      return set_err(c, DBSRG_ERANGE, "UPDATE_HV: bound index out of range");
    const int i = c->h_icb[(ich - 1) + (size_t)c->nch * (ip - 1)];
    if (i < 1 || i > c->iicb) return set_err(c, DBSRG_ERANGE, "UPDATE_HV: ich, ip out of range");
    hvterms.push_back({i, StTerm{0, cidx, vi, 0}});
    return DBSRG_OK;
  }
  int hb(int ic, int jc, int cidx) {
    if (ic > c->npert || jc > c->npert || ic <= 0 || jc <= 0)
      return set_err(c, DBSRG_ERANGE, "UPDATE_HB: index is out of range");
    const int i = c->h_ibb[(ic - 1) + (size_t)c->npert * (jc - 1)];
    if (i < 1 || i > c->iibb) return set_err(c, DBSRG_ERANGE, "UPDATE_HB: ic, jc out of range");
    scterms.push_back({(0LL << 40) + (i - 1), StTerm{0, cidx, 0, i - 1}});
    return DBSRG_OK;
  }
  // Target_h(ich, jch, C, CC): arr 1 adds the slot to htarg, 2 to otarg
  int target(int ich, int jch, int cidx, int arr) {
    if (c->ntarg <= 0) return DBSRG_OK;  // no targets given: nothing to update
    if (ich < 0 || jch < 0 || ich > c->nch || jch > c->nch)
      return set_err(c, DBSRG_ERANGE, "Target_h: channel out of range");
    if (ich < 1 || jch < 1) return DBSRG_OK;
    if (c->h_icc[(ich - 1) + (size_t)c->nch * (jch - 1)] == 0) return DBSRG_OK;
    const int it = c->h_iptar[ich - 1], jt = c->h_iptar[jch - 1];
    const int i = std::max(it, jt), j = std::min(it, jt);
    if (j < 1 || i > c->ntarg) return set_err(c, DBSRG_ERANGE, "Target_h: target out of range");
    const int ij = (i - 1) * i / 2 + j;
    scterms.push_back({((long long)arr << 40) + (ij - 1), StTerm{0, cidx, arr, ij - 1}});
    return DBSRG_OK;
  }
  // the overlap vector V_ch of code io = io1*ibo + io2 (KBORT restated)
  int vch(int io, int *vi) {
    const int o1 = io / DBSRG_IBO, o2 = io % DBSRG_IBO;
    if (o1 < 1 || o1 > c->nbf || o2 < 1 || o2 > c->nbf)
      return set_err(c, DBSRG_ERANGE, "KBORT = 0: orbital index out of range");
    const int ich = c->h_ipbs[o1 - 1];
    if (ich < 1 || ich > c->nch) return set_err(c, DBSRG_ERANGE, "KBORT = 0: not a channel orbital");
    *vi = o2 - 1;
    return DBSRG_OK;
  }
  int chan_of(int io) const { return c->h_ipbs[io / DBSRG_IBO - 1]; }
};

template <class T>
int fetch(dbsrg_ctx *c, std::vector<T> &out, const T *src, int n) {
  out.resize(n);
  if (!src) {
    std::fill(out.begin(), out.end(), T(0));
    return DBSRG_OK;
  }
  if (is_device_ptr(src)) {
    DBSRG_TRY(c, cudaMemcpy(out.data(), src, sizeof(T) * n, cudaMemcpyDeviceToHost));
  } else {
    std::memcpy(out.data(), src, sizeof(T) * n);
  }
  return DBSRG_OK;
}

}  // namespace

int plan_structures(dbsrg_ctx *c, int icase, int itype, int kpol, int n, const int *ipt,
                    const int *k1, const int *k2, const int *k3, const int *k4,
                    const double *cdata, int blo0, int nwin, int nw, void *dev,
                    cudaStream_t ss, StructPlan **out, const int *wstart) {
  const int ns = c->g.ns, ks = c->g.ks, nbf = c->nbf;
  int rc;
  auto P = std::unique_ptr<StructPlan>(new StructPlan());
  P->icase = icase;
  P->itype = itype;
  P->kpol = kpol;
  P->n = n;
  P->nbf = nbf;
  // the list in IPT order, on the host
  std::vector<int> h1, h2, h3, h4, hipt;
  std::vector<double> hc;
  if ((rc = fetch(c, h1, k1, n)) || (rc = fetch(c, h2, k2, n)) || (rc = fetch(c, h3, k3, n)) ||
      (rc = fetch(c, h4, k4, n)) || (rc = fetch(c, hc, cdata, n)))
    return rc;
  if (ipt) {
    if ((rc = fetch(c, hipt, ipt, n))) return rc;
    std::vector<int> t1(n), t2(n), t3(n), t4(n);
    std::vector<double> tc(n);
    for (int j = 0; j < n; j++) {
      const int i = hipt[j];
      if (i < 1 || i > n) return set_err(c, DBSRG_ERANGE, "IPT entry out of range");
      t1[j] = h1[i - 1]; t2[j] = h2[i - 1]; t3[j] = h3[i - 1]; t4[j] = h4[i - 1];
      tc[j] = hc[i - 1];
    }
    h1.swap(t1); h2.swap(t2); h3.swap(t3); h4.swap(t4); hc.swap(tc);
  }
  for (int e = 0; e < n; e++)
    if (!std::isfinite(hc[e])) return set_err(c, DBSRG_EINVAL, "non-finite coefficient in list");
  Builder B{c, blo0, nwin, nw, wstart, {}, {}, {}};
  auto orb_ok = [&](int o) { return o >= 1 && o <= nbf; };
  std::vector<int2> pots, vjobs, ljobs;
  std::vector<int> epot(n, -1), ej1(n, 0), ej2(n, 0), elv(n, -1);
  std::map<int, int> potix;
  std::map<long long, int> vix, lix;
  auto pot_of = [&](int key, int *pi) -> int {
    const int a = key / DBSRG_IBO, b = key % DBSRG_IBO;
    if (!orb_ok(a) || !orb_ok(b)) return set_err(c, DBSRG_ERANGE, "orbital index out of range in list");
    auto it = potix.find(key);
    if (it == potix.end()) {
      it = potix.emplace(key, (int)pots.size()).first;
      pots.push_back(make_int2(a, b));
    }
    *pi = it->second;
    return DBSRG_OK;
  };
  auto kap_slot = [&](int orb) -> int {  // 0-based slot of orbital orb's kappa, -1 none
    if ((int)c->h_kbs.size() < nbf) return -1;
    const int kap = c->h_kbs[orb - 1];
    for (int k = 0; k < c->nkap; k++)
      if (c->h_kap[k] == kap) return k;
    return -1;
  };
  auto lvec_of = [&](int orb, int slot) -> int {
    const long long key = (long long)orb * 64 + slot;
    auto it = lix.find(key);
    if (it == lix.end()) {
      it = lix.emplace(key, (int)ljobs.size()).first;
      ljobs.push_back(make_int2(orb, slot));
    }
    return it->second;
  };

  // ---- the case (R_data.f90:68-86; S_data.f90:73-106)
  if (icase == 2 || icase == 3) {
    const bool R = icase == 2;
    const int at = R ? 0 : itype / 10, it = R ? itype : itype % 10;
    if (R && (kpol < 0 || kpol > c->mk)) return set_err(c, DBSRG_ERANGE, "R_data: kpol out of range");
    if (!R && (kpol < 0 || kpol > c->mk + 1))
      return set_err(c, DBSRG_ERANGE, "S_data: kpol out of range");
    P->family = R ? 0 : 1;
    P->na = R ? 4 : 1;
    P->sym = R ? 's' : 'n';
    P->kb = R ? ks : 2 * ks - 1;
    P->sum_amb = it == 1;
    P->bav = it >= 2;
    if (R) {
      P->icv = it == 1 ? 2 : 1;
      for (int a = 0; a < 4; a++) {
        int ip1, ip2, jp1, jp2;
        switch (a) {
          case 0: ip1 = 1; ip2 = 1; jp1 = 1; jp2 = 1; break;
          case 1: ip1 = 2; ip2 = 2; jp1 = 2; jp2 = 2; break;
          case 2: ip1 = 1; ip2 = 1; jp1 = 2; jp2 = 2; break;
          default: ip1 = 2; ip2 = 2; jp1 = 1; jp2 = 1; break;
        }
        P->ttype[a] = a;
        if (it == 1) {  // density of K1 on (ip1,ip2), convol case 2, K2 on (jp1,jp2)
          P->dc1[a] = ip1; P->dc2[a] = ip2; P->ec1[a] = jp1; P->ec2[a] = jp2;
        } else {  // density of K1 on (jp1,jp2), convol case 1, BAV of p(ip1) into half ip2
          P->dc1[a] = jp1; P->dc2[a] = jp2; P->ipo[a] = ip1; P->ipv[a] = ip2;
        }
      }
      P->dir = 'r';
    } else {
      int ip1, ip2, jp1, jp2, in;
      char sv = 'r';
      if (at == 0) {
        switch (it) {
          case 1: ip1 = 1; ip2 = 2; jp1 = 1; jp2 = 2; in = 2; break;
          case 2: ip1 = 1; ip2 = 2; jp1 = 1; jp2 = 2; in = 1; sv = 'r'; break;
          case 3: ip1 = 1; ip2 = 2; jp1 = 1; jp2 = 2; in = 2; sv = 'r'; break;
          case 4: ip1 = 2; ip2 = 1; jp1 = 1; jp2 = 2; in = 1; sv = 'l'; break;
          default: ip1 = 2; ip2 = 1; jp1 = 1; jp2 = 2; in = 2; sv = 'l'; break;
        }
      } else {
        switch (it) {
          case 1: ip1 = 1; ip2 = 2; jp1 = 2; jp2 = 1; in = 2; break;
          case 2: ip1 = 1; ip2 = 2; jp1 = 2; jp2 = 1; in = 1; sv = 'r'; break;
          case 3: ip1 = 2; ip2 = 1; jp1 = 1; jp2 = 2; in = 2; sv = 'r'; break;
          case 4: ip1 = 2; ip2 = 1; jp1 = 2; jp2 = 1; in = 1; sv = 'l'; break;
          default: ip1 = 1; ip2 = 2; jp1 = 1; jp2 = 2; in = 2; sv = 'l'; break;
        }
      }
      P->ttype[0] = at;
      P->icv = in;
      P->dir = sv;
      if (it == 1) {
        P->dc1[0] = ip1; P->dc2[0] = ip2; P->ec1[0] = jp1; P->ec2[0] = jp2;
      } else {  // BAV of p(ip2) into half ip2 (S_data.f90:205-211)
        P->dc1[0] = jp1; P->dc2[0] = jp2; P->ipo[0] = ip2; P->ipv[0] = ip2;
      }
    }
    // entries: potentials, per-entry jobs
    std::vector<int> vq(n, -1);
    for (int e = 0; e < n; e++) {
      int pi;
      if ((rc = pot_of(h1[e], &pi))) return rc;
      epot[e] = pi;
      if (it == 1) {
        const int j1 = h2[e] / DBSRG_IBO, j2 = h2[e] % DBSRG_IBO;
        if (!orb_ok(j1) || !orb_ok(j2))
          return set_err(c, DBSRG_ERANGE, "orbital index out of range in list");
        ej1[e] = j1;
        ej2[e] = j2;
      } else {
        if (!orb_ok(h2[e])) return set_err(c, DBSRG_ERANGE, "orbital index out of range in list");
        const long long key = (long long)pi * (nbf + 1) + h2[e];
        auto f = vix.find(key);
        if (f == vix.end()) {
          f = vix.emplace(key, (int)vjobs.size()).first;
          vjobs.push_back(make_int2(pi, h2[e]));
        }
        vq[e] = f->second;
      }
    }
    P->npot = (int)pots.size();
    P->npv = (int)vjobs.size();
    // terms, atype by atype (Gen_matrix calls R_data per atype), entries in order
    for (int a = 0; a < P->na; a++)
      for (int e = 0; e < n; e++) {
        const int cidx = a * n + e;
        if (it == 1) {  // route by ic = -k3, jc = -k4 (R_data.f90:116-158)
          const int ic = -h3[e], jc = -h4[e], io = -ic, jo = -jc;
          int vi, wi;
          if (ic > 0 && jc > 0) {
            rc = B.hb(ic, jc, cidx);
          } else if (ic < 0 && jc > 0) {
            if (!(rc = B.vch(io, &vi))) rc = B.hv(B.chan_of(io), jc, vi, cidx);
          } else if (ic < 0 && jc < 0) {
            if (!(rc = B.vch(io, &vi)) && !(rc = B.vch(jo, &wi)))
              rc = B.hw(B.chan_of(io), B.chan_of(jo), vi, wi, cidx);
          } else if (ic < 0 && jc == 0) {
            const int o1 = io / DBSRG_IBO, o2 = io % DBSRG_IBO;
            if (!orb_ok(o1) || !orb_ok(o2))
              return set_err(c, DBSRG_ERANGE, "orbital index out of range in list");
            const int ich = c->h_ipbs[o1 - 1], jch = c->h_ipbs[o2 - 1];
            rc = B.target(ich, jch, cidx, 1);
            if (!rc && c->iitar > 0 && ich != jch) rc = B.hx(ich, jch, 0, cidx);
          } else {
            rc = set_err(c, DBSRG_EINVAL, R ? "R_data: unknown structure for itype=1"
                                            : "S_data: unknown structure for itype=1");
          }
        } else {  // ich = k3, io = k4 (R_data.f90:189-206)
          const int ich = h3[e], io = h4[e];
          const int vi = nbf + a * P->npv + vq[e];
          int wi;
          if (io > 0) {
            if (!(rc = B.vch(io, &wi))) rc = B.hw(ich, B.chan_of(io), vi, wi, cidx);
          } else if (io < 0) {
            rc = B.hv(ich, -io, vi, cidx);
          } else {
            rc = set_err(c, DBSRG_EINVAL, R ? "R_data: unknown structure for itype=2"
                                            : "S_data: unknown structure for itype 2-5");
          }
        }
        if (rc) return rc;
      }
    P->copyc = it >= 2;
  } else if (icase == 1) {
    if (c->nkap < 1 || (int)c->h_kbs.size() < nbf)
      return set_err(c, DBSRG_ESTATE, "L_data: no one-electron matrices (dbsrg_set_dhl)");
    P->lval = itype == 1;
    P->lvec = itype <= 2;
    P->copyc = itype >= 2;
    for (int e = 0; e < n; e++) {
      if (std::fabs(hc[e]) < c->eps_c) continue;  // L_data.f90:48,90,115
      const int cidx = e;
      int vi, wi;
      if (itype == 1) {
        const int i1 = h1[e], i2 = h2[e];
        if (!orb_ok(i1) || !orb_ok(i2))
          return set_err(c, DBSRG_ERANGE, "orbital index out of range in list");
        const int ks1 = kap_slot(i1);
        if (ks1 < 0) return set_err(c, DBSRG_EINVAL, "L_data: no one-electron matrix for kappa");
        ej1[e] = i1;
        elv[e] = lvec_of(i2, ks1);
        const int ic = h3[e], jc = h4[e];
        if (ic > 0 && jc > 0) {
          rc = B.hb(ic, jc, cidx);
        } else if (ic < 0 && jc > 0) {
          if (!(rc = B.vch(-ic, &vi))) rc = B.hv(B.chan_of(-ic), jc, vi, cidx);
        } else if (ic < 0 && jc < 0) {
          if (!(rc = B.vch(-ic, &vi)) && !(rc = B.vch(-jc, &wi)))
            rc = B.hw(B.chan_of(-ic), B.chan_of(-jc), vi, wi, cidx);
        } else if (ic < 0 && jc == 0) {
          const int o1 = (-ic) / DBSRG_IBO, o2 = (-ic) % DBSRG_IBO;
          if (!orb_ok(o1) || !orb_ok(o2))
            return set_err(c, DBSRG_ERANGE, "orbital index out of range in list");
          const int ich = c->h_ipbs[o1 - 1], jch = c->h_ipbs[o2 - 1];
          rc = DBSRG_OK;
          if (c->iitar > 0 && ich != jch) rc = B.hx(ich, jch, 0, cidx);
          if (!rc) rc = B.target(ich, jch, cidx, 1);
        } else {
          rc = set_err(c, DBSRG_EINVAL, "L_data: wrong combination of ic,jc for itype=1");
        }
      } else if (itype == 2) {
        const int i1 = h1[e], ich = h2[e], jc = h3[e];
        if (!orb_ok(i1)) return set_err(c, DBSRG_ERANGE, "orbital index out of range in list");
        const int ks1 = kap_slot(i1);
        if (ks1 < 0) return set_err(c, DBSRG_EINVAL, "L_data: no one-electron matrix for kappa");
        const int lv = lvec_of(i1, ks1);
        elv[e] = lv;
        vi = -1 - lv;  // resolved to the pool index below
        if (jc > 0) {
          rc = B.hv(ich, jc, vi, cidx);
        } else if (jc < 0) {
          if (!(rc = B.vch(-jc, &wi))) rc = B.hw(ich, B.chan_of(-jc), vi, wi, cidx);
        } else {
          rc = set_err(c, DBSRG_EINVAL, "L_data: wrong value jc = 0 for itype=2");
        }
      } else {
        const int i1 = h1[e], j1 = h2[e];
        if (!orb_ok(i1) || !orb_ok(j1))
          return set_err(c, DBSRG_ERANGE, "orbital index out of range in list");
        const int ich = c->h_ipbs[i1 - 1], jch = c->h_ipbs[j1 - 1];
        if (c->h_kbs[i1 - 1] != c->h_kbs[j1 - 1])
          return set_err(c, DBSRG_EINVAL, "L_data: different kappa, itype=3");
        const int ks1 = kap_slot(i1);
        if (ks1 < 0) return set_err(c, DBSRG_EINVAL, "L_data: unknown kappa, itype=3");
        if (ich == jch || c->iitar > 1)
          rc = B.hx(ich, jch, 1 + ks1, cidx);
        else if (c->check_target == 1)
          rc = B.target(ich, jch, cidx, 2);
      }
      if (rc) return rc;
    }
    P->nlv = (int)ljobs.size();
    // L vectors follow the overlap vectors in the pool
    for (auto &bt : B.bterms) {
      if (bt.second.kind <= 2 && bt.second.a < 0) bt.second.a = nbf + (-1 - bt.second.a);
      if (bt.second.kind <= 2 && bt.second.b < 0) bt.second.b = nbf + (-1 - bt.second.b);
    }
    for (auto &ht : B.hvterms)
      if (ht.second.a < 0) ht.second.a = nbf + (-1 - ht.second.a);
  } else if (icase == 0) {
    P->copyc = true;
    for (int e = 0; e < n; e++) {
      if (std::fabs(hc[e]) < c->eps_c) continue;  // O_data.f90:35,42,66
      int vi;
      if (itype == 1) {
        rc = B.hb(h1[e], h2[e], e);
      } else if (itype == 2) {
        if (!(rc = B.vch(h1[e], &vi))) rc = B.hv(B.chan_of(h1[e]), h2[e], vi, e);
      } else {  // itype 4
        const int o1 = h1[e] / DBSRG_IBO, o2 = h1[e] % DBSRG_IBO;
        if (!orb_ok(o1) || !orb_ok(o2))
          return set_err(c, DBSRG_ERANGE, "orbital index out of range in list");
        const int ich = c->h_ipbs[o1 - 1], jch = c->h_ipbs[o2 - 1];
        rc = B.target(ich, jch, e, 2);
        if (!rc && c->iitar > 1 && ich != jch) rc = B.hx(ich, jch, 0, e);
      }
      if (rc) return rc;
    }
  } else {
    return set_err(c, DBSRG_EINVAL, "unsupported icase");
  }

  // ---- groups: block terms per window (block order, terms in list order)
  std::stable_sort(B.bterms.begin(), B.bterms.end(),
                   [](const std::pair<int, StTerm> &x, const std::pair<int, StTerm> &y) {
                     return x.first < y.first;
                   });
  std::stable_sort(B.hvterms.begin(), B.hvterms.end(),
                   [](const std::pair<int, StTerm> &x, const std::pair<int, StTerm> &y) {
                     return x.first < y.first;
                   });
  std::stable_sort(B.scterms.begin(), B.scterms.end(),
                   [](const std::pair<long long, StTerm> &x, const std::pair<long long, StTerm> &y) {
                     return x.first < y.first;
                   });
  std::vector<int> blist, bstart, hvcol, hvstart, scstart;
  std::vector<StTerm> bt, ht, st;
  P->wb.assign(nw + 1, 0);
  for (size_t t = 0; t < B.bterms.size(); t++) {
    if (t == 0 || B.bterms[t].first != B.bterms[t - 1].first) {
      blist.push_back(B.bterms[t].first);
      bstart.push_back((int)t);
      P->wb[B.wof(B.bterms[t].first) + 1]++;
    }
    bt.push_back(B.bterms[t].second);
  }
  bstart.push_back((int)bt.size());
  for (int w = 0; w < nw; w++) P->wb[w + 1] += P->wb[w];
  for (size_t t = 0; t < B.hvterms.size(); t++) {
    if (t == 0 || B.hvterms[t].first != B.hvterms[t - 1].first) {
      hvcol.push_back(B.hvterms[t].first);
      hvstart.push_back((int)t);
    }
    ht.push_back(B.hvterms[t].second);
  }
  hvstart.push_back((int)ht.size());
  for (size_t t = 0; t < B.scterms.size(); t++) {
    if (t == 0 || B.scterms[t].first != B.scterms[t - 1].first) scstart.push_back((int)t);
    st.push_back(B.scterms[t].second);
  }
  scstart.push_back((int)st.size());
  P->nhv = (int)hvcol.size();
  P->nsc = (int)scstart.size() - 1;
  P->wfirst = B.wof(1);
  P->any_block = !bt.empty();

  // ---- device copies (plan memory)
  const size_t N = (size_t)n + 1, na = P->na;
  if (bt.size() > 2 * N * na || ht.size() > 2 * N * na || st.size() > 2 * N * na)
    return set_err(c, DBSRG_ECUDA, "structure terms overflow");
  char *base = (char *)dev;
  auto take = [&](size_t bytes) {
    char *p = base;
    base += al256(bytes);
    return (void *)p;
  };
  P->lcd = (double *)take(sizeof(double) * N);
  P->Ce = (double *)take(sizeof(double) * N * na);
  P->pots = (int2 *)take(sizeof(int2) * N);
  P->vjobs = (int2 *)take(sizeof(int2) * N);
  P->ljobs = (int2 *)take(sizeof(int2) * N);
  P->epot = (int *)take(sizeof(int) * N);
  P->ej1 = (int *)take(sizeof(int) * N);
  P->ej2 = (int *)take(sizeof(int) * N);
  P->elv = (int *)take(sizeof(int) * N);
  P->terms = (StTerm *)take(sizeof(StTerm) * 2 * N * na);
  P->hvterms = (StTerm *)take(sizeof(StTerm) * 2 * N * na);
  P->scterms = (StTerm *)take(sizeof(StTerm) * 2 * N * na);
  P->blist = (int *)take(sizeof(int) * (2 * N * na + 2));
  P->bstart = P->blist + blist.size();
  P->hvcol = (int *)take(sizeof(int) * (2 * N * na + 2));
  P->hvstart = P->hvcol + hvcol.size();
  P->scstart = (int *)take(sizeof(int) * (2 * N * na + 2));
  if ((size_t)((char *)base - (char *)dev) > structure_plan_bytes(c, icase, itype, n))
    return set_err(c, DBSRG_ECUDA, "structure plan overflow");
  auto up = [&](void *dst, const void *src, size_t bytes) -> int {
    return bytes ? copy_in_s(c, dst, src, bytes, ss) : DBSRG_OK;
  };
  if ((rc = up(P->lcd, hc.data(), sizeof(double) * n)) ||
      (rc = up(P->pots, pots.data(), sizeof(int2) * pots.size())) ||
      (rc = up(P->vjobs, vjobs.data(), sizeof(int2) * vjobs.size())) ||
      (rc = up(P->ljobs, ljobs.data(), sizeof(int2) * ljobs.size())) ||
      (rc = up(P->epot, epot.data(), sizeof(int) * n)) ||
      (rc = up(P->ej1, ej1.data(), sizeof(int) * n)) ||
      (rc = up(P->ej2, ej2.data(), sizeof(int) * n)) ||
      (rc = up(P->elv, elv.data(), sizeof(int) * n)) ||
      (rc = up(P->terms, bt.data(), sizeof(StTerm) * bt.size())) ||
      (rc = up(P->hvterms, ht.data(), sizeof(StTerm) * ht.size())) ||
      (rc = up(P->scterms, st.data(), sizeof(StTerm) * st.size())) ||
      (rc = up(P->blist, blist.data(), sizeof(int) * blist.size())) ||
      (rc = up(P->bstart, bstart.data(), sizeof(int) * bstart.size())) ||
      (rc = up(P->hvcol, hvcol.data(), sizeof(int) * hvcol.size())) ||
      (rc = up(P->hvstart, hvstart.data(), sizeof(int) * hvstart.size())) ||
      (rc = up(P->scstart, scstart.data(), sizeof(int) * scstart.size())))
    return rc;
  // the host vectors must outlive the asynchronous copies
  DBSRG_TRY(c, cudaStreamSynchronize(ss));
  (void)ns;
  *out = P.release();
  return DBSRG_OK;
}

int exec_structures(dbsrg_ctx *c, const StructPlan &P, int w, bool prep) {
  const DeviceGrid &g = c->g;
  const int ns = g.ns, ks = g.ks, ms = g.ms, n = P.n, nbf = P.nbf;
  cudaStream_t st = c->stream;
  int rc;
  const int g0 = prep ? 0 : P.wb[w], g1 = prep ? 0 : P.wb[w + 1];
  const bool first = !prep && w == P.wfirst;
  const bool work = prep ? (P.any_block || P.nhv || P.nsc)
                         : (g1 > g0 || (first && (P.nhv > 0 || P.nsc > 0)));
  if (!work) return DBSRG_OK;
  // the full tables the potentials read (FP64 in every form)
  const double *tabs[4] = {nullptr, nullptr, nullptr, nullptr};
  if (P.family >= 0)
    for (int a = 0; a < P.na; a++) {
      rc = P.family == 0 ? get_rtable(c, P.ttype[a], P.kpol, &tabs[a])
                         : get_stable(c, P.ttype[a], P.kpol, &tabs[a]);
      if (rc) return rc;
    }
  if (prep) return DBSRG_OK;
  if (P.nlv > 0 && !c->hd) return set_err(c, DBSRG_ESTATE, "L_data: no one-electron matrices");
  // scratch: pair densities and potentials, then the vector pool
  const size_t per = (size_t)ns * P.kb;
  const size_t nvec = (size_t)nbf + (size_t)P.na * P.npv + P.nlv;
  const size_t xb = al256(sizeof(double) * per * std::max(P.npot, 1));
  if ((rc = ensure_scratch(c, 2 * xb + sizeof(double) * nvec * ms))) return rc;
  double *X = (double *)c->scratch;
  double *Y = (double *)((char *)c->scratch + xb);
  double *pool = (double *)((char *)c->scratch + 2 * xb);
  DBSRG_RUN(c, "k_st_vch", k_st_vch<<<(2 * ns * nbf + 255) / 256, 256, 0, st>>>(
                               ns, nbf, g.fpbs, g.fqbs, c->pq, pool));
  if (P.copyc)
    DBSRG_RUN(c, "k_st_copyc", k_st_copyc<<<(n * P.na + 255) / 256, 256, 0, st>>>(
                                   n, P.na, P.lcd, P.Ce));
  if (P.family >= 0 && P.npot > 0) {
    for (int a = 0; a < P.na; a++) {
      for (int p0 = 0; p0 < P.npot; p0 += 65535) {  // grid y limit
        const int np = std::min(65535, P.npot - p0);
        dim3 gd((unsigned)((per + 255) / 256), (unsigned)np);
        DBSRG_RUN(c, "k_st_density",
                  k_st_density<<<gd, 256, 0, st>>>(ns, ks, P.sym, P.kb, np, P.pots + p0,
                                                   P.dc1[a], P.dc2[a], c->pq, X + per * p0));
      }
      // convol case icv of every pair density with the full table
      if ((rc = band_contract(c, P.kb, P.icv, tabs[a], P.npot, X, Y))) return rc;
      if (P.sum_amb)
        DBSRG_RUN(c, "k_st_sumamb",
                  k_st_sumamb<<<(n + 7) / 8, 256, 0, st>>>(ns, ks, P.sym, P.kb, n, P.epot, P.ej1,
                                                           P.ej2, P.ec1[a], P.ec2[a], c->pq, Y,
                                                           P.lcd, P.Ce + (size_t)a * n));
      for (int q0 = 0; P.bav && q0 < P.npv; q0 += 65535) {
        const int nq = std::min(65535, P.npv - q0);
        dim3 gb((unsigned)((ns + 127) / 128), (unsigned)nq);
        DBSRG_RUN(c, "k_st_bav",
                  k_st_bav<<<gb, 128, 0, st>>>(
                      ns, ks, P.sym, P.dir, P.kb, nq, P.vjobs + q0, P.ipo[a], P.ipv[a], c->pq, Y,
                      pool + (size_t)ms * (nbf + (size_t)a * P.npv + q0)));
      }
    }
  }
  if (P.nlv > 0) {
    double *lpool = pool + (size_t)ms * (nbf + (size_t)P.na * P.npv);
    for (int l0 = 0; l0 < P.nlv; l0 += 65535) {
      const int nl = std::min(65535, P.nlv - l0);
      dim3 gl((unsigned)((ms + 127) / 128), (unsigned)nl);
      DBSRG_RUN(c, "k_st_lvec", k_st_lvec<<<gl, 128, 0, st>>>(ms, nl, P.ljobs + l0, c->hd, c->pq,
                                                              lpool + (size_t)ms * l0));
    }
    if (P.lval)
      DBSRG_RUN(c, "k_st_lval", k_st_lval<<<(n + 7) / 8, 256, 0, st>>>(
                                    ms, n, P.ej1, P.elv, c->pq, lpool, P.lcd, P.Ce));
  }
  // terms of this window's blocks
  for (int t = g0; t < g1; t += 65535) {
    const int nb = std::min(65535, g1 - t);
    dim3 grid((unsigned)((ms + 127) / 128), (unsigned)((ms + 31) / 32), (unsigned)nb);
    DBSRG_RUN(c, "k_st_block_terms",
              k_st_block_terms<<<grid, 128, 0, st>>>(ms, P.blist + t, P.bstart + t, P.terms,
                                                     P.Ce, pool, g.fppqq, c->hd, hch_base(c)));
  }
  if (first && P.nhv > 0) {
    if (!c->hcp) return set_err(c, DBSRG_ESTATE, "no perturbers allocated");
    for (int t = 0; t < P.nhv; t += 65535) {
      dim3 grid((unsigned)((ms + 127) / 128), (unsigned)std::min(65535, P.nhv - t));
      DBSRG_RUN(c, "k_st_hv_terms",
                k_st_hv_terms<<<grid, 128, 0, st>>>(ms, P.hvcol + t, P.hvstart + t, P.hvterms,
                                                    P.Ce, pool, c->hcp));
    }
  }
  if (first && P.nsc > 0)  // one thread per scalar: a 1-D grid of ceil(nsc/128) blocks
    DBSRG_RUN(c, "k_st_scalar_terms",
              k_st_scalar_terms<<<(P.nsc + 127) / 128, 128, 0, st>>>(
                  P.nsc, P.scstart, P.scterms, P.Ce, c->hp, c->htarg, c->otarg));
  return DBSRG_OK;
}

int zero_structures(dbsrg_ctx *c) {
  const size_t ms = c->g.ms;
  if (c->hcp) DBSRG_TRY(c, cudaMemsetAsync(c->hcp, 0, sizeof(double) * ms * c->iicb, c->stream));
  if (c->hp) DBSRG_TRY(c, cudaMemsetAsync(c->hp, 0, sizeof(double) * c->iibb, c->stream));
  const size_t nt = (size_t)c->ntarg * (c->ntarg + 1) / 2;
  if (c->htarg) DBSRG_TRY(c, cudaMemsetAsync(c->htarg, 0, sizeof(double) * nt, c->stream));
  if (c->otarg) DBSRG_TRY(c, cudaMemsetAsync(c->otarg, 0, sizeof(double) * nt, c->stream));
  return DBSRG_OK;
}

void free_structures(dbsrg_ctx *c) {
  for (double **p : {&c->hcp, &c->hp, &c->htarg, &c->otarg, &c->hd}) {
    if (*p) cudaFree(*p);
    *p = nullptr;
  }
}

// ---------------------------------------------------------------------------
// C ABI of the matrix parts beside hch
#define ST_SETTLE(c)               \
  do {                             \
    if ((c)->pending) {            \
      int _r = drain(c);           \
      if (_r) return _r;           \
    }                              \
  } while (0)

extern "C" {

int dbsrg_alloc_perturbers(dbsrg_ctx *c, int npert, const int *icb, int iicb, const int *ibb,
                           int iibb) {
  if (!c) return DBSRG_EINVAL;
  if (!c->hch) return set_err(c, DBSRG_ESTATE, "no matrix allocated");
  if (npert < 0 || (npert > 0 && (!icb || !ibb || iicb < 0 || iibb < 0)))
    return set_err(c, DBSRG_EINVAL, "bad perturber arguments");
  cudaSetDevice(c->device);
  ST_SETTLE(c);
  graph_drop(c);  // frees memory a captured assembly names
  for (double **p : {&c->hcp, &c->hp}) {
    if (*p) cudaFree(*p);
    *p = nullptr;
  }
  c->npert = c->iicb = c->iibb = 0;
  c->h_icb.clear();
  c->h_ibb.clear();
  if (npert == 0) return DBSRG_OK;
  std::vector<int> a((size_t)c->nch * npert), b((size_t)npert * npert);
  int rc;
  if ((rc = fetch(c, a, icb, (int)a.size())) || (rc = fetch(c, b, ibb, (int)b.size()))) return rc;
  for (int v : a)
    if (v < 0 || v > iicb) return set_err(c, DBSRG_ERANGE, "icb entry out of range");
  for (int v : b)
    if (v < 0 || v > iibb) return set_err(c, DBSRG_ERANGE, "ibb entry out of range");
  const size_t ms = c->g.ms;
  DBSRG_TRY(c, cudaMalloc((void **)&c->hcp, sizeof(double) * ms * std::max(iicb, 1)));
  DBSRG_TRY(c, cudaMalloc((void **)&c->hp, sizeof(double) * std::max(iibb, 1)));
  c->npert = npert;
  c->iicb = iicb;
  c->iibb = iibb;
  c->h_icb.swap(a);
  c->h_ibb.swap(b);
  if ((rc = zero_structures(c))) return rc;
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  return DBSRG_OK;
}

int dbsrg_get_perturbers(dbsrg_ctx *c, double *hcp, double *hp) {
  if (!c) return DBSRG_EINVAL;
  cudaSetDevice(c->device);
  ST_SETTLE(c);
  if (c->npert == 0) return set_err(c, DBSRG_ESTATE, "no perturbers allocated");
  int rc;
  if (hcp && (rc = copy_out(c, hcp, c->hcp, sizeof(double) * c->g.ms * c->iicb))) return rc;
  if (hp && (rc = copy_out(c, hp, c->hp, sizeof(double) * c->iibb))) return rc;
  return DBSRG_OK;
}

int dbsrg_set_targets(dbsrg_ctx *c, int ntarg, const int *iptar, int iitar, int check_target) {
  if (!c) return DBSRG_EINVAL;
  if (!c->hch) return set_err(c, DBSRG_ESTATE, "no matrix allocated");
  if (ntarg < 0 || (ntarg > 0 && !iptar)) return set_err(c, DBSRG_EINVAL, "bad target arguments");
  cudaSetDevice(c->device);
  ST_SETTLE(c);
  graph_drop(c);  // frees memory a captured assembly names
  for (double **p : {&c->htarg, &c->otarg}) {
    if (*p) cudaFree(*p);
    *p = nullptr;
  }
  c->ntarg = 0;
  c->iitar = iitar;
  c->check_target = check_target;
  c->h_iptar.clear();
  if (ntarg == 0) return DBSRG_OK;
  std::vector<int> t(c->nch);
  int rc;
  if ((rc = fetch(c, t, iptar, c->nch))) return rc;
  for (int v : t)
    if (v < 1 || v > ntarg) return set_err(c, DBSRG_ERANGE, "iptar entry out of range");
  const size_t nt = (size_t)ntarg * (ntarg + 1) / 2;
  DBSRG_TRY(c, cudaMalloc((void **)&c->htarg, sizeof(double) * nt));
  DBSRG_TRY(c, cudaMalloc((void **)&c->otarg, sizeof(double) * nt));
  c->ntarg = ntarg;
  c->h_iptar.swap(t);
  if ((rc = zero_structures(c))) return rc;
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  return DBSRG_OK;
}

int dbsrg_get_targets(dbsrg_ctx *c, double *htarg, double *otarg) {
  if (!c) return DBSRG_EINVAL;
  cudaSetDevice(c->device);
  ST_SETTLE(c);
  if (c->ntarg == 0) return set_err(c, DBSRG_ESTATE, "no targets set");
  const size_t nt = (size_t)c->ntarg * (c->ntarg + 1) / 2;
  int rc;
  if (htarg && (rc = copy_out(c, htarg, c->htarg, sizeof(double) * nt))) return rc;
  if (otarg && (rc = copy_out(c, otarg, c->otarg, sizeof(double) * nt))) return rc;
  return DBSRG_OK;
}

int dbsrg_set_dhl(dbsrg_ctx *c, int nkap, const int *kap_list, const double *hd, const int *kbs) {
  if (!c) return DBSRG_EINVAL;
  if (c->nbf < 1) return set_err(c, DBSRG_ESTATE, "no orbitals set");
  if (nkap < 0 || nkap > 64 || (nkap > 0 && (!kap_list || !hd || !kbs)))
    return set_err(c, DBSRG_EINVAL, "bad one-electron arguments");
  cudaSetDevice(c->device);
  ST_SETTLE(c);
  graph_drop(c);  // frees memory a captured assembly names
  if (c->hd) cudaFree(c->hd);
  c->hd = nullptr;
  c->nkap = 0;
  c->h_kap.clear();
  c->h_kbs.clear();
  if (nkap == 0) return DBSRG_OK;
  std::vector<int> kl(nkap), kb(c->nbf);
  int rc;
  if ((rc = fetch(c, kl, kap_list, nkap)) || (rc = fetch(c, kb, kbs, c->nbf))) return rc;
  const size_t bytes = sizeof(double) * c->g.ms * c->g.ms * nkap;
  DBSRG_TRY(c, cudaMalloc((void **)&c->hd, bytes));
  if ((rc = copy_in(c, c->hd, hd, bytes))) return rc;
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  c->nkap = nkap;
  c->h_kap.swap(kl);
  c->h_kbs.swap(kb);
  return DBSRG_OK;
}

int dbsrg_set_eps_c(dbsrg_ctx *c, double eps_c) {
  if (!c) return DBSRG_EINVAL;
  if (!(eps_c >= 0.0)) return set_err(c, DBSRG_EINVAL, "eps_c < 0");
  ST_SETTLE(c);
  c->eps_c = eps_c;
  return DBSRG_OK;
}

int dbsrg_update_hw(dbsrg_ctx *c, int ich, int jch, const double *v, const double *w, double cc) {
  if (!c) return DBSRG_EINVAL;
  if (!c->hch) return set_err(c, DBSRG_ESTATE, "no matrix allocated");
  if (!v || !w) return set_err(c, DBSRG_EINVAL, "null vector");
  cudaSetDevice(c->device);
  ST_SETTLE(c);
  if (ich < 1 || jch < 1 || ich > c->nch || jch > c->nch)
    return set_err(c, DBSRG_ERANGE, "UPDATE_HW: channel out of range");
  const int b = c->h_icc[(ich - 1) + (size_t)c->nch * (jch - 1)];
  if (b < 1 || b > c->iicc) return set_err(c, DBSRG_ERANGE, "UPDATE_HW: i out of range");
  if (!in_window(c, b)) return DBSRG_OK;
  const int ms = c->g.ms;
  int rc;
  if ((rc = ensure_scratch2(c, sizeof(double) * 2 * ms))) return rc;
  double *dv = (double *)c->scratch2, *dw = dv + ms;
  if ((rc = copy_in(c, dv, v, sizeof(double) * ms)) || (rc = copy_in(c, dw, w, sizeof(double) * ms)))
    return rc;
  const int kind = ich > jch ? 0 : (ich < jch ? 1 : 2);
  const size_t nn = (size_t)ms * ms;
  DBSRG_RUN(c, "k_st_hw1", k_st_hw1<<<(unsigned)((nn + 255) / 256), 256, 0, c->stream>>>(
                               ms, kind, cc, dv, dw, hch_base(c) + (size_t)(b - 1) * nn));
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  return DBSRG_OK;
}

int dbsrg_update_hv(dbsrg_ctx *c, int ich, int ip, const double *v, double cc) {
  if (!c) return DBSRG_EINVAL;
  if (!v) return set_err(c, DBSRG_EINVAL, "null vector");
  cudaSetDevice(c->device);
  ST_SETTLE(c);
  if (ich < 1 || ich > c->nch)
    return set_err(c, DBSRG_ERANGE, "UPDATE_HV: channel index is out of range");
  if (ip < 1 || ip > c->npert)
    return set_err(c, DBSRG_ERANGE, "UPDATE_HV: bound index is out of range");
  const int i = c->h_icb[(ich - 1) + (size_t)c->nch * (ip - 1)];
  if (i < 1 || i > c->iicb) return set_err(c, DBSRG_ERANGE, "UPDATE_HV: ich, ip out of range");
  const int ms = c->g.ms;
  int rc;
  if ((rc = ensure_scratch2(c, sizeof(double) * ms))) return rc;
  if ((rc = copy_in(c, c->scratch2, v, sizeof(double) * ms))) return rc;
  DBSRG_RUN(c, "k_st_hv1", k_st_hv1<<<(ms + 255) / 256, 256, 0, c->stream>>>(
                               ms, cc, (const double *)c->scratch2, c->hcp + (size_t)ms * (i - 1)));
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  return DBSRG_OK;
}

int dbsrg_update_hb(dbsrg_ctx *c, int ic, int jc, double cc) {
  if (!c) return DBSRG_EINVAL;
  cudaSetDevice(c->device);
  ST_SETTLE(c);
  if (ic > c->npert || jc > c->npert || ic <= 0 || jc <= 0)
    return set_err(c, DBSRG_ERANGE, "UPDATE_HB: index is out of range");
  const int i = c->h_ibb[(ic - 1) + (size_t)c->npert * (jc - 1)];
  if (i < 1 || i > c->iibb) return set_err(c, DBSRG_ERANGE, "UPDATE_HB: ic, jc out of range");
  DBSRG_RUN(c, "k_st_hb1", k_st_hb1<<<1, 32, 0, c->stream>>>(cc, c->hp + (i - 1)));
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  return DBSRG_OK;
}

int dbsrg_scale_matrix(dbsrg_ctx *c, double s) {
  if (!c) return DBSRG_EINVAL;
  if (!c->hch) return set_err(c, DBSRG_ESTATE, "no matrix allocated");
  cudaSetDevice(c->device);
  ST_SETTLE(c);
  const size_t ms = c->g.ms;
  struct {
    double *p;
    size_t n;
  } parts[] = {{c->hch, ms * ms * (size_t)c->wcap}, {c->hcp, ms * (size_t)c->iicb},
               {c->hp, (size_t)c->iibb}};
  for (auto &q : parts) {
    if (!q.p || q.n == 0) continue;
    const unsigned nb = (unsigned)std::min<size_t>((q.n + 255) / 256, (size_t)c->nsm * 8);
    DBSRG_RUN(c, "k_st_scale", k_st_scale<<<nb, 256, 0, c->stream>>>(q.n, s, q.p));
  }
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  return DBSRG_OK;
}

}  // extern "C"
