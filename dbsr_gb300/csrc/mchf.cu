// mchf.cu -- DBSR_MCHF's SCF potential matrices (mchf_matrix.f90) assembled
// by the same kernels as the channel blocks.
//
// mchf_matrix(i) (mchf_matrix.f90:2-251), for an orbital outside the core:
//  * the one-electron entries give qsum(i) = S (at least qsum_min = 1e-8,
//    MOD_dbsr_mchf.f90:55) and the cross terms CI(j); rhs starts as
//    dhl sum_j v_j CI(j) / S / 2 (v_j = (P_j; Q_j), Get_pv_df);
//  * every R^k entry in which orbital i appears is sorted by the pattern of
//    its positions (:98-135) into direct (-1), exchange (-2), Newton (-3)
//    and right-hand-side (orbital j > 0) entries (Add_id4_data, restated as
//    appending to the list of its k), with coefficient C / S;
//  * direct: convol case 1 of the 's' densities of p(:,jj,id3) and
//    p(:,jj,id4) into quadrant (ii,ii); exchange: convol case 4 of the 'x'
//    densities of p(:,ii,id3) and p(:,jj,id4) into (ii,jj); both through
//    the SCF Update_hs.  Those are R_data's itype 3 and itype 4 lists of a
//    one-channel block with K2 = id3, K3 = id4 (the density components of
//    R_data.f90:77-86 and the quadrants of :255-273), the correspondence
//    that hf.cu states for hf_matrix;
//  * right-hand side: for every orbital j, the entries of j as a direct
//    list on their own (one-channel block), whose (ii,ii) quadrant is
//    sum_jj Full_mat_sym(convol case 1 of the densities of type (ii,jj));
//    rhs += that block times v_j (the MATMUL of :201-203 for both ii);
//  * Newton term (newton != 0): per k and type (ii,jj), convol case 4 of
//    the 'x' density of p(:,jj,id3), p(:,jj,id4) of the LAST -3 entry with
//    a nonzero coefficient, unweighted, into hx (ii,jj): the reference
//    writes the convolution of x (the last density) over its weighted sum
//    xx (Convol(ns,ks,xx,x,4,...), :216), and this follows it;
//  * rhs into hfm (:223-241) when irhs > 0 and sum |rhs| >= 1e-8:
//    hfm += SS fppqq + rhs vv^T + vv rhs^T with SS = -rhs.v_i, vv = fppqq v_i,
//    and rhs = 0; then hfm = dhl + hfm, rhs = -rhs, e(i) = v_i.(hfm v_i - rhs).
// core_matrix(i) (:255-346), for a core orbital: hfm = (qsum(i) hd + direct
// and exchange lists with a(i,j,k), b(i,j,k) times qsum(i) qsum(j), or
// qsum(i)(qsum(i)-1) for j = i) / qsum(i), and hx from the exchange lists of
// 2 a(i,i,k) qsum(i)(qsum(i)-1) with K2 = K3 = i, / qsum(i).
// The lists run in the precision form dbsrg_set_precision selected; the
// Newton term runs the FP64 table contraction (k_exchange).
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.cuh"

namespace {

// v = (P_io; Q_io) of orbital io (1-based) from pq(ns, 2, nbf)
__global__ void k_orbital_vec(int ns, const double *pq, int io, double *v) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < 2 * ns) v[q] = pq[(size_t)2 * ns * (io - 1) + q];
}

// y(r) += sum_q H(r,q) v(q) (q ascending), H ms x ms
__global__ void k_mv_acc(int ms, const double *H, const double *v, double *y) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= ms) return;
  double s = 0.0;
  for (int q = 0; q < ms; q++) s = s + H[r + (size_t)ms * q] * v[q];
  y[r] = y[r] + s;
}

// X(i,j) = p1(i) p2(j), the 'x' density
__global__ void k_outer(int ns, const double *p1, const double *p2, double *X) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (size_t)ns * ns) return;
  X[q] = p1[q % ns] * p2[q / ns];
}

// the SCF Update_hs of a full ns x ns result: Y/2 into quadrant (ii,jj) and
// its transpose halved into (jj,ii), in that order per element
__global__ void k_half_update(int ns, int ms, const double *Y, int ii, int jj, double *H) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (size_t)ns * ns) return;
  const int r = (int)(q % ns), c = (int)(q / ns);
  double *h1 = H + (size_t)(ii - 1) * ns + r + (size_t)ms * ((jj - 1) * ns + c);
  double *h2 = H + (size_t)(jj - 1) * ns + r + (size_t)ms * ((ii - 1) * ns + c);
  if (ii == jj) {
    *h1 = *h1 + Y[q] / 2.0;
    *h1 = *h1 + Y[(size_t)c + (size_t)ns * r] / 2.0;
  } else {
    *h1 = *h1 + Y[q] / 2.0;
    *h2 = *h2 + Y[(size_t)c + (size_t)ns * r] / 2.0;
  }
}

__device__ double block_sum(double x, double *sm) {
  sm[threadIdx.x] = x;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) sm[threadIdx.x] = sm[threadIdx.x] + sm[threadIdx.x + h];
    __syncthreads();
  }
  const double s = sm[0];
  __syncthreads();
  return s;
}

// one block: sum |rhs| (below 1e-8: rhs = 0), and for irhs > 0 with a
// nonzero rhs SS = -rhs.v and vv = F v; scal = {apply, SS}
__global__ void __launch_bounds__(1024) k_rhs_prep(int ms, int irhs, double *rhs, const double *v,
                                                   const double *F, double *vv, double *scal) {
  __shared__ double sm[1024];
  double a = 0.0;
  for (int r = threadIdx.x; r < ms; r += blockDim.x) a += fabs(rhs[r]);
  const double srhs = block_sum(a, sm);
  if (srhs < 1e-8)
    for (int r = threadIdx.x; r < ms; r += blockDim.x) rhs[r] = 0.0;
  const bool apply = irhs > 0 && srhs >= 1e-8;
  double b = 0.0;
  for (int r = threadIdx.x; r < ms; r += blockDim.x) b += rhs[r] * v[r];
  const double SS = -block_sum(b, sm);
  for (int r = threadIdx.x; r < ms; r += blockDim.x) {
    double s = 0.0;
    for (int q = 0; q < ms; q++) s = s + F[r + (size_t)ms * q] * v[q];
    vv[r] = s;
  }
  if (threadIdx.x == 0) {
    scal[0] = apply ? 1.0 : 0.0;
    scal[1] = SS;
  }
}

// H = dhl + (H [+ SS F + rhs vv^T + vv rhs^T])
__global__ void k_hfm_final(int ms, double *H, const double *dhl, const double *F,
                            const double *rhs, const double *vv, const double *scal) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (size_t)ms * ms) return;
  const int a = (int)(q % ms), b = (int)(q / ms);
  double h = H[q];
  if (scal[0] != 0.0) {
    h = h + scal[1] * F[q];
    h = h + rhs[a] * vv[b] + rhs[b] * vv[a];
  }
  H[q] = dhl[q] + h;
}

// one block: rhs = -(applied ? 0 : rhs); e = v.(H v - rhs)
__global__ void __launch_bounds__(1024) k_energy(int ms, const double *H, const double *v,
                                                 double *rhs, const double *scal, double *e) {
  __shared__ double sm[1024];
  double acc = 0.0;
  for (int r = threadIdx.x; r < ms; r += blockDim.x) {
    const double x = scal[0] != 0.0 ? 0.0 : rhs[r];
    rhs[r] = -x;
    double s = 0.0;
    for (int q = 0; q < ms; q++) s = s + H[r + (size_t)ms * q] * v[q];
    acc += v[r] * (s + x);
  }
  const double t = block_sum(acc, sm);
  if (threadIdx.x == 0) *e = t;
}

struct Id4 {
  int id2, id3, id4;
  double c;
};

// one list of the one-channel block: K1 = channel pair (1,1), K2 = id3,
// K3 = id4, K4 = 0
int run_list(dbsrg_ctx *c, int itype, int k, const std::vector<const Id4 *> &e) {
  if (e.empty()) return DBSRG_OK;
  std::vector<int> k1(e.size(), DBSRG_IBO + 1), k2(e.size()), k3(e.size()), k4(e.size(), 0);
  std::vector<double> cd(e.size());
  for (size_t q = 0; q < e.size(); q++) {
    k2[q] = e[q]->id3;
    k3[q] = e[q]->id4;
    cd[q] = e[q]->c;
  }
  return dbsrg_gen_matrix(c, 2, itype, k, (int)e.size(), nullptr, k1.data(), k2.data(), k3.data(),
                          k4.data(), cd.data());
}

struct DevBufs {
  double *p = nullptr;
  ~DevBufs() {
    if (p) cudaFree(p);
  }
};

int check_one_channel(dbsrg_ctx *c, int iorb, int kmax, const char *who) {
  if (!c->hmem || c->nch != 1 || c->iicc != 1 || c->wcap < 1)
    return set_err(c, DBSRG_ESTATE, std::string(who) + ": the context must hold a one-channel matrix");
  if (iorb < 1 || iorb > c->nbf) return set_err(c, DBSRG_ERANGE, std::string(who) + ": orbital index");
  if (kmax < 0 || kmax > c->mk) return set_err(c, DBSRG_ERANGE, std::string(who) + ": kmax above mk");
  return DBSRG_OK;
}

}  // namespace

extern "C" int dbsrg_mchf_matrix(dbsrg_ctx *c, int iorb, int kmax, int nl, const int *li1,
                                 const int *li2, const double *lc, int nr, const int *rk,
                                 const int *ri1, const int *ri2, const int *ri3, const int *ri4,
                                 const double *rcoef, const double *dhl, int irhs, int newton,
                                 double eps_c, double *hfm, double *rhs, double *hx, double *e,
                                 double *qsum) {
  if (!c) return DBSRG_EINVAL;
  if (nl < 0 || nr < 0 || (nl > 0 && (!li1 || !li2 || !lc)) ||
      (nr > 0 && (!rk || !ri1 || !ri2 || !ri3 || !ri4 || !rcoef)) || !dhl || !hfm || !rhs || !e ||
      !qsum || (newton && !hx))
    return set_err(c, DBSRG_EINVAL, "mchf_matrix: null argument");
  for (const void *p : {(const void *)li1, (const void *)li2, (const void *)lc, (const void *)rk,
                        (const void *)ri1, (const void *)ri2, (const void *)ri3,
                        (const void *)ri4, (const void *)rcoef, (const void *)e, (const void *)qsum})
    if (p && is_device_ptr(p))
      return set_err(c, DBSRG_EINVAL, "mchf_matrix: lists, e and qsum are host arrays");
  int rc0 = check_one_channel(c, iorb, kmax, "mchf_matrix");
  if (rc0) return rc0;
  const int nbf = c->nbf, i = iorb, ns = c->g.ns, ms = c->g.ms;
  for (int m = 0; m < nl; m++)
    if (li1[m] < 1 || li1[m] > nbf || li2[m] < 1 || li2[m] > nbf)
      return set_err(c, DBSRG_ERANGE, "mchf_matrix: orbital index in the L entries");
  for (int m = 0; m < nr; m++)
    if (rk[m] < 0 || ri1[m] < 1 || ri1[m] > nbf || ri2[m] < 1 || ri2[m] > nbf || ri3[m] < 1 ||
        ri3[m] > nbf || ri4[m] < 1 || ri4[m] > nbf)
      return set_err(c, DBSRG_ERANGE, "mchf_matrix: index in the R^k entries");
  // ---- one-electron entries: S and CI (:59-73)
  double S = 0.0;
  std::vector<double> CI(nbf, 0.0);
  for (int m = 0; m < nl; m++) {
    const int i1 = li1[m], i2 = li2[m];
    if (i1 == i && i2 == i)
      S = S + lc[m];
    else if (i1 == i)
      CI[i2 - 1] = CI[i2 - 1] + lc[m];
    else if (i2 == i)
      CI[i1 - 1] = CI[i1 - 1] + lc[m];
  }
  if (std::fabs(S) < 1e-8) S = 1e-8;
  *qsum = S;
  // ---- the id4 entries of every k (:86-137)
  std::vector<std::vector<Id4>> ids(kmax + 1);
  for (int m = 0; m < nr; m++) {
    const int k = rk[m];
    if (k > kmax) continue;
    const int i1 = ri1[m], i2 = ri2[m], i3 = ri3[m], i4 = ri4[m];
    const double C = rcoef[m] / S;
    if (std::fabs(C) < eps_c) continue;
    const int code = (i == i1) * 1000 + (i == i2) * 100 + (i == i3) * 10 + (i == i4);
    auto add = [&](int t, int a, int b, double v) { ids[k].push_back({t, a, b, v}); };
    switch (code) {
      case 1111: add(-1, i1, i3, 2 * C); add(-3, i1, i3, 4 * C); break;
      case 1010: add(-1, i2, i4, C); break;
      case 101: add(-1, i1, i3, C); break;
      case 1001: add(-2, i2, i3, C); break;
      case 1100: add(-2, i3, i4, C); break;
      case 110: add(-2, i1, i4, C); break;
      case 11: add(-2, i1, i2, C); break;
      case 111: add(-1, i1, i3, C); add(-2, i1, i3, C / 2); add(-3, i1, i3, 3 * C / 2); break;
      case 1011: add(-1, i2, i4, C); add(-2, i2, i4, C / 2); add(-3, i2, i4, 3 * C / 2); break;
      case 1101: add(-1, i1, i3, C); add(-2, i1, i3, C / 2); add(-3, i1, i3, 3 * C / 2); break;
      case 1110: add(-1, i2, i4, C); add(-2, i2, i4, C / 2); add(-3, i2, i4, 3 * C / 2); break;
      case 1000: add(i3, i2, i4, C / 2); break;
      case 100: add(i4, i1, i3, C / 2); break;
      case 10: add(i1, i2, i4, C / 2); break;
      case 1: add(i2, i1, i3, C / 2); break;
      default: break;
    }
  }
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  // device buffers: rhs, v, vv, w (ms each), scal (2), dhl, hx (ms x ms),
  // X, Y (ns x ns)
  const size_t mm = (size_t)ms * ms, nn = (size_t)ns * ns;
  DevBufs buf;
  if (cudaMalloc(&buf.p, 8 * (4 * (size_t)ms + 2 + 2 * mm + 2 * nn))) {
    cudaGetLastError();
    return set_err(c, DBSRG_ENOMEM, "mchf_matrix: allocation failed");
  }
  double *d_rhs = buf.p, *d_v = d_rhs + ms, *d_vv = d_v + ms, *d_w = d_vv + ms;
  double *d_scal = d_w + ms, *d_dhl = d_scal + 2, *d_hx = d_dhl + mm, *d_X = d_hx + mm,
         *d_Y = d_X + nn;
  int rc;
  if ((rc = copy_in(c, d_dhl, dhl, mm * 8))) return rc;
  if (cudaMemsetAsync(d_rhs, 0, 8 * (size_t)ms, st) || cudaMemsetAsync(d_hx, 0, 8 * mm, st))
    return set_err(c, DBSRG_ECUDA, "mchf_matrix: memset failed");
  const unsigned gm = (unsigned)((ms + 127) / 128);
  // rhs = dhl vv, vv = sum_j v_j CI(j) / S / 2 (:75-83), formed on the host
  // from the orbitals' device copy in the reference's order
  bool anyci = false;
  for (double x : CI) anyci = anyci || x != 0.0;
  if (anyci) {
    std::vector<double> hpq((size_t)2 * ns * nbf), vv(ms, 0.0);
    if ((rc = copy_out(c, hpq.data(), c->pq, hpq.size() * 8))) return rc;
    for (int io = 1; io <= nbf; io++) {
      if (CI[io - 1] == 0.0) continue;
      const double *p = hpq.data() + (size_t)2 * ns * (io - 1);
      for (int q = 0; q < ms; q++) vv[q] = vv[q] + p[q] * CI[io - 1] / S / 2.0;
    }
    if ((rc = copy_in(c, d_vv, vv.data(), 8 * (size_t)ms))) return rc;
    DBSRG_RUN(c, "k_mv_acc", k_mv_acc<<<gm, 128, 0, st>>>(ms, d_dhl, d_vv, d_rhs));
  }
  // ---- right-hand side of every orbital j (:187-205)
  for (int j = 1; j <= nbf; j++) {
    bool any = false;
    for (int k = 0; k <= kmax && !any; k++)
      for (const Id4 &x : ids[k]) any = any || x.id2 == j;
    if (!any) continue;
    if ((rc = dbsrg_zero_matrix(c))) return rc;
    for (int k = 0; k <= kmax; k++) {
      std::vector<const Id4 *> e3;
      for (const Id4 &x : ids[k])
        if (x.id2 == j) e3.push_back(&x);
      if ((rc = run_list(c, 3, k, e3))) return rc;
    }
    if ((rc = drain(c))) return rc;
    DBSRG_RUN(c, "k_orbital_vec", k_orbital_vec<<<gm, 128, 0, st>>>(ns, c->pq, j, d_v));
    DBSRG_RUN(c, "k_mv_acc", k_mv_acc<<<gm, 128, 0, st>>>(ms, c->hch, d_v, d_rhs));
  }
  // ---- Newton term (:209-221): the last -3 density of each k, unweighted
  if (newton) {
    static const int ttype[2][2] = {{0, 2}, {3, 1}};
    const unsigned gn = (unsigned)((nn + 255) / 256);
    for (int k = 0; k <= kmax; k++) {
      const Id4 *last = nullptr;
      for (const Id4 &x : ids[k])
        if (x.id2 == -3 && x.c != 0.0) last = &x;
      if (!last) continue;
      for (int ii = 1; ii <= 2; ii++)
        for (int jj = 1; jj <= 2; jj++) {
          const double *tab;
          if ((rc = get_rtable(c, ttype[ii - 1][jj - 1], k, &tab))) return rc;
          const double *p1 = c->pq + (size_t)2 * ns * (last->id3 - 1) + (size_t)ns * (jj - 1);
          const double *p2 = c->pq + (size_t)2 * ns * (last->id4 - 1) + (size_t)ns * (jj - 1);
          DBSRG_RUN(c, "k_outer", k_outer<<<gn, 256, 0, st>>>(ns, p1, p2, d_X));
          if ((rc = exchange_contract(c, tab, 1, d_X, d_Y))) return rc;
          DBSRG_RUN(c, "k_half_update",
                    k_half_update<<<gn, 256, 0, st>>>(ns, ms, d_Y, ii, jj, d_hx));
        }
    }
  }
  // ---- direct and exchange lists (:150-185)
  if ((rc = dbsrg_zero_matrix(c))) return rc;
  for (int k = 0; k <= kmax; k++) {
    std::vector<const Id4 *> e1, e2;
    for (const Id4 &x : ids[k]) {
      if (x.c == 0.0) continue;
      if (x.id2 == -1) e1.push_back(&x);
      if (x.id2 == -2) e2.push_back(&x);
    }
    if ((rc = run_list(c, 3, k, e1))) return rc;
    if ((rc = run_list(c, 4, k, e2))) return rc;
  }
  if ((rc = drain(c))) return rc;
  // ---- rhs into hfm, the final matrix and the energy (:223-249)
  const double *F = c->g.fppqq;
  DBSRG_RUN(c, "k_orbital_vec", k_orbital_vec<<<gm, 128, 0, st>>>(ns, c->pq, i, d_v));
  DBSRG_RUN(c, "k_rhs_prep",
            k_rhs_prep<<<1, 1024, 0, st>>>(ms, irhs, d_rhs, d_v, F, d_vv, d_scal));
  DBSRG_RUN(c, "k_hfm_final",
            k_hfm_final<<<(unsigned)((mm + 255) / 256), 256, 0, st>>>(ms, c->hch, d_dhl, F, d_rhs,
                                                                       d_vv, d_scal));
  DBSRG_RUN(c, "k_energy", k_energy<<<1, 1024, 0, st>>>(ms, c->hch, d_v, d_rhs, d_scal, d_w));
  if ((rc = copy_out(c, hfm, c->hch, mm * 8))) return rc;
  if ((rc = copy_out(c, rhs, d_rhs, 8 * (size_t)ms))) return rc;
  if (newton && (rc = copy_out(c, hx, d_hx, mm * 8))) return rc;
  if ((rc = copy_out(c, e, d_w, 8))) return rc;
  return DBSRG_OK;
}

extern "C" int dbsrg_mchf_core(dbsrg_ctx *c, int iorb, int kmax, const double *a, const double *b,
                               const double *qsum, const double *hd, int newton, double *hfm,
                               double *hx) {
  if (!c) return DBSRG_EINVAL;
  if (!a || !b || !qsum || !hd || !hfm || (newton && !hx))
    return set_err(c, DBSRG_EINVAL, "mchf_core: null argument");
  if (is_device_ptr(a) || is_device_ptr(b) || is_device_ptr(qsum))
    return set_err(c, DBSRG_EINVAL, "mchf_core: a, b and qsum are host arrays");
  int rc = check_one_channel(c, iorb, kmax, "mchf_core");
  if (rc) return rc;
  const int nbf = c->nbf, i = iorb, ms = c->g.ms;
  const double qi = qsum[i - 1];
  if (!(qi != 0.0) || !std::isfinite(qi))
    return set_err(c, DBSRG_EINVAL, "mchf_core: qsum(i) must be finite and nonzero");
  const size_t mm = (size_t)ms * ms;
  auto coef = [&](const double *t, int j, int k) {
    double v = t[(j - 1) + (size_t)nbf * k];
    return i != j ? v * qi * qsum[j - 1] : v * qi * (qi - 1);
  };
  std::vector<Id4> ent;
  std::vector<const Id4 *> e;
  // hfm: direct (a) and exchange (b) lists with K2 = K3 = j, j ascending
  if ((rc = dbsrg_zero_matrix(c))) return rc;
  for (int k = 0; k <= kmax; k++)
    for (int itype = 3; itype <= 4; itype++) {
      ent.clear();
      for (int j = 1; j <= nbf; j++) {
        const double v = coef(itype == 3 ? a : b, j, k);
        if (v != 0.0) ent.push_back({0, j, j, v});
      }
      e.clear();
      for (const Id4 &x : ent) e.push_back(&x);
      if ((rc = run_list(c, itype, k, e))) return rc;
    }
  // qsum(i) hd, then the division by qsum(i) as a product with its
  // reciprocal (within one rounding of the reference's division)
  if ((rc = dbsrg_update_hx(c, 1, 1, hd, qi))) return rc;
  if ((rc = dbsrg_scale_matrix(c, 1.0 / qi))) return rc;
  if ((rc = copy_out(c, hfm, c->hch, mm * 8))) return rc;
  if (newton) {
    if ((rc = dbsrg_zero_matrix(c))) return rc;
    for (int k = 0; k <= kmax; k++) {
      double v = 2.0 * a[(i - 1) + (size_t)nbf * k];
      if (v == 0.0) continue;
      v = v * qi * (qi - 1);
      ent.assign(1, Id4{0, i, i, v});
      e.assign(1, &ent[0]);
      if ((rc = run_list(c, 4, k, e))) return rc;
    }
    if ((rc = dbsrg_scale_matrix(c, 1.0 / qi))) return rc;
    if ((rc = copy_out(c, hx, c->hch, mm * 8))) return rc;
  }
  return DBSRG_OK;
}
