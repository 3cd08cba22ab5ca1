// hf.cu -- the SCF potential matrix of one orbital (DBSR_HF hf_matrix,
// hf_matrix.f90:2-70, the Coulomb part) assembled by the same kernels as the
// channel blocks.
//
// hf_matrix(i) adds, for every table type (ii,jj) and multipole k,
//   direct:   convol case 1 of sum_j a(i,j,k) (doubled for j = i) times the
//             's' density of p(:,jj,j) with itself, into quadrant (ii,ii);
//   exchange: convol case 4 of sum_j b(i,j,k) times the 'x' density of
//             p(:,ii,j) and p(:,jj,j), into quadrant (ii,jj);
// both through Update_hs (half into (ii,jj), half transposed into (jj,ii)),
// then hfm = (qsum dhl + that) / qsum.  That is R_data's itype 3 (direct)
// and itype 4 (exchange) lists of a single diagonal channel block (ich = jch)
// with entries K2 = K3 = j: the same densities, tables and quadrants for
// all four PQ types (R_data.f90:77-86, 214-277; Gen_matrix runs one list
// over all four), and UPDATE_HS halves a diagonal block the same way
// (updates.f90:110-179).  Convol cases 3 (R_data) and 4 (hf_matrix) add
// the same products for 's','s' tables (dbsr_lib_dbs.f90:2344-2470, the
// four updates of one table element permuted).  So the potential matrix is
// one dbsrg_gen_matrix call per list on a one-channel matrix, in whichever
// form dbsrg_set_precision selected.
//
// The Breit part (hf_matrix_breit, hf_matrix.f90:91-163, added before the
// division by qsum when mbreit = 2) is the same with S^k tables: for
// itype 0 (ppqq) / 1 (pqqp), k and int = 1..4, the rk4 entries of the orbital
// (kr1 = k + 1000 itype; i = kr3 with int = kr2 and j = kr4, or i = kr4 with
// int = kint(kr2) and j = kr3) give the coefficients of density(p(jp1,j),
// p(jp2,j)), contracted by convol_sk case int into quadrant (ip1,ip2) with
// Update_hs.  Those are S_data's ktypes 10 itype + 5 + int (structures 6-9,
// whose ip/jp and convol cases S_data.f90:74-97 lists identically) on the
// one-channel block with K2 = K3 = j -- for int 1 and 2.  For int 3 and 4
// hf_matrix_breit passes the storage 'x','x' to convol_sk, which has no
// branch for it (dbsr_lib_dbs.f90:2610-2700: only 's','s', 'l','l', 'n','n',
// 'n','l' and 'l','n' are contracted) and returns zeros: the reference's
// Breit exchange terms add nothing, so no list is made for them.
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.cuh"

namespace {

__global__ void k_div(size_t n, double q, double *x) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = x[i] / q;
}

}  // namespace

extern "C" int dbsrg_hf_matrix(dbsrg_ctx *c, int iorb, int kmax, const double *a,
                               const double *b, double qsum, const double *dhl, double *hfm) {
  if (!c) return DBSRG_EINVAL;
  if (!a || !b || !hfm) return set_err(c, DBSRG_EINVAL, "hf_matrix: null argument");
  if (is_device_ptr(a) || is_device_ptr(b))
    return set_err(c, DBSRG_EINVAL, "hf_matrix: a and b are host arrays");
  if (!c->hmem || c->nch != 1 || c->iicc != 1 || c->wcap < 1)
    return set_err(c, DBSRG_ESTATE, "hf_matrix: the context must hold a one-channel matrix");
  if (iorb < 1 || iorb > c->nbf) return set_err(c, DBSRG_ERANGE, "hf_matrix: orbital index");
  if (kmax < 0 || kmax > c->mk) return set_err(c, DBSRG_ERANGE, "hf_matrix: kmax above mk");
  if (!(qsum != 0.0) || !std::isfinite(qsum))
    return set_err(c, DBSRG_EINVAL, "hf_matrix: qsum must be finite and nonzero");
  int rc = dbsrg_zero_matrix(c);
  if (rc) return rc;
  const int nbf = c->nbf;
  std::vector<int> k1, k2, k4;
  std::vector<double> cd;
  for (int k = 0; k <= kmax; k++)
    for (int itype = 3; itype <= 4; itype++) {
      const double *coef = itype == 3 ? a : b;
      k1.clear();
      k2.clear();
      cd.clear();
      for (int j = 1; j <= nbf; j++) {
        double v = coef[(j - 1) + (size_t)nbf * k];
        if (v == 0.0) continue;
        if (itype == 3 && j == iorb) v = v + v;
        k1.push_back(DBSRG_IBO + 1);  // channel pair (1,1)
        k2.push_back(j);
        cd.push_back(v);
      }
      if (cd.empty()) continue;
      k4.assign(k1.size(), 0);
      // entries sorted by (K1,K2,K3,K4) as Add_matrix leaves them: j ascending
      rc = dbsrg_gen_matrix(c, 2, itype, k, (int)cd.size(), nullptr, k1.data(), k2.data(),
                            k2.data(), k4.data(), cd.data());
      if (rc) return rc;
    }
  // Breit part from the rk4 entries of dbsrg_hf_breit_list (hf_matrix.f90:64)
  static const int kint[4] = {2, 1, 4, 3};
  const size_t nrk = c->hf_crk.size();
  for (int itype = 0; nrk && itype <= 1; itype++)
    for (int k = 0; k <= kmax; k++)
      for (int in = 1; in <= 2; in++) {  // int 3/4: zero in the reference (above)
        std::vector<std::pair<int, double>> ent;  // (j, crk) in entry order
        for (size_t ik = 0; ik < nrk; ik++) {
          if (c->hf_kr1[ik] != k + 1000 * itype) continue;
          int jnt, j;
          if (iorb == c->hf_kr3[ik]) {
            jnt = c->hf_kr2[ik];
            j = c->hf_kr4[ik];
          } else if (iorb == c->hf_kr4[ik]) {
            jnt = kint[c->hf_kr2[ik] - 1];
            j = c->hf_kr3[ik];
          } else {
            continue;
          }
          if (jnt == in) ent.push_back({j, c->hf_crk[ik]});
        }
        if (ent.empty()) continue;
        // sorted by K2 = K3 = j as Add_matrix leaves a list
        std::stable_sort(ent.begin(), ent.end(),
                         [](const std::pair<int, double> &x, const std::pair<int, double> &y) {
                           return x.first < y.first;
                         });
        k1.assign(ent.size(), DBSRG_IBO + 1);
        k2.resize(ent.size());
        cd.resize(ent.size());
        for (size_t q = 0; q < ent.size(); q++) {
          k2[q] = ent[q].first;
          cd[q] = ent[q].second;
        }
        k4.assign(ent.size(), 0);
        rc = dbsrg_gen_matrix(c, 3, 10 * itype + 5 + in, k, (int)cd.size(), nullptr, k1.data(),
                              k2.data(), k2.data(), k4.data(), cd.data());
        if (rc) return rc;
      }
  if (dhl && (rc = dbsrg_update_hx(c, 1, 1, dhl, qsum))) return rc;
  if ((rc = dbsrg_get_block(c, 1, 1, hfm))) return rc;
  const size_t n = (size_t)c->g.ms * c->g.ms;
  if (is_device_ptr(hfm)) {
    DBSRG_RUN(c, "k_div", k_div<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, qsum, hfm));
    DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  } else {
    for (size_t q = 0; q < n; q++) hfm[q] = hfm[q] / qsum;
  }
  return DBSRG_OK;
}

extern "C" int dbsrg_hf_breit_list(dbsrg_ctx *c, int nrk, const int *kr1, const int *kr2,
                                   const int *kr3, const int *kr4, const double *crk) {
  if (!c) return DBSRG_EINVAL;
  if (nrk < 0 || (nrk > 0 && (!kr1 || !kr2 || !kr3 || !kr4 || !crk)))
    return set_err(c, DBSRG_EINVAL, "hf_breit_list: bad arguments");
  for (int i = 0; i < nrk; i++) {
    if (kr2[i] < 1 || kr2[i] > 4) return set_err(c, DBSRG_ERANGE, "hf_breit_list: kr2 outside 1..4");
    if (kr1[i] < 0 || kr1[i] % 1000 > c->mk + 1 || kr1[i] / 1000 > 1)
      return set_err(c, DBSRG_ERANGE, "hf_breit_list: kr1 outside k + 1000 itype");
    if (kr3[i] < 1 || kr3[i] > c->nbf || kr4[i] < 1 || kr4[i] > c->nbf)
      return set_err(c, DBSRG_ERANGE, "hf_breit_list: orbital index");
    if (!std::isfinite(crk[i])) return set_err(c, DBSRG_EINVAL, "hf_breit_list: non-finite crk");
  }
  c->hf_kr1.assign(kr1, kr1 + nrk);
  c->hf_kr2.assign(kr2, kr2 + nrk);
  c->hf_kr3.assign(kr3, kr3 + nrk);
  c->hf_kr4.assign(kr4, kr4 + nrk);
  c->hf_crk.assign(crk, crk + nrk);
  return DBSRG_OK;
}
