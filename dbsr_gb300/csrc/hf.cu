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
