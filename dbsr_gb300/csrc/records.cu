// records.cu -- the dbsr_mat.nnn write-out of DBSR_MAT3 from the
// device-resident matrix:
//  * dbsrg_record_header: SUB1's records after Diag_channels
//    (sub1.f90:164-168): (ns, nch, npert, nsp, nsq), (nsol), (jpsol(0:nch)),
//    (eval(1:nsol)), (the channel solutions diag(1:ms, 1:ipsol(ich), ich)
//    of every channel, one record);
//  * dbsrg_record_matrix: Record_matrix (record_matrix.f90:2-60): for every
//    channel pair ich > jch with a block whose largest element is at least
//    1e-20, the records (ich, jch) and c(1:ni, 1:nj) = D_ich^T H D_jch;
//    for every channel-perturber vector with such an element, (nch+ip, ich)
//    and w(1:ni) = D_ich^T hcp(:, k); for every nonzero perturber-perturber
//    element, (nch+ip, nch+jp) and hp(k); then (0, 0); with icase = 0 the
//    overlaps array of the check that follows (Check_mat);
//  * dbsrg_record_acf: the closing records (mk) and (bcf(nch, nch, 0:mk))
//    (sub1.f90:286-287).
// Records are Fortran sequential unformatted records as gfortran writes
// them: a 4-byte length, the bytes, the same 4-byte length, all in the
// machine's byte order.  The block transformation runs on the device
// (dbsrg_channel_basis, which leaves hch transformed); the device-to-host
// copies carry only the ni x nj corners that are written.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "internal.cuh"

extern "C" int dbsrg_channel_basis(dbsrg_ctx *c, const double *sol, const int *nsol, double *out);

namespace {

// out[b] = max |x| over the n elements of column b of X (n x nb, ld n)
__global__ void k_col_maxabs(size_t n, const double *X, double *out) {
  __shared__ double sm[256];
  const double *x = X + n * blockIdx.x;
  double m = 0.0;
  for (size_t i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(x[i]));
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + h]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sm[0];
}

// w(i, r) = sum_m D(m, i, ich_r) hcp(m, k_r), i < ni_r, for the rows r of
// the channel-perturber records (one block per row), in the order of
// record_matrix.f90:43 (m ascending)
__global__ void k_pert_rows(int ms, const int *rows, const double *D, const double *hcp,
                            double *W) {
  const int r = blockIdx.x;
  const int ich = rows[3 * r], k = rows[3 * r + 1], ni = rows[3 * r + 2];
  const double *d = D + (size_t)ms * ms * (ich - 1);
  const double *h = hcp + (size_t)ms * (k - 1);
  for (int i = threadIdx.x; i < ni; i += blockDim.x) {
    double s = 0.0;
    for (int m = 0; m < ms; m++) s = s + d[m + (size_t)ms * i] * h[m];
    W[(size_t)ms * r + i] = s;
  }
}

bool put_record(FILE *f, const void *p, size_t n) {
  if (n > 0x7fffffffu) return false;
  const int32_t len = (int32_t)n;
  return fwrite(&len, 4, 1, f) == 1 && (n == 0 || fwrite(p, 1, n, f) == n) &&
         fwrite(&len, 4, 1, f) == 1;
}

bool put_ints(FILE *f, std::initializer_list<int32_t> v) {
  std::vector<int32_t> a(v);
  return put_record(f, a.data(), a.size() * 4);
}

}  // namespace

extern "C" int dbsrg_record_header(dbsrg_ctx *c, const char *path, int nsp, int nsq,
                                   const double *sol, const double *eval, const int *nsol) {
  if (!c) return DBSRG_EINVAL;
  if (!path || !sol || !eval || !nsol) return set_err(c, DBSRG_EINVAL, "record_header: null argument");
  if (is_device_ptr(eval) || is_device_ptr(nsol))
    return set_err(c, DBSRG_EINVAL, "record_header: eval and nsol are host arrays");
  if (!c->hmem) return set_err(c, DBSRG_ESTATE, "record_header: no matrix allocated");
  const int ms = c->g.ms, nch = c->nch;
  for (int i = 0; i < nch; i++)
    if (nsol[i] < 0 || nsol[i] > ms) return set_err(c, DBSRG_ERANGE, "record_header: nsol");
  // the solutions on the host (ms x ms per channel)
  std::vector<double> hs;
  const double *S = sol;
  if (is_device_ptr(sol)) {
    hs.resize((size_t)ms * ms * nch);
    int rc = copy_out(c, hs.data(), sol, hs.size() * 8);
    if (rc) return rc;
    S = hs.data();
  }
  std::vector<int32_t> jpsol(nch + 1, 0);
  for (int i = 1; i <= nch; i++) jpsol[i] = jpsol[i - 1] + nsol[i - 1];
  const int ntot = jpsol[nch];
  std::vector<double> ev, dv;
  ev.reserve(ntot);
  dv.reserve((size_t)ms * ntot);
  for (int ich = 1; ich <= nch; ich++)
    for (int js = 1; js <= nsol[ich - 1]; js++) {
      ev.push_back(eval[(js - 1) + (size_t)ms * (ich - 1)]);
      const double *col = S + (size_t)ms * (js - 1) + (size_t)ms * ms * (ich - 1);
      dv.insert(dv.end(), col, col + ms);
    }
  FILE *f = fopen(path, "wb");  // rewind(nui) and the first write truncate
  if (!f) return set_err(c, DBSRG_EIO, "record_header: cannot open file");
  bool ok = put_ints(f, {c->g.ns, nch, c->npert, nsp, nsq}) && put_ints(f, {ntot}) &&
            put_record(f, jpsol.data(), jpsol.size() * 4) &&
            put_record(f, ev.data(), ev.size() * 8) && put_record(f, dv.data(), dv.size() * 8);
  ok = (fclose(f) == 0) && ok;
  return ok ? DBSRG_OK : set_err(c, DBSRG_EIO, "record_header: write failed");
}

extern "C" int dbsrg_record_matrix(dbsrg_ctx *c, const double *sol, const int *nsol, int icase,
                                   const char *path, double *overlaps) {
  if (!c) return DBSRG_EINVAL;
  if (!sol || !nsol || !path) return set_err(c, DBSRG_EINVAL, "record_matrix: null argument");
  if (is_device_ptr(nsol) || (overlaps && is_device_ptr(overlaps)))
    return set_err(c, DBSRG_EINVAL, "record_matrix: nsol and overlaps are host arrays");
  if (!c->hmem || c->wcap < c->iicc)
    return set_err(c, DBSRG_ESTATE, "record_matrix: the whole matrix must be held");
  const int ms = c->g.ms, nch = c->nch, npert = c->npert;
  for (int i = 0; i < nch; i++)
    if (nsol[i] < 0 || nsol[i] > ms) return set_err(c, DBSRG_ERANGE, "record_matrix: nsol");
  cudaSetDevice(c->device);
  int rc = drain(c);
  if (rc) return rc;
  cudaStream_t st = c->stream;
  const size_t blk = (size_t)ms * ms;
  const int no = nch + npert;  // overlaps(no, no)
  // the largest element of every block and perturber vector, before the
  // transformation (record_matrix.f90:18, 36)
  double *dmax = nullptr, *dD = nullptr, *dW = nullptr;
  int *drows = nullptr;
  const int nmax = c->iicc + std::max(c->iicb, 0);
  auto cleanup = [&]() {
    for (void *p : {(void *)dmax, (void *)dD, (void *)dW, (void *)drows})
      if (p) cudaFree(p);
  };
  if (cudaMalloc(&dmax, sizeof(double) * std::max(nmax, 1))) {
    cudaGetLastError();
    return set_err(c, DBSRG_ENOMEM, "record_matrix: allocation failed");
  }
  if (c->iicc > 0)
    DBSRG_RUN(c, "k_col_maxabs", k_col_maxabs<<<c->iicc, 256, 0, st>>>(blk, c->hch, dmax));
  if (npert > 0 && c->iicb > 0)
    DBSRG_RUN(c, "k_col_maxabs",
              k_col_maxabs<<<c->iicb, 256, 0, st>>>((size_t)ms, c->hcp, dmax + c->iicc));
  std::vector<double> hmax(std::max(nmax, 1));
  if ((rc = copy_out(c, hmax.data(), dmax, sizeof(double) * nmax))) {
    cleanup();
    return rc;
  }
  // the solutions on the device, once, for the perturber rows
  const double *D = sol;
  if (!is_device_ptr(sol)) {
    if (cudaMalloc(&dD, blk * nch * 8)) {
      cudaGetLastError();
      cleanup();
      return set_err(c, DBSRG_ENOMEM, "record_matrix: allocation failed");
    }
    if ((rc = copy_in(c, dD, sol, blk * nch * 8))) {
      cleanup();
      return rc;
    }
    D = dD;
  }
  // channel-perturber rows: (ich, k, ni) of every record, then w on the device
  std::vector<int> rows, rinfo;  // rinfo: ich, ip per row
  for (int ich = 1; npert > 0 && ich <= nch; ich++)
    for (int ip = 1; ip <= npert; ip++) {
      const int k = c->h_icb[(ich - 1) + (size_t)nch * (ip - 1)];
      if (k < 1 || hmax[c->iicc + k - 1] < 1e-20) continue;
      rows.insert(rows.end(), {ich, k, nsol[ich - 1]});
      rinfo.insert(rinfo.end(), {ich, ip});
    }
  const int nrows = (int)rinfo.size() / 2;
  std::vector<double> hw((size_t)ms * nrows);
  if (nrows > 0) {
    if (cudaMalloc(&drows, sizeof(int) * rows.size()) || cudaMalloc(&dW, 8 * hw.size())) {
      cudaGetLastError();
      cleanup();
      return set_err(c, DBSRG_ENOMEM, "record_matrix: allocation failed");
    }
    if ((rc = copy_in(c, drows, rows.data(), sizeof(int) * rows.size()))) {
      cleanup();
      return rc;
    }
    DBSRG_RUN(c, "k_pert_rows", k_pert_rows<<<nrows, 128, 0, st>>>(ms, drows, D, c->hcp, dW));
    if ((rc = copy_out(c, hw.data(), dW, 8 * hw.size()))) {
      cleanup();
      return rc;
    }
  }
  // the blocks: c = D_ich^T H D_jch in place (top-left ni x nj corner)
  if ((rc = dbsrg_channel_basis(c, D, nsol, nullptr))) {
    cleanup();
    return rc;
  }
  FILE *f = fopen(path, "ab");
  if (!f) {
    cleanup();
    return set_err(c, DBSRG_EIO, "record_matrix: cannot open file");
  }
  bool ok = true;
  std::vector<double> cb;
  for (int ich = 2; ok && ich <= nch; ich++)
    for (int jch = 1; ok && jch < ich; jch++) {
      const int k = c->h_icc[(ich - 1) + (size_t)nch * (jch - 1)];
      if (k < 1 || hmax[k - 1] < 1e-20) continue;
      const int ni = nsol[ich - 1], nj = nsol[jch - 1];
      cb.assign((size_t)ni * nj, 0.0);
      if (ni > 0 && nj > 0) {
        if (cudaMemcpy2DAsync(cb.data(), (size_t)ni * 8, c->hch + (size_t)(k - 1) * blk,
                              (size_t)ms * 8, (size_t)ni * 8, nj, cudaMemcpyDeviceToHost,
                              st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
          fclose(f);
          cleanup();
          return set_err(c, DBSRG_ECUDA, "record_matrix: block copy failed");
        }
      }
      ok = put_ints(f, {ich, jch}) && put_record(f, cb.data(), cb.size() * 8);
      if (icase == 0 && overlaps) {
        double m = 0.0;
        for (double x : cb) m = std::max(m, std::fabs(x));
        overlaps[(ich - 1) + (size_t)no * (jch - 1)] = m;
      }
    }
  for (int r = 0; ok && r < nrows; r++) {
    const int ich = rinfo[2 * r], ip = rinfo[2 * r + 1], ni = nsol[ich - 1];
    const double *w = hw.data() + (size_t)ms * r;
    if (icase == 0 && overlaps) {
      double m = 0.0;
      for (int i = 0; i < ni; i++) m = std::max(m, std::fabs(w[i]));
      overlaps[(nch + ip - 1) + (size_t)no * (ich - 1)] = m;
    }
    ok = put_ints(f, {nch + ip, ich}) && put_record(f, w, (size_t)ni * 8);
  }
  if (ok && npert > 0 && c->iibb > 0) {
    std::vector<double> hp(c->iibb);
    if ((rc = copy_out(c, hp.data(), c->hp, 8 * hp.size()))) {
      fclose(f);
      cleanup();
      return rc;
    }
    for (int ip = 1; ok && ip <= npert; ip++)
      for (int jp = 1; ok && jp <= ip; jp++) {
        const int k = c->h_ibb[(ip - 1) + (size_t)npert * (jp - 1)];
        if (k < 1 || hp[k - 1] == 0.0) continue;
        ok = put_ints(f, {ip + nch, jp + nch}) && put_record(f, &hp[k - 1], 8);
        if (icase == 0 && overlaps)
          overlaps[(nch + ip - 1) + (size_t)no * (nch + jp - 1)] = std::fabs(hp[k - 1]);
      }
  }
  ok = ok && put_ints(f, {0, 0});  // the end of the matrix
  ok = (fclose(f) == 0) && ok;
  cleanup();
  return ok ? DBSRG_OK : set_err(c, DBSRG_EIO, "record_matrix: write failed");
}

extern "C" int dbsrg_record_acf(dbsrg_ctx *c, const char *path, const double *bcf) {
  if (!c) return DBSRG_EINVAL;
  if (!path || !bcf) return set_err(c, DBSRG_EINVAL, "record_acf: null argument");
  if (is_device_ptr(bcf)) return set_err(c, DBSRG_EINVAL, "record_acf: bcf is a host array");
  if (!c->hmem) return set_err(c, DBSRG_ESTATE, "record_acf: no matrix allocated");
  FILE *f = fopen(path, "ab");
  if (!f) return set_err(c, DBSRG_EIO, "record_acf: cannot open file");
  const size_t n = (size_t)c->nch * c->nch * (c->mk + 1);
  bool ok = put_ints(f, {c->mk}) && put_record(f, bcf, n * 8);
  ok = (fclose(f) == 0) && ok;
  return ok ? DBSRG_OK : set_err(c, DBSRG_EIO, "record_acf: write failed");
}
