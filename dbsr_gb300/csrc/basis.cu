// basis.cu -- the channel basis of DBSR_MAT3's write-out, on the
// device-resident matrix:
//  * Diag_channels (diag.f90:2-81): per channel, the diagonal block of H and
//    of the overlap restricted to the B-splines the zero conditions keep
//    (iprm, zero_cond.f90:2-56), the generalized symmetric eigenproblem
//    H c = E B c (LAPACK DSYGV there, cuSOLVER sygvd here), the solutions
//    with Edmin <= E <= Edmax and |E| >= Egap, restored to the full B-spline
//    net and signed so that their largest component is positive;
//  * Record_matrix (record_matrix.f90:14-26): every off-diagonal block
//    replaced by c = D_ich^T H D_jch: in the split form as split-BF16
//    tcgen05 products (sgemm.cu), otherwise two DGEMMs through cuBLAS.
// cuSOLVER and cuBLAS are loaded on first use (dlopen), so the assembly
// library itself does not depend on them.
#include <cublas_v2.h>
#include <cusolverDn.h>
#include <dlfcn.h>

#include <cmath>
#include <mutex>
#include <vector>

#include "internal.cuh"

namespace {

struct LinAlg {
  bool ok = false;
  std::string why;
  cusolverStatus_t (*sv_create)(cusolverDnHandle_t *) = nullptr;
  cusolverStatus_t (*sv_destroy)(cusolverDnHandle_t) = nullptr;
  cusolverStatus_t (*sv_stream)(cusolverDnHandle_t, cudaStream_t) = nullptr;
  cusolverStatus_t (*sygvd_size)(cusolverDnHandle_t, cusolverEigType_t, cusolverEigMode_t,
                                 cublasFillMode_t, int, const double *, int, const double *, int,
                                 const double *, int *) = nullptr;
  cusolverStatus_t (*sygvd)(cusolverDnHandle_t, cusolverEigType_t, cusolverEigMode_t,
                            cublasFillMode_t, int, double *, int, double *, int, double *,
                            double *, int, int *) = nullptr;
  cublasStatus_t (*bl_create)(cublasHandle_t *) = nullptr;
  cublasStatus_t (*bl_destroy)(cublasHandle_t) = nullptr;
  cublasStatus_t (*bl_stream)(cublasHandle_t, cudaStream_t) = nullptr;
  cublasStatus_t (*dgemm)(cublasHandle_t, cublasOperation_t, cublasOperation_t, int, int, int,
                          const double *, const double *, int, const double *, int,
                          const double *, double *, int) = nullptr;
};

void *open_first(const char *const *names) {
  for (int i = 0; names[i]; i++)
    if (void *h = dlopen(names[i], RTLD_NOW | RTLD_LOCAL)) return h;
  return nullptr;
}

LinAlg &linalg() {
  static LinAlg L;
  static std::once_flag once;
  std::call_once(once, [] {
    static const char *sv_names[] = {"libcusolver.so.12", "libcusolver.so", nullptr};
    static const char *bl_names[] = {"libcublas.so.13", "libcublas.so", nullptr};
    void *sv = open_first(sv_names), *bl = open_first(bl_names);
    if (!sv || !bl) {
      L.why = "cuSOLVER or cuBLAS not found";
      return;
    }
    auto get = [&](void *h, const char *n) { return dlsym(h, n); };
    L.sv_create = (decltype(L.sv_create))get(sv, "cusolverDnCreate");
    L.sv_destroy = (decltype(L.sv_destroy))get(sv, "cusolverDnDestroy");
    L.sv_stream = (decltype(L.sv_stream))get(sv, "cusolverDnSetStream");
    L.sygvd_size = (decltype(L.sygvd_size))get(sv, "cusolverDnDsygvd_bufferSize");
    L.sygvd = (decltype(L.sygvd))get(sv, "cusolverDnDsygvd");
    L.bl_create = (decltype(L.bl_create))get(bl, "cublasCreate_v2");
    L.bl_destroy = (decltype(L.bl_destroy))get(bl, "cublasDestroy_v2");
    L.bl_stream = (decltype(L.bl_stream))get(bl, "cublasSetStream_v2");
    L.dgemm = (decltype(L.dgemm))get(bl, "cublasDgemm_v2");
    L.ok = L.sv_create && L.sv_destroy && L.sv_stream && L.sygvd_size && L.sygvd &&
           L.bl_create && L.bl_destroy && L.bl_stream && L.dgemm;
    if (!L.ok) L.why = "cuSOLVER/cuBLAS entry points missing";
  });
  return L;
}

// dst(n x n) = src(idx, idx) of an ms x ms column-major block
__global__ void k_gather_sub(int ms, int n, const int *idx, const double *src, double *dst) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n * n) return;
  const int i = q % n, j = q / n;
  dst[q] = src[(size_t)idx[i] + (size_t)ms * idx[j]];
}

// selected eigenvectors (columns sel[s] of V, n x n) back on the full
// B-spline net (zero at removed B-splines), signed so that the first
// component of largest modulus is positive (maxloc, diag.f90:61-62); one
// block per solution
__global__ void k_restore_solutions(int ms, int n, const int *idx, const double *V,
                                    const int *sel, double *out) {
  __shared__ double sv[256];
  __shared__ int si[256];
  const int s = blockIdx.x, t = threadIdx.x;
  const double *v = V + (size_t)n * sel[s];
  double best = -1.0;
  int bi = 0x7fffffff;
  for (int i = t; i < n; i += blockDim.x) {
    const double a = fabs(v[i]);
    if (a > best || (a == best && idx[i] < bi)) {
      best = a;
      bi = idx[i];
    }
  }
  sv[t] = best;
  si[t] = bi;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (t < h && (sv[t + h] > sv[t] || (sv[t + h] == sv[t] && si[t + h] < si[t]))) {
      sv[t] = sv[t + h];
      si[t] = si[t + h];
    }
    __syncthreads();
  }
  const int pos = si[0];
  __shared__ double sign;
  if (t == 0) {
    sign = 1.0;
    for (int i = 0; i < n; i++)
      if (idx[i] == pos) sign = v[i] < 0.0 ? -1.0 : 1.0;
  }
  __syncthreads();
  double *o = out + (size_t)ms * s;
  for (int j = t; j < ms; j += blockDim.x) o[j] = 0.0;
  __syncthreads();
  for (int i = t; i < n; i += blockDim.x) o[idx[i]] = sign * v[i];
}

struct Handles {
  cusolverDnHandle_t sv = nullptr;
  cublasHandle_t bl = nullptr;
};

int handles(dbsrg_ctx *c, Handles &h) {
  LinAlg &L = linalg();
  if (!L.ok) return set_err(c, DBSRG_ESTATE, "channel basis: " + L.why);
  if (!c->sv_handle) {
    cusolverDnHandle_t s;
    if (L.sv_create(&s) != CUSOLVER_STATUS_SUCCESS)
      return set_err(c, DBSRG_ECUDA, "cusolverDnCreate failed");
    c->sv_handle = s;
  }
  if (!c->bl_handle) {
    cublasHandle_t b;
    if (L.bl_create(&b) != CUBLAS_STATUS_SUCCESS)
      return set_err(c, DBSRG_ECUDA, "cublasCreate failed");
    c->bl_handle = b;
  }
  h.sv = (cusolverDnHandle_t)c->sv_handle;
  h.bl = (cublasHandle_t)c->bl_handle;
  L.sv_stream(h.sv, c->stream);
  L.bl_stream(h.bl, c->stream);
  return DBSRG_OK;
}

}  // namespace

void basis_release(dbsrg_ctx *c) {
  LinAlg &L = linalg();
  if (!L.ok) return;
  if (c->sv_handle) L.sv_destroy((cusolverDnHandle_t)c->sv_handle);
  if (c->bl_handle) L.bl_destroy((cublasHandle_t)c->bl_handle);
  c->sv_handle = c->bl_handle = nullptr;
}

extern "C" int dbsrg_diag_channels(dbsrg_ctx *c, const double *bdiag, const int *iprm,
                                   double emin, double emax, double egap, double *sol,
                                   double *eval, int *nsol) {
  if (!c) return DBSRG_EINVAL;
  if (!bdiag || !iprm || !sol || !eval || !nsol)
    return set_err(c, DBSRG_EINVAL, "diag_channels: null argument");
  if (is_device_ptr(eval) || is_device_ptr(nsol) || is_device_ptr(iprm))
    return set_err(c, DBSRG_EINVAL, "diag_channels: iprm, eval and nsol are host arrays");
  if (!c->hmem || c->wcap < c->iicc)
    return set_err(c, DBSRG_ESTATE, "diag_channels: the whole matrix must be held");
  cudaSetDevice(c->device);
  int rc = drain(c);
  if (rc) return rc;
  Handles h;
  if ((rc = handles(c, h))) return rc;
  LinAlg &L = linalg();
  const int ms = c->g.ms, nch = c->nch;
  const size_t blk = (size_t)ms * ms;
  cudaStream_t st = c->stream;
  // device work: B (ms x ms), A and B compact, W, index, selection, work,
  // info, and the restored solutions of one channel
  double *dB = nullptr, *dA = nullptr, *dBc = nullptr, *dW = nullptr, *dS = nullptr;
  int *dI = nullptr, *dSel = nullptr, *dInfo = nullptr;
  double *dWork = nullptr;
  int lwork = 0;
  auto cleanup = [&]() {
    for (void *p : {(void *)dB, (void *)dA, (void *)dBc, (void *)dW, (void *)dS, (void *)dI,
                    (void *)dSel, (void *)dInfo, (void *)dWork})
      if (p) cudaFree(p);
  };
  auto fail = [&](int code, const char *msg) {
    cudaStreamSynchronize(st);
    cleanup();
    return set_err(c, code, msg);
  };
  if (cudaMalloc(&dB, blk * 8) || cudaMalloc(&dA, blk * 8) || cudaMalloc(&dBc, blk * 8) ||
      cudaMalloc(&dW, ms * 8) || cudaMalloc(&dS, blk * 8) || cudaMalloc(&dI, ms * 4) ||
      cudaMalloc(&dSel, ms * 4) || cudaMalloc(&dInfo, 4)) {
    cudaGetLastError();
    return fail(DBSRG_ENOMEM, "diag_channels: allocation failed");
  }
  if (L.sygvd_size(h.sv, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                   ms, dA, ms, dBc, ms, dW, &lwork) != CUSOLVER_STATUS_SUCCESS ||
      cudaMalloc(&dWork, (size_t)std::max(lwork, 1) * 8)) {
    cudaGetLastError();
    return fail(DBSRG_ECUDA, "diag_channels: workspace");
  }
  const bool host_out = !is_device_ptr(sol);
  std::vector<double> w(ms);
  for (int ich = 1; ich <= nch; ich++) {
    nsol[ich - 1] = 0;
    const int k = c->h_icc[(ich - 1) + (size_t)nch * (ich - 1)];
    double *so = sol + (size_t)(ich - 1) * blk;
    double *ev = eval + (size_t)(ich - 1) * ms;  // host
    std::fill(ev, ev + ms, 0.0);
    if (host_out)
      std::fill(so, so + blk, 0.0);
    else
      cudaMemsetAsync(so, 0, blk * 8, st);
    if (k < 1) continue;
    // B-splines kept by the zero conditions (iprm, host)
    std::vector<int> idx;
    for (int j = 0; j < ms; j++)
      if (iprm[(size_t)(ich - 1) * ms + j] != 0) idx.push_back(j);
    const int n = (int)idx.size();
    if (n == 0) continue;
    if ((rc = copy_in(c, dB, bdiag + (size_t)(ich - 1) * blk, blk * 8))) return fail(rc, "copy");
    if ((rc = copy_in(c, dI, idx.data(), sizeof(int) * n))) return fail(rc, "copy");
    const unsigned g = (unsigned)(((size_t)n * n + 255) / 256);
    DBSRG_RUN(c, "k_gather_sub",
              k_gather_sub<<<g, 256, 0, st>>>(ms, n, dI, c->hch + (size_t)(k - 1) * blk, dA));
    DBSRG_RUN(c, "k_gather_sub", k_gather_sub<<<g, 256, 0, st>>>(ms, n, dI, dB, dBc));
    if (L.sygvd(h.sv, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n,
                dA, n, dBc, n, dW, dWork, lwork, dInfo) != CUSOLVER_STATUS_SUCCESS)
      return fail(DBSRG_ECUDA, "diag_channels: cusolverDnDsygvd failed");
    int info = 0;
    cudaMemcpyAsync(&info, dInfo, 4, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(w.data(), dW, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return fail(DBSRG_ECUDA, "diag_channels");
    if (info != 0) return fail(DBSRG_ECUDA, "channel diagonalization failed");
    // solutions in the energy window (diag.f90:46-50), ascending
    std::vector<int> sel;
    for (int i = 0; i < n; i++)
      if (w[i] >= emin && w[i] <= emax && std::fabs(w[i]) >= egap) sel.push_back(i);
    const int ks = (int)sel.size();
    nsol[ich - 1] = ks;
    if (ks == 0) continue;
    for (int s = 0; s < ks; s++) ev[s] = w[sel[s]];
    if ((rc = copy_in(c, dSel, sel.data(), sizeof(int) * ks))) return fail(rc, "copy");
    DBSRG_RUN(c, "k_restore_solutions",
              k_restore_solutions<<<ks, 256, 0, st>>>(ms, n, dI, dA, dSel, host_out ? dS : so));
    if (host_out) {
      cudaMemcpyAsync(so, dS, sizeof(double) * ms * ks, cudaMemcpyDeviceToHost, st);
      if (cudaStreamSynchronize(st) != cudaSuccess) return fail(DBSRG_ECUDA, "diag_channels");
    }
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail(DBSRG_ECUDA, "diag_channels");
  cleanup();
  return DBSRG_OK;
}

extern "C" int dbsrg_channel_basis(dbsrg_ctx *c, const double *sol, const int *nsol,
                                   double *out) {
  if (!c) return DBSRG_EINVAL;
  if (!sol || !nsol) return set_err(c, DBSRG_EINVAL, "channel_basis: null argument");
  if (!c->hmem || c->wcap < c->iicc)
    return set_err(c, DBSRG_ESTATE, "channel_basis: the whole matrix must be held");
  cudaSetDevice(c->device);
  int rc = drain(c);
  if (rc) return rc;
  Handles h;
  if ((rc = handles(c, h))) return rc;
  LinAlg &L = linalg();
  const int ms = c->g.ms, nch = c->nch;
  const size_t blk = (size_t)ms * ms;
  cudaStream_t st = c->stream;
  for (int i = 0; i < nch; i++)
    if (nsol[i] < 0 || nsol[i] > ms) return set_err(c, DBSRG_ERANGE, "channel_basis: nsol");
  // the solutions on the device (ms x ms per channel) and one product buffer
  const double *D = sol;
  double *dD = nullptr, *dWt = nullptr;
  if (!is_device_ptr(sol)) {
    if (cudaMalloc(&dD, blk * nch * 8)) {
      cudaGetLastError();
      return set_err(c, DBSRG_ENOMEM, "channel_basis: allocation failed");
    }
    if ((rc = copy_in(c, dD, sol, blk * nch * 8))) {
      cudaFree(dD);
      return rc;
    }
    D = dD;
  }
  if (cudaMalloc(&dWt, blk * 8)) {
    cudaGetLastError();
    if (dD) cudaFree(dD);
    return set_err(c, DBSRG_ENOMEM, "channel_basis: allocation failed");
  }
  if (c->precision == DBSRG_SPLIT_BF16) {  // split-BF16 tensor-core products (sgemm.cu)
    rc = split_channel_basis(c, D, nsol);
    cudaStreamSynchronize(st);
    cudaFree(dWt);
    if (dD) cudaFree(dD);
    if (rc) return rc;
    if (out) return copy_out(c, out, c->hch, blk * c->iicc * 8);
    return DBSRG_OK;
  }
  const double one = 1.0, zero = 0.0;
  int bad = 0;
  // c = D_ich^T H D_jch for every block of a channel pair ich > jch, in place
  for (int ich = 2; ich <= nch && !bad; ich++)
    for (int jch = 1; jch < ich && !bad; jch++) {
      const int k = c->h_icc[(ich - 1) + (size_t)nch * (jch - 1)];
      if (k < 1) continue;
      const int ni = nsol[ich - 1], nj = nsol[jch - 1];
      double *H = c->hch + (size_t)(k - 1) * blk;
      const double *Di = D + (size_t)(ich - 1) * blk, *Dj = D + (size_t)(jch - 1) * blk;
      if (ni > 0 && nj > 0)
        bad |= L.dgemm(h.bl, CUBLAS_OP_T, CUBLAS_OP_N, ni, ms, ms, &one, Di, ms, H, ms, &zero,
                       dWt, ni) != CUBLAS_STATUS_SUCCESS;
      bad |= cudaMemsetAsync(H, 0, blk * 8, st) != cudaSuccess;
      if (ni > 0 && nj > 0)
        bad |= L.dgemm(h.bl, CUBLAS_OP_N, CUBLAS_OP_N, ni, nj, ms, &one, dWt, ni, Dj, ms, &zero,
                       H, ms) != CUBLAS_STATUS_SUCCESS;
    }
  const cudaError_t e = cudaStreamSynchronize(st);
  cudaFree(dWt);
  if (dD) cudaFree(dD);
  if (bad || e != cudaSuccess) return set_err(c, DBSRG_ECUDA, "channel_basis: DGEMM failed");
  if (out) return copy_out(c, out, c->hch, blk * c->iicc * 8);
  return DBSRG_OK;
}
