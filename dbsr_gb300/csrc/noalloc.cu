// noalloc.cu -- the exchange contraction of one channel-pair segment with
// no device allocation at all, for callers that cannot call cudaMalloc:
// host programs that must fix their GPU memory footprint when they load the
// library (a partition of device memory agreed between MPI ranks sharing a
// GPU, or a service whose own pool reserves all memory up front), and loops
// that cannot take the device-wide synchronisation an allocation or a free
// may bring.  Every other entry point of this library
// grows its own scratch with cudaMalloc on demand; this one uses instead a
// file-scope device array of fixed size, so its memory is reserved once, on
// every GPU that loads the library, until the process exits.
//
// Limits and sharing:
//   * ns <= DBSRG_NOALLOC_MAX_NS (512): the accumulated exchange density
//     of one segment, ns x ns FP64, lives in g_density_scratch (2 MiB);
//   * all calls on a device share that array, and each call overwrites it
//     completely before reading it; calls whose work overlaps on the GPU
//     (different streams, or host threads) race on it and must be ordered
//     by the caller;
//   * the first call on a device (with that device current) looks up the
//     device address of the array with cudaGetSymbolAddress.  The address
//     belongs to the device's context of that moment: do not use the entry
//     point after a cudaDeviceReset of the device in the same process;
//   * the call is synchronous: it waits on its stream for its own kernels
//     and for the read-back of its error word before it returns.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/dbsrg.h"

#define DBSRG_NOALLOC_MAX_NS 512
#define NA_MAXDEV 64
#define NA_MAXKS 16

// scratch of the accumulated density (ns x ns, column-major) and an error
// word for entries whose orbital indices are out of range
static __device__ __align__(256) double g_density_scratch[DBSRG_NOALLOC_MAX_NS * DBSRG_NOALLOC_MAX_NS];
static __device__ __align__(256) int g_noalloc_err[64];

static double *g_scratch_addr[NA_MAXDEV];
static int *g_err_addr[NA_MAXDEV];
static bool g_ready[NA_MAXDEV];
static std::mutex g_setup_mutex;

namespace {

// xx(i,j) = sum_e c_e * P1_e(i) * P2_e(j): the 'x' density (density,
// dbsr_lib_dbs.f90:2880-2884) accumulated over the entries of one segment
// in list order (R_data.f90:252-255).  Every element is written.
__global__ void k_na_density(int ns, int nbf, int jp1, int jp2, int n, const int *k2,
                             const int *k3, const double *cd, const double *pq, double *xx,
                             int *err) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ns * ns) return;
  int i = q % ns, j = q / ns;
  double acc = 0.0;
  for (int e = 0; e < n; e++) {
    int a = k2[e], b = k3[e];
    if (a < 1 || a > nbf || b < 1 || b > nbf) {
      if (q == 0) atomicExch(err, 1);
      continue;
    }
    double p1 = pq[(size_t)i + (size_t)ns * (jp1 - 1) + (size_t)2 * ns * (a - 1)];
    double p2 = pq[(size_t)j + (size_t)ns * (jp2 - 1) + (size_t)2 * ns * (b - 1)];
    acc = acc + cd[e] * (p1 * p2);
  }
  xx[q] = acc;
}

// convol case 3 with 's','s' storage (dbsr_lib_dbs.f90:2344-2356) as a
// gather: a(x,y) sums the four symmetric images of the table entries that
// the reference scatters into it.
__global__ void k_na_exchange(int ns, int ks, const double *__restrict__ rkb,
                              const double *__restrict__ d, double *__restrict__ out) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ns * ns) return;
  const int x = q % ns + 1, y = q / ns + 1;
  auto T = [&](int i, int j, int ip, int jp) -> double {
    return rkb[(size_t)(i - 1) + (size_t)ns * ((size_t)(j - 1) +
               (size_t)ns * ((size_t)(ip - 1) + (size_t)ks * (size_t)(jp - 1)))];
  };
  auto D = [&](int i, int j) -> double { return d[(size_t)(i - 1) + (size_t)ns * (j - 1)]; };
  double acc = 0.0;
  for (int jp = 1; jp <= ks; jp++)
    for (int ip = 1; ip <= ks; ip++) {
      if (y - jp + 1 >= 1 && x + ip - 1 <= ns)
        acc = fma(T(x, y - jp + 1, ip, jp), D(x + ip - 1, y - jp + 1), acc);
      if (ip > 1 && x - ip + 1 >= 1 && y - jp + 1 >= 1)
        acc = fma(T(x - ip + 1, y - jp + 1, ip, jp), D(x - ip + 1, y - jp + 1), acc);
      if (jp > 1 && x + ip - 1 <= ns && y + jp - 1 <= ns)
        acc = fma(T(x, y, ip, jp), D(x + ip - 1, y + jp - 1), acc);
      if (ip > 1 && jp > 1 && x - ip + 1 >= 1 && y + jp - 1 <= ns)
        acc = fma(T(x - ip + 1, y, ip, jp), D(x - ip + 1, y + jp - 1), acc);
    }
  out[q] = acc;
}

__global__ void k_na_clear(int *err) {
  if (threadIdx.x == 0) err[0] = 0;
}

// device address of the static arrays for the current device (set-up on
// the first call per device, with that device current)
int noalloc_setup(double **scr, int **err) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAXDEV) return DBSRG_ECUDA;
  std::lock_guard<std::mutex> lk(g_setup_mutex);
  if (!g_ready[dev]) {
    void *p = nullptr, *e = nullptr;
    if (cudaGetSymbolAddress(&p, g_density_scratch) != cudaSuccess) return DBSRG_ECUDA;
    if (cudaGetSymbolAddress(&e, g_noalloc_err) != cudaSuccess) return DBSRG_ECUDA;
    g_scratch_addr[dev] = (double *)p;
    g_err_addr[dev] = (int *)e;
    g_ready[dev] = true;
  }
  *scr = g_scratch_addr[dev];
  *err = g_err_addr[dev];
  return DBSRG_OK;
}

}  // namespace

extern "C" int dbsrg_exchange_segment_noalloc(int ns, int ks, const double *rkb,
                                              const double *pq, int nbf, int jp1, int jp2,
                                              int n, const int *k2, const int *k3,
                                              const double *cdata, double *out,
                                              void *stream) {
  if (ns < 1 || ks < 1 || ks > NA_MAXKS || ns < ks || nbf < 1 || n < 0 || !rkb || !pq ||
      !out || (n > 0 && (!k2 || !k3 || !cdata)) || jp1 < 1 || jp1 > 2 || jp2 < 1 || jp2 > 2)
    return DBSRG_EINVAL;
  if (ns > DBSRG_NOALLOC_MAX_NS) return DBSRG_ERANGE;  // beyond the static scratch
  double *scr = nullptr;
  int *err = nullptr;
  int rc = noalloc_setup(&scr, &err);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int nn = ns * ns, nb = (nn + 255) / 256;
  // each launch reports its own status (cudaLaunchKernel), so an error left
  // behind by an earlier call of the process is not taken for this one's
  {
    void *a[] = {&err};
    if (cudaLaunchKernel((const void *)k_na_clear, dim3(1), dim3(32), a, 0, st) != cudaSuccess)
      return DBSRG_ECUDA;
  }
  {
    void *a[] = {(void *)&ns, &nbf, &jp1, &jp2, &n, (void *)&k2, (void *)&k3,
                 (void *)&cdata, (void *)&pq, &scr, &err};
    if (cudaLaunchKernel((const void *)k_na_density, dim3(nb), dim3(256), a, 0, st) !=
        cudaSuccess)
      return DBSRG_ECUDA;
  }
  {
    void *a[] = {(void *)&ns, (void *)&ks, (void *)&rkb, &scr, &out};
    if (cudaLaunchKernel((const void *)k_na_exchange, dim3(nb), dim3(256), a, 0, st) !=
        cudaSuccess)
      return DBSRG_ECUDA;
  }
  int h = 0;
  if (cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return DBSRG_ECUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return DBSRG_ECUDA;
  return h ? DBSRG_ERANGE : DBSRG_OK;
}
