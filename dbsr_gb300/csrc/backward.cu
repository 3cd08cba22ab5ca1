// backward.cu -- the energy functional E = sum_e c_e R^k_e(a,b;c,d) over the
// bound orbitals and its gradient with respect to their P/Q B-spline
// coefficients (the direct potentials DBSR_HF and DBSR_MCHF build in their
// SCF step, hf_matrix.f90:2-163).
//
// R^k(a,b;c,d) (rk, dbsr_lib_dbs.f90:3981-4022) sums four table types t with
// electron-1 basis A_t and electron-2 basis B_t (0 PP|PP, 1 QQ|QQ,
// 2 PP|QQ, 3 QQ|PP): R_t = rho1^T T_t rho2 with rho1 the symmetric band
// density of (a,c) in basis A_t and rho2 that of (b,d) in basis B_t.  The
// direct pair potential Kd_t[(b,d)] (factor.cu; the convol case 1 of T_t
// with rho2) is the potential rho2 makes for electron 1, so
//   R_t = sum over the band of rho1 * Kd_t[(b,d)],
//   dR_t/d f_a = Kd_t[(b,d)]~ f_c,  dR_t/d f_c = Kd_t[(b,d)]~ f_a  (basis A_t)
// with K~ the symmetric band matrix of the 's' storage.  The tables are
// symmetric under exchanging the electrons with types 2 and 3 swapped, so
// the potential of rho1 for electron 2 is Kd_swap(t)[(a,c)]:
//   dR_t/d f_b = Kd_swap(t)[(a,c)]~ f_d,  dR_t/d f_d = ... f_b  (basis B_t).
// The pair potentials are built from the cell moments and diagonal cells,
// recomputed when the tables were released.  Every gradient term is a
// vector of ns; the terms are summed per (orbital, component) in entry order
// from a host-built list, so the result is deterministic without atomics.
#include "internal.cuh"

#include <algorithm>
#include <numeric>

namespace {

// electron-1 / electron-2 basis of table type t (1 P, 2 Q), and the type with
// the electrons exchanged
__host__ __device__ inline int TA(int t) { return (t == 0 || t == 2) ? 1 : 2; }
__host__ __device__ inline int TB(int t) { return (t == 0 || t == 3) ? 1 : 2; }
__host__ __device__ inline int SWAP(int t) { return t < 2 ? t : 5 - t; }

struct KdTypes {
  const double *K[4];  // Kd_t[pair][ns*ks], 's' storage
};

// R_e = sum_t sum_{i,ip} rho1_t(i,ip) Kd_t[(b,d)](i,ip), one warp per entry
__global__ void k_rk_energy(int n, int ns, int ks, int nb, const int *ent, const int *ia,
                            const int *ib, const int *ic, const int *id, const int *bmap,
                            const double *pq, KdTypes kd, double *R) {
  const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) / 32), lane = threadIdx.x % 32;
  if (w >= n) return;
  const int e = ent[w];
  const int a = ia[e], b = ib[e], c = ic[e], d = id[e];
  const int pair2 = bmap[b - 1] * nb + bmap[d - 1];
  const size_t per = (size_t)ns * ks;
  double acc = 0.0;
  for (int t = 0; t < 4; t++) {
    const double *fa = pq + (size_t)2 * ns * (a - 1) + (size_t)ns * (TA(t) - 1);
    const double *fc = pq + (size_t)2 * ns * (c - 1) + (size_t)ns * (TA(t) - 1);
    const double *K = kd.K[t] + (size_t)pair2 * per;
    for (int i = lane; i < ns; i += 32) {
      const double ai = fa[i], ci = fc[i];
      double s = K[i] * (ai * ci);
      for (int ip = 2; ip <= ks && i + ip - 1 < ns; ip++) {
        const int j = i + ip - 1;
        s = fma(K[i + (size_t)ns * (ip - 1)], ai * fc[j] + fa[j] * ci, s);
      }
      acc += s;
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) R[e] = acc;
}

// E = sum_e c_e R_e in a fixed order (one block, fixed tree)
__global__ void k_energy_sum(int n, const double *c, const double *R, double *E) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int e = threadIdx.x; e < n; e += 256) s = fma(c[e], R[e], s);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *E = sh[0];
}

// gradient terms: T[(e*4 + t)*4 + role][m] = c_e (K~ f)(m) with
// role 0: target a, K = Kd_t[(b,d)], f = f_c (basis A_t); 1: target c, f = f_a;
// role 2: target b, K = Kd_swap(t)[(a,c)], f = f_d (basis B_t); 3: target d, f = f_b
__global__ void k_rk_grad_terms(int n, int ns, int ks, int nb, const int *ia, const int *ib,
                                const int *ic, const int *id, const double *coef,
                                const int *bmap, const double *pq, KdTypes kd, double *T) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (size_t)n * 16 * ns) return;
  const int m = (int)(q % ns), r = (int)(q / ns) % 4, t = (int)(q / ns / 4) % 4;
  const int e = (int)(q / ((size_t)ns * 16));
  const int a = ia[e], b = ib[e], c = ic[e], d = id[e];
  const int pr = r < 2 ? bmap[b - 1] * nb + bmap[d - 1] : bmap[a - 1] * nb + bmap[c - 1];
  const int comp = r < 2 ? TA(t) : TB(t);
  const int src = r == 0 ? c : r == 1 ? a : r == 2 ? d : b;
  const double *K = kd.K[r < 2 ? t : SWAP(t)] + (size_t)pr * ns * ks;
  const double *f = pq + (size_t)2 * ns * (src - 1) + (size_t)ns * (comp - 1);
  double acc = 0.0;
  for (int j = max(0, m - ks + 1); j <= min(ns - 1, m + ks - 1); j++) {
    const int lo = min(m, j), dl = abs(m - j);
    acc = fma(K[lo + (size_t)ns * dl], f[j], acc);
  }
  T[q] = coef[e] * acc;
}

// grad[(o, comp, m)] = sum over the term list of (o, comp), in list order
__global__ void k_rk_grad_reduce(int ns, int nbf, const int *lstart, const int *lidx,
                                 const double *T, double *grad) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (size_t)ns * 2 * nbf) return;
  const int m = (int)(q % ns);
  const int oc = (int)(q / ns);  // o * 2 + comp (pq layout)
  double acc = 0.0;
  for (int l = lstart[oc]; l < lstart[oc + 1]; l++) acc += T[(size_t)lidx[l] * ns + m];
  grad[q] = acc;
}

}  // namespace

extern "C" int dbsrg_backward(dbsrg_ctx *c, int n, const int *k, const int *i1, const int *i2,
                              const int *i3, const int *i4, const double *coef, double *energy,
                              double *grad) {
  if (!c) return DBSRG_EINVAL;
  int rc;
  if (n < 0 || (n > 0 && (!k || !i1 || !i2 || !i3 || !i4 || !coef)) || !energy)
    return set_err(c, DBSRG_EINVAL, "backward: bad arguments");
  if (!c->pq) return set_err(c, DBSRG_ESTATE, "backward: no orbitals set");
  cudaSetDevice(c->device);
  if (c->pending && (rc = drain(c))) return rc;
  const int ns = c->g.ns, ks = c->g.ks, nbf = c->nbf, nb = c->nbound;
  cudaStream_t st = c->stream;
  // the entries on the host (small: integer keys and coefficients)
  std::vector<int> hk(n), h1(n), h2(n), h3(n), h4(n);
  std::vector<double> hc(n);
  auto fetch = [&](void *dst, const void *src, size_t bytes) -> int {
    if (!bytes) return DBSRG_OK;
    DBSRG_TRY(c, cudaMemcpy(dst, src, bytes,
                            is_device_ptr(src) ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost));
    return DBSRG_OK;
  };
  const size_t ib = sizeof(int) * (size_t)n;
  if ((rc = fetch(hk.data(), k, ib)) || (rc = fetch(h1.data(), i1, ib)) ||
      (rc = fetch(h2.data(), i2, ib)) || (rc = fetch(h3.data(), i3, ib)) ||
      (rc = fetch(h4.data(), i4, ib)) || (rc = fetch(hc.data(), coef, sizeof(double) * n)))
    return rc;
  for (int e = 0; e < n; e++) {
    for (int o : {h1[e], h2[e], h3[e], h4[e]})
      if (o < 1 || o > nbf || c->h_bmap[o - 1] < 0)
        return set_err(c, DBSRG_EINVAL, "backward: orbitals must be bound orbitals 1..nbf");
    if (hk[e] < 0 || hk[e] > 63) return set_err(c, DBSRG_ERANGE, "backward: k out of range");
  }
  if (nb < 1 || nb > 64)
    return set_err(c, DBSRG_EINVAL, "backward: 1..64 bound orbitals (ipbs = 0)");
  // device arrays: entries, per-k entry order, R, terms, term lists, E
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return hk[x] < hk[y]; });
  // term lists per (orbital, component): (e*4 + t)*4 + role in entry order
  std::vector<int> cnt((size_t)2 * nbf + 1, 0);
  auto target = [&](int e, int t, int r) {
    const int o = r == 0 ? h1[e] : r == 1 ? h3[e] : r == 2 ? h2[e] : h4[e];
    const int comp = r < 2 ? TA(t) : TB(t);
    return (o - 1) * 2 + (comp - 1);
  };
  const bool want_grad = grad != nullptr;
  std::vector<int> lstart((size_t)2 * nbf + 1, 0), lidx;
  if (want_grad) {
    for (int e = 0; e < n; e++)
      for (int t = 0; t < 4; t++)
        for (int r = 0; r < 4; r++) cnt[target(e, t, r) + 1]++;
    for (int i = 0; i < 2 * nbf; i++) lstart[i + 1] = lstart[i] + cnt[i + 1];
    lidx.resize((size_t)16 * n);
    std::vector<int> fill(lstart.begin(), lstart.end() - 1);
    for (int e = 0; e < n; e++)
      for (int t = 0; t < 4; t++)
        for (int r = 0; r < 4; r++) lidx[fill[target(e, t, r)]++] = (e * 4 + t) * 4 + r;
  }
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t tn = want_grad ? (size_t)n * 16 * ns : 0;
  const size_t bytes = 6 * al(ib) + 2 * al(sizeof(double) * (size_t)n) + al(sizeof(double) * tn) +
                       al(sizeof(int) * lstart.size()) + al(sizeof(int) * lidx.size()) +
                       al(sizeof(double) * (size_t)ns * 2 * nbf) + 256;
  if ((rc = ensure_scratch(c, bytes))) return rc;
  char *base = (char *)c->scratch;
  auto take = [&](size_t b) {
    char *p = base;
    base += al(b);
    return (void *)p;
  };
  int *dk = (int *)take(ib), *d1 = (int *)take(ib), *d2 = (int *)take(ib), *d3 = (int *)take(ib),
      *d4 = (int *)take(ib), *dord = (int *)take(ib);
  double *dc = (double *)take(sizeof(double) * n), *dR = (double *)take(sizeof(double) * n);
  double *dT = (double *)take(sizeof(double) * tn);
  int *dls = (int *)take(sizeof(int) * lstart.size()), *dli = (int *)take(sizeof(int) * lidx.size());
  double *dG = (double *)take(sizeof(double) * (size_t)ns * 2 * nbf);
  double *dE = (double *)take(sizeof(double));
  if ((rc = copy_in(c, dk, hk.data(), ib)) || (rc = copy_in(c, d1, h1.data(), ib)) ||
      (rc = copy_in(c, d2, h2.data(), ib)) || (rc = copy_in(c, d3, h3.data(), ib)) ||
      (rc = copy_in(c, d4, h4.data(), ib)) || (rc = copy_in(c, dord, order.data(), ib)) ||
      (rc = copy_in(c, dc, hc.data(), sizeof(double) * n)))
    return rc;
  if (want_grad &&
      ((rc = copy_in(c, dls, lstart.data(), sizeof(int) * lstart.size())) ||
       (rc = copy_in(c, dli, lidx.data(), sizeof(int) * lidx.size()))))
    return rc;
  // per multipole: the four pair potentials, then energy and gradient terms
  for (int lo = 0; lo < n;) {
    int hi = lo;
    while (hi < n && hk[order[hi]] == hk[order[lo]]) hi++;
    const int kp = hk[order[lo]];
    KdTypes kd{};
    for (int t = 0; t < 4; t++)
      if ((rc = get_pairpot_direct(c, 0, t, kp, 1, TB(t), TB(t), &kd.K[t]))) return rc;
    const int m = hi - lo;
    DBSRG_RUN(c, "k_rk_energy",
              k_rk_energy<<<(unsigned)((m * 32 + 255) / 256), 256, 0, st>>>(
                  m, ns, ks, nb, dord + lo, d1, d2, d3, d4, c->bmap, c->pq, kd, dR));
    if (want_grad) {
      // the terms of the entries of this multipole: one launch per entry run
      // (entries of one k are contiguous in 'order' but not in the arrays)
      std::vector<int> run(order.begin() + lo, order.begin() + hi);
      std::sort(run.begin(), run.end());
      for (size_t s0 = 0; s0 < run.size();) {
        size_t s1 = s0 + 1;
        while (s1 < run.size() && run[s1] == run[s1 - 1] + 1) s1++;
        const int e0 = run[s0], ne = (int)(s1 - s0);
        const size_t nt = (size_t)ne * 16 * ns;
        DBSRG_RUN(c, "k_rk_grad_terms",
                  k_rk_grad_terms<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(
                      ne, ns, ks, nb, d1 + e0, d2 + e0, d3 + e0, d4 + e0, dc + e0, c->bmap,
                      c->pq, kd, dT + (size_t)e0 * 16 * ns));
        s0 = s1;
      }
    }
    lo = hi;
  }
  if (n > 0) DBSRG_RUN(c, "k_energy_sum", k_energy_sum<<<1, 256, 0, st>>>(n, dc, dR, dE));
  else DBSRG_TRY(c, cudaMemsetAsync(dE, 0, sizeof(double), st));
  if (want_grad) {
    const size_t ng = (size_t)ns * 2 * nbf;
    DBSRG_RUN(c, "k_rk_grad_reduce",
              k_rk_grad_reduce<<<(unsigned)((ng + 255) / 256), 256, 0, st>>>(ns, nbf, dls, dli,
                                                                             dT, dG));
    if ((rc = copy_out(c, grad, dG, sizeof(double) * ng))) return rc;
  }
  return copy_out(c, energy, dE, sizeof(double));
}
