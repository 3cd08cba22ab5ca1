// orth.cu -- DBS_ORTH (DBSR_MAT3/dbs_orth.f90:2-84): orthogonality of the
// channel functions to chosen bound orbitals, imposed on the assembled
// matrix by Bentley's projection (J. Phys. B 27 (1994) 637):
//     H(ich,jch) -> (1 - A_ich) H(ich,jch) (1 - A_jch^T),
//     A_c = sum_{j in O(c)} w_j v_j^T,   v_j = (P_j; Q_j),   w_j = B v_j,
// B = blockdiag(fpbs, fqbs) (Get_pv / Get_qv with bpq, read_data.f90:144-145)
// and O(c) the bound orbitals channel c is made orthogonal to (the caller's
// mask; the reference takes the bound orbitals of the channel's kappa with
// IBORT = 0, dbs_orth.f90:39-43).
//
// The reference applies the row update (matmul(aa,x)) when its channel loop
// reaches ich and the column update (matmul(x,bb)) when it reaches jch, as
// full ms x ms products on every block of the channel's row.  The two
// updates commute, so here every stored block (ich >= jch, row channel
// a = ich, column channel b = jch) is transformed once through the rank-|O|
// factors:
//     T1 = V_a^T X   (|O_a| x ms)      T2 = X V_b   (ms x |O_b|)
//     T1' = T1 - (T1 V_b) W_b^T
//     X'  = X - W_a T1' - T2 W_b^T      (= X - W_a T1 - T2 W_b^T + W_a S W_b^T)
// FP64 throughout; every sum runs in a fixed order (no atomics), so the
// result is deterministic.
#include <vector>

#include "internal.cuh"

namespace {

constexpr int OCH = 4;  // orbitals per chunk of the dot-product kernels

// one stored block and its two channels' orbital lists (indices into the
// V/W columns) and scratch offsets
struct OrthBlock {
  int blk;     // 1-based block number
  int a0, na;  // row channel: orbitals olist[a0 .. a0+na)
  int b0, nb;  // column channel
  long long t1, t2;  // scratch offsets (doubles) of T1 (na x ms) and T2 (ms x nb)
};

// V(:,u) = (P; Q) of bound orbital orb[u], W(:,u) = fppqq V(:,u); one
// thread per (row r, orbital u)
__global__ void k_orth_vw(int ns, int nu, const int *orb, const double *pq, const double *fppqq,
                          double *V, double *W) {
  const int ms = 2 * ns;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ms * nu) return;
  const int r = q % ms, u = q / ms;
  const double *p = pq + (size_t)2 * ns * (orb[u] - 1);  // (P; Q) are contiguous
  V[q] = p[r];
  double acc = 0.0;
  for (int c = 0; c < ms; c++) acc = fma(fppqq[r + (size_t)ms * c], p[c], acc);
  W[q] = acc;
}

// T1(j,c) = sum_r V(r, a_j) X(r,c): one warp per column c, lanes over rows,
// a fixed shuffle tree per sum
__global__ void k_orth_t1(int ms, const OrthBlock *bl, const int *olist, const double *V,
                          const double *hch, double *scr) {
  const OrthBlock B = bl[blockIdx.y];
  if (B.na == 0) return;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int c = blockIdx.x * (blockDim.x / 32) + warp;
  if (c >= ms) return;
  const double *x = hch + (size_t)(B.blk - 1) * ms * ms + (size_t)ms * c;
  double *t1 = scr + B.t1;
  for (int j0 = 0; j0 < B.na; j0 += OCH) {
    double acc[OCH] = {0.0, 0.0, 0.0, 0.0};
    const double *v[OCH];
#pragma unroll
    for (int u = 0; u < OCH; u++)
      v[u] = V + (size_t)ms * olist[B.a0 + min(j0 + u, B.na - 1)];
    for (int r = lane; r < ms; r += 32) {
      const double xv = x[r];
#pragma unroll
      for (int u = 0; u < OCH; u++) acc[u] = fma(v[u][r], xv, acc[u]);
    }
#pragma unroll
    for (int u = 0; u < OCH; u++) {
      double s = acc[u];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0 && j0 + u < B.na) t1[(size_t)(j0 + u) + (size_t)B.na * c] = s;
    }
  }
}

// T2(r,l) = sum_c X(r,c) V(c, b_l): one thread per row, columns in order
// (consecutive threads read consecutive rows of a column)
__global__ void k_orth_t2(int ms, const OrthBlock *bl, const int *olist, const double *V,
                          const double *hch, double *scr) {
  const OrthBlock B = bl[blockIdx.y];
  if (B.nb == 0) return;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= ms) return;
  const double *x = hch + (size_t)(B.blk - 1) * ms * ms + r;
  double *t2 = scr + B.t2;
  for (int l0 = 0; l0 < B.nb; l0 += OCH) {
    double acc[OCH] = {0.0, 0.0, 0.0, 0.0};
    const double *v[OCH];
#pragma unroll
    for (int u = 0; u < OCH; u++)
      v[u] = V + (size_t)ms * olist[B.b0 + min(l0 + u, B.nb - 1)];
    for (int c = 0; c < ms; c++) {
      const double xv = x[(size_t)ms * c];
#pragma unroll
      for (int u = 0; u < OCH; u++) acc[u] = fma(xv, v[u][c], acc[u]);
    }
#pragma unroll
    for (int u = 0; u < OCH; u++)
      if (l0 + u < B.nb) t2[r + (size_t)ms * (l0 + u)] = acc[u];
  }
}

// T1' = T1 - S W_b^T with S = T1 V_b (na x nb), per block: one CTA, S in
// shared memory (warp per element, fixed shuffle tree), then one thread per
// element of T1
constexpr int MAXO = 32;
__global__ void k_orth_s(int ms, const OrthBlock *bl, const int *olist, const double *V,
                         const double *W, double *scr) {
  const OrthBlock B = bl[blockIdx.x];
  if (B.na == 0 || B.nb == 0) return;
  __shared__ double S[MAXO * MAXO];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, nw = blockDim.x / 32;
  double *t1 = scr + B.t1;
  for (int e = warp; e < B.na * B.nb; e += nw) {
    const int j = e % B.na, l = e / B.na;
    const double *v = V + (size_t)ms * olist[B.b0 + l];
    double acc = 0.0;
    for (int c = lane; c < ms; c += 32) acc = fma(t1[(size_t)j + (size_t)B.na * c], v[c], acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) S[j + MAXO * l] = acc;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < B.na * ms; e += blockDim.x) {
    const int j = e % B.na, c = e / B.na;
    double s = 0.0;
    for (int l = 0; l < B.nb; l++)
      s = fma(S[j + MAXO * l], W[(size_t)c + (size_t)ms * olist[B.b0 + l]], s);
    t1[e] = t1[e] - s;
  }
}

// X' = X - W_a T1' - T2 W_b^T: one thread per row r and UCOLS columns;
// per element the row terms (orbitals of a) then the column terms (of b),
// each in list order
constexpr int UCOLS = 8;
__global__ void k_orth_update(int ms, const OrthBlock *bl, const int *olist, const double *W,
                              const double *scr, double *hch) {
  const OrthBlock B = bl[blockIdx.z];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c0 = blockIdx.y * UCOLS, nc = min(UCOLS, ms - c0);
  if (r >= ms) return;
  double *x = hch + (size_t)(B.blk - 1) * ms * ms + r + (size_t)ms * c0;
  const double *t1 = scr + B.t1 + (size_t)B.na * c0, *t2 = scr + B.t2 + r;
  double d[UCOLS];
#pragma unroll
  for (int k = 0; k < UCOLS; k++) d[k] = 0.0;
  for (int j = 0; j < B.na; j++) {
    const double w = W[r + (size_t)ms * olist[B.a0 + j]];
#pragma unroll
    for (int k = 0; k < UCOLS; k++)
      if (k < nc) d[k] = fma(w, t1[(size_t)j + (size_t)B.na * k], d[k]);
  }
  for (int l = 0; l < B.nb; l++) {
    const double t = t2[(size_t)ms * l];
    const double *wb = W + (size_t)ms * olist[B.b0 + l] + c0;
#pragma unroll
    for (int k = 0; k < UCOLS; k++)
      if (k < nc) d[k] = fma(t, wb[k], d[k]);
  }
#pragma unroll
  for (int k = 0; k < UCOLS; k++)
    if (k < nc) x[(size_t)ms * k] -= d[k];
}

}  // namespace

extern "C" int dbsrg_orth_channels(dbsrg_ctx *c, const int *iort) {
  if (!c) return DBSRG_EINVAL;
  if (!iort) return set_err(c, DBSRG_EINVAL, "orth_channels: null argument");
  if (is_device_ptr(iort)) return set_err(c, DBSRG_EINVAL, "orth_channels: iort is a host array");
  if (!c->hmem || c->wcap < c->iicc)
    return set_err(c, DBSRG_ESTATE, "orth_channels: the whole matrix must be held");
  if (!c->pq || c->nbf < 1) return set_err(c, DBSRG_ESTATE, "orth_channels: no orbitals");
  cudaSetDevice(c->device);
  int rc = drain(c);
  if (rc) return rc;
  const int ns = c->g.ns, ms = c->g.ms, nch = c->nch, nbf = c->nbf;
  // orbitals used by any channel, and each channel's list of them
  std::vector<int> ucol(nbf, -1), orb;
  std::vector<int> cstart(nch + 1, 0), olist;
  for (int ich = 0; ich < nch; ich++) {
    cstart[ich] = (int)olist.size();
    for (int j = 0; j < nbf; j++) {
      if (!iort[j + (size_t)nbf * ich]) continue;
      if (c->h_ipbs[j] != 0)
        return set_err(c, DBSRG_EINVAL, "orth_channels: orthogonality to a non-bound orbital");
      if (ucol[j] < 0) {
        ucol[j] = (int)orb.size();
        orb.push_back(j + 1);
      }
      olist.push_back(ucol[j]);
    }
    if ((int)olist.size() - cstart[ich] > MAXO)
      return set_err(c, DBSRG_ERANGE, "orth_channels: more than 32 orbitals for one channel");
  }
  cstart[nch] = (int)olist.size();
  if (orb.empty()) return DBSRG_OK;
  // stored blocks with a condition on either side
  std::vector<OrthBlock> blocks;
  long long off = 0;
  for (int ich = 1; ich <= nch; ich++)
    for (int jch = 1; jch <= ich; jch++) {
      const int k = c->h_icc[(ich - 1) + (size_t)nch * (jch - 1)];
      if (k < 1) continue;
      OrthBlock b{};
      b.blk = k;
      b.a0 = cstart[ich - 1];
      b.na = cstart[ich] - cstart[ich - 1];
      b.b0 = cstart[jch - 1];
      b.nb = cstart[jch] - cstart[jch - 1];
      if (b.na == 0 && b.nb == 0) continue;
      b.t1 = off;
      off += (long long)b.na * ms;
      b.t2 = off;
      off += (long long)b.nb * ms;
      blocks.push_back(b);
    }
  if (blocks.empty()) return DBSRG_OK;
  cudaStream_t st = c->stream;
  const int nu = (int)orb.size();
  // chunks of at most 65535 blocks (grid y/z limit) whose scratch stays below
  // 1 GB (a block needs at most 2 x 32 x ms doubles), offsets rebased to each
  // chunk's first element
  const long long cap = std::min(off, 1LL << 27);
  std::vector<size_t> cuts{0};
  for (size_t i = 0, first = 0; i < blocks.size(); i++) {
    const long long base = blocks[first].t1;
    if (blocks[i].t2 + (long long)blocks[i].nb * ms - base > cap || i - first >= 65535) {
      cuts.push_back(i);
      first = i;
    }
  }
  cuts.push_back(blocks.size());
  for (size_t k = 0; k + 1 < cuts.size(); k++) {
    const long long base = blocks[cuts[k]].t1;
    for (size_t i = cuts[k]; i < cuts[k + 1]; i++) {
      blocks[i].t1 -= base;
      blocks[i].t2 -= base;
    }
  }
  int *dorb = nullptr, *dol = nullptr;
  double *dV = nullptr, *dW = nullptr, *dscr = nullptr;
  OrthBlock *dbl = nullptr;
  auto cleanup = [&]() {
    for (void *p : {(void *)dorb, (void *)dol, (void *)dV, (void *)dW, (void *)dscr, (void *)dbl})
      if (p) cudaFree(p);
  };
  if (cudaMalloc(&dorb, sizeof(int) * nu) || cudaMalloc(&dol, sizeof(int) * olist.size()) ||
      cudaMalloc(&dV, sizeof(double) * ms * nu) || cudaMalloc(&dW, sizeof(double) * ms * nu) ||
      cudaMalloc(&dscr, sizeof(double) * cap) ||
      cudaMalloc(&dbl, sizeof(OrthBlock) * blocks.size())) {
    cudaGetLastError();
    cleanup();
    return set_err(c, DBSRG_ENOMEM, "orth_channels: allocation failed");
  }
  auto fail = [&](int code, const char *msg) {
    cudaStreamSynchronize(st);
    cleanup();
    return set_err(c, code, msg);
  };
  if ((rc = copy_in(c, dorb, orb.data(), sizeof(int) * nu))) return fail(rc, "copy");
  if ((rc = copy_in(c, dol, olist.data(), sizeof(int) * olist.size()))) return fail(rc, "copy");
  if ((rc = copy_in(c, dbl, blocks.data(), sizeof(OrthBlock) * blocks.size())))
    return fail(rc, "copy");
  DBSRG_RUN(c, "k_orth_vw",
            k_orth_vw<<<(unsigned)((ms * nu + 255) / 256), 256, 0, st>>>(ns, nu, dorb, c->pq,
                                                                         c->g.fppqq, dV, dW));
  for (size_t k = 0; k + 1 < cuts.size(); k++) {
    const OrthBlock *cb = dbl + cuts[k];
    const unsigned nbk = (unsigned)(cuts[k + 1] - cuts[k]);
    DBSRG_RUN(c, "k_orth_t1",
              k_orth_t1<<<dim3((unsigned)((ms + 7) / 8), nbk), 256, 0, st>>>(ms, cb, dol, dV,
                                                                              c->hch, dscr));
    DBSRG_RUN(c, "k_orth_t2",
              k_orth_t2<<<dim3((unsigned)((ms + 127) / 128), nbk), 128, 0, st>>>(ms, cb, dol, dV,
                                                                                 c->hch, dscr));
    DBSRG_RUN(c, "k_orth_s", k_orth_s<<<nbk, 256, 0, st>>>(ms, cb, dol, dV, dW, dscr));
    DBSRG_RUN(c, "k_orth_update",
              k_orth_update<<<dim3((unsigned)((ms + 127) / 128),
                                   (unsigned)((ms + UCOLS - 1) / UCOLS), nbk),
                              128, 0, st>>>(ms, cb, dol, dW, dscr, c->hch));
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail(DBSRG_ECUDA, "orth_channels");
  cleanup();
  return DBSRG_OK;
}
