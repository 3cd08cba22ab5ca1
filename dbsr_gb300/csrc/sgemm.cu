// sgemm.cu -- FP64-accurate matrix products as split-BF16 tcgen05 products,
// for the block transformation of Record_matrix (record_matrix.f90:14-26):
// c = D_ich^T H D_jch for every block of a channel pair ich > jch, as
//   W^T = (D_ich^T H)^T   and   c = W D_jch.
//
// Operands.  Both GEMMs are C(r, c) = sum_k A(r, k) B(k, c) with the rows of
// A and the columns of B given as vectors contiguous in k ("vectors": the
// columns of D, of H and of W^T).  Every vector is cut into K chunks of 32;
// every chunk gets its own exponent e with 2^(e-1) > its largest modulus
// and six balanced base-256 digits per element (tc_common.cuh), stored as
// [chunk][slice][32-vector tile][32 x 32 BF16, canonical K-major layout],
// the exponents as [chunk][vector].  The digits of D_ch serve as A of the
// first product (its columns are the rows of D_ch^T) and as B of the second
// (the columns of D_ch).
//
// Products.  One CTA per 128 x 32 output tile walks the K chunks: a producer
// thread bulk-copies the six A slices (128 x 32) and B slices (32 x 32) of a
// chunk into one of two shared-memory stages and issues the 42 MMAs
// (21 slice pairs of order i + j <= 5, two K steps of 16) into one of two
// TMEM accumulator sets; eight epilogue warps read the six orders of the
// set (exact integers below 2^22), recombine them into int64
// I = sum_g D_g 256^(5-g) at the chunk's scale 2^(e_r + e_c - 56), and add
// I >> 5 into an int64 sum kept at the largest scale met so far (smaller
// scales shifted right: bits below 2^-51 of the largest one dropped; with
// |I| < 2^59 a chunk, the sum of up to 256 chunks stays inside int64).  The
// sum is converted to FP64 once.  Error: about 32 2^-48 of max|A| max|B|
// over each chunk, summed over the chunks.
#include <cuda_bf16.h>

#include <algorithm>
#include <vector>

#include "internal.cuh"
#include "tc_common.cuh"

using namespace tc;

namespace {

constexpr int TILE = 32 * 32;               // BF16 elements of a 32-vector digit tile
constexpr uint32_t A_BYTES = 4 * TILE * 2;  // one slice of a 128-row A operand
constexpr uint32_t B_BYTES = TILE * 2;      // one slice of a 32-column B operand
constexpr int SHIFT = 5;                    // right shift of each chunk's integer
constexpr int NCW = 8;                      // epilogue warps
constexpr int NTHR = 32 * (NCW + 1);        // + one producer warp
constexpr unsigned long long WAIT_NS = 2000000000ull;

constexpr int ZERO_EXP = -20000;  // exponent of an all-zero chunk
constexpr int NO_EXP = -100000;   // the empty sum

// digits of R vectors of K elements (vector r at X + r ldx, contiguous),
// rows padded to NR*32 and K to nk*32 with zeros: out [nk][TS][NR][TILE],
// chunk exponents ex[nk][NR*32].  One warp per vector; lanes 4q..4q+3 hold
// the four groups of 8 elements of one chunk.
__global__ void k_vec_digits(int R, int K, const double *X, size_t ldx, int NR, int nk,
                             __nv_bfloat16 *out, int *ex) {
  const int r = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (r >= NR * 32) return;  // whole warps
  const double *x = X + (size_t)r * ldx;
  const bool live = r < R;
  const int rt = r >> 5, rr = r & 31;
  const size_t sl = (size_t)NR * TILE;
  for (int g0 = 0; g0 < nk * 4; g0 += 32) {
    const int g = g0 + lane, kc = g >> 2, kg = g & 3;
    const bool gv = g < nk * 4;
    double v[8];
    double m = 0.0;
#pragma unroll
    for (int t = 0; t < 8; t++) {
      const int k = 32 * kc + 8 * kg + t;
      v[t] = live && gv && k < K ? x[k] : 0.0;
      m = fmax(m, fabs(v[t]));
    }
    m = fmax(m, __shfl_xor_sync(0xffffffffu, m, 1));
    m = fmax(m, __shfl_xor_sync(0xffffffffu, m, 2));
    const int e = m == 0.0 ? ZERO_EXP : scale_exp(m);
    if (!gv) continue;
    if (kg == 0) ex[(size_t)kc * NR * 32 + r] = e;
    float d[8][TS];
#pragma unroll
    for (int t = 0; t < 8; t++) digits(v[t], e, d[t]);
    __nv_bfloat16 *base = out + (size_t)kc * TS * sl + (size_t)rt * TILE + core_off(rr, 8 * kg);
#pragma unroll
    for (int i = 0; i < TS; i++) {
      __align__(16) __nv_bfloat16 h[8];
#pragma unroll
      for (int t = 0; t < 8; t++) h[t] = __float2bfloat16_rn(d[t][i]);
      *(uint4 *)(base + (size_t)i * sl) = *(const uint4 *)h;
    }
  }
}

struct GemmJob {
  const __nv_bfloat16 *A, *B;  // digits, [nk][TS][NRa|NRb][TILE]
  const int *ea, *eb;          // chunk exponents, [nk][NRa*32] and [nk][NRb*32]
  double *C;                   // C(r, c) at C[r*sr + c*sc]
  long long sr, sc;
  int M, N, NRa, NRb;
};

__device__ __forceinline__ void mbar_arrive1(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(mbar) : "memory");
}

// blockIdx.y: job; blockIdx.x: tile (mt, nt) of its M x N output
__global__ void __launch_bounds__(NTHR) k_sgemm(const GemmJob *jobs, int nk, int *err) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char *sA = smraw;                  // [2][TS][A_BYTES]
  unsigned char *sB = sA + 2 * TS * A_BYTES;  // [2][TS][B_BYTES]
  __shared__ __align__(8) uint64_t bar_ld[2], bar_mma[2], bar_free[2];
  __shared__ uint32_t tmem_base;
  __shared__ int s_abort;
  const GemmJob jb = jobs[blockIdx.y];
  const int ntn = (jb.N + 31) / 32;
  const int mt = blockIdx.x / ntn, nt = blockIdx.x % ntn;
  if (mt * 128 >= jb.M || nt * 32 >= jb.N) return;  // uniform per CTA, before any barrier
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  if (tid == 0) {
    for (int b = 0; b < 2; b++) {
      mbar_init(smem_u32(&bar_ld[b]), 1);
      mbar_init(smem_u32(&bar_mma[b]), 1);
      mbar_init(smem_u32(&bar_free[b]), NCW);
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    s_abort = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tbase = tmem_base;
  volatile int *abort_flag = &s_abort;
  const size_t sla = (size_t)jb.NRa * TILE, slb = (size_t)jb.NRb * TILE;

  if (warp == NCW) {
    // ---------------------------------------------------------- producer
    if (lane == 0) {
      long long issued = -1, done = -1, last_mma = -1;
      bool fail = false;
      auto loads = [&](int kc) {
        const int s = kc & 1;
        const uint32_t lb = smem_u32(&bar_ld[s]);
        mbar_expect_tx(lb, TS * (A_BYTES + B_BYTES));
        const __nv_bfloat16 *a = jb.A + (size_t)kc * TS * sla + (size_t)4 * mt * TILE;
        const __nv_bfloat16 *b = jb.B + (size_t)kc * TS * slb + (size_t)nt * TILE;
        for (int i = 0; i < TS; i++) {
          bulk_g2s(smem_u32(sA + (size_t)(s * TS + i) * A_BYTES), a + (size_t)i * sla, A_BYTES, lb);
          bulk_g2s(smem_u32(sB + (size_t)(s * TS + i) * B_BYTES), b + (size_t)i * slb, B_BYTES, lb);
        }
        issued = kc;
      };
      loads(0);
      for (int kc = 0; kc < nk; kc++) {
        const int s = kc & 1;
        const uint32_t n = (uint32_t)(kc >> 1);
        if (kc + 1 < nk) {  // stage (kc+1)&1 was last read by the MMAs of kc-1
          if (kc >= 1 && !mbar_wait(smem_u32(&bar_mma[(kc - 1) & 1]), ((kc - 1) >> 1) & 1, WAIT_NS)) {
            fail = true;
            break;
          }
          loads(kc + 1);
        }
        if (!mbar_wait(smem_u32(&bar_ld[s]), n & 1, WAIT_NS)) {
          fail = true;
          break;
        }
        done = kc;
        // TMEM set s was last read by the epilogue for chunk kc-2
        if (kc >= 2 && !mbar_wait(smem_u32(&bar_free[s]), (n - 1) & 1, WAIT_NS)) {
          fail = true;
          break;
        }
        fence_after();
        constexpr uint32_t idesc = make_idesc(128, 32);
        const uint64_t ad0 = make_desc(smem_u32(sA + (size_t)s * TS * A_BYTES), 128, 512);
        const uint64_t bd0 = make_desc(smem_u32(sB + (size_t)s * TS * B_BYTES), 128, 512);
#pragma unroll
        for (int g = 0; g < TS; g++) {
          const uint32_t dt = tbase + (uint32_t)(s * 256 + g * 32);
#pragma unroll
          for (int i = 0; i <= g; i++)
#pragma unroll
            for (int kk = 0; kk < 2; kk++)
              mma_bf16(dt, ad0 + ((i * A_BYTES + kk * 256) >> 4),
                       bd0 + (((g - i) * B_BYTES + kk * 256) >> 4), idesc,
                       (i == 0 && kk == 0) ? 0u : 1u);
        }
        mma_commit(smem_u32(&bar_mma[s]));
        last_mma = kc;
      }
      if (fail) {
        *abort_flag = 1;
        atomicExch(err, 1);
        for (long long k = done + 1; k <= issued; k++)  // copies in flight land first
          mbar_wait(smem_u32(&bar_ld[k & 1]), (uint32_t)((k >> 1) & 1), WAIT_NS);
      }
      if (last_mma >= 0)
        mbar_wait(smem_u32(&bar_mma[last_mma & 1]), (uint32_t)((last_mma >> 1) & 1), WAIT_NS);
    }
  } else {
    // ---------------------------------------------------------- epilogue
    // warp w reads TMEM lanes 32 (w & 3) .. +31 (rows) and columns 16 (w >> 2)
    const int lg = warp & 3, ch = warp >> 2;
    const int r = mt * 128 + lg * 32 + lane;  // < NRa*32: A rows are padded to 128
    long long acc[16];
    int cur[16];
#pragma unroll
    for (int c = 0; c < 16; c++) acc[c] = 0, cur[c] = NO_EXP;
    bool dead = false;
    // the chunk's row exponent and its 16 column exponents (64-byte aligned),
    // loaded one chunk ahead of their use
    int er_n;
    int4 en[4];
    auto exps = [&](int kc) {
      er_n = jb.ea[(size_t)kc * jb.NRa * 32 + r];
      const int4 *ep =
          reinterpret_cast<const int4 *>(jb.eb + (size_t)kc * jb.NRb * 32 + nt * 32 + ch * 16);
#pragma unroll
      for (int u = 0; u < 4; u++) en[u] = ep[u];
    };
    exps(0);
    for (int kc = 0; kc < nk; kc++) {
      const int s = kc & 1;
      const uint32_t n = (uint32_t)(kc >> 1);
      const int er = er_n;
      const int ec[16] = {en[0].x, en[0].y, en[0].z, en[0].w, en[1].x, en[1].y, en[1].z, en[1].w,
                          en[2].x, en[2].y, en[2].z, en[2].w, en[3].x, en[3].y, en[3].z, en[3].w};
      if (kc + 1 < nk) exps(kc + 1);
      if (!dead && *abort_flag) dead = true;
      bool ok = !dead && mbar_wait(smem_u32(&bar_mma[s]), n & 1, WAIT_NS);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) {
        if (!dead) {
          dead = true;
          *abort_flag = 1;
          if (lane == 0) atomicExch(err, 1);
        }
        continue;
      }
      fence_after();
      int P[3][16];
      const uint32_t col = tbase + ((uint32_t)(lg * 32) << 16) + (uint32_t)(s * 256 + ch * 16);
#pragma unroll
      for (int k = 0; k < 3; k++) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
          uint32_t v0[8], v1[8];
          tmem_ld8(col + 64 * k + 8 * h, v0);
          tmem_ld8(col + 64 * k + 32 + 8 * h, v1);
          tmem_wait_ld();
          // orders 2k and 2k+1: bits(D + 1.5 2^23) = D + 0x4B400000 for |D| < 2^22
#pragma unroll
          for (int c = 0; c < 8; c++)
            P[k][8 * h + c] =
                (int)(((uint32_t)__float_as_uint(__uint_as_float(v0[c]) + 12582912.0f) << 8) +
                      (uint32_t)__float_as_uint(__uint_as_float(v1[c]) + 12582912.0f) -
                      257u * 0x4B400000u);
        }
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive1(smem_u32(&bar_free[s]));
#pragma unroll
      for (int c = 0; c < 16; c++) {
        const long long I = ((long long)P[0][c] * 4294967296LL + (long long)P[1][c] * 65536LL +
                             (long long)P[2][c]) >> SHIFT;
        const int se = er + ec[c];
        if (se > cur[c]) {  // the sum raised to the larger scale
          const int up = se - cur[c];
          acc[c] = up < 63 ? acc[c] >> up : 0;
          cur[c] = se;
        }
        const int sh = cur[c] - se;
        if (sh < 63) acc[c] += I >> sh;
      }
    }
    if (!dead && r < jb.M) {
#pragma unroll
      for (int c = 0; c < 16; c++) {
        const int cc = nt * 32 + ch * 16 + c;
        if (cc < jb.N)
          jb.C[(long long)r * jb.sr + (long long)cc * jb.sc] =
              i64_to_f64(acc[c], cur[c] - 8 * (TS + 1) + SHIFT);
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tbase), "r"(512));
}

struct Buf {
  void *p = nullptr;
  ~Buf() {
    if (p) cudaFree(p);
  }
  bool alloc(size_t n) {
    if (cudaMalloc(&p, std::max<size_t>(n, 16)) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return false;
    }
    return true;
  }
};

}  // namespace

// c = D_ich^T H D_jch for every block of a channel pair ich > jch, in place
// (ni x nj corner, the rest zero); D on the device (ms x ms per channel)
int split_channel_basis(dbsrg_ctx *c, const double *D, const int *nsol) {
  const int ms = c->g.ms, nch = c->nch;
  // vectors padded to whole 128-row A tiles, K to whole chunks of 32
  const int NR = 4 * ((ms + 127) / 128), nk = (ms + 31) / 32;
  if (nk > 256) return set_err(c, DBSRG_EINVAL, "channel_basis: ms above 8192");
  const size_t blk = (size_t)ms * ms;
  const size_t dsz = (size_t)nk * TS * NR * TILE;  // BF16 elements of one digit operand
  cudaStream_t st = c->stream;
  // the blocks to transform
  std::vector<int> bi, bj, bk;
  for (int ich = 2; ich <= nch; ich++)
    for (int jch = 1; jch < ich; jch++) {
      const int k = c->h_icc[(ich - 1) + (size_t)nch * (jch - 1)];
      if (k < 1) continue;
      bi.push_back(ich);
      bj.push_back(jch);
      bk.push_back(k);
    }
  if (bk.empty()) return DBSRG_OK;
  // digits of every channel's solutions (columns of D_ch)
  Buf dD, eD, err;
  const size_t esz = (size_t)nk * NR * 32;  // chunk exponents of one operand
  if (!dD.alloc(dsz * 2 * nch) || !eD.alloc(sizeof(int) * esz * nch) || !err.alloc(4))
    return set_err(c, DBSRG_ENOMEM, "channel_basis: digit allocation failed");
  __nv_bfloat16 *Dd = (__nv_bfloat16 *)dD.p;
  int *De = (int *)eD.p;
  cudaMemsetAsync(err.p, 0, 4, st);
  const unsigned gv = (unsigned)((NR * 32 + 7) / 8);  // 8 vectors (warps) a block
  for (int ch = 1; ch <= nch; ch++)
    DBSRG_RUN(c, "k_vec_digits",
              k_vec_digits<<<gv, 256, 0, st>>>(nsol[ch - 1], ms, D + (size_t)(ch - 1) * blk, ms,
                                                NR, nk, Dd + dsz * (ch - 1),
                                                De + esz * (ch - 1)));
  // blocks in batches: digits of H's columns, W^T (ms x ni), digits of W's rows
  const size_t per_blk = 2 * dsz * 2 + blk * 8 + 2 * sizeof(int) * esz;
  size_t freeb = 0, totb = 0;
  cudaMemGetInfo(&freeb, &totb);
  int nb = (int)std::max<size_t>(1, std::min<size_t>(256, (freeb / 4) / per_blk));
  nb = std::min<int>(nb, (int)bk.size());
  Buf dH, dW, dWd, eH, eW, dJ;
  if (!dH.alloc(dsz * 2 * nb) || !dW.alloc(blk * 8 * nb) || !dWd.alloc(dsz * 2 * nb) ||
      !eH.alloc(sizeof(int) * esz * nb) || !eW.alloc(sizeof(int) * esz * nb) ||
      !dJ.alloc(sizeof(GemmJob) * nb))
    return set_err(c, DBSRG_ENOMEM, "channel_basis: product allocation failed");
  const size_t smem = 2 * TS * (A_BYTES + B_BYTES);
  int rc;
  if ((rc = raise_smem_limit(c, (const void *)k_sgemm, smem))) return rc;
  std::vector<GemmJob> jobs(nb);
  const int tiles = ((ms + 127) / 128) * ((ms + 31) / 32);
  for (size_t b0 = 0; b0 < bk.size(); b0 += nb) {
    const int n = (int)std::min<size_t>(nb, bk.size() - b0);
    // H columns -> digits (B of the first product)
    for (int q = 0; q < n; q++) {
      double *H = c->hch + (size_t)(bk[b0 + q] - 1) * blk;
      DBSRG_RUN(c, "k_vec_digits",
                k_vec_digits<<<gv, 256, 0, st>>>(ms, ms, H, ms, NR, nk,
                                                  (__nv_bfloat16 *)dH.p + dsz * q,
                                                  (int *)eH.p + esz * q));
    }
    // W^T(k, r) = sum_m H(m, k) D_ich(m, r): A = D_ich^T (rows r), B = H (columns k),
    // stored transposed: element (r, k) at Wt[k + ms r]
    int jn = 0;
    for (int q = 0; q < n; q++) {
      const int ich = bi[b0 + q], ni = nsol[ich - 1];
      if (ni == 0) continue;
      GemmJob &j = jobs[jn++];
      j.A = Dd + dsz * (ich - 1);
      j.ea = De + esz * (ich - 1);
      j.B = (__nv_bfloat16 *)dH.p + dsz * q;
      j.eb = (int *)eH.p + esz * q;
      j.C = (double *)dW.p + blk * q;
      j.sr = ms;
      j.sc = 1;
      j.M = ni;
      j.N = ms;
      j.NRa = NR;
      j.NRb = NR;
    }
    if (jn > 0) {
      if ((rc = copy_in(c, dJ.p, jobs.data(), sizeof(GemmJob) * jn))) return rc;
      DBSRG_RUN(c, "k_sgemm",
                k_sgemm<<<dim3((unsigned)tiles, (unsigned)jn), NTHR, smem, st>>>(
                    (const GemmJob *)dJ.p, nk, (int *)err.p));
    }
    // W rows (columns of W^T) -> digits (A of the second product)
    for (int q = 0; q < n; q++) {
      const int ni = nsol[bi[b0 + q] - 1];
      DBSRG_RUN(c, "k_vec_digits",
                k_vec_digits<<<gv, 256, 0, st>>>(ni, ms, (double *)dW.p + blk * q, ms, NR, nk,
                                                  (__nv_bfloat16 *)dWd.p + dsz * q,
                                                  (int *)eW.p + esz * q));
    }
    // c = W D_jch into the zeroed block (column-major, ld ms)
    jn = 0;
    for (int q = 0; q < n; q++) {
      double *H = c->hch + (size_t)(bk[b0 + q] - 1) * blk;
      cudaMemsetAsync(H, 0, blk * 8, st);
      const int ni = nsol[bi[b0 + q] - 1], jch = bj[b0 + q], nj = nsol[jch - 1];
      if (ni == 0 || nj == 0) continue;
      GemmJob &j = jobs[jn++];
      j.A = (__nv_bfloat16 *)dWd.p + dsz * q;
      j.ea = (int *)eW.p + esz * q;
      j.B = Dd + dsz * (jch - 1);
      j.eb = De + esz * (jch - 1);
      j.C = H;
      j.sr = 1;
      j.sc = ms;
      j.M = ni;
      j.N = nj;
      j.NRa = NR;
      j.NRb = NR;
    }
    if (jn > 0) {
      // the job table is rewritten only after the first product has read it
      if ((rc = copy_in(c, dJ.p, jobs.data(), sizeof(GemmJob) * jn))) return rc;
      DBSRG_RUN(c, "k_sgemm",
                k_sgemm<<<dim3((unsigned)tiles, (unsigned)jn), NTHR, smem, st>>>(
                    (const GemmJob *)dJ.p, nk, (int *)err.p));
    }
  }
  int herr = 0;
  cudaMemcpyAsync(&herr, err.p, 4, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess)
    return set_err(c, DBSRG_ECUDA, "channel_basis: tensor-core products failed");
  if (herr) return set_err(c, DBSRG_ETIMEOUT, "channel_basis: a product pipeline wait ran out");
  return DBSRG_OK;
}
