// farfield_tc.cu -- far-field product of the factored exchange on the
// tcgen05 tensor cores in split precision.
//
// out(x,y) = sum_a U(x,a) Z(a,y) over the bound orbitals a (K = nb <= 32),
// written only where |y - x| >= 9 (the band is gathered in FP64 elsewhere).
//
// Splitting (exact):  U(x,a) = 2^eu(x) * sum_i u_i(x,a) 2^-8(i+1) with
// integer digits |u_i| <= 255 (i = 0..S-1), eu(x) a power-of-two scale per
// row; Z(a,y) likewise with a scale per column.  Every digit is an integer of
// at most 8 significant bits, hence exact in BF16.  For each order
// g = i + j <= S-1 the tensor cores accumulate
//     D_g = sum_{i+j=g} sum_a u_i(x,a) z_j(a,y)
// in FP32: all partial sums are integers below (g+1)*nb*255^2 < 2^24, so the
// FP32 accumulation is exact.  The epilogue forms the integer
//     I = sum_g D_g 2^(8(S-1-g))   (exact in int64)
// and writes out = 2^(eu+ez-8(S+1)) * I in FP64.  The only rounding is the
// truncation of the digit expansions after S slices (relative 2^-8S of the
// row/column scales times nb) and the final int64 -> FP64 rounding.
//
// One CTA computes a 128 x 32 output tile: warp 0 allocates 256 TMEM
// columns (S=6 accumulators of 32 FP32 columns), the CTA stages the S
// digit slices of U (128 x 32 each) and Z (32 x 32 each) in shared memory in
// the canonical no-swizzle K-major layout, one thread issues the 42
// tcgen05.mma (kind::f16, BF16 x BF16 -> FP32, M=128, N=32, K=16) and
// commits them to an mbarrier; all four warps then read their 32 TMEM lanes.
// Waits are bounded: on a timeout the kernel records an error word, waits
// once more (bounded) for its MMAs, frees its TMEM and returns.
#include <cuda_bf16.h>

#include "internal.cuh"

namespace {

constexpr int TS = 6;       // digit slices per operand
constexpr int TM = 128;     // tile rows (x)
constexpr int TN = 32;      // tile columns (y)
constexpr int TK = 32;      // padded orbital dimension
constexpr int FARD = 9;     // far field |y - x| >= 9
constexpr int A_SLICE = TM * TK;   // bf16 elements per A slice tile
constexpr int B_SLICE = TN * TK;   // bf16 elements per B slice tile
constexpr int TMEM_COLS = 256;     // >= TS * TN, power of two
constexpr unsigned long long WAIT_LIMIT = 1ull << 26;

// offset of element (r, k) of a rows x 32 tile in the canonical K-major,
// no-swizzle layout: 8x8 core matrices (128 bytes), core matrix (r/8, k/8)
// at ((r/8)*4 + k/8) * 64 elements
__device__ __forceinline__ int core_off(int r, int k) {
  return (((r >> 3) * 4 + (k >> 3)) << 6) + ((r & 7) << 3) + (k & 7);
}

// digits of v / 2^e, |v / 2^e| < 1: S integers with |d| <= 255, the base-256
// expansion of trunc(|v| 2^(8S-e)) with the sign of v.  Done on the bit
// pattern with integer instructions (the FP64 pipe of this GPU is narrow);
// it equals the sequential w*=256, d=trunc(w), w-=d expansion exactly.
__device__ __forceinline__ void digits(double v, int e, float *d) {
  long long bits = __double_as_longlong(v);
  int ev = (int)((bits >> 52) & 0x7FF);
  unsigned long long W = 0;
  if (ev != 0) {  // zero and subnormals (far below every scale here) give 0
    unsigned long long mant = (unsigned long long)(bits & ((1LL << 52) - 1)) | (1ULL << 52);
    int s = ev - 1075 - e + 8 * TS;  // W = mant * 2^s, |v / 2^e| < 1 => s < -4
    if (s >= 0)
      W = 0;  // cannot happen for |v / 2^e| < 1; kept for safety
    else if (-s < 64)
      W = mant >> (-s);
  }
  const float sg = bits < 0 ? -1.0f : 1.0f;
#pragma unroll
  for (int i = 0; i < TS; i++) d[i] = sg * (float)((W >> (8 * (TS - 1 - i))) & 255ULL);
}

__device__ __forceinline__ int scale_exp(double m) {  // m >= 0: 2^e > m
  if (m == 0.0) return 0;
  int e;
  frexp(m, &e);  // m = f * 2^e, f in [0.5, 1)
  return e;
}

// U (ns x nb, column-major) -> slices A[tile][slice][128x32] + eu[x]
__global__ void k_split_rows(int ns, int nb, const double *U, __nv_bfloat16 *A, int *eu) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int ntile = (ns + TM - 1) / TM;
  if (x >= ntile * TM) return;
  int tile = x / TM, r = x % TM;
  double m = 0.0;
  if (x < ns)
    for (int a = 0; a < nb; a++) m = fmax(m, fabs(U[(size_t)x + (size_t)ns * a]));
  int e = scale_exp(m);
  if (x < ns) eu[x] = e;
  for (int a = 0; a < TK; a++) {
    float d[TS];
    double v = (x < ns && a < nb) ? U[(size_t)x + (size_t)ns * a] : 0.0;
    digits(v, e, d);
    for (int i = 0; i < TS; i++)
      A[((size_t)tile * TS + i) * A_SLICE + core_off(r, a)] = __float2bfloat16_rn(d[i]);
  }
}

// Z (per slot: nb x ns, Z[a + nb*y]) -> B[slot][ytile][slice][32x32] + ez[slot][y]
__global__ void k_split_cols(int ns, int nb, int nm, const double *Z, __nv_bfloat16 *B, int *ez) {
  int y = blockIdx.x * blockDim.x + threadIdx.x;
  int slot = blockIdx.y;
  int nty = (ns + TN - 1) / TN;
  if (y >= nty * TN) return;
  int tile = y / TN, cidx = y % TN;
  const double *Zs = Z + (size_t)slot * nb * ns;
  double m = 0.0;
  if (y < ns)
    for (int a = 0; a < nb; a++) m = fmax(m, fabs(Zs[(size_t)a + (size_t)nb * y]));
  int e = scale_exp(m);
  if (y < ns) ez[(size_t)slot * ns + y] = e;
  __nv_bfloat16 *Bt = B + (((size_t)slot * nty + tile) * TS) * B_SLICE;
  for (int a = 0; a < TK; a++) {
    float d[TS];
    double v = (y < ns && a < nb) ? Zs[(size_t)a + (size_t)nb * y] : 0.0;
    digits(v, e, d);
    for (int i = 0; i < TS; i++) Bt[(size_t)i * B_SLICE + core_off(cidx, a)] = __float2bfloat16_rn(d[i]);
  }
}

// ---- tcgen05 / mbarrier helpers (inline PTX) --------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: canonical K-major layout, no swizzle;
// LBO = byte distance between core matrices along K, SBO = along M/N
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  return d;                // base offset 0, swizzle mode 0 (none)
}

// instruction descriptor: kind::f16, A/B BF16, D F32, both K-major, M, N
__host__ __device__ constexpr uint32_t make_idesc(int m, int n) {
  return (1u << 4)               // D format F32
         | (1u << 7)             // A format BF16
         | (1u << 10)            // B format BF16
         | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc,
                                         uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
        "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
        "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// exact int64 -> FP64 times 2^sh (the value is far inside the normal range)
__device__ __forceinline__ double i64_scaled(long long I, int sh) {
  if (I == 0) return 0.0;
  double d = __ll2double_rn(I);
  long long b = __double_as_longlong(d);
  int ex = (int)((b >> 52) & 0x7FF) + sh;
  if (ex <= 0 || ex >= 0x7FF) return ldexp(d, sh);
  b = (b & ~(0x7FFLL << 52)) | ((long long)ex << 52);
  return __longlong_as_double(b);
}

// mode 0: upper far field (y - x >= 9); 1: lower far field (x - y >= 9)
__global__ void __launch_bounds__(128) k_far_tc(int ns, int nm, int mode,
                                                const __nv_bfloat16 *__restrict__ A,
                                                const int *__restrict__ eu,
                                                const __nv_bfloat16 *__restrict__ B,
                                                const int *__restrict__ ez, double *Y, size_t per,
                                                int *err) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  __nv_bfloat16 *sA = (__nv_bfloat16 *)smraw;            // TS * A_SLICE
  __nv_bfloat16 *sB = sA + TS * A_SLICE;                  // TS * B_SLICE
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const int tx = blockIdx.x, ty = blockIdx.y, slot = blockIdx.z;
  const int x0 = tx * TM, y0 = ty * TN;
  const int nty = (ns + TN - 1) / TN;
  // skip tiles with no far-field element of this mode
  if (mode == 0 ? ((y0 + TN - 1) - x0 < FARD) : ((x0 + TM - 1) - y0 < FARD)) return;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;

  // stage operands (16-byte vector copies)
  {
    const uint4 *gA = (const uint4 *)(A + (size_t)tx * TS * A_SLICE);
    uint4 *dA = (uint4 *)sA;
    for (int i = threadIdx.x; i < TS * A_SLICE / 8; i += blockDim.x) dA[i] = gA[i];
    const uint4 *gB = (const uint4 *)(B + ((size_t)slot * nty + ty) * TS * B_SLICE);
    uint4 *dB = (uint4 *)sB;
    for (int i = threadIdx.x; i < TS * B_SLICE / 8; i += blockDim.x) dB[i] = gB[i];
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  // make the operand stores visible to the tensor cores' async proxy
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tbase = tmem_base;

  if (threadIdx.x == 0) {
    const uint32_t idesc = make_idesc(TM, TN);
    const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
    for (int g = 0; g < TS; g++) {
      const uint32_t dt = tbase + (uint32_t)(g * TN);
      int first = 1;
      for (int i = 0; i <= g; i++) {
        const int jsl = g - i;
        for (int kk = 0; kk < TK / 16; kk++) {
          // k-step kk covers core-matrix columns 2kk, 2kk+1 (LBO = 128 B apart)
          uint64_t ad = make_desc(a0 + (uint32_t)(i * A_SLICE * 2 + kk * 256), 128, 512);
          uint64_t bd = make_desc(b0 + (uint32_t)(jsl * B_SLICE * 2 + kk * 256), 128, 512);
          mma_bf16(dt, ad, bd, idesc, first ? 0u : 1u);
          first = 0;
        }
      }
    }
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
            smem_u32(&mbar))
        : "memory");
  }
  // bounded wait for the MMAs
  bool done = false;
  for (unsigned long long it = 0; it < WAIT_LIMIT; it++)
    if (mbar_try(smem_u32(&mbar), 0)) {
      done = true;
      break;
    }
  if (!done) {
    if (lane == 0) atomicExch(err, 1);
    for (unsigned long long it = 0; it < WAIT_LIMIT; it++)
      if (mbar_try(smem_u32(&mbar), 0)) break;
  }
  done = __all_sync(0xffffffffu, done);  // tcgen05.ld is warp-collective
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");

  if (done) {
    // epilogue: lane = tile row, 32 columns; Horner over the slice orders
    const int x = x0 + warp * 32 + lane;
    long long I[TN];
#pragma unroll
    for (int cc = 0; cc < TN; cc++) I[cc] = 0;
    for (int g = 0; g < TS; g++) {
      uint32_t v[32];
      tmem_ld32(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)(g * TN), v);
#pragma unroll
      for (int cc = 0; cc < TN; cc++)
        I[cc] = (I[cc] << 8) + (long long)__float2ll_rn(__uint_as_float(v[cc]));
    }
    if (x < ns) {
      const int ex = eu[x];
      double *Ys = Y + (size_t)slot * per;
      const int *ezs = ez + (size_t)slot * ns;
#pragma unroll
      for (int cc = 0; cc < TN; cc++) {
        const int y = y0 + cc;
        const int d = y - x;
        if (y < ns && (mode == 0 ? d >= FARD : d <= -FARD))
          Ys[(size_t)x + (size_t)ns * y] = i64_scaled(I[cc], ex + ezs[y] - 8 * (TS + 1));
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tbase),
                 "r"(TMEM_COLS));
}

}  // namespace

// Far field of one chunk of segments on the tensor cores.  U/Ul are shared
// by the chunk; Z/Zl hold nb x ns per slot.  Writes the far-field elements
// of Y (per slot stride per); nb must be <= 32 (TK).
int farfield_tc(dbsrg_ctx *c, int ns, int nb, int nm, const double *U, const double *Ul,
                const double *Z, const double *Zl, double *Y, size_t per) {
  if (nb > TK) return set_err(c, DBSRG_EINVAL, "split far field: at most 32 bound orbitals");
  const int ntx = (ns + TM - 1) / TM, nty = (ns + TN - 1) / TN;
  // digit slices and scales in their own arena
  size_t a_el = (size_t)ntx * TS * A_SLICE, b_el = (size_t)nm * nty * TS * B_SLICE;
  size_t bytes = (2 * a_el + 2 * b_el) * sizeof(__nv_bfloat16) +
                 (2 * (size_t)ns + 2 * (size_t)nm * ns) * sizeof(int) + 64 * sizeof(int) + 4096;
  int rc = ensure_tcscratch(c, bytes);
  if (rc) return rc;
  char *p = (char *)c->tcscratch;
  auto take = [&](size_t n) { char *q = p; p += (n + 255) & ~(size_t)255; return (void *)q; };
  __nv_bfloat16 *Au = (__nv_bfloat16 *)take(a_el * 2), *Al = (__nv_bfloat16 *)take(a_el * 2);
  __nv_bfloat16 *Bz = (__nv_bfloat16 *)take(b_el * 2), *Bl = (__nv_bfloat16 *)take(b_el * 2);
  int *eu = (int *)take(ns * 4), *eul = (int *)take(ns * 4);
  int *ez = (int *)take((size_t)nm * ns * 4), *ezl = (int *)take((size_t)nm * ns * 4);
  int *err = (int *)take(64 * 4);
  cudaStream_t st = c->stream;
  DBSRG_TRY(c, cudaMemsetAsync(err, 0, sizeof(int), st));
  const size_t smem = (size_t)TS * (A_SLICE + B_SLICE) * sizeof(__nv_bfloat16);
  DBSRG_TRY(c, cudaFuncSetAttribute(k_far_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
  for (int mode = 0; mode < (Ul ? 2 : 1); mode++) {
    const double *Um = mode == 0 ? U : Ul;
    const double *Zm = mode == 0 ? Z : Zl;
    __nv_bfloat16 *Am = mode == 0 ? Au : Al, *Bm = mode == 0 ? Bz : Bl;
    int *eum = mode == 0 ? eu : eul, *ezm = mode == 0 ? ez : ezl;
    DBSRG_RUN(c, "k_split_rows",
              k_split_rows<<<(ntx * TM + 127) / 128, 128, 0, st>>>(ns, nb, Um, Am, eum));
    dim3 gs((unsigned)((nty * TN + 127) / 128), (unsigned)nm);
    DBSRG_RUN(c, "k_split_cols", k_split_cols<<<gs, 128, 0, st>>>(ns, nb, nm, Zm, Bm, ezm));
    dim3 gm((unsigned)ntx, (unsigned)nty, (unsigned)nm);
    DBSRG_RUN(c, "k_far_tc",
              k_far_tc<<<gm, 128, smem, st>>>(ns, nm, mode, Am, eum, Bm, ezm, Y, per, err));
  }
  int h = 0;
  DBSRG_TRY(c, cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  DBSRG_TRY(c, cudaStreamSynchronize(st));
  if (h) return set_err(c, DBSRG_ETIMEOUT, "tensor-core far field: MMA completion wait ran out");
  return DBSRG_OK;
}
