// tc_common.cuh -- inline-PTX helpers of the split-BF16 tcgen05 kernels:
// digit expansion, shared-memory matrix descriptors, MMA issue, mbarriers,
// bulk copies, TMEM loads, and the exact integer recombination.
//
// Split scheme.  An FP64 value v with |v| < 2^(e-1) is written as
//     v = 2^e * sum_{i<TS} d_i 2^(-8(i+1)) + r,   |d_i| <= 128, |r| < 2^(e-8TS)
// with balanced base-256 digits d_i (integers of at most 8 significant bits,
// exact in BF16).  A product sum over K <= 32 terms of two such expansions,
// taken per order g = i + j (i + j <= TS-1), is an integer
//     D_g = sum_{i+j=g} sum_k d_i(k) d'_j(k),  |D_g| <= TS*32*128^2 < 2^22,
// which the FP32 accumulation of the tensor cores holds exactly.  The
// epilogue converts each D_g exactly (magic-number add) and recombines
// I = sum_g D_g 256^(TS-1-g) in int64; the product sum is 2^(e+e'-8(TS+1)) I.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace tc {

constexpr int TS = 6;  // digit slices per operand

// offset (elements) of (r, k) in a tile of rows x 32 BF16 in the canonical
// K-major no-swizzle layout: 8x8 core matrices of 128 bytes, core (r/8, k/8)
// at ((r/8)*4 + k/8) * 64 elements.  Consecutive 32-row tiles stacked give
// the same layout for 64, 96 or 128 rows.
__device__ __forceinline__ int core_off(int r, int k) {
  return (((r >> 3) * 4 + (k >> 3)) << 6) + ((r & 7) << 3) + (k & 7);
}

// exponent e with 2^(e-1) > m >= 0 (0 for m == 0)
__device__ __forceinline__ int scale_exp(double m) {
  if (m == 0.0) return 0;
  int e;
  frexp(m, &e);  // m = f 2^e, f in [0.5, 1)
  return e + 1;
}

// the balanced base-256 digits of W < 2^(8TS-1) with sign neg: from the
// least significant digit, digits >= 128 taking -256 and a carry; the
// leading digit then stays in [0, 128]
__device__ __forceinline__ void digits_of(unsigned long long W, bool neg, float *d) {
  int carry = 0;
  int q[TS];
#pragma unroll
  for (int i = TS - 1; i >= 1; i--) {
    int t = (int)((W >> (8 * (TS - 1 - i))) & 255ULL) + carry;
    carry = t >= 128 ? 1 : 0;
    q[i] = t - 256 * carry;
  }
  q[0] = (int)((W >> (8 * (TS - 1))) & 255ULL) + carry;  // W < 2^(8TS-1): in [0, 128]
  const float sg = neg ? -1.0f : 1.0f;
#pragma unroll
  for (int i = 0; i < TS; i++) d[i] = sg * (float)q[i];
}

// balanced digits of v / 2^e (|v / 2^e| < 1/2): W = trunc(|v| 2^(8TS-e)) < 2^(8TS-1).
// Integer instructions on the bit pattern only.
__device__ __forceinline__ void digits(double v, int e, float *d) {
  const long long bits = __double_as_longlong(v);
  const int ev = (int)((bits >> 52) & 0x7FF);
  unsigned long long W = 0;
  if (ev != 0) {  // zero and subnormals (far below every scale here) give 0
    const unsigned long long mant = (unsigned long long)(bits & ((1LL << 52) - 1)) | (1ULL << 52);
    const int s = ev - 1075 - e + 8 * TS;  // W = mant * 2^s
    if (s >= 0)
      W = 0;  // |v| >= 2^e: excluded by the choice of e
    else if (-s < 64)
      W = mant >> (-s);
  }
  digits_of(W, bits < 0, d);
}

// trunc(f 2^sh) toward zero as int64, for |f 2^sh| < 2^62 (zero and
// subnormal f give 0)
__device__ __forceinline__ long long f32_fixed(float f, int sh) {
  const int b = __float_as_int(f);
  const int ex = (b >> 23) & 0xFF;
  if (ex == 0) return 0;
  const long long m = (long long)((b & 0x7FFFFF) | 0x800000);
  const int s = ex - 150 + sh;  // f 2^sh = m 2^s
  const long long v = s >= 0 ? (s < 39 ? m << s : 0) : (-s < 63 ? m >> (-s) : 0);
  return b < 0 ? -v : v;
}

// the same digits for a float-float value hi + lo (|hi| < 2^(e-1), |lo| at
// most half an ulp of hi) without FP64 arithmetic: both words to int64 fixed
// point with 15 bits below the last digit (exact but for the bits of lo
// beyond them), summed, W the integer part of the magnitude
constexpr int FFX = 15;
__device__ __forceinline__ void digits_ff(float hi, float lo, int e, float *d) {
  const int sh = 8 * TS - e + FFX;
  const long long X = f32_fixed(hi, sh) + f32_fixed(lo, sh);
  const bool neg = X < 0;
  digits_of((unsigned long long)(neg ? -X : X) >> FFX, neg, d);
}

// exponent e with 2^(e-1) > |hi + lo| from the float-float high words' maximum
// m: any float below 2^E is at most (1 - 2^-24) 2^E, so hi + lo stays below
// 2^E too (0 for m == 0)
__device__ __forceinline__ int scale_exp_ff(float m) {
  if (m == 0.0f) return 0;
  int e;
  frexpf(m, &e);
  return e + 1;
}

// exact int32 of an FP32 integer |f| < 2^22
__device__ __forceinline__ int f2i_exact(float f) {
  return __float_as_int(f + 12582912.0f) - 0x4B400000;
}

// I * 2^sh outside the normal range of FP64 (never produced by the scales
// here); kept out of line so the common path stays short
static __device__ __noinline__ double i64_scale_slow(long long I, int sh) {
  return ldexp(__ll2double_rn(I), sh);
}

// FP64 of I * 2^sh: the conversion of I rounded to nearest, then the
// scale 2^sh added to the exponent field (one conversion on the FP64 pipe
// and a few integer instructions)
__device__ __forceinline__ double i64_to_f64(long long I, int sh) {
  if (I == 0) return 0.0;
  const double d = __ll2double_rn(I);
  const long long bits = __double_as_longlong(d);
  const int ex = (int)((bits >> 52) & 0x7FF) + sh;
  if (ex <= 0 || ex >= 0x7FF) return i64_scale_slow(I, sh);
  return __longlong_as_double(bits + ((long long)sh << 52));
}

// v / 2 by the exponent field (normal v; zero stays zero)
__device__ __forceinline__ double half_f64(double v) {
  const long long b = __double_as_longlong(v);
  const int ex = (int)((b >> 52) & 0x7FF);
  if (ex <= 1) return v * 0.5;  // zero and the bottom of the range
  return __longlong_as_double(b - (1LL << 52));
}

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

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
      : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(mbar), "r"(count));
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

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// wait for the phase of the given parity; false after limit_ns nanoseconds
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity,
                                          unsigned long long limit_ns) {
  if (mbar_try(mbar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  while (!mbar_try(mbar, parity))
    if (globaltimer() - t0 > limit_ns) return false;
  return true;
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(bytes)
               : "memory");
}

// 1-D bulk copy global -> shared completing on an mbarrier (16-byte aligned
// addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes,
                                         uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&v)[8]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}

}  // namespace tc
