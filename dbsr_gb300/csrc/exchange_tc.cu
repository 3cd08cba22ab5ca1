// exchange_tc.cu -- the exchange cases (convol cases 3/4: R_data itype 4,
// S_data itypes 8/9) of the split-precision form: far field on the tcgen05
// tensor cores, near band, and the scatter into hch in one persistent kernel.
//
// For every owner block of a chunk and every quadrant that receives
// contributions (UPDATE_HS, updates.f90:110-179) the quadrant is cut into
// 128 x 32 tiles.  A tile becomes hch + f * (sum of its terms): a term is one
// segment's exchange result y taken directly or transposed (the ich < jch
// order, and the second half of the ich == jch case), f = 1/2 for ich == jch
// and 1 otherwise.  A term's far field is a split-BF16 product
//   direct:      y(x,y) = U(x,:) Z_s(:,y)        where y - x >= 9
//                         Ul(x,:) Zl_s(:,y)      where x - y >= 9 (R^k only)
//   transposed:  y(y,x) = Z_s(:,x)^T U(y,:)^T    where x - y >= 9
//                         Zl_s(:,x)^T Ul(y,:)^T  where y - x >= 9 (R^k only)
// (U, Ul, V, Vl the far-field vectors of the table, Z_s = C_s V^T with C_s
// the segment's coefficients over bound-orbital pairs) and its near band
// |y - x| <= 8 the sum over the segment's entries of the band pair
// potentials, both built in factor.cu.
//
// Operands are digit tiles in HBM (tc_common.cuh): U per table, Z per
// segment slot, each [slice][32-row tile][32 x 32 BF16, canonical K-major
// layout], so a 128-row A operand is four consecutive tiles of a slice and a
// 32-row B operand is one tile.  The K dimension of a tile is 32 bound
// orbitals; with more, the orbitals are cut into chunks of 32 (nbk of them),
// every chunk its own digit operand with its own row/column exponents, and
// a term's product is taken once per chunk (the chunks' products summed
// exactly in the int64 accumulators like the products of different terms).  One CTA per SM walks the tile list.
// One producer thread loads the operands two products ahead with 1-D bulk
// copies (cp.async.bulk completing on an mbarrier), issues each product's 42 MMAs (21 slice
// pairs x 2 K-steps of M=128 N=32 K=16) into one of two TMEM accumulator sets
// and commits them to a second mbarrier, while sixteen warps recombine the
// previous product out of the other set (warp w reads TMEM lanes 32(w%4)..
// and columns 8(w/4)..).  hch is read and written once per tile; no atomics.
// Every wait is bounded (2 s): on a timeout the kernel records an error word,
// waits (bounded) for its own copies and MMAs in flight, frees its TMEM and
// returns.
#include "internal.cuh"
#include "tc_common.cuh"
#include "ff.cuh"

namespace {

using namespace tc;

constexpr int FAR = 9, BAND = 8, NDB = 17;
constexpr int TILE = 32 * 32;                   // BF16 elements of a 32-row digit tile
constexpr uint32_t A_BYTES = 4 * TILE * 2;      // one slice of a 128-row operand
constexpr uint32_t B_BYTES = TILE * 2;          // one slice of a 32-row operand
constexpr int MAXT = 4;                         // terms per tile
constexpr int MAX_NBK = 4;                      // chunks of 32 bound orbitals (128 in all)
// staged band rows per diagonal: a tile's 32 columns meet 32 rows of each
// diagonal, plus one on each side for the 16-byte alignment of the copies
constexpr int BR = 34;
// limit of the waits for the kernel's own copies and MMAs before it exits
// (the pipeline waits use the context's limit, 2 s by default)
constexpr unsigned long long WAIT_NS = 2000000000ull;

// digits of 8 values (columns 8kg .. 8kg+7 of a 32-wide row, row exponent
// e) into a digit operand laid out [slice][32-row tile][TILE]
__device__ __forceinline__ void write_digit_group(__nv_bfloat16 *D, int NR, int row, int kg,
                                                  const double *vals8, int e) {
  const int rt = row >> 5, r = row & 31;
  float d[8][TS];
#pragma unroll
  for (int t = 0; t < 8; t++) digits(vals8[t], e, d[t]);
#pragma unroll
  for (int i = 0; i < TS; i++) {
    __align__(16) __nv_bfloat16 h[8];
#pragma unroll
    for (int t = 0; t < 8; t++) h[t] = __float2bfloat16_rn(d[t][i]);
    *(uint4 *)(D + ((size_t)i * NR + rt) * TILE + core_off(r, 8 * kg)) = *(const uint4 *)h;
  }
}

// the same for 8 normalised float-float values (no FP64 arithmetic)
__device__ __forceinline__ void write_digit_group_ff(__nv_bfloat16 *D, int NR, int row, int kg,
                                                     const float2 *vals8, int e) {
  const int rt = row >> 5, r = row & 31;
  float d[8][TS];
#pragma unroll
  for (int t = 0; t < 8; t++) digits_ff(vals8[t].x, vals8[t].y, e, d[t]);
#pragma unroll
  for (int i = 0; i < TS; i++) {
    __align__(16) __nv_bfloat16 h[8];
#pragma unroll
    for (int t = 0; t < 8; t++) h[t] = __float2bfloat16_rn(d[t][i]);
    *(uint4 *)(D + ((size_t)i * NR + rt) * TILE + core_off(r, 8 * kg)) = *(const uint4 *)h;
  }
}

// digits of one 32-wide row (values vals[0..31], row exponent e)
__device__ __forceinline__ void write_digit_row(__nv_bfloat16 *D, int NR, int row,
                                                const double *vals, int e) {
#pragma unroll
  for (int kg = 0; kg < 4; kg++) write_digit_group(D, NR, row, kg, vals + 8 * kg, e);
}

// exponents of one digit operand: NR*32 row exponents, then the NR maxima
// over its 32-row tiles
constexpr int EXP_PER_ROWTILE = 33;

// U (ns x nb, column-major), orbital chunk blockIdx.y (orbitals 32c ..
// 32c+31) -> digit operand [chunk][slice][NR][TILE] and exponents
// [chunk][NR*33]
__global__ void k_udigits(int ns, int nb, int NR, const double *U, __nv_bfloat16 *Dall,
                          int *euall) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int ck = blockIdx.y;
  if (x >= NR * 32) return;
  __nv_bfloat16 *D = Dall + (size_t)ck * TS * NR * TILE;
  int *eu = euall + (size_t)ck * NR * EXP_PER_ROWTILE;
  double vals[32];
  double m = 0.0;
#pragma unroll
  for (int k = 0; k < 32; k++) {
    const int o = 32 * ck + k;
    vals[k] = (x < ns && o < nb) ? U[(size_t)x + (size_t)ns * o] : 0.0;
    m = fmax(m, fabs(vals[k]));
  }
  const int e = scale_exp(m);
  eu[x] = e;
  const int et = __reduce_max_sync(0xffffffffu, e);  // a warp is one 32-row tile
  if ((threadIdx.x & 31) == 0) eu[NR * 32 + x / 32] = et;
  write_digit_row(D, NR, x, vals, e);
}

struct ZArgs {
  int ns, nb, nbk, NR, nm, lower;
  const float2 *V[4], *Vl[4], *Kb[4];  // float-float copies
  const int *members;
  const SegInfo *info;
  const int *pairs;
  const float2 *cd;
  __nv_bfloat16 *Zd;  // [a][mode][slot][chunk][slice][NR][TILE]
  int *ez;            // [a][mode][slot][chunk][NR*33]
  double *Yb;         // [a][slot][ns*17]
};

// Per segment slot and atype, one thread per row y (ZROWS rows a block):
//   Z_s(k,y) = sum_{e in s, first orbital k} c_e V(y, second orbital)  (Zl with Vl)
//   Yb_s(y,d) = sum_e c_e Kb(pair_e; y, d)                             (near band)
// as float-float sums (ff.cuh), then the digits of Z (and Zl) and their row
// exponents.  The sums read the pair potentials of every entry: the kernel
// is bound by those reads (L2 and HBM), not by its arithmetic.
constexpr int ZROWS = 32;  // one warp per block: one 32-row digit tile
// ONE: at most 32 bound orbitals (one chunk)
template <bool ONE>
__global__ void __launch_bounds__(ZROWS) k_zdigits(const ZArgs z) {
  // [mode][nb][ZROWS] float-float: per thread one column; sized by the bound
  // orbitals (and the modes) in use, which sets how many blocks share an SM
  extern __shared__ float2 zs[];
  const int t = threadIdx.x, y = blockIdx.x * ZROWS + t, slot = blockIdx.y, a = blockIdx.z;
  const int ns = z.ns, nb = z.nb;
  float2 *z0 = zs, *z1 = zs + nb * ZROWS;
  for (int k = 0; k < nb; k++) {
    z0[k * ZROWS + t] = make_float2(0.0f, 0.0f);
    if (z.lower) z1[k * ZROWS + t] = make_float2(0.0f, 0.0f);
  }
  const SegInfo si = z.info[z.members[slot]];
  const float2 *V = z.V[a], *Vl = z.lower ? z.Vl[a] : nullptr, *Kb = z.Kb[a];
  const size_t kper = (size_t)ns * NDB;
  float bh[NDB], bl[NDB];
#pragma unroll
  for (int d = 0; d < NDB; d++) bh[d] = bl[d] = 0.0f;
  if (y < ns) {
    // the next entry's pair index and coefficient are loaded while this
    // entry's potentials are summed
    int pr_n = si.start < si.end ? z.pairs[si.start] : 0;
    float2 c_n = si.start < si.end ? z.cd[si.start] : make_float2(0.0f, 0.0f);
    for (int e = si.start; e < si.end; e++) {
      const int pr = pr_n, oa = pr / nb, ob = pr - oa * nb;
      const float2 c = c_n;
      if (e + 1 < si.end) {
        pr_n = z.pairs[e + 1];
        c_n = z.cd[e + 1];
      }
      const float2 *kb = Kb + (size_t)pr * kper + y;
      float2 kv[NDB];
#pragma unroll
      for (int d = 0; d < NDB; d++) kv[d] = kb[(size_t)ns * d];
      {
        float2 acc = z0[oa * ZROWS + t];
        ffa::mac(c, V[(size_t)y + (size_t)ns * ob], acc.x, acc.y);
        z0[oa * ZROWS + t] = acc;
      }
      if (Vl) {
        float2 acc = z1[oa * ZROWS + t];
        ffa::mac(c, Vl[(size_t)y + (size_t)ns * ob], acc.x, acc.y);
        z1[oa * ZROWS + t] = acc;
      }
#pragma unroll
      for (int d = 0; d < NDB; d++) ffa::mac(c, kv[d], bh[d], bl[d]);
    }
    double *yb = z.Yb + ((size_t)a * z.nm + slot) * kper + y;
#pragma unroll
    for (int d = 0; d < NDB; d++) yb[(size_t)ns * d] = ffa::value(bh[d], bl[d]);
  }
  const size_t sl = (size_t)z.NR * TILE;
  for (int mode = 0; mode < (z.lower ? 2 : 1); mode++) {
    float2 *zz = mode ? z1 : z0;
    // per chunk of 32 orbitals: each sum renormalised in place (TwoSum:
    // hi + lo unchanged, |lo| at most half an ulp of hi), the row exponent
    // from the high words, the digits 8 columns at a time
    for (int ck = 0; ck < (ONE ? 1 : z.nbk); ck++) {
      float m = 0.0f;
      for (int k = 32 * ck; k < (ONE ? nb : min(nb, 32 * ck + 32)); k++) {
        const float2 v = zz[k * ZROWS + t];
        const float s = v.x + v.y, bp = s - v.x;
        zz[k * ZROWS + t] = make_float2(s, (v.x - (s - bp)) + (v.y - bp));
        m = fmaxf(m, fabsf(s));
      }
      const int e = scale_exp_ff(m);
      const size_t op = ((size_t)(a * 2 + mode) * z.nm + slot) * (ONE ? 1 : z.nbk) + ck;
      z.ez[op * z.NR * EXP_PER_ROWTILE + y] = e;
      const int et = __reduce_max_sync(0xffffffffu, e);  // a warp is one 32-row tile
      if ((t & 31) == 0) z.ez[op * z.NR * EXP_PER_ROWTILE + z.NR * 32 + y / 32] = et;
      for (int kg = 0; kg < 4; kg++) {
        float2 vals[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
          const int k = 32 * ck + 8 * kg + u;
          vals[u] = k < nb ? zz[k * ZROWS + t] : make_float2(0.0f, 0.0f);
        }
        write_digit_group_ff(z.Zd + op * TS * sl, z.NR, y, kg, vals, e);
      }
    }
  }
}

struct XArgs {
  int ns, NR, ntx, nty, nm, na, lower;
  int nbk;                     // chunks of 32 bound orbitals (products per term and field)
  int nrows;                   // (quadrant record, x tile) rows of 128 x ns
  const __nv_bfloat16 *Ud[4];  // per atype: [mode][chunk][slice][NR][TILE]
  const int *eu[4];            // per atype: [mode][chunk][NR*33]
  const __nv_bfloat16 *Zd;     // [a][mode][slot][chunk][slice][NR][TILE]
  const int *ez;               // [a][mode][slot][chunk][NR*33]
  const double *Yb;            // [a][slot][ns*17]
  const XQuad *xq;
  double *hch;
  int *err;
  unsigned long long wait_ns;  // limit of the pipeline waits
  int inject_wait;             // test: the epilogue first waits on a barrier nobody completes
};

// one row (quadrant record, x tile): the quadrant's terms, term code
// t = atype | transposed << 2 | member slot << 3
struct Row {
  int blk, qr, qc, nt, half, tx;
  int tc[MAXT];
};

__device__ __forceinline__ void load_row(const XArgs &p, int row, Row &r) {
  const int4 *q = reinterpret_cast<const int4 *>(p.xq + row / p.ntx);
  const int4 v0 = q[0], v1 = q[1], v2 = q[2];  // blk qr qc nt | half t0 t1 t2 | t3 . . .
  r.tx = row % p.ntx;
  r.blk = v0.x;
  r.qr = v0.y;
  r.qc = v0.z;
  r.nt = min(v0.w, MAXT);
  r.half = v1.x;
  r.tc[0] = v1.y;
  r.tc[1] = v1.z;
  r.tc[2] = v1.w;
  r.tc[3] = v2.x;
}

// term code of term t (a select chain keeps the codes in registers)
__device__ __forceinline__ int term_code(const Row &r, int t) {
  return t == 0 ? r.tc[0] : t == 1 ? r.tc[1] : t == 2 ? r.tc[2] : r.tc[3];
}

// products of tile (tx, ty), packed 3 bits each (term | mode << 2): per term
// the upper field of its result and, for R^k, the lower one, where the tile
// meets them.  *band: the tile meets the near band |y - x| <= 8.
__device__ __forceinline__ uint32_t tile_products(const XArgs &p, const Row &r, int ty, int &np,
                                                  bool &band) {
  const int x0 = r.tx * 128, y0 = ty * 32;
  const bool up = (y0 + 31) - x0 >= FAR, lo = (x0 + 127) - y0 >= FAR;
  uint32_t codes = 0;
  np = 0;
#pragma unroll
  for (int t = 0; t < MAXT; t++) {
    if (t >= r.nt) break;
    const bool tra = (term_code(r, t) >> 2) & 1;
    if (tra ? lo : up) codes |= (uint32_t)t << (3 * np++);
    if (p.lower && (tra ? up : lo)) codes |= (uint32_t)(t | 4) << (3 * np++);
  }
  band = (y0 + 31) - x0 >= -BAND && y0 - (x0 + 127) <= BAND;
  return codes;
}

// first staged row of diagonal dd (y - x = dd - BAND) of a direct term's
// band for the tile at (x0, ty0): rows x = y - (dd - BAND) of the columns
// y in ty0 .. ty0+31 within the tile's rows, rounded down to even
__device__ __forceinline__ int band_row0(int x0, int ty0, int dd) {
  return max(ty0 + BAND - dd, x0) & ~1;
}

// the producer's walk over the products of its rows (tiles without
// products skipped): row, tile ty, field product pc of np (the codes) and
// orbital chunk ck of nbk, and the row's terms
struct ProdIt {
  int row, ty, pc, np, ck;
  uint32_t codes;
  Row r;
};

// advance to the next product (orbital chunks innermost); false when the
// CTA's rows are done
__device__ __forceinline__ bool prod_next(const XArgs &p, int nbk, ProdIt &it) {
  if (it.row >= p.nrows) return false;
  if (++it.ck < nbk) return true;
  it.ck = 0;
  it.pc++;
  while (it.pc >= it.np) {
    if (++it.ty >= p.nty) {
      it.row += gridDim.x;
      if (it.row >= p.nrows) return false;
      load_row(p, it.row, it.r);
      it.ty = 0;
    }
    bool band;
    it.codes = tile_products(p, it.r, it.ty, it.np, band);
    it.pc = 0;
  }
  return true;
}

// digit operands of the current product: A (128 rows of the tile) and B
// (32 columns), each [slice][32-row tile][TILE] with slices sl apart
__device__ __forceinline__ void prod_operands(const XArgs &p, int nbk, const ProdIt &it, size_t sl,
                                              const __nv_bfloat16 *&As,
                                              const __nv_bfloat16 *&Bs) {
  const int ck = it.ck;
  const int pcode = (it.codes >> (3 * it.pc)) & 7, t = pcode & 3, m = pcode >> 2;
  const int tc = term_code(it.r, t), a = tc & 3, tra = (tc >> 2) & 1, slot = tc >> 3;
  const __nv_bfloat16 *Ub = p.Ud[a] + ((size_t)m * nbk + ck) * TS * sl;
  const __nv_bfloat16 *Zb =
      p.Zd + (((size_t)(a * 2 + m) * p.nm + slot) * nbk + ck) * TS * sl;
  As = (tra ? Zb : Ub) + (size_t)4 * it.r.tx * TILE;
  Bs = (tra ? Ub : Zb) + (size_t)it.ty * TILE;
}

constexpr int NCW = 16;               // consumer (epilogue) warps
constexpr int CPT = 32 / (NCW / 4);   // tile columns per consumer thread
constexpr int WPROD = NCW;            // producer warp
constexpr int WSTAGE = NCW + 1;       // stager warp
constexpr int NTHR = 32 * (NCW + 2);
static_assert(TS == 6, "the epilogue pairs the six orders");

__device__ __forceinline__ void consumers_sync() {
  asm volatile("bar.sync 1, %0;\n" ::"n"(32 * NCW) : "memory");
}

// 8-byte asynchronous copy global -> shared; zero fill when !valid
__device__ __forceinline__ void cp_async8(uint32_t dst, const void *src, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src),
               "r"(valid ? 8 : 0)
               : "memory");
}

// hch[dst .. dst + bytes) += smem[src ..] as one asynchronous bulk
// reduction (FP64 add in L2, one add per element: the same rounding as an
// FP64 add on the SM); 16-byte aligned addresses, bytes a multiple of 16
__device__ __forceinline__ void bulk_reduce_add_f64(double *dst, uint32_t src, uint32_t bytes) {
  asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.add.f64 [%0], [%1], %2;\n" ::"l"(dst),
               "r"(src), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(mbar) : "memory");
}

// Warp-specialised, one CTA per SM walking rows (quadrant record, x tile)
// of 128 x ns; every role walks the same tile sequence.
//  * producer (warp NCW, one lane): issues the bulk loads of the next
//    product (once the MMAs of the previous one completed; the 128-row A
//    operand only when neither A slot holds it already), then waits for this
//    product's operands and for the consumers to have read the TMEM set two
//    products back, issues the MMAs and commits them;
//  * stager (warp NCW+1, even ns): per tile waits until the consumers are
//    done with the tile two back, adds that tile's results into hch with
//    one asynchronous bulk reduction per column (cp.reduce.async.bulk
//    .add.f64: the FP64 add happens in L2, so hch is neither loaded into the
//    SM nor added there), waits until the reduction has read the buffer,
//    then bulk-loads the band rows of the new tile's terms (one copy per
//    lane) into the buffers that tile used, a tile ahead of the consumers;
//  * consumers (warps 0..NCW-1): per product read the TMEM set, release it
//    and add the product into int64 accumulators; per tile convert, add the
//    band, write the results into the tile's result buffer and release it.
//    (Odd ns: the consumers stage hch and the band themselves with 8-byte
//    copies and write hch + result to global memory.)
// 18 warps: two SM sub-partitions hold 5 of them, and a sub-partition has
// 16384 registers, so at most 96 registers a thread.  Four consumer warps per
// sub-partition hide each other's TMEM and integer latencies.
//
// ONE: at most 32 bound orbitals (one orbital chunk, nbk = 1).
template <bool ONE>
__global__ void __maxnreg__(96) k_xfused(const XArgs p) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char *sA = smraw;                          // [2][TS][A_BYTES]
  unsigned char *sB = sA + 2 * TS * A_BYTES;          // [2][TS][B_BYTES]
  double *sband = (double *)(sB + 2 * TS * B_BYTES);  // [2][MAXT][NDB][BR]
  double *shch = sband + (size_t)2 * MAXT * NDB * BR; // [2][32 columns][128 rows]
  __shared__ __align__(8) uint64_t bar_ld[2], bar_mma[2], bar_free[2], bar_tile[2], bar_sfree[2];
  __shared__ __align__(8) uint64_t bar_never;  // completed by nobody (the injected timeout)
  __shared__ uint32_t tmem_base;
  __shared__ int s_abort;
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  if (tid == 0) {
    for (int b = 0; b < 2; b++) {
      mbar_init(smem_u32(&bar_ld[b]), 1);
      mbar_init(smem_u32(&bar_mma[b]), 1);
      mbar_init(smem_u32(&bar_free[b]), NCW);
      mbar_init(smem_u32(&bar_tile[b]), 1);
      mbar_init(smem_u32(&bar_sfree[b]), NCW);
    }
    mbar_init(smem_u32(&bar_never), 1);
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
  const size_t sl = (size_t)p.NR * TILE;  // elements per slice of a digit operand
  const size_t ms = 2 * (size_t)p.ns;
  const int EX = p.NR * EXP_PER_ROWTILE;  // exponents per digit operand
  const int nbk = ONE ? 1 : p.nbk;
  // even ns: every hch column and band row of a tile starts on a 16-byte
  // boundary and is staged by 1-D bulk copies; odd ns: 8-byte cp.async
  const bool bulk = (p.ns % 2) == 0;
  volatile int *abort_flag = &s_abort;

  if (warp == WPROD) {
    // ------------------------------------------------------------ producer
    // Product q reads B slot q & 1 and one of two A slots, chosen by the A
    // operand's address (kept while it repeats: U rows of a direct term are
    // the same for every tile of a row and every row of the CTA).  The loads
    // of product q + 1 are issued before the MMAs of product q wait for
    // theirs, so the copies of two products are in flight at once.
    if (lane == 0) {
      ProdIt it;
      it.row = (int)blockIdx.x - (int)gridDim.x;
      it.ty = p.nty - 1;
      it.pc = 0;
      it.np = 0;
      it.ck = nbk - 1;  // the first prod_next moves to the first product
      it.codes = 0;
      const __nv_bfloat16 *aKey[2] = {nullptr, nullptr};  // A operand held by each A slot
      int aslot[2] = {0, 0};                              // A slot of products q & 1
      long long ld_issued = -1, ld_done = -1, mma_last = -1;
      bool fail = false;
      // bulk loads of product qq into B slot qq & 1 and an A slot
      auto issue_loads = [&](long long qq) {
        const __nv_bfloat16 *As, *Bs;
        prod_operands(p, nbk, it, sl, As, Bs);
        const int bq = (int)(qq & 1);
        int s;
        if (aKey[0] == As)
          s = 0;
        else if (aKey[1] == As)
          s = 1;
        else  // the slot that product qq - 1 (MMAs not yet issued) does not read
          s = qq == 0 ? 0 : 1 - aslot[(qq - 1) & 1];
        const bool needA = aKey[s] != As;
        const uint32_t la = smem_u32(&bar_ld[bq]);
        mbar_expect_tx(la, TS * (B_BYTES + (needA ? A_BYTES : 0)));
        for (int i = 0; i < TS; i++) {
          if (needA)
            bulk_g2s(smem_u32(sA + (size_t)(s * TS + i) * A_BYTES), As + (size_t)i * sl, A_BYTES,
                     la);
          bulk_g2s(smem_u32(sB + (size_t)(bq * TS + i) * B_BYTES), Bs + (size_t)i * sl, B_BYTES,
                   la);
        }
        aKey[s] = As;
        aslot[bq] = s;
        ld_issued = qq;
      };
      bool more = prod_next(p, nbk, it);
      if (more) issue_loads(0);
      for (long long q = 0; more; q++) {
        if (*abort_flag) {
          fail = true;
          break;
        }
        const int b = (int)(q & 1);
        const uint32_t n = (uint32_t)(q >> 1);
        // loads of product q + 1: its B slot (and an A slot other than
        // product q's) were last read by product q - 1 or earlier
        const bool more1 = prod_next(p, nbk, it);
        if (more1) {
          if (q >= 1 &&
              !mbar_wait(smem_u32(&bar_mma[(q - 1) & 1]), (uint32_t)(((q - 1) >> 1) & 1),
                         p.wait_ns)) {
            fail = true;
            break;
          }
          issue_loads(q + 1);
        }
        // MMAs of product q
        if (!mbar_wait(smem_u32(&bar_ld[b]), n & 1, p.wait_ns)) {
          fail = true;
          break;
        }
        ld_done = q;
        if (q >= 2 && !mbar_wait(smem_u32(&bar_free[b]), (n - 1) & 1, p.wait_ns)) {
          fail = true;
          break;
        }
        fence_after();
        constexpr uint32_t idesc = make_idesc(128, 32);
        // descriptors of the slots; operand offsets added to the address
        // field (shared addresses stay below 2^18 bytes: no carry)
        const uint64_t ad0 =
            make_desc(smem_u32(sA + (size_t)aslot[b] * TS * A_BYTES), 128, 512);
        const uint64_t bd0 = make_desc(smem_u32(sB + (size_t)b * TS * B_BYTES), 128, 512);
#pragma unroll
        for (int g = 0; g < TS; g++) {
          const uint32_t dt = tbase + (uint32_t)(b * 256 + g * 32);
#pragma unroll
          for (int i = 0; i <= g; i++)
#pragma unroll
            for (int kk = 0; kk < 2; kk++)
              mma_bf16(dt, ad0 + ((i * A_BYTES + kk * 256) >> 4),
                       bd0 + (((g - i) * B_BYTES + kk * 256) >> 4), idesc,
                       (i == 0 && kk == 0) ? 0u : 1u);
        }
        mma_commit(smem_u32(&bar_mma[b]));
        mma_last = q;
        more = more1;
      }
      if (fail) {
        *abort_flag = 1;
        atomicExch(p.err, 1);
        // copies still in flight land before the CTA exits
        for (long long k = ld_done + 1; k <= ld_issued; k++)
          mbar_wait(smem_u32(&bar_ld[k & 1]), (uint32_t)((k >> 1) & 1), WAIT_NS);
      }
      // every MMA of this CTA completes before its TMEM is freed
      if (mma_last >= 0)
        mbar_wait(smem_u32(&bar_mma[mma_last & 1]), (uint32_t)((mma_last >> 1) & 1), WAIT_NS);
    }
  } else if (warp == WSTAGE) {
    // ------------------------------------------------------------ stager
    if (bulk) {
      // two buffer pairs (the results and the band rows of a tile): tile n
      // takes pair n & 1 once the consumers have released tile n - 2 and
      // its results have been reduced into hch, so the band copies of the
      // next tile overlap the consumers' current one
      uint32_t nst = 0;  // tiles staged
      long long last_n[2] = {-1, -1};
      bool fail = false;
      // the hch columns of the tile each buffer holds the results of: the
      // tile's first column in hch, its rows and columns
      double *pdst[2] = {nullptr, nullptr};
      int prow[2] = {0, 0}, pcol[2] = {0, 0};
      // add buffer s's results into hch once the consumers have written them
      // (waited before), and wait until the reduction has read the buffer
      auto reduce = [&](int s) {
        if (pdst[s] && *abort_flag == 0) {
          if (lane < pcol[s])
            bulk_reduce_add_f64(pdst[s] + ms * (size_t)lane,
                                smem_u32(shch + (size_t)s * 32 * 128 + (size_t)lane * 128),
                                (uint32_t)prow[s] * 8);
          asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
          asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
        }
        pdst[s] = nullptr;
        __syncwarp();
      };
      Row r;
      for (int row = blockIdx.x; row < p.nrows && !fail; row += gridDim.x) {
        load_row(p, row, r);
        const int x0 = r.tx * 128, nrow = min(128, p.ns - x0);
        const double *hq = p.hch + (size_t)(r.blk - 1) * ms * ms + (size_t)(r.qr - 1) * p.ns +
                           ms * (size_t)(r.qc - 1) * p.ns;
        for (int ty = 0; ty < p.nty; ty++) {
          int np;
          bool band;
          tile_products(p, r, ty, np, band);
          if (np == 0 && !band) continue;
          const int ty0 = ty * 32, ncol = min(32, p.ns - ty0), s = nst & 1;
          bool ok = *abort_flag == 0;
          if (ok && nst >= 2)
            ok = mbar_wait(smem_u32(&bar_sfree[s]), ((nst >> 1) - 1) & 1, p.wait_ns);
          ok = __all_sync(0xffffffffu, ok);
          if (!ok) {
            fail = true;
            break;
          }
          reduce(s);  // tile nst - 2's results, before the buffer is reused
          // rows of diagonal dd of a direct term's band: band_row0 .. hi | 1
          // (both even-aligned ends inside the tile's rows and below ns)
          const int hib = min(x0 + 127, p.ns - 1);
          double *sb = sband + (size_t)s * MAXT * NDB * BR;
          const uint32_t tb = smem_u32(&bar_tile[s]);
          if (lane == 0) {
            uint32_t bytes = 0;  // the band rows (hch is added by a bulk reduction)
            if (band)
              for (int t = 0; t < r.nt; t++) {
                if ((term_code(r, t) >> 2) & 1) {
                  bytes += NDB * 8 * ncol;
                } else {
                  for (int dd = 0; dd < NDB; dd++) {
                    const int lo = band_row0(x0, ty0, dd),
                              hi = min(ty0 + 31 + BAND - dd, hib) | 1;
                    if (hi > lo) bytes += (uint32_t)(hi - lo + 1) * 8;
                  }
                }
              }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            mbar_expect_tx(tb, bytes);
          }
          __syncwarp();
          pdst[s] = const_cast<double *>(hq) + ms * (size_t)ty0 + x0;
          prow[s] = nrow;
          pcol[s] = ncol;
          if (band)
            for (int k = lane; k < NDB * r.nt; k += 32) {
              const int t = k / NDB, dd = k % NDB, tc = term_code(r, t);
              const bool tra = (tc >> 2) & 1;
              const double *yb =
                  p.Yb + ((size_t)(tc & 3) * p.nm + (tc >> 3)) * (size_t)p.ns * NDB +
                  (size_t)p.ns * dd;
              const uint32_t dst = smem_u32(sb + ((size_t)t * NDB + dd) * BR);
              if (tra) {
                bulk_g2s(dst, yb + ty0, (uint32_t)ncol * 8, tb);
              } else {
                const int lo = band_row0(x0, ty0, dd), hi = min(ty0 + 31 + BAND - dd, hib) | 1;
                if (hi > lo) bulk_g2s(dst, yb + lo, (uint32_t)(hi - lo + 1) * 8, tb);
              }
            }
          last_n[s] = nst;
          nst++;
        }
      }
      // the results of the last two staged tiles, once their consumers are done
      for (long long k = (long long)nst - 2; !fail && k < (long long)nst; k++) {
        if (k < 0) continue;
        const int s = (int)(k & 1);
        bool ok = mbar_wait(smem_u32(&bar_sfree[s]), (uint32_t)((k >> 1) & 1), p.wait_ns);
        ok = __all_sync(0xffffffffu, ok);
        if (!ok) {
          fail = true;
          break;
        }
        reduce(s);
      }
      if (fail && lane == 0) {
        *abort_flag = 1;
        atomicExch(p.err, 1);
      }
      // the reductions complete, and the copies of the last staged tiles
      // land, before the CTA exits
      asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
      if (lane == 0)
        for (int s = 0; s < 2; s++)
          if (last_n[s] >= 0)
            mbar_wait(smem_u32(&bar_tile[s]), (uint32_t)((last_n[s] >> 1) & 1), WAIT_NS);
    }
  } else {
    // ------------------------------------------------------------ consumers
    // Thread (lane group lg, column group cg) owns row x of the tile and CPT
    // columns.  Product p scales element (x, y) by 2^(er_p(x) + ec_p(y)); the
    // thread sums its products exactly in int64 aligned to one exponent, the
    // largest row + column exponent of the products added so far (right
    // shifts drop bits below 2^-56 of the largest scale), and converts each
    // sum to FP64 once.
    const int lg = warp & 3, cg = warp >> 2, xl = lg * 32 + lane;
    bool dead = false;
    if (p.inject_wait) {  // a wait that runs out: the kernel must abort cleanly
      const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&bar_never), 0, p.wait_ns));
      if (!ok) {
        dead = true;
        *abort_flag = 1;
        if (lane == 0) atomicExch(p.err, 1);
      }
    }
    uint32_t q = 0, ntile = 0;
    Row r;
    long long Iacc[CPT];
    for (int row = blockIdx.x; row < p.nrows; row += gridDim.x) {
      load_row(p, row, r);
      const int x = r.tx * 128 + xl, x0 = r.tx * 128;
      const bool row_ok = x < p.ns;
      const double *hq = p.hch + (size_t)(r.blk - 1) * ms * ms + (size_t)(r.qr - 1) * p.ns +
                         ms * (size_t)(r.qc - 1) * p.ns;
      for (int ty = 0; ty < p.nty; ty++) {
        int np;
        bool band;
        const uint32_t codes = tile_products(p, r, ty, np, band);
        if (np == 0 && !band) continue;
        const int y0 = ty * 32 + cg * CPT, ty0 = ty * 32;
        double *h = const_cast<double *>(hq) + ms * (size_t)y0 + x;
        // this tile's staging buffers (the stager alternates two of them)
        const int sbuf = bulk ? (int)(ntile & 1) : 0;
        const double *sh = shch + (size_t)sbuf * 32 * 128;
        double *sbt = sband + (size_t)sbuf * MAXT * NDB * BR;
#pragma unroll
        for (int c = 0; c < CPT; c++) Iacc[c] = 0;
        if (!bulk) {  // odd ns: the consumers stage hch and the band themselves
#pragma unroll
          for (int c = 0; c < CPT; c++) {
            const bool ok = row_ok && y0 + c < p.ns;
            cp_async8(smem_u32(sh + (size_t)(cg * CPT + c) * 128 + xl), ok ? h + ms * c : p.hch,
                      ok);
          }
          if (band) {
            for (int t = 0; t < r.nt; t++) {
              const int tc = term_code(r, t);
              const double *yb =
                  p.Yb + ((size_t)(tc & 3) * p.nm + (tc >> 3)) * (size_t)p.ns * NDB;
              double *sb = sbt + (size_t)t * NDB * BR;
              if (!((tc >> 2) & 1)) {  // rows x of y, diagonals y - x (band_row0 on)
                for (int e = tid; e < NDB * BR; e += 32 * NCW) {
                  const int dd = e / BR, rr = band_row0(x0, ty0, dd) + e % BR,
                            yy = rr + dd - BAND;
                  const bool ok = rr < p.ns && rr < x0 + 128 && yy >= 0 && yy < p.ns;
                  cp_async8(smem_u32(sb + e), ok ? yb + rr + (size_t)p.ns * dd : yb, ok);
                }
              } else {  // rows y of y, diagonals x - y
                for (int e = tid; e < NDB * 32; e += 32 * NCW) {
                  const int dd = e / 32, rr = ty0 + e % 32, xx = rr + dd - BAND;
                  const bool ok = rr < p.ns && xx >= 0 && xx < p.ns;
                  cp_async8(smem_u32(sb + dd * BR + e % 32), ok ? yb + rr + (size_t)p.ns * dd : yb,
                            ok);
                }
              }
            }
          }
          asm volatile("cp.async.commit_group;\n" ::: "memory");
        }
        // per element the exponent the int64 sum is kept at: the largest
        // row + column exponent of the products added so far
        int cur[CPT];
#pragma unroll
        for (int c = 0; c < CPT; c++) cur[c] = -100000;
        // products of the tile: field product fp of the codes, orbital chunk
        // ck (innermost)
        for (int pc = 0, fp = 0, ck = 0; fp < np;
             pc++, q++, (++ck == nbk ? (ck = 0, fp++) : 0)) {
          const int b = q & 1;
          const uint32_t n = q >> 1;
          const int pcode = (codes >> (3 * fp)) & 7, m = pcode >> 2;
          const int tc = term_code(r, pcode & 3), a = tc & 3, tra = (tc >> 2) & 1;
          const int *eua = p.eu[a] + ((size_t)m * nbk + ck) * EX;
          const int *ezs = p.ez + (((size_t)(a * 2 + m) * p.nm + (tc >> 3)) * nbk + ck) * EX;
          const int er = tra ? ezs[x] : eua[x];
          // column exponents: 8 ints at a 32-byte aligned offset
          const int4 *ep = reinterpret_cast<const int4 *>((tra ? eua : ezs) + y0);
          const int4 e0 = ep[0], e1 = ep[1];
          const int ec[CPT] = {e0.x, e0.y, e0.z, e0.w, e1.x, e1.y, e1.z, e1.w};
          // the product's far field: y - x >= FAR (sg = 1) or x - y >= FAR (sg = -1)
          const int sg = (tra ^ m) ? -1 : 1;
          if (!dead && *abort_flag) dead = true;
          bool ok = !dead && mbar_wait(smem_u32(&bar_mma[b]), n & 1, p.wait_ns);
          ok = __all_sync(0xffffffffu, ok);
          if (!ok) {
            if (!dead) {
              dead = true;
              *abort_flag = 1;
              if (lane == 0) atomicExch(p.err, 1);
            }
            continue;
          }
          fence_after();
          // orders 2k and 2k+1 of the product: bits(D + 1.5 2^23) = D + 1.5 2^23
          // (as an integer) exactly for |D| < 2^22; wrap-around unsigned
          // arithmetic leaves P_k = 256 D_2k + D_2k+1
          int P[3][CPT];
          const uint32_t col =
              tbase + ((uint32_t)(lg * 32) << 16) + (uint32_t)(b * 256 + cg * CPT);
          {
            // the six orders' columns loaded together, one wait
            uint32_t v[TS][CPT];
#pragma unroll
            for (int g = 0; g < TS; g++) tmem_ld8(col + 32 * g, v[g]);
            tmem_wait_ld();
#pragma unroll
            for (int k = 0; k < 3; k++)
#pragma unroll
              for (int c = 0; c < CPT; c++)
                P[k][c] =
                    (int)(((uint32_t)__float_as_uint(__uint_as_float(v[2 * k][c]) + 12582912.0f)
                           << 8) +
                          (uint32_t)__float_as_uint(__uint_as_float(v[2 * k + 1][c]) + 12582912.0f) -
                          257u * 0x4B400000u);
          }
          fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(smem_u32(&bar_free[b]));
#pragma unroll
          for (int c = 0; c < CPT; c++) {
            // I = sum_g D_g 256^(TS-1-g) = P0 2^32 + P1 2^16 + P2
            const long long I = (long long)P[0][c] * 4294967296LL +
                                (long long)P[1][c] * 65536LL + (long long)P[2][c];
            const int d = (y0 + c) - x, se = er + ec[c];
            if (sg * d >= FAR) {
              if (pc == 0) {  // the tile's first product: the sum starts at its exponent
                Iacc[c] = I;
                cur[c] = se;
              } else {
                if (se > cur[c]) {  // raise the sum to the new exponent
                  const int up = se - cur[c];
                  Iacc[c] = up < 63 ? Iacc[c] >> up : 0;
                  cur[c] = se;
                }
                const int sh = cur[c] - se;
                if (sh < 63) Iacc[c] += I >> sh;
              }
            }
          }
        }
        // to FP64 (the factor 1/2 of ich == jch in the exponent), near band,
        // and the write of the tile: one FP64 add per element
        double val[CPT];
#pragma unroll
        for (int c = 0; c < CPT; c++)
          val[c] = cur[c] > -100000 ? i64_to_f64(Iacc[c], cur[c] - 8 * (TS + 1) - r.half) : 0.0;
        if (bulk) {
          const bool ok =
              dead || mbar_wait(smem_u32(&bar_tile[sbuf]), (ntile >> 1) & 1, p.wait_ns);
          if (!ok) {
            dead = true;
            *abort_flag = 1;
            atomicExch(p.err, 1);
          }
        } else {
          asm volatile("cp.async.wait_group 0;\n" ::: "memory");
          if (band) consumers_sync();
        }
        if (band) {
#pragma unroll
          for (int c = 0; c < CPT; c++) {
            const int y = y0 + c, d = y - x;
            if (d < -BAND || d > BAND || !row_ok || y >= p.ns) continue;
            for (int t = 0; t < r.nt; t++) {
              const double *sb = sbt + (size_t)t * NDB * BR;
              const double bv =
                  ((term_code(r, t) >> 2) & 1)
                      ? sb[(BAND - d) * BR + (y - ty0)]
                      : sb[(d + BAND) * BR + (x - band_row0(x0, ty0, d + BAND))];
              val[c] += r.half ? half_f64(bv) : bv;
            }
          }
        }
        if (bulk) {
          // the results into the buffer; the stager adds the buffer into hch
          // (one bulk reduction per column) before the buffer is reused
          if (!dead) {
            double *so = const_cast<double *>(sh);
#pragma unroll
            for (int c = 0; c < CPT; c++) so[(size_t)(cg * CPT + c) * 128 + xl] = val[c];
          }
          asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
          __syncwarp();
          if (lane == 0) mbar_arrive(smem_u32(&bar_sfree[sbuf]));
          ntile++;
        } else {
          if (row_ok && !dead) {
#pragma unroll
            for (int c = 0; c < CPT; c++)
              if (y0 + c < p.ns) h[ms * c] = sh[(size_t)(cg * CPT + c) * 128 + xl] + val[c];
          }
          if (band) consumers_sync();
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tbase), "r"(512));
}

}  // namespace

bool build_xquads(int na, const int *ii, const int *jj, const std::vector<int> &mem,
                  const std::vector<int> &own, const std::vector<SegInfo> &hinfo,
                  std::vector<XQuad> &out) {
  for (int os : own) {
    const SegInfo &si = hinfo[mem[os]];
    const int ps = si.partner >= 0 ? os + 1 : -1;
    for (int q = 0; q < 4; q++) {
      XQuad r{};
      r.blk = si.blk;
      r.qr = q % 2 + 1;
      r.qc = q / 2 + 1;
      for (int a = 0; a < na; a++)
        for (int pass = 0; pass < 2; pass++) {
          const int slot = pass == 0 ? os : ps;
          if (slot < 0) break;
          const SegInfo &sj = hinfo[mem[slot]];
          const bool eq = sj.ich == sj.jch;
          const bool dir = (sj.ich > sj.jch || eq) && r.qr == ii[a] && r.qc == jj[a];
          const bool tra = (sj.ich < sj.jch && r.qr == ii[a] && r.qc == jj[a]) ||
                           (eq && r.qr == jj[a] && r.qc == ii[a]);
          if (eq) r.half = 1;
          for (int k = 0; k < 2; k++) {
            if (!(k == 0 ? dir : tra)) continue;
            if (r.nt == MAXT) return false;
            r.term[r.nt++] = a | k << 2 | slot << 3;
          }
        }
      if (r.nt > 0) out.push_back(r);
    }
  }
  return true;
}

// algorithmic work of one k_xfused launch: the read-modify-write of hch over
// every tile that receives a product or a band term (16 bytes per element),
// and the tensor-core FLOPs of its products (42 MMAs of 128 x 32 x 16)
static void xfused_work(const XQuad *hxq, int nxq, int ns, int lower, int nbk, double &bytes,
                        double &flops) {
  bytes = flops = 0.0;
  if (!hxq) return;
  const int ntx = (ns + 127) / 128, nty = (ns + 31) / 32;
  for (int i = 0; i < nxq; i++) {
    const XQuad &r = hxq[i];
    for (int tx = 0; tx < ntx; tx++)
      for (int ty = 0; ty < nty; ty++) {
        const int x0 = tx * 128, y0 = ty * 32;
        const bool up = (y0 + 31) - x0 >= FAR, lo = (x0 + 127) - y0 >= FAR;
        int np = 0;
        for (int t = 0; t < r.nt && t < MAXT; t++) {
          const bool tra = (r.term[t] >> 2) & 1;
          np += (tra ? lo : up) + (lower && (tra ? up : lo));
        }
        const bool band = (y0 + 31) - x0 >= -BAND && y0 - (x0 + 127) <= BAND;
        if (np == 0 && !band) continue;
        bytes += 16.0 * std::min(128, ns - x0) * std::min(32, ns - y0);
        flops += (double)np * nbk * (TS * (TS + 1)) * 2.0 * 128 * 32 * 16;
      }
  }
}

int split_exchange(dbsrg_ctx *c, const SplitExchange &x) {
  const int ns = c->g.ns, nb = c->nbound;
  if (nb < 1 || nb > 32 * MAX_NBK)
    return set_err(c, DBSRG_EINVAL, "split exchange: 1..128 bound orbitals");
  const int nbk = (nb + 31) / 32;  // chunks of 32 bound orbitals
  if (x.na < 1 || x.na > 4 || x.nm < 1 || (x.nxq < 1 && !x.prep)) return DBSRG_OK;
  cudaStream_t st = c->stream;
  int rc0;
  const int ntx = (ns + 127) / 128, NR = 4 * ntx, nty = (ns + 31) / 32;
  const size_t sl = (size_t)NR * TILE;
  // digits of U (and Ul) per table, cached with the far-field vectors
  for (int a = 0; a < x.na; a++) {
    FarField *f = const_cast<FarField *>(x.far[a]);
    if (f->Ud) continue;
    void *d = nullptr;
    const size_t bytes = 2 * (size_t)nbk * TS * sl * sizeof(__nv_bfloat16) +
                         2 * (size_t)nbk * NR * EXP_PER_ROWTILE * sizeof(int);
    if (!(d = cache_alloc(c, bytes))) {
      return set_err(c, DBSRG_ENOMEM, "digit allocation failed");
    }
    f->Ud = d;
    f->eu = (int *)((char *)d + 2 * (size_t)nbk * TS * sl * sizeof(__nv_bfloat16));
    for (int m = 0; m < (f->Ul ? 2 : 1); m++)
      DBSRG_RUN(c, "k_udigits",
                k_udigits<<<dim3((unsigned)((NR * 32 + 127) / 128), (unsigned)nbk), 128, 0, st>>>(
                    ns, nb, NR, m ? f->Ul : f->U,
                    (__nv_bfloat16 *)f->Ud + (size_t)m * nbk * TS * sl,
                    f->eu + (size_t)m * nbk * NR * EXP_PER_ROWTILE));
  }
  const size_t mv = (size_t)ns * nb;
  if (x.prep) {  // float-float far-field vectors, then nothing per chunk
    for (int a = 0; a < x.na; a++) {
      const float2 *v;
      if (x.lower && !x.far[a]->Vl) return set_err(c, DBSRG_EINVAL, "split exchange: no lower field");
      if ((rc0 = ff_of(c, x.far[a]->V, mv, &v))) return rc0;
      if (x.lower && (rc0 = ff_of(c, x.far[a]->Vl, mv, &v))) return rc0;
    }
    return DBSRG_OK;
  }
  // per chunk: Z digits, exponents, band rows, error word
  const size_t zel = (size_t)x.na * 2 * x.nm * nbk * TS * sl;
  const size_t zex = (size_t)x.na * 2 * x.nm * nbk * NR * EXP_PER_ROWTILE;
  const size_t ybn = (size_t)x.na * x.nm * ns * NDB;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t bytes = al(zel * 2) + al(zex * 4) + al(ybn * 8);
  int rc = ensure_tcscratch(c, bytes);
  if (rc) return rc;
  char *q = (char *)c->tcscratch;
  __nv_bfloat16 *Zd = (__nv_bfloat16 *)q;
  int *ez = (int *)(q + al(zel * 2));
  double *Yb = (double *)(q + al(zel * 2) + al(zex * 4));
  if (!c->kerr) {  // read and cleared at the end of the Gen_matrix call
    DBSRG_TRY(c, cudaMalloc((void **)&c->kerr, sizeof(int)));
    DBSRG_TRY(c, cudaMemsetAsync(c->kerr, 0, sizeof(int), st));
  }
  ZArgs z{};
  z.ns = ns;
  z.nb = nb;
  z.nbk = nbk;
  z.NR = NR;
  z.nm = x.nm;
  z.lower = x.lower;
  if (!x.cdf) return set_err(c, DBSRG_EINVAL, "split exchange: no float-float coefficients");
  for (int a = 0; a < x.na; a++) {
    if (x.lower && !x.far[a]->Vl) return set_err(c, DBSRG_EINVAL, "split exchange: no lower field");
    if ((rc = ff_of(c, x.far[a]->V, mv, &z.V[a]))) return rc;
    if (x.lower && (rc = ff_of(c, x.far[a]->Vl, mv, &z.Vl[a]))) return rc;
    z.Kb[a] = x.Kbf[a];
  }
  z.members = x.members;
  z.info = x.info;
  z.pairs = x.pairs;
  z.cd = x.cdf;
  z.Zd = Zd;
  z.ez = ez;
  z.Yb = Yb;
  const size_t zsm = (size_t)(x.lower ? 2 : 1) * nb * ZROWS * sizeof(float2);
  const void *zk = nbk == 1 ? (const void *)k_zdigits<true> : (const void *)k_zdigits<false>;
  if ((rc = raise_smem_limit(c, zk, zsm))) return rc;
  // executed work: per PQ type, row and entry one multiply-add per field
  // (Z, and Zl for R^k) and per band diagonal (17), float-float; the entry's
  // band potential values (17 float-float pairs a row) read, the digits and
  // band rows written
  const double zf = 2.0 * x.na * ns * (1.0 + x.lower + NDB) * (double)x.nent;
  const double zb = 8.0 * x.na * ns * ((1.0 + x.lower + NDB) * (double)x.nent +
                                       NDB * (double)x.nm) +
                    2.0 * TS * (double)x.na * (1 + x.lower) * x.nm * nbk * NR * TILE;
  // every row of the operand, zeros past ns
  const dim3 gz((unsigned)(NR * 32 / ZROWS), (unsigned)x.nm, (unsigned)x.na);
  if (nbk == 1)
    DBSRG_RUN_W(c, "k_zdigits", zb, zf, k_zdigits<true><<<gz, ZROWS, zsm, st>>>(z));
  else
    DBSRG_RUN_W(c, "k_zdigits", zb, zf, k_zdigits<false><<<gz, ZROWS, zsm, st>>>(z));
  XArgs p{};
  p.ns = ns;
  p.NR = NR;
  p.ntx = ntx;
  p.nty = nty;
  p.nm = x.nm;
  p.na = x.na;
  p.lower = x.lower;
  p.nbk = nbk;
  p.nrows = x.nxq * ntx;
  for (int a = 0; a < x.na; a++) {
    p.Ud[a] = (const __nv_bfloat16 *)x.far[a]->Ud;
    p.eu[a] = x.far[a]->eu;
  }
  p.Zd = Zd;
  p.ez = ez;
  p.Yb = Yb;
  p.xq = x.xq;
  p.hch = hch_base(c);
  p.err = c->kerr;
  p.wait_ns = c->wait_ns;
  p.inject_wait = c->inject_wait ? 1 : 0;
  const size_t smem = 2 * TS * (size_t)(A_BYTES + B_BYTES) +
                      ((size_t)2 * MAXT * NDB * BR + 2 * 32 * 128) * sizeof(double);
  const void *xk = nbk == 1 ? (const void *)k_xfused<true> : (const void *)k_xfused<false>;
  if ((rc = raise_smem_limit(c, xk, smem))) return rc;
  const int nblk = std::min(p.nrows, std::max(1, c->nsm));
  double wbytes = 0.0, wflops = 0.0;
  if (c->timing) xfused_work(x.hxq, x.nxq, ns, x.lower, nbk, wbytes, wflops);
  if (nbk == 1)
    DBSRG_RUN_W(c, "k_xfused", wbytes, wflops,
                k_xfused<true><<<(unsigned)nblk, NTHR, smem, st>>>(p));
  else
    DBSRG_RUN_W(c, "k_xfused", wbytes, wflops,
                k_xfused<false><<<(unsigned)nblk, NTHR, smem, st>>>(p));
  return DBSRG_OK;
}
