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
// 32-row B operand is one tile.  One CTA per SM walks the tile list.
// Thread 0 loads the next product's operands with 1-D bulk copies
// (cp.async.bulk completing on an mbarrier), issues its 42 MMAs (21 slice
// pairs x 2 K-steps of M=128 N=32 K=16) into one of two TMEM accumulator sets
// and commits them to a second mbarrier, while the eight warps recombine the
// previous product out of the other set (warp w reads TMEM lanes 32(w%4)..
// and columns 16(w/4)..).  hch is read and written once per tile; no atomics.
// Every wait is bounded (2 s): on a timeout the kernel records an error word,
// waits (bounded) for its own copies and MMAs in flight, frees its TMEM and
// returns.
#include "internal.cuh"
#include "tc_common.cuh"

namespace {

using namespace tc;

constexpr int FAR = 9, BAND = 8, NDB = 17;
constexpr int TILE = 32 * 32;                   // BF16 elements of a 32-row digit tile
constexpr uint32_t A_BYTES = 4 * TILE * 2;      // one slice of a 128-row operand
constexpr uint32_t B_BYTES = TILE * 2;          // one slice of a 32-row operand
constexpr int MAXT = 4;                         // terms per tile
constexpr unsigned long long WAIT_NS = 2000000000ull;

// digits of one 32-wide row (values vals[0..31], row exponent e) into a
// digit operand laid out [slice][32-row tile][TILE]
__device__ __forceinline__ void write_digit_row(__nv_bfloat16 *D, int NR, int row,
                                                const double *vals, int e) {
  const int rt = row >> 5, r = row & 31;
#pragma unroll
  for (int kg = 0; kg < 4; kg++) {
    float d[8][TS];
#pragma unroll
    for (int t = 0; t < 8; t++) digits(vals[8 * kg + t], e, d[t]);
#pragma unroll
    for (int i = 0; i < TS; i++) {
      __align__(16) __nv_bfloat16 h[8];
#pragma unroll
      for (int t = 0; t < 8; t++) h[t] = __float2bfloat16_rn(d[t][i]);
      *(uint4 *)(D + ((size_t)i * NR + rt) * TILE + core_off(r, 8 * kg)) = *(const uint4 *)h;
    }
  }
}

// U (ns x nb, column-major) -> digit operand [slice][NR][TILE] and row exponents
__global__ void k_udigits(int ns, int nb, int NR, const double *U, __nv_bfloat16 *D, int *eu) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= NR * 32) return;
  double vals[32];
  double m = 0.0;
#pragma unroll
  for (int k = 0; k < 32; k++) {
    vals[k] = (x < ns && k < nb) ? U[(size_t)x + (size_t)ns * k] : 0.0;
    m = fmax(m, fabs(vals[k]));
  }
  const int e = scale_exp(m);
  eu[x] = e;
  write_digit_row(D, NR, x, vals, e);
}

struct ZArgs {
  int ns, nb, NR, nm, lower;
  const double *V[4], *Vl[4], *Kb[4];
  const int *members;
  const SegInfo *info;
  const int *pairs;
  const double *cd;
  __nv_bfloat16 *Zd;  // [a][mode][slot][slice][NR][TILE]
  int *ez;            // [a][mode][slot][NR*32]
  double *Yb;         // [a][slot][ns*17]
};

// Per segment slot and atype, one thread per row y:
//   Z_s(k,y) = sum_{e in s, first orbital k} c_e V(y, second orbital)  (Zl with Vl)
//   Yb_s(y,d) = sum_e c_e Kb(pair_e; y, d)                             (near band)
// then the digits of Z (and Zl) and their row exponents.
__global__ void __launch_bounds__(128) k_zdigits(const ZArgs z) {
  extern __shared__ double zs[];  // [2][32][128]: per thread one column
  const int t = threadIdx.x, y = blockIdx.x * 128 + t, slot = blockIdx.y, a = blockIdx.z;
  const int ns = z.ns, nb = z.nb;
  double *z0 = zs, *z1 = zs + 32 * 128;
  for (int k = 0; k < 32; k++) {
    z0[k * 128 + t] = 0.0;
    z1[k * 128 + t] = 0.0;
  }
  const SegInfo si = z.info[z.members[slot]];
  const double *V = z.V[a], *Vl = z.lower ? z.Vl[a] : nullptr, *Kb = z.Kb[a];
  const size_t kper = (size_t)ns * NDB;
  double band[NDB];
#pragma unroll
  for (int d = 0; d < NDB; d++) band[d] = 0.0;
  if (y < ns) {
    for (int e = si.start; e < si.end; e++) {
      const int pr = z.pairs[e], oa = pr / nb, ob = pr - oa * nb;
      const double c = z.cd[e];
      z0[oa * 128 + t] = fma(c, V[(size_t)y + (size_t)ns * ob], z0[oa * 128 + t]);
      if (Vl) z1[oa * 128 + t] = fma(c, Vl[(size_t)y + (size_t)ns * ob], z1[oa * 128 + t]);
      const double *kb = Kb + (size_t)pr * kper + y;
#pragma unroll
      for (int d = 0; d < NDB; d++) band[d] = fma(c, kb[(size_t)ns * d], band[d]);
    }
    double *yb = z.Yb + ((size_t)a * z.nm + slot) * kper + y;
#pragma unroll
    for (int d = 0; d < NDB; d++) yb[(size_t)ns * d] = band[d];
  }
  const size_t sl = (size_t)z.NR * TILE;
  for (int mode = 0; mode < (z.lower ? 2 : 1); mode++) {
    const double *zz = mode ? z1 : z0;
    double vals[32];
    double m = 0.0;
#pragma unroll
    for (int k = 0; k < 32; k++) {
      vals[k] = zz[k * 128 + t];
      m = fmax(m, fabs(vals[k]));
    }
    const int e = scale_exp(m);
    const size_t op = (size_t)(a * 2 + mode) * z.nm + slot;
    z.ez[op * z.NR * 32 + y] = e;
    write_digit_row(z.Zd + op * TS * sl, z.NR, y, vals, e);
  }
}

struct XArgs {
  int ns, NR, ntx, nty, nm, na, lower;
  long long nitems;
  const __nv_bfloat16 *Ud[4];  // per atype: [mode][slice][NR][TILE]
  const int *eu[4];            // per atype: [mode][NR*32]
  const __nv_bfloat16 *Zd;     // [a][mode][slot][slice][NR][TILE]
  const int *ez;               // [a][mode][slot][NR*32]
  const double *Yb;            // [a][slot][ns*17]
  int ii[4], jj[4];
  const int *members;
  const int *pqlist;           // owner slot * 4 + quadrant
  const SegInfo *info;
  double *hch;
  int *err;
};

struct Plan {
  int ok, tx, ty, qr, qc, blk, nt, half, np, band;
  int ta[MAXT], tslot[MAXT], ttra[MAXT];
  int pt[2 * MAXT], pm[2 * MAXT];
};

// terms and products of one tile (the term order of k_scatter_x: atype-major,
// owner then partner)
__device__ void make_plan(const XArgs &p, long long item, Plan &pl) {
  pl.ok = 0;
  pl.nt = 0;
  pl.np = 0;
  if (item >= p.nitems) return;
  const long long per = (long long)p.ntx * p.nty;
  const int pqi = (int)(item / per), rem = (int)(item % per);
  pl.tx = rem / p.nty;
  pl.ty = rem % p.nty;
  const int code = p.pqlist[pqi], oslot = code >> 2, quad = code & 3;
  pl.qr = quad % 2 + 1;
  pl.qc = quad / 2 + 1;
  const SegInfo si = p.info[p.members[oslot]];
  pl.blk = si.blk;
  const int pslot = si.partner >= 0 ? oslot + 1 : -1;
  pl.half = 0;
  for (int a = 0; a < p.na; a++)
    for (int pass = 0; pass < 2; pass++) {
      const int slot = pass == 0 ? oslot : pslot;
      if (slot < 0) break;
      const SegInfo sj = p.info[p.members[slot]];
      const bool eq = sj.ich == sj.jch;
      const bool dir = (sj.ich > sj.jch || eq) && pl.qr == p.ii[a] && pl.qc == p.jj[a];
      const bool tra = (sj.ich < sj.jch && pl.qr == p.ii[a] && pl.qc == p.jj[a]) ||
                       (eq && pl.qr == p.jj[a] && pl.qc == p.ii[a]);
      if (eq) pl.half = 1;
      for (int k = 0; k < 2; k++) {
        if (!(k == 0 ? dir : tra)) continue;
        if (pl.nt == MAXT) {
          atomicExch(p.err, 2);
          continue;
        }
        pl.ta[pl.nt] = a;
        pl.tslot[pl.nt] = slot;
        pl.ttra[pl.nt] = k;
        pl.nt++;
      }
    }
  const int x0 = pl.tx * 128, y0 = pl.ty * 32;
  const bool up = (y0 + 31) - x0 >= FAR, lo = (x0 + 127) - y0 >= FAR;
  for (int t = 0; t < pl.nt; t++) {
    const bool r0 = pl.ttra[t] ? lo : up;  // upper field of the term's result
    const bool r1 = p.lower && (pl.ttra[t] ? up : lo);
    if (r0) {
      pl.pt[pl.np] = t;
      pl.pm[pl.np++] = 0;
    }
    if (r1) {
      pl.pt[pl.np] = t;
      pl.pm[pl.np++] = 1;
    }
  }
  pl.band = (y0 + 31) - x0 >= -BAND && y0 - (x0 + 127) <= BAND;
  pl.ok = 1;
}

__global__ void __launch_bounds__(256, 1) k_xfused(const XArgs p) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char *sA = smraw;                          // [2][TS][A_BYTES]
  unsigned char *sB = sA + 2 * TS * A_BYTES;          // [2][TS][B_BYTES]
  double *sband = (double *)(sB + 2 * TS * B_BYTES);  // [MAXT][NDB][128]
  __shared__ __align__(8) uint64_t bar_ld[2], bar_mma[2];
  __shared__ uint32_t tmem_base;
  __shared__ Plan sp[2];
  __shared__ int s_abort;
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  const int lg = warp & 3, hf = warp >> 2;
  if (tid == 0) {
    for (int b = 0; b < 2; b++) {
      mbar_init(smem_u32(&bar_ld[b]), 1);
      mbar_init(smem_u32(&bar_mma[b]), 1);
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
  const size_t sl = (size_t)p.NR * TILE;  // elements per slice of a digit operand

  // thread 0 state of the asynchronous work in flight
  long long ld_pending = -1, mma_pending = -1;  // product index of an unfinished load / commit

  auto issue = [&](const Plan &pl, int pc, uint32_t P) -> bool {
    const int b = P & 1;
    const uint32_t par = (P >> 1) & 1;
    const int t = pl.pt[pc], m = pl.pm[pc], a = pl.ta[t], slot = pl.tslot[t];
    const __nv_bfloat16 *Ub = p.Ud[a] + (size_t)m * TS * sl;
    const __nv_bfloat16 *Zb = p.Zd + ((size_t)(a * 2 + m) * p.nm + slot) * TS * sl;
    const __nv_bfloat16 *As = (pl.ttra[t] ? Zb : Ub) + (size_t)4 * pl.tx * TILE;
    const __nv_bfloat16 *Bs = (pl.ttra[t] ? Ub : Zb) + (size_t)pl.ty * TILE;
    const uint32_t la = smem_u32(&bar_ld[b]);
    mbar_expect_tx(la, TS * (A_BYTES + B_BYTES));
    for (int i = 0; i < TS; i++) {
      bulk_g2s(smem_u32(sA + (size_t)(b * TS + i) * A_BYTES), As + (size_t)i * sl, A_BYTES, la);
      bulk_g2s(smem_u32(sB + (size_t)(b * TS + i) * B_BYTES), Bs + (size_t)i * sl, B_BYTES, la);
    }
    ld_pending = P;
    if (!mbar_wait(la, par, WAIT_NS)) return false;
    ld_pending = -1;
    const uint32_t idesc = make_idesc(128, 32);
    const uint32_t a0 = smem_u32(sA + (size_t)b * TS * A_BYTES);
    const uint32_t b0 = smem_u32(sB + (size_t)b * TS * B_BYTES);
    for (int g = 0; g < TS; g++) {
      const uint32_t dt = tbase + (uint32_t)(b * 256 + g * 32);
      uint32_t acc = 0;
      for (int i = 0; i <= g; i++)
        for (int kk = 0; kk < 2; kk++) {
          const uint64_t ad = make_desc(a0 + (uint32_t)(i * A_BYTES + kk * 256), 128, 512);
          const uint64_t bd = make_desc(b0 + (uint32_t)((g - i) * B_BYTES + kk * 256), 128, 512);
          mma_bf16(dt, ad, bd, idesc, acc);
          acc = 1;
        }
    }
    mma_commit(smem_u32(&bar_mma[b]));
    mma_pending = P;
    return true;
  };

  double tacc[16];
#pragma unroll
  for (int c = 0; c < 16; c++) tacc[c] = 0.0;

  auto epilogue = [&](const Plan &pl, int pc, uint32_t P) -> bool {
    const int b = P & 1;
    const uint32_t par = (P >> 1) & 1;
    const bool ok = mbar_wait(smem_u32(&bar_mma[b]), par, WAIT_NS);
    // tcgen05.ld is warp-collective: a warp reads only when all its lanes saw completion
    if (!__all_sync(0xffffffffu, ok)) return false;
    fence_after();
    uint32_t v[TS][16];
#pragma unroll
    for (int g = 0; g < TS; g++)
      tmem_ld16(tbase + ((uint32_t)(lg * 32) << 16) + (uint32_t)(b * 256 + g * 32 + hf * 16), v[g]);
    tmem_wait_ld();
    const int t = pl.pt[pc], m = pl.pm[pc], a = pl.ta[t], slot = pl.tslot[t], tra = pl.ttra[t];
    const int x = pl.tx * 128 + lg * 32 + lane;
    const int *eua = p.eu[a] + (size_t)m * p.NR * 32;
    const int *ezs = p.ez + ((size_t)(a * 2 + m) * p.nm + slot) * p.NR * 32;
    const int erow = (tra ? ezs[x] : eua[x]) - 8 * (TS + 1);
    const int y0 = pl.ty * 32 + hf * 16;
    const int *ecol = tra ? eua : ezs;
#pragma unroll
    for (int c = 0; c < 16; c++) {
      const int y = y0 + c, d = y - x;
      const bool in = tra ? (m == 0 ? d <= -FAR : d >= FAR) : (m == 0 ? d >= FAR : d <= -FAR);
      if (in && x < p.ns && y < p.ns) {
        long long I = 0;
#pragma unroll
        for (int g = 0; g < TS; g++) I = I * 256 + (long long)f2i_exact(__uint_as_float(v[g][c]));
        tacc[c] += i64_scaled(I, erow + ecol[y]);
      }
    }
    return true;
  };

  auto finish = [&](const Plan &pl) {
    const int x0 = pl.tx * 128, y0 = pl.ty * 32, xl = lg * 32 + lane, x = x0 + xl;
    const int ns = p.ns;
    if (pl.band) {
      for (int t = 0; t < pl.nt; t++) {
        const double *yb = p.Yb + ((size_t)pl.ta[t] * p.nm + pl.tslot[t]) * (size_t)ns * NDB;
        double *sb = sband + (size_t)t * NDB * 128;
        if (!pl.ttra[t]) {  // rows x of y, diagonals y - x
          for (int q = tid; q < NDB * 128; q += 256) {
            const int dd = q / 128, r = x0 + q % 128, yy = r + dd - BAND;
            sb[q] = (r < ns && yy >= 0 && yy < ns) ? yb[r + (size_t)ns * dd] : 0.0;
          }
        } else {  // rows y of y, diagonals x - y
          for (int q = tid; q < NDB * 32; q += 256) {
            const int dd = q / 32, r = y0 + q % 32, xx = r + dd - BAND;
            sb[q] = (r < ns && xx >= 0 && xx < ns) ? yb[r + (size_t)ns * dd] : 0.0;
          }
        }
      }
      __syncthreads();
#pragma unroll
      for (int c = 0; c < 16; c++) {
        const int y = y0 + hf * 16 + c, d = y - x;
        if (d < -BAND || d > BAND || x >= ns || y >= ns) continue;
        for (int t = 0; t < pl.nt; t++) {
          const double *sb = sband + (size_t)t * NDB * 128;
          tacc[c] += pl.ttra[t] ? sb[(BAND - d) * 32 + (y - y0)] : sb[(d + BAND) * 128 + xl];
        }
      }
    }
    if ((pl.np > 0 || pl.band) && x < ns) {
      const int ms = 2 * ns;
      double *hb = p.hch + (size_t)(pl.blk - 1) * ms * ms + (size_t)(pl.qr - 1) * ns +
                   (size_t)ms * (pl.qc - 1) * ns + x;
#pragma unroll
      for (int c = 0; c < 16; c++) {
        const int y = y0 + hf * 16 + c;
        if (y < ns) {
          double *h = hb + (size_t)ms * y;
          *h = *h + (pl.half ? 0.5 * tacc[c] : tacc[c]);
        }
      }
    }
#pragma unroll
    for (int c = 0; c < 16; c++) tacc[c] = 0.0;
  };

  long long item = blockIdx.x;
  int ci = 0, pc = 0;
  uint32_t P = 0;
  if (tid == 0) {
    make_plan(p, item, sp[0]);
    if (sp[0].ok && sp[0].np > 0 && !issue(sp[0], 0, 0)) s_abort = 1;
  }
  fence_before();
  __syncthreads();
  fence_after();
  while (!s_abort && sp[ci].ok) {
    const Plan &cur = sp[ci];
    const bool last = cur.np == 0 || pc == cur.np - 1;
    if (tid == 0) {
      if (!last) {
        if (!issue(cur, pc + 1, P + 1)) s_abort = 1;
      } else {
        Plan &nx = sp[ci ^ 1];
        make_plan(p, item + gridDim.x, nx);
        if (nx.ok && nx.np > 0 && !issue(nx, 0, P + (cur.np > 0 ? 1u : 0u))) s_abort = 1;
      }
    }
    if (cur.np > 0 && !epilogue(cur, pc, P)) s_abort = 1;
    if (last) finish(cur);
    fence_before();
    __syncthreads();
    fence_after();
    if (cur.np > 0) P++;
    if (last) {
      ci ^= 1;
      item += gridDim.x;
      pc = 0;
    } else {
      pc++;
    }
  }
  if (s_abort && tid == 0) {
    atomicExch(p.err, 1);
    // bounded waits for this CTA's own copies and MMAs still in flight
    if (ld_pending >= 0)
      mbar_wait(smem_u32(&bar_ld[ld_pending & 1]), (uint32_t)((ld_pending >> 1) & 1), WAIT_NS);
    if (mma_pending >= 0)
      mbar_wait(smem_u32(&bar_mma[mma_pending & 1]), (uint32_t)((mma_pending >> 1) & 1), WAIT_NS);
  }
  fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tbase), "r"(512));
}

}  // namespace

int split_exchange(dbsrg_ctx *c, const SplitExchange &x) {
  const int ns = c->g.ns, nb = c->nbound;
  if (nb < 1 || nb > 32) return set_err(c, DBSRG_EINVAL, "split exchange: 1..32 bound orbitals");
  if (x.na < 1 || x.na > 4 || x.nm < 1 || x.npq < 1) return DBSRG_OK;
  cudaStream_t st = c->stream;
  const int ntx = (ns + 127) / 128, NR = 4 * ntx, nty = (ns + 31) / 32;
  const size_t sl = (size_t)NR * TILE;
  // digits of U (and Ul) per table, cached with the far-field vectors
  for (int a = 0; a < x.na; a++) {
    FarField *f = const_cast<FarField *>(x.far[a]);
    if (f->Ud) continue;
    void *d = nullptr;
    const size_t bytes = 2 * TS * sl * sizeof(__nv_bfloat16) + 2 * (size_t)NR * 32 * sizeof(int);
    if (cudaMalloc(&d, bytes) != cudaSuccess) {
      cudaGetLastError();
      return set_err(c, DBSRG_ENOMEM, "digit allocation failed");
    }
    f->Ud = d;
    f->eu = (int *)((char *)d + 2 * TS * sl * sizeof(__nv_bfloat16));
    for (int m = 0; m < (f->Ul ? 2 : 1); m++)
      DBSRG_RUN(c, "k_udigits",
                k_udigits<<<(unsigned)((NR * 32 + 127) / 128), 128, 0, st>>>(
                    ns, nb, NR, m ? f->Ul : f->U, (__nv_bfloat16 *)f->Ud + (size_t)m * TS * sl,
                    f->eu + (size_t)m * NR * 32));
  }
  // per chunk: Z digits, exponents, band rows, error word
  const size_t zel = (size_t)x.na * 2 * x.nm * TS * sl;
  const size_t zex = (size_t)x.na * 2 * x.nm * NR * 32;
  const size_t ybn = (size_t)x.na * x.nm * ns * NDB;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t bytes = al(zel * 2) + al(zex * 4) + al(ybn * 8) + 256;
  int rc = ensure_tcscratch(c, bytes);
  if (rc) return rc;
  char *q = (char *)c->tcscratch;
  __nv_bfloat16 *Zd = (__nv_bfloat16 *)q;
  int *ez = (int *)(q + al(zel * 2));
  double *Yb = (double *)(q + al(zel * 2) + al(zex * 4));
  int *err = (int *)(q + al(zel * 2) + al(zex * 4) + al(ybn * 8));
  DBSRG_TRY(c, cudaMemsetAsync(err, 0, sizeof(int), st));
  ZArgs z{};
  z.ns = ns;
  z.nb = nb;
  z.NR = NR;
  z.nm = x.nm;
  z.lower = x.lower;
  for (int a = 0; a < x.na; a++) {
    z.V[a] = x.far[a]->V;
    z.Vl[a] = x.far[a]->Vl;
    z.Kb[a] = x.Kb[a];
    if (x.lower && !x.far[a]->Vl) return set_err(c, DBSRG_EINVAL, "split exchange: no lower field");
  }
  z.members = x.members;
  z.info = x.info;
  z.pairs = x.pairs;
  z.cd = x.cd;
  z.Zd = Zd;
  z.ez = ez;
  z.Yb = Yb;
  const size_t zsm = 2 * 32 * 128 * sizeof(double);
  DBSRG_TRY(c, cudaFuncSetAttribute(k_zdigits, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)zsm));
  DBSRG_RUN(c, "k_zdigits",
            k_zdigits<<<dim3((unsigned)ntx, (unsigned)x.nm, (unsigned)x.na), 128, zsm, st>>>(z));
  XArgs p{};
  p.ns = ns;
  p.NR = NR;
  p.ntx = ntx;
  p.nty = nty;
  p.nm = x.nm;
  p.na = x.na;
  p.lower = x.lower;
  p.nitems = (long long)x.npq * ntx * nty;
  for (int a = 0; a < x.na; a++) {
    p.Ud[a] = (const __nv_bfloat16 *)x.far[a]->Ud;
    p.eu[a] = x.far[a]->eu;
    p.ii[a] = x.ii[a];
    p.jj[a] = x.jj[a];
  }
  p.Zd = Zd;
  p.ez = ez;
  p.Yb = Yb;
  p.members = x.members;
  p.pqlist = x.pqlist;
  p.info = x.info;
  p.hch = c->hch;
  p.err = err;
  const size_t smem = 2 * TS * (size_t)(A_BYTES + B_BYTES) + (size_t)MAXT * NDB * 128 * sizeof(double);
  DBSRG_TRY(c, cudaFuncSetAttribute(k_xfused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
  const long long nblk = std::min<long long>(p.nitems, (long long)std::max(1, c->nsm));
  DBSRG_RUN(c, "k_xfused", k_xfused<<<(unsigned)nblk, 256, smem, st>>>(p));
  int h = 0;
  DBSRG_TRY(c, cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  DBSRG_TRY(c, cudaStreamSynchronize(st));
  if (h == 1) return set_err(c, DBSRG_ETIMEOUT, "tensor-core exchange: a completion wait ran out");
  if (h) return set_err(c, DBSRG_ECUDA, "tensor-core exchange: inconsistent tile terms");
  return DBSRG_OK;
}
