// assemble.cu -- the plain-FP64 Gen_matrix path: density accumulation per
// channel-pair segment, contraction with the R^k/S^k tables and the ordered
// scatter into the channel-pair blocks, following
//   R_data itype 3/4  DBSR_MAT3/R_data.f90:56-86, 214-277
//   S_data itype 6-9  DBSR_MAT3/S_data.f90:67-113, 240-274
//   O_data itype 3    DBSR_MAT3/O_data.f90:50-61
//   UPDATE_HS/HW/HX   DBSR_MAT3/updates.f90:79-216
//
// Work decomposition (one Gen_matrix call):
//   1. the list is copied to the device in Add_matrix (IPT) order;
//   2. k_segments marks the runs of equal K1 (one channel pair each) --
//      the reference flushes a segment when the next K1 differs;
//   3. k_density_acc forms xx = sum_e c_e * density(e) for every segment
//      and atype, entries in list order;
//   4. the contraction: band products (convol cases 1/2) as a tiled FP64
//      product over all segments sharing one table, exchange (cases 3/4)
//      as a gather per output element batched over segments;
//   5. k_scatter adds the results into hch.  One thread owns one hch
//      element and applies the contributions in the reference's order
//      (atype-major, then list order), so no atomics are needed and the
//      result is deterministic.
#include <memory>

#include "internal.cuh"
#include "ff.cuh"

#include <algorithm>
#include <cmath>
#include <functional>

namespace {

constexpr int kSegChunk = 256;  // segments per pass of the plain contraction


// ---------------------------------------------------------------------------
// list gather into IPT order
__global__ void k_gather(int n, const int *ipt, const int *k1, const int *k2, const int *k3,
                         const double *c, int *o1, int *o2, int *o3, double *oc) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  int i = ipt ? ipt[e] - 1 : e;
  o1[e] = k1[i];
  o2[e] = k2[i];
  o3[e] = k3[i];
  oc[e] = c[i];
}

// segment starts: positions where K1 differs from the previous entry.
// Single thread block; counts per thread chunk, block scan, then writes.
__global__ void k_segments(int n, const int *k1, int *seg_start, int *nseg_out) {
  __shared__ int cnt[1024];
  int tid = threadIdx.x, nt = blockDim.x;
  int chunk = (n + nt - 1) / nt;
  int lo = tid * chunk, hi = min(n, lo + chunk);
  int c = 0;
  for (int p = lo; p < hi; p++)
    if (p == 0 || k1[p] != k1[p - 1]) c++;
  cnt[tid] = c;
  __syncthreads();
  // inclusive scan (Hillis-Steele)
  for (int off = 1; off < nt; off <<= 1) {
    int v = tid >= off ? cnt[tid - off] : 0;
    __syncthreads();
    cnt[tid] += v;
    __syncthreads();
  }
  int base = cnt[tid] - c;
  for (int p = lo; p < hi; p++)
    if (p == 0 || k1[p] != k1[p - 1]) seg_start[base++] = p;
  if (tid == nt - 1) {
    seg_start[cnt[tid]] = n;
    *nseg_out = cnt[tid];
  }
}

// the coefficients as float-float pairs (split form gather-sums)
__global__ void k_cd_ff(int n, const double *cd, float2 *cdf) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) cdf[e] = ffa::split(cd[e]);
}

// bound-orbital indices of every entry must address pq(:,:,1:nbf) (err 1),
// and every coefficient must be finite (err 3)
__global__ void k_check_orbitals(int n, const int *k2, const int *k3, const double *cd, int nbf,
                                 int *err) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  if (k2[e] < 1 || k2[e] > nbf || k3[e] < 1 || k3[e] > nbf) atomicExch(err, 1);
  if (!isfinite(cd[e])) atomicExch(err, 3);
}

// decode segments, look up blocks, pair up segments of the same block
__global__ void k_seg_info(int nseg, const int *seg_start, const int *k1, int nch, int iicc,
                           const int *icc, SegInfo *info, int *err) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  SegInfo si;
  si.start = seg_start[s];
  si.end = seg_start[s + 1];
  int key = k1[si.start];
  si.ich = key / DBSRG_IBO;
  si.jch = key % DBSRG_IBO;
  si.blk = 0;
  si.partner = -1;
  si.owner = 1;
  if (si.ich < 1 || si.jch < 1 || si.ich > nch || si.jch > nch) {
    atomicExch(err, 1);
  } else {
    int b = icc[(si.ich - 1) + (size_t)nch * (si.jch - 1)];
    if (b < 1 || b > iicc)
      atomicExch(err, 2);
    else
      si.blk = b;
    if (si.ich != si.jch) {
      // the swapped pair maps to the same block; binary search its K1
      int want = si.jch * DBSRG_IBO + si.ich;
      int lo = 0, hi = nseg - 1;
      while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        int v = k1[seg_start[mid]];
        if (v == want) {
          si.partner = mid;
          break;
        }
        if (v < want)
          lo = mid + 1;
        else
          hi = mid - 1;
      }
      if (si.partner >= 0 && si.partner < s) si.owner = 0;
    }
  }
  info[s] = si;
}

// ---------------------------------------------------------------------------
// density accumulation (density, dbsr_lib_dbs.f90:2834-2891; the
// xx = xx + cdata*dd loops of R_data.f90:217-220 / S_data.f90:244-246).
// xx layout: [atype][segment][ns*ncol], column-major per segment.
struct DensSpec {
  int jp1[4], jp2[4];  // components (1 P, 2 Q) of the two bound orbitals
};

__global__ void k_density_acc(int ns, int ks, char sym, int ncol, int na, DensSpec spec,
                              int nm, const int *members, const SegInfo *info, const int *k2,
                              const int *k3, const double *cd, const double *pq,
                              double *xx) {
  size_t per = (size_t)ns * ncol;
  size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= per) return;
  const int slot = blockIdx.y;
  int s = members[slot];
  int a = blockIdx.z;
  int i = (int)(q % ns) + 1, j = (int)(q / ns) + 1;  // 1-based (i,j) of d(i,j)
  const SegInfo si = info[s];
  const double *P1base = pq + (size_t)ns * (spec.jp1[a] - 1);
  const double *P2base = pq + (size_t)ns * (spec.jp2[a] - 1);
  double acc = 0.0;
  for (int e = si.start; e < si.end; e++) {
    const double *p1 = P1base + (size_t)2 * ns * (k2[e] - 1) - 1;  // 1-based view
    const double *p2 = P2base + (size_t)2 * ns * (k3[e] - 1) - 1;
    double d;
    if (sym == 's') {
      if (j == 1)
        d = p1[i] * p2[i];
      else if (i <= ns - j + 1)
        d = p1[i] * p2[i + j - 1] + p1[i + j - 1] * p2[i];
      else
        d = 0.0;
    } else if (sym == 'n') {
      int imin = max(1, 1 + ks - j), imax = min(ns, ns + ks - j);
      d = (i >= imin && i <= imax) ? p1[i] * p2[i + j - ks] : 0.0;
    } else {
      d = p1[i] * p2[j];
    }
    acc = acc + cd[e] * d;
  }
  xx[((size_t)a * nm + slot) * per + q] = acc;
}

// ---------------------------------------------------------------------------
// band contraction, convol cases 1 and 2 (dbsr_lib_dbs.f90:2243-2338 and
// :2517-2608): for every segment n of the chunk
//   case 1: a(i,ip) = sum_{j,jp} d(j,jp) rkb(i,j,ip,jp)
//   case 2: a(j,jp) = sum_{i,ip} d(i,ip) rkb(i,j,ip,jp)
// as one product over all segments that share the table: rows r=(i,ip),
// columns n, contraction over (j,jp).  Tiles: 64 rows x 64 segments x 16,
// 256 threads with 4x4 outputs each.
constexpr int GBM = 64, GBN = 64, GBK = 16;

__global__ void __launch_bounds__(256) k_band_contract(int ns, int kb, int icase,
                                                      const double *__restrict__ rkb,
                                                      int nsg, const double *__restrict__ X,
                                                      double *__restrict__ A) {
  __shared__ double Rs[GBK][GBM + 1];
  __shared__ double Xs[GBK][GBN + 1];
  const int nrt = (ns + GBM - 1) / GBM;  // row tiles per band column
  const int rt = blockIdx.x % nrt;
  const int obp = blockIdx.x / nrt;  // output band column (ip for case 1)
  const int n0 = blockIdx.y * GBN;
  const int r0 = rt * GBM;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const size_t per = (size_t)ns * kb;
  const size_t ns2 = (size_t)ns * ns;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = 0.0;
  for (int cbp = 0; cbp < kb; cbp++) {  // contracted band column
    for (int c0 = 0; c0 < ns; c0 += GBK) {
      // table tile: rows r0..r0+63 (output index), cols c0..c0+15
      for (int q = threadIdx.x; q < GBK * GBM; q += 256) {
        int rr = q % GBM, cc = q / GBM;
        int r = r0 + rr, cidx = c0 + cc;
        double v = 0.0;
        if (r < ns && cidx < ns) {
          size_t off;
          if (icase == 1)  // rkb(r, cidx, obp, cbp)
            off = (size_t)r + (size_t)ns * cidx + ns2 * ((size_t)obp + (size_t)kb * cbp);
          else  // rkb(cidx, r, cbp, obp)
            off = (size_t)cidx + (size_t)ns * r + ns2 * ((size_t)cbp + (size_t)kb * obp);
          v = rkb[off];
        }
        Rs[cc][rr] = v;
      }
      for (int q = threadIdx.x; q < GBK * GBN; q += 256) {
        int cc = q % GBK, nn = q / GBK;
        int cidx = c0 + cc, n = n0 + nn;
        double v = 0.0;
        if (cidx < ns && n < nsg) v = X[(size_t)n * per + cidx + (size_t)ns * cbp];
        Xs[cc][nn] = v;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < GBK; kk++) {
        double rv[4], xv[4];
#pragma unroll
        for (int a = 0; a < 4; a++) rv[a] = Rs[kk][ty * 4 + a];
#pragma unroll
        for (int b = 0; b < 4; b++) xv[b] = Xs[kk][tx * 4 + b];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
          for (int b = 0; b < 4; b++) acc[a][b] = fma(rv[a], xv[b], acc[a][b]);
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int a = 0; a < 4; a++) {
    int r = r0 + ty * 4 + a;
    if (r >= ns) continue;
#pragma unroll
    for (int b = 0; b < 4; b++) {
      int n = n0 + tx * 4 + b;
      if (n < nsg) A[(size_t)n * per + r + (size_t)ns * obp] = acc[a][b];
    }
  }
}

// ---------------------------------------------------------------------------
// exchange contraction, convol case 3 with 's','s' storage
// (dbsr_lib_dbs.f90:2344-2356) and cases 3/4 with 'n','n' storage
// (:2370-2378, :2418-2426; convol_sk :2632-2640, :2690-2698), written as a
// gather: one thread owns output a(x,y) of NB segments and sums the table
// entries that the reference scatters into it.
constexpr int XNB = 4;

__global__ void __launch_bounds__(256) k_exchange(int ns, int ks, int mode, int nsg,
                                                 const double *__restrict__ rkb,
                                                 const double *__restrict__ D,
                                                 double *__restrict__ A) {
  size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nn = (size_t)ns * ns;
  if (q >= nn) return;
  const int x = (int)(q % ns) + 1, y = (int)(q / ns) + 1;  // 1-based output (x,y)
  const int sb = blockIdx.y * XNB;
  const int nb = min(XNB, nsg - sb);
  const double *Db = D + (size_t)sb * nn;
  double acc[XNB];
#pragma unroll
  for (int b = 0; b < XNB; b++) acc[b] = 0.0;
  auto TB = [&](int i, int j, int ip, int jp, int kb) -> double {
    return __ldg(&rkb[(size_t)(i - 1) + (size_t)ns * ((size_t)(j - 1) +
                       (size_t)ns * ((size_t)(ip - 1) + (size_t)kb * (size_t)(jp - 1)))]);
  };
  auto DV = [&](int b, int i, int j) -> double {
    return __ldg(&Db[(size_t)b * nn + (size_t)(i - 1) + (size_t)ns * (size_t)(j - 1)]);
  };
  if (mode == 0) {  // R table, 's','s', case 3: four symmetric terms
    for (int jp = 1; jp <= ks; jp++) {
      for (int ip = 1; ip <= ks; ip++) {
        // T1: a(i,jj) += c*d(ii,j), i=x, jj=y -> j=y-jp+1, ii=x+ip-1
        if (y - jp + 1 >= 1 && x + ip - 1 <= ns) {
          double c = TB(x, y - jp + 1, ip, jp, ks);
#pragma unroll
          for (int b = 0; b < XNB; b++)
            if (b < nb) acc[b] = fma(c, DV(b, x + ip - 1, y - jp + 1), acc[b]);
        }
        // T2 (ip>1): a(ii,jj) += c*d(i,j): ii=x -> i=x-ip+1, jj=y -> j=y-jp+1
        if (ip > 1 && x - ip + 1 >= 1 && y - jp + 1 >= 1) {
          double c = TB(x - ip + 1, y - jp + 1, ip, jp, ks);
#pragma unroll
          for (int b = 0; b < XNB; b++)
            if (b < nb) acc[b] = fma(c, DV(b, x - ip + 1, y - jp + 1), acc[b]);
        }
        // T3 (jp>1): a(i,j) += c*d(ii,jj): i=x, j=y
        if (jp > 1 && x + ip - 1 <= ns && y + jp - 1 <= ns) {
          double c = TB(x, y, ip, jp, ks);
#pragma unroll
          for (int b = 0; b < XNB; b++)
            if (b < nb) acc[b] = fma(c, DV(b, x + ip - 1, y + jp - 1), acc[b]);
        }
        // T4 (ip>1,jp>1): a(ii,j) += c*d(i,jj): ii=x -> i=x-ip+1, j=y
        if (ip > 1 && jp > 1 && x - ip + 1 >= 1 && y + jp - 1 <= ns) {
          double c = TB(x - ip + 1, y, ip, jp, ks);
#pragma unroll
          for (int b = 0; b < XNB; b++)
            if (b < nb) acc[b] = fma(c, DV(b, x - ip + 1, y + jp - 1), acc[b]);
        }
      }
    }
  } else {  // S table 'n','n' (kb = 2ks-1)
    const int kb = 2 * ks - 1;
    for (int jp = 1; jp <= kb; jp++) {
      for (int ip = 1; ip <= kb; ip++) {
        if (mode == 1) {
          // case 3: a(i,jj) += c*d(ii,j), i=x, jj=y -> j=y-jp+ks, ii=x+ip-ks
          int j = y - jp + ks, ii = x + ip - ks;
          if (j < max(1, 1 + ks - jp) || j > min(ns, ns + ks - jp)) continue;
          if (x < max(1, 1 + ks - ip) || x > min(ns, ns + ks - ip)) continue;
          double c = TB(x, j, ip, jp, kb);
#pragma unroll
          for (int b = 0; b < XNB; b++)
            if (b < nb) acc[b] = fma(c, DV(b, ii, j), acc[b]);
        } else {
          // case 4: a(ii,j) += c*d(i,jj), ii=x -> i=x-ip+ks, j=y, jj=y+jp-ks
          int i = x - ip + ks, jj = y + jp - ks;
          if (y < max(1, 1 + ks - jp) || y > min(ns, ns + ks - jp)) continue;
          if (i < max(1, 1 + ks - ip) || i > min(ns, ns + ks - ip)) continue;
          double c = TB(i, y, ip, jp, kb);
#pragma unroll
          for (int b = 0; b < XNB; b++)
            if (b < nb) acc[b] = fma(c, DV(b, i, jj), acc[b]);
        }
      }
    }
  }
  for (int b = 0; b < nb; b++) A[(size_t)(sb + b) * nn + q] = acc[b];
}

// ---------------------------------------------------------------------------
// ordered scatter into hch (UPDATE_HS, updates.f90:110-179).
struct ScatterSpec {
  int na;           // number of contribution sets (atypes) in order
  int ii[4], jj[4]; // target quadrant of each set
  char sym;         // storage of the results: 's', 'n' or 'x'
  int ncol;         // columns of one result
};

__device__ __forceinline__ double yval(const double *d, int ns, int ks, char sym, int i, int j) {
  // element (i,j) (1-based) of the ns x ns matrix y built from d
  if (sym == 'x') return d[(size_t)(i - 1) + (size_t)ns * (j - 1)];
  if (sym == 's') {
    int lo = min(i, j), dlt = abs(i - j);
    if (dlt >= ks) return 0.0;
    return d[(size_t)(lo - 1) + (size_t)ns * dlt];
  }
  int jp = j - i + ks;  // 'n'
  if (jp < 1 || jp > 2 * ks - 1) return 0.0;
  return d[(size_t)(i - 1) + (size_t)ns * (jp - 1)];
}

// index space: mode 0 (full): the ms x ms block; mode 1 (band): the four
// quadrants x ns rows x (2ks-1) diagonals.
__global__ void k_scatter(int ns, int ks, int mode, ScatterSpec sp, int nm, const int *members,
                          const int *own_slots, const SegInfo *info, const double *Y,
                          double *hch) {
  const int ms = 2 * ns;
  const int oslot = own_slots[blockIdx.y];
  const int s = members[oslot];
  const SegInfo si = info[s];
  if (si.blk < 1) return;
  // the partner, if any, is stored in the next member slot
  const int pslot = (si.partner >= 0) ? oslot + 1 : -1;
  size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  int r, c;  // 0-based position in the ms x ms block
  if (mode == 0) {
    if (q >= (size_t)ms * ms) return;
    r = (int)(q % ms);
    c = (int)(q / ms);
  } else {
    const int nd = 2 * ks - 1;
    if (q >= (size_t)4 * ns * nd) return;
    int quad = (int)(q / ((size_t)ns * nd));
    int rem = (int)(q % ((size_t)ns * nd));
    int lr = rem % ns, off = rem / ns - (ks - 1);
    int lc = lr + off;
    if (lc < 0 || lc >= ns) return;
    r = (quad & 1) * ns + lr;
    c = (quad >> 1) * ns + lc;
  }
  const int qr = r / ns + 1, qc = c / ns + 1;
  const int lr = r % ns + 1, lc = c % ns + 1;
  const size_t per = (size_t)ns * sp.ncol;
  bool touched = false;
  double val = 0.0;
  double *h = hch + (size_t)(si.blk - 1) * ms * ms + (size_t)r + (size_t)ms * c;
  for (int a = 0; a < sp.na; a++) {
    for (int pass = 0; pass < 2; pass++) {
      int slot = pass == 0 ? oslot : pslot;
      if (slot < 0) break;
      const SegInfo sj = info[members[slot]];
      const double *d = Y + ((size_t)a * nm + slot) * per;
      const int ii = sp.ii[a], jj = sp.jj[a];
      if (sj.ich > sj.jch) {
        if (qr == ii && qc == jj) {
          if (!touched) { val = *h; touched = true; }
          val = val + yval(d, ns, ks, sp.sym, lr, lc);
        }
      } else if (sj.jch > sj.ich) {
        if (qr == ii && qc == jj) {
          if (!touched) { val = *h; touched = true; }
          val = val + yval(d, ns, ks, sp.sym, lc, lr);
        }
      } else {
        if (qr == ii && qc == jj) {
          if (!touched) { val = *h; touched = true; }
          val = val + yval(d, ns, ks, sp.sym, lr, lc) / 2.0;
        }
        if (qr == jj && qc == ii) {
          if (!touched) { val = *h; touched = true; }
          val = val + yval(d, ns, ks, sp.sym, lc, lr) / 2.0;
        }
      }
    }
  }
  if (touched) *h = val;
}

// asymptotic coefficients (UPDATE_ACF, R_data.f90:223-240): one warp per
// owner segment (owners have distinct blocks); per atype 0, 1 and per
// segment (the owner, then its partner) the lanes sum every 32nd entry and
// a butterfly combines the lanes, and the sum is added to acf in that order.
constexpr int ACF_WARPS = 4;  // warps per block
__global__ void k_acf(int nseg_owner, const int *owners, const SegInfo *info, int kpol,
                      int nbf, const int *k2, const int *k3, const double *cd,
                      const double *quad, double *acf, int iicc) {
  const int lane = threadIdx.x & 31;
  const int t = blockIdx.x * ACF_WARPS + threadIdx.x / 32;
  if (t >= nseg_owner) return;
  const int s = owners[t];
  const SegInfo si = info[s];
  if (si.blk < 1) return;
  double *dst = acf + (size_t)(si.blk - 1) + (size_t)iicc * kpol;
  for (int a = 0; a < 2; a++) {
    for (int pass = 0; pass < 2; pass++) {
      const int ss = pass == 0 ? s : si.partner;
      if (pass == 1 && ss < 0) break;
      const SegInfo sj = info[ss];
      double CA = 0.0;
      for (int e = sj.start + lane; e < sj.end; e += 32) {
        const double S =
            quad[(size_t)(k2[e] - 1) + (size_t)nbf * ((k3[e] - 1) + (size_t)nbf * a)];
        CA = CA + cd[e] * S;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) CA += __shfl_xor_sync(0xffffffffu, CA, o);
      if (lane == 0) *dst = *dst + CA;
    }
  }
}


// ---------------------------------------------------------------------------
// O_data itype 3 (<i|.><.|j>, O_data.f90:50-61) with UPDATE_HW
// (updates.f90:183-216).  V_ch is restated as the B-spline overlap vector
// of the bound orbital: v(1:ns) = fpbs*P, v(ns+1:ms) = fqbs*Q.
__global__ void k_vch(int ns, int nbf, const double *fpbs, const double *fqbs,
                      const double *pq, double *vch) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= 2 * ns * nbf) return;
  int i = q % (2 * ns), b = q / (2 * ns);
  int comp = i / ns, ii = i % ns;
  const double *F = comp == 0 ? fpbs : fqbs;
  const double *p = pq + (size_t)2 * ns * b + (size_t)ns * comp;
  double s = 0.0;
  for (int j = 0; j < ns; j++) s += F[(size_t)ii + (size_t)ns * j] * p[j];
  vch[q] = s;
}

// One thread per row r of a touched block and 32 consecutive columns: the
// entries of the block in list order, each a rank-1 term with the row factor
// formed once (one FMA per element and entry):
//   ich > jch: C v(r) w(c);  ich < jch: C w(r) v(c);
//   ich = jch: C/2 (v(r) w(c) + v(c) w(r))
__global__ void k_overlap_update(int ns, const int *tlist, const int *bstart, const int *order,
                                 const int *k1, const int *k2, const double *cd,
                                 const int *ipbs, const double *vch, double *hch) {
  constexpr int NC = 32;
  const int ms = 2 * ns;
  const int b = tlist[blockIdx.z];
  const int e0 = bstart[b], e1 = bstart[b + 1];
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c0 = blockIdx.y * NC;
  if (e0 == e1 || r >= ms) return;
  const int ncol = min(NC, ms - c0);
  double *h = hch + (size_t)(b - 1) * ms * ms + r + (size_t)ms * c0;
  double val[NC];
#pragma unroll
  for (int j = 0; j < NC; j++) val[j] = j < ncol ? h[(size_t)ms * j] : 0.0;
  for (int t = e0; t < e1; t++) {
    const int e = order[t];
    const int i1 = k1[e] / DBSRG_IBO, i2 = k1[e] % DBSRG_IBO;
    const int j1 = k2[e] / DBSRG_IBO, j2 = k2[e] % DBSRG_IBO;
    const int ich = ipbs[i1 - 1], jch = ipbs[j1 - 1];
    const double *v = vch + (size_t)ms * (i2 - 1);
    const double *w = vch + (size_t)ms * (j2 - 1);
    const double C = cd[e];
    if (ich != jch) {
      const double *u = ich > jch ? w : v;  // column vector
      const double a = C * (ich > jch ? v[r] : w[r]);
#pragma unroll
      for (int j = 0; j < NC; j++)
        if (j < ncol) val[j] = fma(a, u[c0 + j], val[j]);
    } else {
      const double a1 = 0.5 * C * v[r], a2 = 0.5 * C * w[r];
#pragma unroll
      for (int j = 0; j < NC; j++)
        if (j < ncol) val[j] = fma(a1, w[c0 + j], fma(a2, v[c0 + j], val[j]));
    }
  }
#pragma unroll
  for (int j = 0; j < NC; j++)
    if (j < ncol) h[(size_t)ms * j] = val[j];
}

// UPDATE_HX (updates.f90:79-106)
__global__ void k_update_hx(int ms, int ich, int jch, const double *d, double cc, double *blk) {
  size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (size_t)ms * ms) return;
  int r = (int)(q % ms), c = (int)(q / ms);
  double x = ich >= jch ? cc * d[q] : cc * d[(size_t)c + (size_t)ms * r];
  blk[q] = blk[q] + x;
}

}  // namespace

// ---------------------------------------------------------------------------
int update_hx(dbsrg_ctx *c, int ich, int jch, const double *d, double cc) {
  const int ms = c->g.ms;
  if (!c->hch) return set_err(c, DBSRG_ESTATE, "no matrix allocated");
  if (ich < 1 || jch < 1 || ich > c->nch || jch > c->nch)
    return set_err(c, DBSRG_ERANGE, "UPDATE_HX: channel out of range");
  int b = c->h_icc[(ich - 1) + (size_t)c->nch * (jch - 1)];
  if (b < 1 || b > c->iicc) return set_err(c, DBSRG_ERANGE, "UPDATE_HX: i out of range");
  if (!in_window(c, b)) return DBSRG_OK;  // the block is assembled in another window
  const double *dd = d;
  size_t bytes = sizeof(double) * (size_t)ms * ms;
  if (!is_device_ptr(d)) {
    int rc = ensure_scratch2(c, bytes);
    if (rc) return rc;
    rc = copy_in(c, c->scratch2, d, bytes);
    if (rc) return rc;
    dd = (const double *)c->scratch2;
  }
  size_t n = (size_t)ms * ms;
  DBSRG_RUN(c, "k_update_hx", k_update_hx<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(
      ms, ich, jch, dd, cc, hch_base(c) + (size_t)(b - 1) * ms * ms));
  DBSRG_TRY(c, cudaStreamSynchronize(c->stream));
  return DBSRG_OK;
}

namespace {

// One coefficient list, set up once and executed per block window.
//  * set-up (plan_list): the list copied in IPT order, its segments and
//    their blocks read back, the case's structure (PQ types, storage,
//    convol case), and the work of every window of a partition of the
//    blocks (windows [blo0 + w*nwin, blo0 + (w+1)*nwin), w < nw): chunks of
//    owner segments with their partners, quadrant records of the split
//    exchange, owners for acf, touched blocks of an overlap list.  All work
//    lists go to the device in one copy.
//  * execution (exec_list): the window's chunks, acf terms or overlap
//    updates on the contraction stream, with the tables (cached) fetched
//    there.
struct Chunk {
  int moff, nm, nown, xoff, nxq;
  long long nent;  // entries of the member segments (executed-work statements)
};
struct ListPlan {
  int icase = 0, itype = 0, kpol = 0, n = 0, nseg = 0;
  bool factored = false, split_x = false;
  int na = 0, icv = 0, tabfam = 0, ncol = 0, kb = 0;
  char sym_d = 's';
  size_t per = 0;
  DensSpec dsp{};
  ScatterSpec ssp{};
  int ttype[4] = {0, 1, 2, 3};
  int *lk1 = nullptr, *lk2 = nullptr, *lk3 = nullptr, *lpair = nullptr;
  double *lcd = nullptr;
  float2 *lcdf = nullptr;  // the coefficients as float-float pairs
  SegInfo *info = nullptr;
  int *work = nullptr;   // chunk members and owner slots | acf owners
  XQuad *dxq = nullptr;  // quadrant records
  double *vch = nullptr;
  int *bstart = nullptr, *tlist = nullptr, *order = nullptr;  // overlap list
  std::vector<Chunk> chunks;
  std::vector<int> wchunk, wown, wtl;  // per window: [w], [w+1] ranges
  std::vector<double> wovl;            // overlap list: executed FLOPs per window
  int own_off = 0;                     // acf owners inside `work`
  std::vector<XQuad> hxq;
  // the structures that are not channel-pair contractions (structures.cu)
  std::shared_ptr<StructPlan> sp;
};

size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

// device bytes of one list's state
size_t plan_bytes(const dbsrg_ctx *c, int icase, int itype, int n) {
  if (is_structure_list(icase, itype)) return structure_plan_bytes(c, icase, itype, n);
  const size_t ib = sizeof(int) * (size_t)n, db = sizeof(double) * (size_t)n;
  size_t t = 8 * al256(ib) + 2 * al256(db) + al256(sizeof(int) * (n + 2)) + al256(64) +
             al256(sizeof(SegInfo) * (size_t)(n + 1)) + al256(sizeof(int) * (size_t)(7 * (n + 1))) +
             al256(sizeof(XQuad) * 4 * (size_t)(n + 1)) + al256(sizeof(float2) * (size_t)n);
  if (icase == 0)
    t += al256(sizeof(double) * (size_t)c->g.ms * c->nbf) +
         al256(sizeof(int) * (2 * (size_t)(c->iicc + 2) + n));
  return t;
}

int plan_list(dbsrg_ctx *c, int icase, int itype, int kpol, int n, const int *ipt,
              const int *k1, const int *k2, const int *k3, const int *k4, const double *cdata,
              int blo0, int nwin, int nw, void *dev, cudaStream_t ss, ListPlan &P,
              const int *wstart = nullptr) {
  const DeviceGrid &g = c->g;
  const int ns = g.ns, ks = g.ks, ms = g.ms;
  int rc;
  P.icase = icase;
  P.itype = itype;
  P.kpol = kpol;
  P.n = n;
  if (is_structure_list(icase, itype)) {
    StructPlan *sp = nullptr;
    rc = plan_structures(c, icase, itype, kpol, n, ipt, k1, k2, k3, k4, cdata, blo0, nwin, nw,
                         dev, ss, &sp, wstart);
    if (rc) return rc;
    P.sp.reset(sp, free_structure_plan);
    return DBSRG_OK;
  }
  // window of block b in the partition, -1 outside it
  auto wof = [&](int b) -> int {
    if (wstart) {
      if (b < wstart[0] || b >= wstart[nw]) return -1;
      return (int)(std::upper_bound(wstart, wstart + nw + 1, b) - wstart) - 1;
    }
    if (b < blo0) return -1;
    const int w = (b - blo0) / nwin;
    return w < nw ? w : -1;
  };
  const size_t ibytes = sizeof(int) * (size_t)n, dbytes = sizeof(double) * (size_t)n;
  char *base = (char *)dev;
  auto take = [&](size_t bytes) {
    char *p = base;
    base += al256(bytes);
    return (void *)p;
  };
  int *dk1 = (int *)take(ibytes), *dk2 = (int *)take(ibytes), *dk3 = (int *)take(ibytes);
  double *dcd = (double *)take(dbytes);
  int *dipt = (int *)take(ibytes);
  P.lk1 = (int *)take(ibytes);
  P.lk2 = (int *)take(ibytes);
  P.lk3 = (int *)take(ibytes);
  P.lcd = (double *)take(dbytes);
  P.lpair = (int *)take(ibytes);  // factored path: bound-orbital pair of each entry
  int *seg_start = (int *)take(sizeof(int) * (size_t)(n + 2));
  int *dscal = (int *)take(64);  // [0]=nseg [1]=err [2]=- [3]=pair err
  P.info = (SegInfo *)take(sizeof(SegInfo) * (size_t)(n + 1));
  // per chunk member segment ids and owner slots (at most 6 ints per
  // segment), then the acf owners (one per segment)
  P.work = (int *)take(sizeof(int) * (size_t)(7 * (n + 1)));
  P.dxq = (XQuad *)take(sizeof(XQuad) * 4 * (size_t)(n + 1));
  P.lcdf = (float2 *)take(sizeof(float2) * (size_t)n);
  if ((rc = copy_in_s(c, dk1, k1, ibytes, ss))) return rc;
  if ((rc = copy_in_s(c, dk2, k2, ibytes, ss))) return rc;
  if ((rc = copy_in_s(c, dk3, k3, ibytes, ss))) return rc;
  if ((rc = copy_in_s(c, dcd, cdata, dbytes, ss))) return rc;
  if (ipt && (rc = copy_in_s(c, dipt, ipt, ibytes, ss))) return rc;
  DBSRG_TRY(c, cudaMemsetAsync(dscal, 0, 64, ss));
  DBSRG_RUN_S(c, ss, "k_gather",
              k_gather<<<(n + 255) / 256, 256, 0, ss>>>(n, ipt ? dipt : nullptr, dk1, dk2, dk3,
                                                        dcd, P.lk1, P.lk2, P.lk3, P.lcd));
  DBSRG_RUN_S(c, ss, "k_cd_ff",
              k_cd_ff<<<(n + 255) / 256, 256, 0, ss>>>(n, P.lcd, P.lcdf));

  // ---- overlaps: entries grouped by block on the host (counting sort, list
  // order kept within a block); entries below eps_c are dropped
  // (mod_dbsr_mat.f90:56)
  if (icase == 0) {
    if (itype != 3) return set_err(c, DBSRG_EINVAL, "O_data: unknown structure (itype)");
    const int iicc = c->iicc;
    P.vch = (double *)take(sizeof(double) * (size_t)ms * c->nbf);
    P.bstart = (int *)take(sizeof(int) * (2 * (size_t)(iicc + 2) + n));
    P.tlist = P.bstart + (iicc + 2);  // blocks with entries, ascending
    P.order = P.tlist + (iicc + 2);
    std::vector<int> hk1(n), hk2(n);
    std::vector<double> hcd(n);
    DBSRG_TRY(c, cudaMemcpyAsync(hk1.data(), P.lk1, ibytes, cudaMemcpyDeviceToHost, ss));
    DBSRG_TRY(c, cudaMemcpyAsync(hk2.data(), P.lk2, ibytes, cudaMemcpyDeviceToHost, ss));
    DBSRG_TRY(c, cudaMemcpyAsync(hcd.data(), P.lcd, dbytes, cudaMemcpyDeviceToHost, ss));
    DBSRG_TRY(c, cudaStreamSynchronize(ss));
    std::vector<int> eblk(n, 0), hstart(iicc + 2, 0), hlist, horder(n);
    for (int e = 0; e < n; e++) {
      if (!std::isfinite(hcd[e])) return set_err(c, DBSRG_EINVAL, "non-finite coefficient in list");
      if (std::fabs(hcd[e]) < c->eps_c) continue;
      const int i1 = hk1[e] / DBSRG_IBO, j1 = hk2[e] / DBSRG_IBO;
      if (i1 < 1 || i1 > c->nbf || j1 < 1 || j1 > c->nbf || hk1[e] % DBSRG_IBO < 1 ||
          hk1[e] % DBSRG_IBO > c->nbf || hk2[e] % DBSRG_IBO < 1 || hk2[e] % DBSRG_IBO > c->nbf)
        return set_err(c, DBSRG_ERANGE, "channel or orbital index out of range in list");
      const int ich = c->h_ipbs[i1 - 1], jch = c->h_ipbs[j1 - 1];
      if (ich < 1 || jch < 1 || ich > c->nch || jch > c->nch)
        return set_err(c, DBSRG_ERANGE, "channel or orbital index out of range in list");
      const int b = c->h_icc[(ich - 1) + (size_t)c->nch * (jch - 1)];
      if (b < 1 || b > iicc) return set_err(c, DBSRG_ERANGE, "channel pair has no block in icc");
      if (wof(b) < 0) continue;
      eblk[e] = b;
      hstart[b + 1]++;
    }
    P.wtl.assign(nw + 1, 0);
    P.wovl.assign(nw, 0.0);
    for (int b = 1; b <= iicc; b++) {
      if (hstart[b + 1] > 0) {
        hlist.push_back(b);
        P.wtl[wof(b) + 1]++;
        // one multiply-add per element and entry (two on diagonal blocks)
        P.wovl[wof(b)] += 2.0 * (double)ms * ms * hstart[b + 1];
      }
      hstart[b + 1] += hstart[b];
    }
    for (int w = 0; w < nw; w++) P.wtl[w + 1] += P.wtl[w];
    {
      std::vector<int> fill(hstart.begin(), hstart.end());
      for (int e = 0; e < n; e++)
        if (eblk[e]) horder[fill[eblk[e]]++] = e;
    }
    if (!hlist.empty()) {
      if ((rc = copy_in_s(c, P.bstart, hstart.data(), sizeof(int) * (iicc + 2), ss))) return rc;
      if ((rc = copy_in_s(c, P.tlist, hlist.data(), sizeof(int) * hlist.size(), ss))) return rc;
      if ((rc = copy_in_s(c, P.order, horder.data(), sizeof(int) * hstart[iicc + 1], ss)))
        return rc;
    }
    return DBSRG_OK;
  }

  // ---- segments (orbital check and segment count read back together)
  DBSRG_RUN_S(c, ss, "k_check_orbitals",
              k_check_orbitals<<<(n + 255) / 256, 256, 0, ss>>>(n, P.lk2, P.lk3, P.lcd, c->nbf,
                                                                dscal + 1));
  DBSRG_RUN_S(c, ss, "k_segments", k_segments<<<1, 1024, 0, ss>>>(n, P.lk1, seg_start, dscal));
  int hs[4] = {0, 0, 0, 0};  // nseg, error, -, bound-pair error
  DBSRG_TRY(c, cudaMemcpyAsync(hs, dscal, 2 * sizeof(int), cudaMemcpyDeviceToHost, ss));
  DBSRG_TRY(c, cudaStreamSynchronize(ss));
  if (hs[1] == 3) return set_err(c, DBSRG_EINVAL, "non-finite coefficient in list");
  if (hs[1]) return set_err(c, DBSRG_ERANGE, "channel or orbital index out of range in list");
  const int nseg = hs[0];
  if (nseg < 1 || nseg > n) return set_err(c, DBSRG_ECUDA, "inconsistent segment count");
  P.nseg = nseg;
  DBSRG_RUN_S(c, ss, "k_seg_info",
              k_seg_info<<<(nseg + 127) / 128, 128, 0, ss>>>(nseg, seg_start, P.lk1, c->nch,
                                                             c->iicc, c->icc, P.info, dscal + 1));

  // ---- the case: PQ types, storage and convol case
  P.factored = c->precision != DBSRG_PLAIN_FP64;
  if (icase == 2) {
    if (itype != 3 && itype != 4) return set_err(c, DBSRG_EINVAL, "R_data: unknown itype");
    if (kpol < 0 || kpol > c->mk) return set_err(c, DBSRG_ERANGE, "R_data: kpol out of range");
    P.na = 4;
    P.tabfam = 0;
    P.icv = itype == 3 ? 1 : 3;
    P.sym_d = itype == 3 ? 's' : 'x';
    for (int a = 0; a < 4; a++) {
      int ip1, ip2, jp1, jp2;
      switch (a) {  // R_data.f90:73-86
        case 0: ip1 = 1; ip2 = 1; jp1 = 1; jp2 = 1; break;
        case 1: ip1 = 2; ip2 = 2; jp1 = 2; jp2 = 2; break;
        case 2: ip1 = 1; ip2 = 1; jp1 = 2; jp2 = 2;
          if (itype == 4) { ip1 = 1; ip2 = 2; jp1 = 1; jp2 = 2; }
          break;
        default: ip1 = 2; ip2 = 2; jp1 = 1; jp2 = 1;
          if (itype == 4) { ip1 = 2; ip2 = 1; jp1 = 2; jp2 = 1; }
          break;
      }
      P.dsp.jp1[a] = jp1; P.dsp.jp2[a] = jp2;
      P.ssp.ii[a] = ip1; P.ssp.jj[a] = ip2;
    }
  } else if (icase == 3) {
    int atype = itype / 10, it = itype % 10;
    if (atype < 0 || atype > 1 || it < 6 || it > 9)
      return set_err(c, DBSRG_EINVAL, "S_data: unknown itype");
    if (kpol < 0 || kpol > c->mk + 1) return set_err(c, DBSRG_ERANGE, "S_data: kpol out of range");
    int ip1, ip2, jp1, jp2, in;  // S_data.f90:74-97
    if (atype == 0) {
      switch (it) {
        case 6: ip1 = 1; ip2 = 2; jp1 = 1; jp2 = 2; in = 1; break;
        case 7: ip1 = 1; ip2 = 2; jp1 = 1; jp2 = 2; in = 2; break;
        case 8: ip1 = 1; ip2 = 2; jp1 = 2; jp2 = 1; in = 3; break;
        default: ip1 = 2; ip2 = 1; jp1 = 1; jp2 = 2; in = 4; break;
      }
    } else {
      switch (it) {
        case 6: ip1 = 1; ip2 = 2; jp1 = 2; jp2 = 1; in = 1; break;
        case 7: ip1 = 2; ip2 = 1; jp1 = 1; jp2 = 2; in = 2; break;
        case 8: ip1 = 1; ip2 = 1; jp1 = 2; jp2 = 2; in = 3; break;
        default: ip1 = 2; ip2 = 2; jp1 = 1; jp2 = 1; in = 4; break;
      }
    }
    P.na = 1;
    P.tabfam = 1;
    P.icv = in;
    P.sym_d = in <= 2 ? 'n' : 'x';
    P.dsp.jp1[0] = jp1; P.dsp.jp2[0] = jp2;
    P.ssp.ii[0] = ip1; P.ssp.jj[0] = ip2;
    P.ttype[0] = atype;
  } else {
    return set_err(c, DBSRG_EINVAL, "unsupported icase");
  }
  P.ssp.na = P.na;
  P.ssp.sym = P.sym_d;
  P.ncol = P.sym_d == 's' ? ks : (P.sym_d == 'n' ? 2 * ks - 1 : ns);
  P.ssp.ncol = P.ncol;
  P.kb = P.tabfam == 0 ? ks : 2 * ks - 1;
  P.per = (size_t)ns * P.ncol;
  P.split_x = P.factored && P.icv >= 3 && c->precision == DBSRG_SPLIT_BF16;

  if (P.factored) {
    // the factored contraction works with ordered pairs of bound orbitals
    if (c->nbound < 1) return set_err(c, DBSRG_ESTATE, "no bound orbitals (ipbs = 0)");
    if ((rc = pair_index(c, n, P.lk2, P.lk3, P.lpair, dscal + 3, ss))) return rc;
  }
  // segment table, segment errors and bound-pair errors in one read-back
  std::vector<SegInfo> hinfo(nseg);
  DBSRG_TRY(c, cudaMemcpyAsync(hs, dscal, 4 * sizeof(int), cudaMemcpyDeviceToHost, ss));
  DBSRG_TRY(c, cudaMemcpyAsync(hinfo.data(), P.info, sizeof(SegInfo) * nseg,
                               cudaMemcpyDeviceToHost, ss));
  DBSRG_TRY(c, cudaStreamSynchronize(ss));
  if (hs[1] == 1) return set_err(c, DBSRG_ERANGE, "channel or orbital index out of range in list");
  if (hs[1] == 2) return set_err(c, DBSRG_ERANGE, "channel pair has no block in icc");
  if (hs[3]) return set_err(c, DBSRG_EINVAL, "factored contraction: K2/K3 must be bound orbitals");
  for (int s = 0; s < nseg; s++) {
    const SegInfo &si = hinfo[s];
    if (si.start < 0 || si.end > n || si.start >= si.end || si.blk < 1 || si.blk > c->iicc ||
        si.partner < -1 || si.partner >= nseg)
      return set_err(c, DBSRG_ECUDA, "inconsistent segment table");
  }

  // ---- chunks of owner segments per window, each owner with its partner (a
  // channel pair listed in both orders maps to one block; both lists
  // contribute to that block in list order within every atype, so they stay
  // in one chunk); owners in list order within a window
  std::vector<std::vector<int>> wseg(nw);
  for (int s = 0; s < nseg; s++) {
    if (!hinfo[s].owner) continue;
    const int w = wof(hinfo[s].blk);
    if (w >= 0) wseg[w].push_back(s);
  }
  const int chunk = !P.factored ? kSegChunk : (P.icv <= 2 ? c->tune_dchunk : c->tune_xchunk);
  std::vector<int> hbuf;
  bool xq_ok = true;
  P.wchunk.assign(nw + 1, 0);
  for (int w = 0; w < nw; w++) {
    std::vector<int> mem, own;  // member segment ids; owner slot positions
    auto close = [&]() {
      if (mem.empty()) return;
      Chunk ch{(int)hbuf.size(), (int)mem.size(), (int)own.size(), (int)P.hxq.size(), 0, 0};
      for (int m : mem) ch.nent += hinfo[m].end - hinfo[m].start;
      hbuf.insert(hbuf.end(), mem.begin(), mem.end());
      hbuf.insert(hbuf.end(), own.begin(), own.end());
      if (P.split_x) {
        xq_ok = xq_ok && build_xquads(P.na, P.ssp.ii, P.ssp.jj, mem, own, hinfo, P.hxq);
        ch.nxq = (int)P.hxq.size() - ch.xoff;
      }
      P.chunks.push_back(ch);
      mem.clear();
      own.clear();
    };
    for (int s : wseg[w]) {
      own.push_back((int)mem.size());
      mem.push_back(s);
      if (hinfo[s].partner >= 0) mem.push_back(hinfo[s].partner);
      if ((int)mem.size() >= chunk - 1) close();
    }
    close();
    P.wchunk[w + 1] = (int)P.chunks.size();
  }
  if (!xq_ok) return set_err(c, DBSRG_ECUDA, "split exchange: a quadrant with more than 4 terms");
  if (P.hxq.size() > 4 * (size_t)(n + 1) || hbuf.size() > 6 * (size_t)(n + 1))
    return set_err(c, DBSRG_ECUDA, "work records overflow");
  // owners of direct R^k (acf), in list order within a window
  P.wown.assign(nw + 1, 0);
  P.own_off = (int)hbuf.size();
  if (icase == 2 && itype == 3)
    for (int w = 0; w < nw; w++) {
      hbuf.insert(hbuf.end(), wseg[w].begin(), wseg[w].end());
      P.wown[w + 1] = P.wown[w] + (int)wseg[w].size();
    }
  if (!hbuf.empty() && (rc = copy_in_s(c, P.work, hbuf.data(), sizeof(int) * hbuf.size(), ss)))
    return rc;
  if (!P.hxq.empty() &&
      (rc = copy_in_s(c, P.dxq, P.hxq.data(), sizeof(XQuad) * P.hxq.size(), ss)))
    return rc;
  return DBSRG_OK;
}

// window w of a planned list on the contraction stream; hch_base(c) must
// address that window's blocks.  prep: build (or find) the tables, pair
// potentials and digit caches that any window of the list reads, and launch
// nothing else (every chunk of a list reads the same ones)
int exec_list(dbsrg_ctx *c, const ListPlan &P, int w, bool prep = false) {
  const DeviceGrid &g = c->g;
  const int ns = g.ns, ks = g.ks, ms = g.ms;
  cudaStream_t st = c->stream;
  int rc;
  if (P.sp) return exec_structures(c, *P.sp, w, prep);
  if (P.icase == 0) {
    if (prep) return DBSRG_OK;
    const int t0 = P.wtl[w], nt = P.wtl[w + 1] - t0;
    if (nt <= 0) return DBSRG_OK;
    // the overlap vectors depend on the orbitals only: built by the first
    // window with blocks of this list, kept by the plan for the later ones
    if (t0 == P.wtl[0])
      DBSRG_RUN(c, "k_vch", k_vch<<<(2 * ns * c->nbf + 255) / 256, 256, 0, st>>>(
                                ns, c->nbf, g.fpbs, g.fqbs, c->pq, P.vch));
    for (int t = 0; t < nt; t += 65535) {  // grid z limit
      const int nz = std::min(65535, nt - t);
      dim3 grid((unsigned)((ms + 127) / 128), (unsigned)((ms + 31) / 32), (unsigned)nz);
      // executed work: the window's multiply-adds, one read-modify-write of
      // every touched block (16 bytes an element)
      const double ob = 16.0 * (double)ms * ms * nz;
      const double of = t == 0 ? P.wovl[w] : 0.0;
      DBSRG_RUN_W(c, "k_overlap_update", ob, of,
                  k_overlap_update<<<grid, 128, 0, st>>>(ns, P.tlist + t0 + t, P.bstart, P.order,
                                                         P.lk1, P.lk2, P.lcd, c->ipbs, P.vch,
                                                         hch_base(c)));
    }
    return DBSRG_OK;
  }
  const int nwp = (int)P.wchunk.size() - 1;
  const int c0 = prep ? 0 : P.wchunk[w], c1 = prep ? P.wchunk[nwp] : P.wchunk[w + 1];
  const int o0 = prep ? 0 : P.wown[w], nown_acf = (prep ? P.wown[nwp] : P.wown[w + 1]) - o0;
  if (c0 == c1 && nown_acf == 0) return DBSRG_OK;
  // tables of the case (cached after the first use)
  const double *tabs[4] = {nullptr, nullptr, nullptr, nullptr};
  for (int a = 0; a < P.na; a++) {
    rc = DBSRG_OK;
    if (P.icase == 2) {
      // the factored path reads only the band |j-i| <= 16 of exchange
      // tables and no table at all for the direct contraction
      if (!P.factored)
        rc = get_rtable(c, a, P.kpol, &tabs[a]);
      else if (P.itype == 4)
        rc = get_band_table(c, 0, a, P.kpol, &tabs[a]);
    } else {
      if (!P.factored)
        rc = get_stable(c, P.ttype[0], P.kpol, &tabs[0]);
      else if (P.icv >= 3)
        rc = get_band_table(c, 1, P.ttype[0], P.kpol, &tabs[0]);
    }
    if (rc) return rc;
  }
  const int na = P.na, icv = P.icv;
  const size_t per = P.per;
  auto run_chunk = [&](const Chunk &ch) -> int {
    const int *mb = P.work + ch.moff, *ob = P.work + ch.moff + ch.nm;
    const int nm = ch.nm, nown = ch.nown;
    int rc2;
    if (P.factored) {
      double *Y = nullptr;
      if (icv >= 3 && !P.split_x && !prep) {
        if ((rc2 = ensure_scratch(c, sizeof(double) * per * na * nm))) return rc2;
        Y = (double *)c->scratch;
      }
      FactorJob job{};
      job.family = P.tabfam;
      job.kpol = P.kpol;
      job.icv = icv;
      job.sym = P.sym_d;
      job.na = na;
      for (int a = 0; a < na; a++) {
        job.types[a] = P.ttype[a];
        job.jp1[a] = P.dsp.jp1[a];
        job.jp2[a] = P.dsp.jp2[a];
        job.ii[a] = P.ssp.ii[a];
        job.jj[a] = P.ssp.jj[a];
        job.tabs[a] = tabs[a];
      }
      job.nm = nm;
      job.members = mb;
      job.nown = nown;
      job.own = ob;
      job.info = P.info;
      job.k2 = P.lk2;
      job.k3 = P.lk3;
      job.pairs = P.lpair;
      job.cd = P.lcd;
      job.cdf = P.lcdf;
      job.Y = Y;
      job.split = c->precision == DBSRG_SPLIT_BF16;
      job.xq = ch.nxq ? P.dxq + ch.xoff : nullptr;
      job.hxq = ch.nxq ? P.hxq.data() + ch.xoff : nullptr;
      job.nxq = ch.nxq;
      job.nent = ch.nent;
      job.prep = prep;
      return factored_contract(c, job);
    }
    if (prep) return DBSRG_OK;
    if ((rc2 = ensure_scratch(c, 2 * sizeof(double) * per * na * nm))) return rc2;
    double *X = (double *)c->scratch;
    double *Y = X + per * na * nm;
    {
      dim3 gd((unsigned)((per + 255) / 256), (unsigned)nm, (unsigned)na);
      DBSRG_RUN(c, "k_density_acc",
                k_density_acc<<<gd, 256, 0, st>>>(ns, ks, P.sym_d, P.ncol, na, P.dsp, nm, mb,
                                                  P.info, P.lk2, P.lk3, P.lcd, c->pq, X));
    }
    for (int a = 0; a < na; a++) {
      const double *Xa = X + (size_t)a * nm * per;
      double *Ya = Y + (size_t)a * nm * per;
      if (icv <= 2) {
        int nrt = (ns + GBM - 1) / GBM;
        dim3 gg((unsigned)(nrt * P.kb), (unsigned)((nm + GBN - 1) / GBN));
        DBSRG_RUN(c, "k_band_contract",
                  k_band_contract<<<gg, 256, 0, st>>>(ns, P.kb, icv, tabs[a], nm, Xa, Ya));
      } else {
        int mode = P.tabfam == 0 ? 0 : (icv == 3 ? 1 : 2);
        dim3 gx((unsigned)(((size_t)ns * ns + 255) / 256), (unsigned)((nm + XNB - 1) / XNB));
        DBSRG_RUN(c, "k_exchange",
                  k_exchange<<<gx, 256, 0, st>>>(ns, ks, mode, nm, tabs[a], Xa, Ya));
      }
    }
    int mode = P.sym_d == 'x' ? 0 : 1;
    size_t space = mode == 0 ? (size_t)ms * ms : (size_t)4 * ns * (2 * ks - 1);
    dim3 gs((unsigned)((space + 255) / 256), (unsigned)nown);
    DBSRG_RUN(c, "k_scatter",
              k_scatter<<<gs, 256, 0, st>>>(ns, ks, mode, P.ssp, nm, mb, ob, P.info, Y,
                                            hch_base(c)));
    return DBSRG_OK;
  };
  for (int k = c0; k < (prep ? std::min(c1, c0 + 1) : c1); k++)
    if ((rc = run_chunk(P.chunks[k]))) return rc;
  if (nown_acf > 0) {
    const double *quad;
    if ((rc = get_quad(c, P.kpol, &quad))) return rc;
    if (prep) return DBSRG_OK;
    DBSRG_RUN(c, "k_acf",
              k_acf<<<(nown_acf + ACF_WARPS - 1) / ACF_WARPS, 32 * ACF_WARPS, 0, st>>>(
                  nown_acf, P.work + P.own_off + o0, P.info, P.kpol, c->nbf, P.lk2, P.lk3, P.lcd,
                  quad, c->acf, c->iicc));
  }
  return DBSRG_OK;
}

}  // namespace

// convol cases 1/2 of nsg band densities X with one full table (k_band_contract)
int band_contract(dbsrg_ctx *c, int kb, int icase, const double *rkb, int nsg, const double *X,
                  double *Y) {
  const int ns = c->g.ns;
  const int nrt = (ns + GBM - 1) / GBM;
  for (int s0 = 0; s0 < nsg; s0 += 65535 * GBN) {
    const int nn = std::min(nsg - s0, 65535 * GBN);
    const size_t off = (size_t)s0 * ns * kb;
    dim3 gg((unsigned)(nrt * kb), (unsigned)((nn + GBN - 1) / GBN));
    DBSRG_RUN(c, "k_band_contract",
              k_band_contract<<<gg, 256, 0, c->stream>>>(ns, kb, icase, rkb, nn, X + off, Y + off));
  }
  return DBSRG_OK;
}

// convol case 3 of nsg full ('x') densities X with one full R^k table
// (k_exchange, 's','s' storage); for these tables case 4 adds the same
// products (dbsr_lib_dbs.f90:2344-2470)
int exchange_contract(dbsrg_ctx *c, const double *rkb, int nsg, const double *X, double *Y) {
  const int ns = c->g.ns, ks = c->g.ks;
  dim3 gx((unsigned)(((size_t)ns * ns + 255) / 256), (unsigned)((nsg + XNB - 1) / XNB));
  DBSRG_RUN(c, "k_exchange", k_exchange<<<gx, 256, 0, c->stream>>>(ns, ks, 0, nsg, rkb, X, Y));
  return DBSRG_OK;
}

namespace {

// The cached inputs of a planned list, built on the table stream of its k;
// the contraction stream waits for them.  overlap: the contraction stream
// holds nothing the builds read (only the kernels of earlier lists of this
// assembly), so they may run beside it.
int prepare_list(dbsrg_ctx *c, const ListPlan &P, bool overlap) {
  if (P.icase == 0 && !P.sp) return DBSRG_OK;
  int rc;
  if (P.factored && !P.sp) {  // shared by the builds of every k
    bool built = false;
    if ((rc = ensure_bound_rows(c, &built))) return rc;
    if (built) overlap = false;
  }
  if (!overlap || c->stream_built || c->timing) {
    // timing mode keeps the builds apart from the contraction kernels, so
    // that each kernel's events time it alone
    DBSRG_TRY(c, cudaEventRecord(c->sready, c->stream));
    for (cudaStream_t b : c->bstream) DBSRG_TRY(c, cudaStreamWaitEvent(b, c->sready, 0));
    c->stream_built = false;
  }
  const int bs = P.kpol & 1;
  const cudaStream_t keep = c->stream;
  c->stream = c->bstream[bs];
  rc = exec_list(c, P, 0, true);
  c->stream = keep;
  if (rc) return rc;
  DBSRG_TRY(c, cudaEventRecord(c->tready[bs], c->bstream[bs]));
  DBSRG_TRY(c, cudaStreamWaitEvent(c->stream, c->tready[bs], 0));
  if (c->timing) {  // the other table stream joins too (nothing else runs beside)
    DBSRG_TRY(c, cudaEventRecord(c->tready[bs ^ 1], c->bstream[bs ^ 1]));
    DBSRG_TRY(c, cudaStreamWaitEvent(c->stream, c->tready[bs ^ 1], 0));
  }
  return DBSRG_OK;
}

}  // namespace

int gen_matrix_plain(dbsrg_ctx *c, int icase, int itype, int kpol, int n, const int *ipt,
                     const int *k1, const int *k2, const int *k3, const int *k4,
                     const double *cdata) {
  if (n <= 0) return DBSRG_OK;
  if (!c->hch) return set_err(c, DBSRG_ESTATE, "no matrix allocated");
  if (!c->pq) return set_err(c, DBSRG_ESTATE, "no orbitals set");
  cudaStream_t st = c->stream;
  int rc;
  // The list state lives in one of two buffers; in the asynchronous mode the
  // set-up runs on the set-up stream once the kernels of the call two back
  // are done with the buffer, while the previous call's kernels run.
  const bool pipe = c->async;
  const int par = c->lpar;
  c->lpar ^= 1;
  cudaStream_t ss = pipe ? c->sstream : st;
  if ((rc = ensure_lstate(c, par, plan_bytes(c, icase, itype, n)))) return rc;
  if (pipe) DBSRG_TRY(c, cudaStreamWaitEvent(ss, c->lfree[par], 0));
  ListPlan P;
  if ((rc = plan_list(c, icase, itype, kpol, n, ipt, k1, k2, k3, k4, cdata, c->wlo, c->wcap, 1,
                      c->lstate[par], ss, P)))
    return rc;
  if (pipe) {  // the contraction waits for the set-up
    DBSRG_TRY(c, cudaEventRecord(c->lready, ss));
    DBSRG_TRY(c, cudaStreamWaitEvent(st, c->lready, 0));
  }
  if ((rc = prepare_list(c, P, pipe && c->pending))) return rc;
  if ((rc = exec_list(c, P, 0))) return rc;
  // the kernels of this call are done with the list state after this point
  DBSRG_TRY(c, cudaEventRecord(c->lfree[par], st));
  if (pipe) {
    c->pending = true;
    return DBSRG_OK;
  }
  return drain(c);  // synchronous mode: wait, and report the tensor-core error word
}

int assemble_windows(dbsrg_ctx *c, int nlists, const dbsrg_list *lists, int nwin, int nslot,
                     const std::function<int(int w, double *slot)> &before,
                     const std::function<int(int w, int blo, int nb, double *slot)> &after,
                     const std::vector<int> *wstart) {
  const int iicc = c->iicc;
  const int nw = wstart ? (int)wstart->size() - 1 : (iicc + nwin - 1) / nwin;
  if (wstart) {
    const std::vector<int> &ws = *wstart;
    if (nw < 1 || ws[0] != 1 || ws[nw] != iicc + 1)
      return set_err(c, DBSRG_EINVAL, "window partition must cover blocks 1..iicc");
    for (int w = 0; w < nw; w++)
      if (ws[w + 1] <= ws[w] || ws[w + 1] - ws[w] > nwin)
        return set_err(c, DBSRG_EINVAL, "window partition: empty or oversized window");
  }
  auto wlo_of = [&](int w) { return wstart ? (*wstart)[w] : 1 + w * nwin; };
  auto wsize = [&](int w) {
    return wstart ? (*wstart)[w + 1] - (*wstart)[w] : std::min(nwin, iicc - w * nwin);
  };
  const size_t blk = (size_t)c->g.ms * c->g.ms;
  std::vector<ListPlan> plans((size_t)nlists);
  std::vector<void *> mem((size_t)nlists, nullptr);
  const double *hch0 = c->hch;
  const int wlo0 = c->wlo, wcap0 = c->wcap;
  auto slot_of = [&](int w) { return c->hmem + (size_t)(w % nslot) * nwin * blk; };
  auto enter = [&](int w) {
    c->hch = slot_of(w);
    c->wlo = wlo_of(w);
    c->wcap = wstart ? wsize(w) : nwin;
  };
  auto body = [&]() -> int {
    int rc;
    // window 0 is executed list by list right after each list's set-up, so
    // the set-up of list l+1 overlaps the kernels of list l
    enter(0);
    if ((rc = before(0, c->hch))) return rc;
    bool prepared = false;  // the builds of the first list wait for the stream
    for (int l = 0; l < nlists; l++) {
      const dbsrg_list &L = lists[l];
      if (L.ncdata < 0) return set_err(c, DBSRG_EINVAL, "ncdata < 0");
      if (L.ncdata == 0) continue;
      if (!L.k1 || !L.k2 || !L.k3 || !L.cdata) return set_err(c, DBSRG_EINVAL, "null list pointer");
      if (!(mem[l] = cache_alloc(c, plan_bytes(c, L.icase, L.itype, L.ncdata))))
        return set_err(c, DBSRG_ENOMEM, "list state allocation failed");
      if ((rc = plan_list(c, L.icase, L.itype, L.kpol, L.ncdata, L.ipt, L.k1, L.k2, L.k3, L.k4,
                          L.cdata, 1, nwin, nw, mem[l], c->sstream, plans[l],
                          wstart ? wstart->data() : nullptr)))
        return rc;
      DBSRG_TRY(c, cudaEventRecord(c->lready, c->sstream));
      DBSRG_TRY(c, cudaStreamWaitEvent(c->stream, c->lready, 0));
      if ((rc = prepare_list(c, plans[l], prepared))) return rc;
      prepared = true;
      if ((rc = exec_list(c, plans[l], 0))) return rc;
    }
    if ((rc = after(0, 1, wsize(0), c->hch))) return rc;
    for (int w = 1; w < nw; w++) {
      enter(w);
      if ((rc = before(w, c->hch))) return rc;
      for (int l = 0; l < nlists; l++)
        if (lists[l].ncdata > 0 && (rc = exec_list(c, plans[l], w))) return rc;
      if ((rc = after(w, wlo_of(w), wsize(w), c->hch))) return rc;
    }
    return DBSRG_OK;
  };
  int rc = body();
  const int rd = drain(c);
  for (void *p : mem) cache_free(c, p);  // pooled for the next assembly
  c->hch = const_cast<double *>(hch0);
  c->wlo = wlo0;
  c->wcap = wcap0;
  return rc ? rc : rd;
}

// ---------------------------------------------------------------------------
// A whole assembly captured as one CUDA graph (dbsrg_graph_capture): every
// list is planned first (segments and chunks need the list read back, which
// a graph cannot do), the cached tables and orbital products are dropped,
// and then the zeroing of the matrix, the builds of every table, pair
// potential and digit operand the lists read, and every contraction and
// scatter are captured from the contraction stream (the table streams join
// through the events of prepare_list).  A replay repeats all of that from
// the orbitals in the context's orbital buffer.
struct GraphState {
  std::vector<ListPlan> plans;
  std::vector<void *> mem;
  cudaGraphExec_t exec = nullptr;
  long long launches = 0;
};

void graph_drop(dbsrg_ctx *c) {
  GraphState *g = c->graph;
  if (!g) return;
  c->graph = nullptr;
  // a replay may be running: its plan memory goes back to the pool only
  // once the stream is idle
  cudaStreamSynchronize(c->stream);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  for (void *p : g->mem) cache_free(c, p);
  delete g;
}

int graph_capture(dbsrg_ctx *c, int nlists, const dbsrg_list *lists) {
  graph_drop(c);
  if (!c->hch) return set_err(c, DBSRG_ESTATE, "no matrix allocated");
  if (!c->pq) return set_err(c, DBSRG_ESTATE, "no orbitals set");
  if (c->hcap < c->iicc) return set_err(c, DBSRG_ESTATE, "graph capture needs the whole matrix");
  if (c->timing) return set_err(c, DBSRG_ESTATE, "graph capture with timing on");
  int rc = drain(c);
  if (rc) return rc;
  free_tables(c);  // rebuilt inside the graph (the buffers stay pooled)
  GraphState *g = new (std::nothrow) GraphState();
  if (!g) return set_err(c, DBSRG_ENOMEM, "graph state");
  g->plans.resize((size_t)nlists);
  g->mem.assign((size_t)nlists, nullptr);
  const double *hch0 = c->hch;
  const int wlo0 = c->wlo;
  c->hch = c->hmem;
  c->wlo = 1;
  auto restore = [&]() {
    c->hch = const_cast<double *>(hch0);
    c->wlo = wlo0;
  };
  auto fail = [&](int r) {
    for (void *p : g->mem) cache_free(c, p);
    delete g;
    restore();
    return r;
  };
  for (int l = 0; l < nlists; l++) {
    const dbsrg_list &L = lists[l];
    if (L.ncdata < 0) return fail(set_err(c, DBSRG_EINVAL, "ncdata < 0"));
    if (L.ncdata == 0) continue;
    if (!L.k1 || !L.k2 || !L.k3 || !L.cdata)
      return fail(set_err(c, DBSRG_EINVAL, "null list pointer"));
    if (!(g->mem[l] = cache_alloc(c, plan_bytes(c, L.icase, L.itype, L.ncdata))))
      return fail(set_err(c, DBSRG_ENOMEM, "list state allocation failed"));
    if ((rc = plan_list(c, L.icase, L.itype, L.kpol, L.ncdata, L.ipt, L.k1, L.k2, L.k3, L.k4,
                        L.cdata, 1, c->iicc, 1, g->mem[l], c->sstream, g->plans[l])))
      return fail(rc);
  }
  DBSRG_TRY(c, cudaStreamSynchronize(c->sstream));
  const long long l0 = c->launches;
  DBSRG_TRY(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
  rc = DBSRG_OK;
  {
    const size_t blk = (size_t)c->g.ms * c->g.ms;
    cudaError_t e = cudaMemsetAsync(c->hmem, 0, sizeof(double) * blk * c->iicc, c->stream);
    if (e == cudaSuccess)
      e = cudaMemsetAsync(c->acf, 0, sizeof(double) * (size_t)c->iicc * (c->mk + 1), c->stream);
    if (e != cudaSuccess) rc = cuda_check(c, e, "graph zeroing");
  }
  if (!rc) rc = zero_structures(c);
  // both table streams join the capture here (a list without table builds,
  // such as an overlap list first, would leave them outside it)
  for (int b = 0; b < 2 && !rc; b++) {
    cudaError_t e = cudaEventRecord(c->sready, c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->bstream[b], c->sready, 0);
    if (e != cudaSuccess) rc = cuda_check(c, e, "graph fork");
  }
  bool prepared = false;
  for (int l = 0; l < nlists && !rc; l++) {
    if (lists[l].ncdata <= 0) continue;
    if ((rc = prepare_list(c, g->plans[l], prepared))) break;
    prepared = true;
    rc = exec_list(c, g->plans[l], 0);
  }
  // both table streams back into the contraction stream (one of them may
  // have joined the capture without work after its last join)
  for (int b = 0; b < 2 && !rc; b++) {
    cudaError_t e = cudaEventRecord(c->tready[b], c->bstream[b]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->tready[b], 0);
    if (e != cudaSuccess) rc = cuda_check(c, e, "graph join");
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(c->stream, &graph);
  if (!rc && ee != cudaSuccess) rc = cuda_check(c, ee, "graph capture");
  if (!rc) {
    const cudaError_t ei = cudaGraphInstantiate(&g->exec, graph, 0);
    if (ei != cudaSuccess) rc = cuda_check(c, ei, "graph instantiate");
  }
  if (graph) cudaGraphDestroy(graph);
  c->stream_built = false;
  if (rc) {
    cudaGetLastError();
    if (g->exec) cudaGraphExecDestroy(g->exec);
    g->exec = nullptr;
    free_tables(c);  // whatever the capture cached was never computed
    return fail(rc);
  }
  g->launches = c->launches - l0;
  c->launches = l0;
  restore();
  c->graph = g;
  return DBSRG_OK;
}

int graph_launch(dbsrg_ctx *c, const double *pq) {
  GraphState *g = c->graph;
  if (!g) return set_err(c, DBSRG_ESTATE, "no captured assembly");
  if (pq) {
    int rc = copy_in(c, c->pq, pq, sizeof(double) * 2 * (size_t)c->g.ns * c->nbf);
    if (rc) return rc;
  }
  DBSRG_TRY(c, cudaGraphLaunch(g->exec, c->stream));
  c->launches += g->launches;
  if (c->async) {
    c->pending = true;
    return DBSRG_OK;
  }
  return drain(c);
}
