// internal.cuh -- shared declarations of the sm_103a assembly library.
//
// Device memory layout (all FP64 arrays keep the reference's Fortran
// column-major order so results can be compared element by element and
// handed back to a Fortran caller without reshuffling):
//   grid:     t(ns+ks), tp, tq, gx/gw(ks), gr/grw/grm(nv,ks),
//             pbsp(nv+1,ks,ksp), qbsp(nv+1,ks,ksq), fpbs/fqbs(ns,ns),
//             fppqq(ms,ms)
//   tables:   R: rkb(ns,ns,ks,ks) per (k,type); S: rkb(ns,ns,2ks-1,2ks-1)
//             per (k,type), built on first use (the irka cache of
//             dbsr_lib_dbs.f90:2919-2925) and kept resident in HBM
//   orbitals: pq(ns,2,nbf)
//   matrix:   hch(ms,ms,iicc), acf(iicc,0:mk), icc(nch,nch)
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "../../include/dbsrg.h"

#define DBSRG_IBO 32768  // packing basis for orbitals, mod_dbsr_mat.f90:61
#define DBSRG_MAXK 16    // largest supported spline order

struct DeviceGrid {
  int ns = 0, ks = 0, ksp = 0, ksq = 0, nv = 0, nsp = 0, nsq = 0, ms = 0;
  double *t = nullptr, *tp = nullptr, *tq = nullptr;
  double *gx = nullptr, *gw = nullptr;
  double *gr = nullptr, *grw = nullptr, *grm = nullptr;
  double *pbsp = nullptr, *qbsp = nullptr;
  double *fpbs = nullptr, *fqbs = nullptr, *fppqq = nullptr;
  // inner Gauss points of the diagonal cells (they depend on the grid only):
  // per interval, for the ks x ks points (outer m, inner i): x, weight,
  // P B-spline values (ksp each), Q B-spline values (ksq each)
  double *tri = nullptr;
};

// resident cell moments and diagonal-cell integrals of one table
struct CellData {
  double *lo1 = nullptr, *hi1 = nullptr, *lo2 = nullptr, *hi2 = nullptr, *rkd = nullptr;
};

// far-field orbital vectors of one exchange table and contraction case:
// U, V (upper field) and Ul, Vl (lower field, R^k only), each (ns, nbound)
struct FarField {
  double *U = nullptr, *V = nullptr, *Ul = nullptr, *Vl = nullptr;
  // split-BF16 digit tiles of U (mode 0) and Ul (mode 1) and their row
  // exponents, built on first use by the tensor-core exchange
  void *Ud = nullptr;
  int *eu = nullptr;
};

// one channel-pair segment of a coefficient list (a run of equal K1)
struct SegInfo {
  int start, end;  // entry range [start,end) in IPT order
  int ich, jch;    // channel pair decoded from K1
  int blk;         // 1-based block from icc, 0 if invalid
  int partner;     // other segment of this list mapping to the same block, or -1
  int owner;       // 1 if this segment applies the block's contributions
};

struct dbsrg_ctx {
  int device = 0;
  int nsm = 0;  // streaming multiprocessors of the device
  cudaStream_t stream = nullptr;
  DeviceGrid g;
  std::string err;
  long long launches = 0;
  int precision = DBSRG_PLAIN_FP64;
  // orbitals
  int nbf = 0;
  double *pq = nullptr;
  int *ipbs = nullptr;
  std::vector<int> h_ipbs;
  // matrix
  int nch = 0, iicc = 0, mk = -1;
  int *icc = nullptr;
  std::vector<int> h_icc;
  double *hch = nullptr;   // the current window's first block
  double *hmem = nullptr;  // the matrix allocation (hcap blocks)
  int hcap = 0;
  double *acf = nullptr;
  // table caches, indexed [k*4+type] (R) and [k*2+type] (S)
  std::vector<double *> rtab, stab;
  // band-limited tables (|j-i| <= DBSRG_TABLE_BAND) for the factored path
  std::vector<double *> rbtab, sbtab;
  std::vector<CellData> rcell, scell;
  // far-field vectors, keyed (k*4+type)*2+case34 (R) / (k*2+type)*2+case34 (S);
  // map nodes keep their addresses while other entries are added
  std::map<size_t, FarField> rfar, sfar;
  // orbital-pair potentials of the factored contraction (direct band results
  // and exchange band results per ordered bound-orbital pair), keyed by
  // pairpot_key(); they depend on the tables and the orbitals
  std::map<long long, double *> ppot;
  // float-float copies (hi, lo) of orbital products for the split form's
  // gather-sums, keyed by the FP64 array they copy; dropped with the
  // orbital products
  std::map<const void *, float2 *> ffc;
  // bound-orbital rows brows[(comp-1)*nbound*ns + a*ns + x] = pq(x+1, comp, b2o[a])
  double *brows = nullptr;
  // bound-orbital map: bmap[orb-1] = dense bound index or -1; nbound
  int nbound = 0;
  int *bmap = nullptr;  // (nbf)
  int *b2o = nullptr;   // (nbound): 1-based orbital of each bound index
  std::vector<int> h_bmap;
  // <a|r^k|b> per component for the asymptotic coefficients, [k]
  std::vector<double *> quad;
  // scratch arena (grown on demand, reused across calls)
  void *scratch = nullptr;
  size_t scratch_bytes = 0;
  void *scratch2 = nullptr;   // list state of one Gen_matrix call
  size_t scratch2_bytes = 0;
  void *tscratch = nullptr;   // table construction (moments, diagonal cells)
  size_t tscratch_bytes = 0;
  void *fscratch = nullptr;   // factored contraction (band densities, Z vectors)
  size_t fscratch_bytes = 0;
  void *tcscratch = nullptr;  // tensor-core far field (digit slices, scales)
  size_t tcscratch_bytes = 0;
  // pair-potential construction (cell sums, cell parts), one per table stream
  void *pscratch[2] = {nullptr, nullptr};
  size_t pscratch_bytes[2] = {0, 0};
  // List pipeline.  The state of one Gen_matrix call (the list in IPT order,
  // segments, chunk members, quadrant records) lives in one of two buffers,
  // alternating per call.  Its set-up (copies, segment kernels, read-backs)
  // runs on sstream once the kernels of the call two back have released the
  // buffer (lfree), and the contraction on stream waits for it (lready), so
  // the host plans one list while the kernels of the previous one run.
  cudaStream_t sstream = nullptr;
  void *lstate[2] = {nullptr, nullptr};
  size_t lstate_bytes[2] = {0, 0};
  cudaEvent_t lfree[2] = {nullptr, nullptr};
  cudaEvent_t lready = nullptr;
  int lpar = 0;
  // Table streams.  The tables, cell data, far fields, digits and pair
  // potentials that a list's contraction reads are built on one of two
  // table streams (the higher priority) before the contraction, which waits
  // for them (tready).  The stream is chosen by the parity of the list's k:
  // everything built for one k (cell data, tables, far fields, digits,
  // quadratures) stays on one stream, and the builds for neighbouring k run
  // side by side, and beside the kernels of earlier lists.
  // When the contraction stream may hold work the builds read (the first
  // list after a state change, the timing mode), both table streams first
  // wait for it (sready).  A pair-potential build made on the contraction
  // stream itself sets stream_built, with the same effect at the next
  // preparation, since it shares pscratch[0].  The bound-orbital rows
  // (shared by every k) are made on the contraction stream before the first
  // preparation that needs them.
  cudaStream_t bstream[2] = {nullptr, nullptr};
  cudaEvent_t tready[2] = {nullptr, nullptr}, sready = nullptr;
  bool stream_built = false;
  // asynchronous mode (dbsrg_set_async): Gen_matrix returns once its kernels
  // are queued; failures of queued kernels surface at the next call that
  // waits (dbsrg_sync, the read-outs, state changes)
  bool async = false;
  bool pending = false;
  // limit of the tensor-core kernels' pipeline waits, and the test switch
  // that makes one of them run out (dbsrg_set_wait_limit,
  // dbsrg_inject_wait_timeout)
  unsigned long long wait_ns = 2000000000ull;
  bool inject_wait = false;
  // cuSOLVER / cuBLAS handles of the channel basis (basis.cu), made on use
  void *sv_handle = nullptr, *bl_handle = nullptr;
  // tuning (dbsrg_set_tuning): segments per chunk of the factored exchange
  // and direct contractions, windows of dbsrg_assemble_to_host
  int tune_xchunk = 256, tune_dchunk = 4096, tune_windows = 8;
  // block window: hch holds blocks wlo .. wlo + wcap - 1 of 1 .. iicc (all
  // of them unless dbsrg_alloc_matrix_window asked for fewer); Gen_matrix
  // skips the segments of blocks outside the window
  int wlo = 1, wcap = 0;
  // assembly straight into host memory (dbsrg_assemble_to_host): windows
  // alternate between two halves of the allocation while a copy stream
  // moves the finished one to the host
  cudaStream_t cstream = nullptr;
  cudaEvent_t cdone[2] = {nullptr, nullptr}, wdone = nullptr;
  // pool of released cache buffers (tables, cell data, far fields, digits,
  // pair potentials), reused by exact size: a rebuild after
  // dbsrg_invalidate_tables allocates nothing; dbsrg_release_tables and
  // allocation failures return the pool to the device
  std::multimap<size_t, void *> pool;
  std::map<void *, size_t> psize;
  // scratch buffers replaced by larger ones while queued work could still
  // read them (grow_buffer); freed with the pool
  std::vector<void *> retired;
  // a captured whole assembly (dbsrg_graph_capture), replayed by
  // dbsrg_graph_launch; dropped by every call that frees or replaces memory
  // it names
  struct GraphState *graph = nullptr;
  // error word of the tensor-core kernels (bounded waits), read whenever the
  // context waits for its stream
  int *kerr = nullptr;
  // pinned staging for host lists
  void *pinned = nullptr;
  size_t pinned_bytes = 0;
  // per-kernel CUDA-event timing (dbsrg_timing): event pairs recorded on
  // the context stream around each named launch, resolved on report
  bool timing = false;
  struct TimedLaunch {
    const char *name;
    cudaEvent_t a, b;
    double bytes, flops;  // algorithmic work of the launch (0: not stated)
  };
  std::vector<TimedLaunch> tev;
  std::vector<cudaEvent_t> evpool;
  // Matrix parts outside hch (structures.cu): perturber vectors hcp(ms,iicb)
  // with icb(nch,npert) and perturber scalars hp(iibb) with ibb(npert,npert)
  // (Alloc_dbsr_matrix, updates.f90:47-72); target interaction and overlap
  // matrices htarg/otarg(ntarg(ntarg+1)/2) with iptar(nch) (Target_h,
  // target_subs.f90:2-31); the one-electron Dirac matrices hd(ms,ms,nkap)
  // of the kappas h_kap and the kappa of every orbital h_kbs (L_data);
  // eps_c of the O and L lists (mod_dbsr_mat.f90:50)
  int npert = 0, iicb = 0, iibb = 0;
  std::vector<int> h_icb, h_ibb;
  double *hcp = nullptr, *hp = nullptr;
  int ntarg = 0, iitar = 0, check_target = 1;
  std::vector<int> h_iptar;
  double *htarg = nullptr, *otarg = nullptr;
  int nkap = 0;
  std::vector<int> h_kap, h_kbs;
  double *hd = nullptr;
  double eps_c = 1.0e-10;
  // rk4 entries of DBSR_HF's Breit energy (dbsrg_hf_breit_list), read by
  // dbsrg_hf_matrix for its Breit part (hf_matrix_breit)
  std::vector<int> hf_kr1, hf_kr2, hf_kr3, hf_kr4;
  std::vector<double> hf_crk;
};

cudaEvent_t event_get(dbsrg_ctx *c);

// block b (1-based) of the matrix is held by the current window
inline bool in_window(const dbsrg_ctx *c, int b) { return b >= c->wlo && b < c->wlo + c->wcap; }
// base the kernels index blocks from, hch + (b - 1) ms^2 for block b: the
// window's storage shifted by its first block (only blocks inside the window
// are ever addressed)
inline double *hch_base(const dbsrg_ctx *c) {
  const size_t shift = (size_t)(c->wlo - 1) * c->g.ms * c->g.ms * sizeof(double);
  return reinterpret_cast<double *>(reinterpret_cast<uintptr_t>(c->hch) - shift);
}

// ---- error helpers -------------------------------------------------------
int set_err(dbsrg_ctx *c, int code, const std::string &msg);
int cuda_check(dbsrg_ctx *c, cudaError_t e, const char *what);
#define DBSRG_TRY(ctx, call)                                \
  do {                                                      \
    cudaError_t _e = (call);                                \
    if (_e != cudaSuccess) return cuda_check(ctx, _e, #call); \
  } while (0)
// After every launch: count it, check the launch, and with the environment
// variable DBSRG_SYNC_CHECK=1 also synchronise so a failing kernel is
// reported by name at its own launch.
bool sync_check_enabled();
#define DBSRG_LAUNCHED(ctx)                                                  \
  do {                                                                       \
    (ctx)->launches++;                                                       \
    cudaError_t _e = cudaGetLastError();                                     \
    if (_e != cudaSuccess) return cuda_check(ctx, _e, "kernel launch");      \
    if (sync_check_enabled()) {                                              \
      _e = cudaStreamSynchronize((ctx)->stream);                             \
      if (_e != cudaSuccess) return cuda_check(ctx, _e, __func__);           \
    }                                                                        \
  } while (0)

// Launch a named kernel on the context stream; with timing enabled the
// launch is bracketed by events (resolved by dbsrg_timing_report) and its
// algorithmic bytes and FLOPs, where stated, are recorded with it.
#define DBSRG_RUN_SW(ctx, strm, name, wbytes, wflops, ...)        \
  do {                                                            \
    cudaEvent_t _ea = nullptr;                                    \
    if ((ctx)->timing) {                                          \
      _ea = event_get(ctx);                                       \
      cudaEventRecord(_ea, (strm));                               \
    }                                                             \
    __VA_ARGS__;                                                  \
    if ((ctx)->timing) {                                          \
      cudaEvent_t _eb = event_get(ctx);                           \
      cudaEventRecord(_eb, (strm));                               \
      (ctx)->tev.push_back({name, _ea, _eb, (double)(wbytes), (double)(wflops)}); \
    }                                                             \
    DBSRG_LAUNCHED(ctx);                                          \
  } while (0)
#define DBSRG_RUN_W(ctx, name, wbytes, wflops, ...) \
  DBSRG_RUN_SW(ctx, (ctx)->stream, name, wbytes, wflops, __VA_ARGS__)
#define DBSRG_RUN(ctx, name, ...) DBSRG_RUN_W(ctx, name, 0, 0, __VA_ARGS__)
#define DBSRG_RUN_S(ctx, strm, name, ...) DBSRG_RUN_SW(ctx, strm, name, 0, 0, __VA_ARGS__)

bool is_device_ptr(const void *p);
// copies n bytes from a host-or-device pointer into device memory dst
int copy_in(dbsrg_ctx *c, void *dst, const void *src, size_t n);
int copy_in_s(dbsrg_ctx *c, void *dst, const void *src, size_t n, cudaStream_t s);
// waits for the set-up, table and contraction streams and reports failures of
// queued kernels
int drain(dbsrg_ctx *c);
// raises the dynamic shared-memory limit of kernel fn on the context's
// device to at least bytes; never lowers it (contexts of a batch launch the
// same kernels concurrently with different sizes), one lock for all
int raise_smem_limit(dbsrg_ctx *c, const void *fn, size_t bytes);
int ensure_lstate(dbsrg_ctx *c, int par, size_t bytes);
// cache buffers through the pool (nullptr when the device is out of memory)
void *cache_alloc(dbsrg_ctx *c, size_t bytes);
void cache_free(dbsrg_ctx *c, void *p);
void pool_trim(dbsrg_ctx *c);
int copy_out(dbsrg_ctx *c, void *dst, const void *src, size_t n);
// scratch arenas (device)
// grows a scratch buffer to at least bytes; the old one is retired, not
// freed (queued work may still use it)
int grow_buffer(dbsrg_ctx *c, void **p, size_t *have, size_t bytes);
int ensure_scratch(dbsrg_ctx *c, size_t bytes);
int ensure_scratch2(dbsrg_ctx *c, size_t bytes);
int ensure_tscratch(dbsrg_ctx *c, size_t bytes);
int ensure_tcscratch(dbsrg_ctx *c, size_t bytes);
int ensure_pscratch(dbsrg_ctx *c, int which, size_t bytes);
// the bound-orbital rows of both components (factor.cu), built once per
// orbital set; *built set when they were made now
int ensure_bound_rows(dbsrg_ctx *c, bool *built);
int ensure_pinned(dbsrg_ctx *c, size_t bytes);
// frees the far-field vectors, pair potentials and bound rows (they depend
// on the orbitals and the tables)
void free_orbital_products(dbsrg_ctx *c);
// the cached tables and orbital products back to the pool (capi.cu)
void free_tables(dbsrg_ctx *c);
// captured whole assembly (assemble.cu): capture (plans every list, then
// captures the table builds and contractions from the contraction stream),
// replay with the orbitals optionally replaced (same size), drop
int graph_capture(dbsrg_ctx *c, int nlists, const dbsrg_list *lists);
int graph_launch(dbsrg_ctx *c, const double *pq);
void graph_drop(dbsrg_ctx *c);
// handles of the channel basis (basis.cu)
void basis_release(dbsrg_ctx *c);
// float-float copy of n doubles at src (cached until the orbital products go)
int ff_of(dbsrg_ctx *c, const double *src, size_t n, const float2 **out);

// ---- tables.cu ------------------------------------------------------------
int build_grid(dbsrg_ctx *c, const double *t_host_or_dev);
int compute_moments(dbsrg_ctx *c, int which, int k, double *rkm_dev);
int compute_diag_cells(dbsrg_ctx *c, int type, int k, double *rkd_dev);
// returns device pointer of the cached table (building it if needed)
int get_rtable(dbsrg_ctx *c, int type, int k, const double **out);
int get_stable(dbsrg_ctx *c, int type, int k, const double **out);
int get_quad(dbsrg_ctx *c, int k, const double **out);
int get_celldata(dbsrg_ctx *c, int family, int type, int k, const CellData **out);
// (ns, 2*DBSRG_TABLE_BAND+1, kb, kb): rkb(i, j-i+DBSRG_TABLE_BAND+1, ip, jp)
#define DBSRG_TABLE_BAND 16
int get_band_table(dbsrg_ctx *c, int family, int type, int k, const double **out);

// ---- assemble.cu ----------------------------------------------------------
int gen_matrix_plain(dbsrg_ctx *c, int icase, int itype, int kpol, int n,
                     const int *ipt, const int *k1, const int *k2,
                     const int *k3, const int *k4, const double *cdata);
int update_hx(dbsrg_ctx *c, int ich, int jch, const double *d, double cc);
// convol cases 1/2 (icase) of nsg band densities X[s][ns*kb] with the full
// table rkb (kb = ks for R, 2ks-1 for S) into Y[s][ns*kb], on the context stream
int band_contract(dbsrg_ctx *c, int kb, int icase, const double *rkb, int nsg, const double *X,
                  double *Y);
// convol case 3 (= 4) of nsg full densities with one full R^k table
int exchange_contract(dbsrg_ctx *c, const double *rkb, int nsg, const double *X, double *Y);
// Record_matrix's c = D_ich^T H D_jch for all blocks ich > jch as split-BF16
// tensor-core products (sgemm.cu); D on the device
int split_channel_basis(dbsrg_ctx *c, const double *D, const int *nsol);
// Every list set up once, then executed window by window over the blocks
// (windows of nwin blocks alternating between nslot slots of the matrix
// allocation; or, with wstart, the windows [wstart[w], wstart[w+1]) of at
// most nwin blocks, wstart[0] = 1 and wstart[nw] = iicc + 1): before(w,
// slot) prepares a slot (on the contraction stream), after(w, blo, nb, slot)
// takes the assembled window.  Drains at the end.
int assemble_windows(dbsrg_ctx *c, int nlists, const dbsrg_list *lists, int nwin, int nslot,
                     const std::function<int(int w, double *slot)> &before,
                     const std::function<int(int w, int blo, int nb, double *slot)> &after,
                     const std::vector<int> *wstart = nullptr);

// ---- structures.cu --------------------------------------------------------
// The list structures whose terms are not channel-pair contractions: R_data
// itypes 1/2, S_data itypes 1-5, L_data itypes 1-3, O_data itypes 1/2/4.
// A list is planned once on the host (entries classified, terms grouped by
// the block, perturber column or scalar they update) and executed per block
// window (its potentials, vectors and coefficients computed, the terms of
// the window's blocks applied; perturber and target terms in the window that
// holds block 1).
struct StructPlan;
bool is_structure_list(int icase, int itype);
size_t structure_plan_bytes(const dbsrg_ctx *c, int icase, int itype, int n);
int plan_structures(dbsrg_ctx *c, int icase, int itype, int kpol, int n, const int *ipt,
                    const int *k1, const int *k2, const int *k3, const int *k4,
                    const double *cdata, int blo0, int nwin, int nw, void *dev,
                    cudaStream_t ss, StructPlan **out, const int *wstart = nullptr);
int exec_structures(dbsrg_ctx *c, const StructPlan &P, int w, bool prep);
void free_structure_plan(StructPlan *P);
// zeroes hcp, hp, htarg, otarg (with the matrix); frees them (destroy)
int zero_structures(dbsrg_ctx *c);
void free_structures(dbsrg_ctx *c);

// ---- factor.cu ------------------------------------------------------------
int ensure_fscratch(dbsrg_ctx *c, size_t bytes);
// One chunk of segments of one list through the factored contraction,
// including its scatter into hch.
struct FactorJob {
  int family;        // 0 R^k, 1 S^k
  int kpol;
  int icv;           // convol case 1..4
  char sym;          // storage of the results: 's', 'n' (band) or 'x' (full)
  int na;            // PQ types (atypes) processed, in order
  int types[4];      // table type of each atype
  int jp1[4], jp2[4];
  int ii[4], jj[4];  // target quadrant of each atype (UPDATE_HS)
  const double *tabs[4];  // band tables of the exchange cases
  int nm;            // member segments of the chunk
  const int *members;
  int nown;          // owner segments of the chunk
  const int *own;    // member slot of each owner
  const SegInfo *info;
  const int *k2, *k3;
  const int *pairs;  // ordered bound-orbital pair index of every entry
  const double *cd;
  const float2 *cdf;  // split form: the coefficients as float-float pairs
  double *Y;         // exchange results [a][slot][ns*ns] (FP64 far field)
  bool split;        // exchange on the tensor cores (split BF16), fused scatter
  int nxq;           // split exchange: (owner block, quadrant) records of the chunk
  const struct XQuad *xq;
  const struct XQuad *hxq;  // host copy of the records (work accounting)
  bool prep;         // build (or find) the cached inputs only, launch no contraction
  long long nent;    // entries of the member segments (executed-work statements)
};
int factored_contract(dbsrg_ctx *c, const FactorJob &job);
// One quadrant of one owner's block in the split exchange and the terms it
// receives (UPDATE_HS, updates.f90:110-179), in the order of k_scatter_x
// (atype-major, owner then partner, direct before transposed).  Term code:
// atype | transposed << 2 | member slot << 3.
struct XQuad {
  int blk, qr, qc, nt, half;
  int term[4];
  int pad[3];
};
static_assert(sizeof(XQuad) == 48, "XQuad is read as three 16-byte vectors");
// records of every quadrant of the owners of one chunk that receives terms;
// false if a quadrant would receive more than four
bool build_xquads(int na, const int *ii, const int *jj, const std::vector<int> &mem,
                  const std::vector<int> &own, const std::vector<SegInfo> &hinfo,
                  std::vector<XQuad> &out);
// exchange_tc.cu entry of the split form
struct SplitExchange {
  int na, nm, lower;
  const FarField *far[4];  // far-field vectors (and digit caches) per atype
  const float2 *Kbf[4];    // band pair potentials per atype (float-float)
  const int *members;
  const XQuad *xq, *hxq;  // device records and their host copy
  int nxq;
  const SegInfo *info;
  const int *pairs;
  const double *cd;
  const float2 *cdf;  // the coefficients as float-float pairs
  bool prep;          // build the digit and float-float caches only
  long long nent;     // entries of the member segments (executed-work statements)
};
int split_exchange(dbsrg_ctx *c, const SplitExchange &x);
// Direct pair potentials of table (family, type, k) for convol case icv with
// density components jp1/jp2: Kd[pair][ns*ncol] over the ordered bound-orbital
// pairs (pair = a*nbound + b), cached until release_tables/set_orbitals.
int get_pairpot_direct(dbsrg_ctx *c, int family, int type, int k, int icv, int jp1, int jp2,
                       const double **out);
// the same potentials as float-float pairs, the diagonal cells contracted in
// float-float arithmetic (the split form's direct sums)
int get_pairpot_direct_ff(dbsrg_ctx *c, int family, int type, int k, int icv, int jp1, int jp2,
                          const float2 **out);
int get_pairpot_direct_any(dbsrg_ctx *c, int family, int type, int k, int icv, int jp1, int jp2,
                           bool ff, const void **out);
// pairs[e] = bmap[K2]*nbound + bmap[K3]; sets *derr when an orbital is not bound
int pair_index(dbsrg_ctx *c, int n, const int *k2, const int *k3, int *pairs, int *derr,
               cudaStream_t s);

// ---- device helpers ---------------------------------------------------------
// Values of the kx B-splines that are nonzero on the interval starting at
// knot tx(kg) (1-based), at point x: the ni=1, nderiv=1 path of zbsplvd /
// zbsplvb (dbsr_lib_dbs.f90:4197-4468).  Explicit round-to-nearest
// intrinsics keep the reference's operation order (no contraction).
__device__ __forceinline__ void bspline_values(const double *tx, int kx,
                                               int kg, double x,
                                               double *biatx) {
  double dr[DBSRG_MAXK], dl[DBSRG_MAXK];
  biatx[0] = 1.0;
  for (int j = 1; j < kx; j++) {
    const int jp1 = j + 1;
    double saved = 0.0;
    dr[j - 1] = __dsub_rn(tx[kg + j - 1], x);
    dl[j - 1] = __dsub_rn(x, tx[kg - j]);
    for (int m = 1; m <= j; m++) {
      double term = __ddiv_rn(biatx[m - 1], __dadd_rn(dr[m - 1], dl[jp1 - m - 1]));
      biatx[m - 1] = __dadd_rn(saved, __dmul_rn(dr[m - 1], term));
      saved = __dmul_rn(dl[jp1 - m - 1], term);
    }
    biatx[jp1 - 1] = saved;
  }
}

// real**integer by binary exponentiation (same method as libgcc's powi)
__device__ __forceinline__ double ipow_d(double x, int m) {
  unsigned int n = m < 0 ? (unsigned)(-m) : (unsigned)m;
  double y = (n % 2) ? x : 1.0;
  while (n >>= 1) {
    x = __dmul_rn(x, x);
    if (n % 2) y = __dmul_rn(y, x);
  }
  return m < 0 ? __ddiv_rn(1.0, y) : y;
}
