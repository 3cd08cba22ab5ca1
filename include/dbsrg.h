/*
 * dbsrg.h -- C ABI of the GB300 (sm_103a) Hamiltonian-block assembly
 * library (libdbsrgpu.so) for DBSR_MAT3.
 *
 * The library replaces the assembly step that DBSR_MAT3 enters through
 *     Subroutine Gen_matrix(itype,kpol)      DBSR_MAT3/gen_matrix.f90:2-17
 * and everything below it:
 *   - B-spline grid and Gauss tables      dbsr_lib_dbs.f90:911-1102
 *   - cell moments and R^k/S^k tables    dbsr_lib_dbs.f90:1234-1720,2898-3936
 *   - density / convol / convol_sk       dbsr_lib_dbs.f90:2208-2891
 *   - R_data / S_data / L_data / O_data DBSR_MAT3/R_data.f90, S_data.f90,
 *     dispatch                          L_data.f90, O_data.f90
 *   - UPDATE_HS/HW/HV/HB/HX/ACF,        DBSR_MAT3/updates.f90:79-292,
 *     Target_h                          target_subs.f90:2-31
 * The Fortran caller keeps its module data; these entry points receive
 * that data explicitly (plain pointers and sizes, Fortran column-major
 * layout, 1-based orbital/channel/block numbers exactly as in the
 * reference), so an iso_c_binding interface block can bind them one to
 * one.  Conventions:
 *   - every entry point returns a dbsrg_status; nonzero means failure and
 *     dbsrg_last_error() gives a message.  The library never aborts; the
 *     Fortran shim stops on nonzero status as the reference does.
 *   - one context per process and thread; calls are serialised on the
 *     context's CUDA stream and return after the work is complete unless
 *     stated otherwise.
 *   - host arrays passed in stay owned by the caller; the library copies
 *     them.  Pointers may also be device pointers (CUDA unified
 *     addressing tells them apart); then no copy is made.
 *   - there is no CPU fallback: without a usable sm_103a device every
 *     call that needs one returns DBSRG_ECUDA.
 */
#ifndef DBSRG_H
#define DBSRG_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dbsrg_ctx dbsrg_ctx;

enum dbsrg_status {
  DBSRG_OK = 0,
  DBSRG_EINVAL = -1,   /* bad argument (the reference would Stop)        */
  DBSRG_ECUDA = -2,    /* CUDA error or no usable device                  */
  DBSRG_ENOMEM = -3,   /* device allocation failed                        */
  DBSRG_ERANGE = -4,   /* index out of range in a list (UPDATE_* checks)  */
  DBSRG_ESTATE = -5,   /* call order violated (e.g. no matrix allocated)  */
  DBSRG_ETIMEOUT = -6, /* a device-side bounded wait ran out              */
  DBSRG_EIO = -7       /* a file of the write-out could not be written     */
};

/* precision / algorithm of the contraction */
enum dbsrg_precision {
  DBSRG_PLAIN_FP64 = 0,  /* the reference's loop structure over the
                            assembled tables, FP64 throughout           */
  DBSRG_SPLIT_BF16 = 1,  /* cell-factored contraction; the exchange far
                            field as split-BF16 tcgen05 products (exact
                            FP32 slice sums, int64 recombination), fused
                            with the band and the scatter; tables, pair
                            potentials, band and block sums in FP64     */
  DBSRG_FACTOR_FP64 = 2  /* the same factored contraction, all FP64      */
};

/* table families for dbsrg_get_table */
enum dbsrg_family { DBSRG_RK = 0, DBSRG_SK = 1 };

typedef struct dbsrg_grid_desc {
  int ns;          /* number of order-ks B-splines                         */
  int ks;          /* order of the knot sequence (9)                       */
  int ksp;         /* order for P (large) components (8)                   */
  int ksq;         /* order for Q (small) components (9)                   */
  const double *t; /* knots t(1:ns+ks), host or device                     */
  int device;      /* CUDA device ordinal                                  */
} dbsrg_grid_desc;

/* Context with the B-spline grid: knots -> Gauss points, B-spline values
 * (pbsp/qbsp), overlap matrices fpbs/fqbs/fppqq, all built on the device.
 * Replaces read_knot_dat/def_grid (grid_type -1, dbsr_lib_dbs.f90:611)
 * + alloc_DBS_gauss (:911) + Def_pbsp/Def_qbsp/Def_pq_arrays (:987-1102). */
int dbsrg_create(dbsrg_ctx **ctx, const dbsrg_grid_desc *desc);
int dbsrg_destroy(dbsrg_ctx *ctx);
const char *dbsrg_last_error(const dbsrg_ctx *ctx);

/* Orbitals pq(ns,2,nbf) (Fortran order, P then Q) and ipbs(nbf), the
 * channel number of a channel orbital or 0 for a bound orbital: the
 * DBS_orbitals_pq module data read by R_data/S_data (R_data.f90:226,255). */
int dbsrg_set_orbitals(dbsrg_ctx *ctx, int nbf, const double *pq,
                       const int *ipbs);

/* Channel-pair matrix in the reference layout hch(ms,ms,iicc), ms=2*ns,
 * with icc(nch,nch) giving the 1-based block of a channel pair (0: not
 * held), and acf(iicc,0:mk).  Replaces Alloc_dbsr_matrix
 * (updates.f90:2-76); the matrix is zeroed. */
int dbsrg_alloc_matrix(dbsrg_ctx *ctx, int nch, const int *icc, int iicc,
                       int mk);
int dbsrg_zero_matrix(dbsrg_ctx *ctx);

/* Streamed output for matrices larger than the device memory (no reference
 * counterpart: Alloc_dbsr_matrix holds all of hch).  The device holds a
 * window of nwin consecutive blocks, blocks blo .. blo+nwin-1 after
 * dbsrg_set_window(blo) (blocks 1 .. nwin after the allocation); acf is
 * held whole.  dbsrg_gen_matrix then adds only the entries of blocks in the
 * window (the others are skipped, not errors), as do dbsrg_update_hx and
 * the overlaps, and dbsrg_get_matrix returns the window's blocks (the last
 * window stops at block iicc).  Running every list once per window and
 * reading each window out assembles the whole matrix; acf is complete after
 * the last window.  dbsrg_set_window zeroes the window. */
int dbsrg_alloc_matrix_window(dbsrg_ctx *ctx, int nch, const int *icc,
                              int iicc, int mk, int nwin);
int dbsrg_set_window(dbsrg_ctx *ctx, int blo);
/* Number of blocks dbsrg_get_matrix returns for the current window. */
int dbsrg_window_blocks(const dbsrg_ctx *ctx);

int dbsrg_set_precision(dbsrg_ctx *ctx, int precision);

/* Drop-in for Gen_matrix(itype,kpol) (gen_matrix.f90:2-17): processes one
 * coefficient list exactly as Add_matrix leaves it (MOD_c_data.f90:318-
 * 368): entries ipt(1:ncdata) index the arrays k1..k4, cdata, sorted by
 * (K1,K2,K3,K4).  ipt may be NULL for the identity order.
 *   icase 0: overlaps O_data (O_data.f90:2-90), itypes 1-4
 *   icase 1: one-electron L_data (L_data.f90:2-145), itypes 1-3; needs
 *            dbsrg_set_dhl
 *   icase 2: R^k R_data (R_data.f90:2-290), itypes 1-4, all four atypes
 *   icase 3: S^k S_data (S_data.f90:2-287), ktype = 10*atype + itype,
 *            itypes 1-9
 * Adds into hch and acf, and into the perturber parts hcp/hp
 * (dbsrg_alloc_perturbers) and the target matrices htarg/otarg
 * (dbsrg_set_targets) where the structure updates them.  The perturber
 * and target terms of a list are added when the current window holds
 * block 1 (always without windows).  Entries the reference would stop on
 * (an index out of range, a perturber term without perturbers, an unknown
 * structure) give DBSRG_ERANGE / DBSRG_EINVAL and nothing of the list is
 * added.  k4 may be NULL (all zero) except for the structures that read it
 * (R and S itype 1 and 2, L itype 1). */
int dbsrg_gen_matrix(dbsrg_ctx *ctx, int icase, int itype, int kpol,
                     int ncdata, const int *ipt, const int *k1,
                     const int *k2, const int *k3, const int *k4,
                     const double *cdata);

/* One coefficient list, as for dbsrg_gen_matrix. */
typedef struct dbsrg_list {
  int icase, itype, kpol, ncdata;
  const int *ipt, *k1, *k2, *k3, *k4;
  const double *cdata;
} dbsrg_list;

/* A batch of independent symmetry blocks (J-parity partial waves), one
 * context each with its own grid, orbitals and matrix: context i's lists
 * are lists[sum(nlists[0..i-1]) ... + nlists[i] - 1], processed in order as
 * by dbsrg_gen_matrix; the contexts run concurrently (one host thread and
 * one CUDA stream each).  Returns the first nonzero status by context
 * index; dbsrg_last_error of that context holds the message.  No
 * counterpart in DBSR_MAT3, which runs one partial wave per process. */
int dbsrg_gen_batch(int nctx, dbsrg_ctx *const *ctxs, const int *nlists,
                    const dbsrg_list *lists);

/* The batch with streamed output, for symmetry blocks whose matrices do not
 * fit in device memory together (or alone): every context holds a window
 * (dbsrg_alloc_matrix_window) and runs its lists once per window, windows
 * in block order; after each window fn(user, i, blo, nblocks, window) gets
 * context i's blocks blo .. blo+nblocks-1 on the device (window: the first
 * of them, ms x ms each, in the hch layout) and may read them (with
 * dbsrg_get_matrix or its own copies) before it returns, when the window is
 * reused.  fn runs on the context's host thread, concurrently for different
 * contexts.  Every list is set up once (segments, chunks per window) and
 * executed window by window.  The windows and acf start from zero; acf is
 * complete at the end.  Returns as dbsrg_gen_batch. */
typedef void (*dbsrg_window_fn)(void *user, int ictx, int blo, int nblocks,
                                const double *window);
int dbsrg_gen_batch_streamed(int nctx, dbsrg_ctx *const *ctxs,
                             const int *nlists, const dbsrg_list *lists,
                             dbsrg_window_fn fn, void *user);

/* The whole assembly of one context straight into a caller's matrix
 * hch_host(ms,ms,iicc) (host, best pinned, or device) and acf_host
 * (iicc,0:mk) (may be NULL): the lists run once per window of at most
 * nwin blocks (nwin <= 0: from the tuned window count; every list is set up
 * once, its work split by window), windows alternating between two halves
 * of the device allocation, and while one window is assembled the previous
 * one is copied out on a separate stream, so the copy hides behind the
 * assembly.  With more than two windows' worth of blocks the first and the
 * last window hold max(1, nwin/8) blocks: the first window's assembly and
 * the last window's copy are what nothing overlaps.
 * The allocation must hold two windows (or nwin >= iicc).  The device
 * matrix is overwritten; acf, and the perturber and target parts when
 * held, are zeroed first and hold the list's terms at the end (read them
 * with dbsrg_get_acf / dbsrg_get_perturbers / dbsrg_get_targets).  Lists
 * are as for dbsrg_gen_batch (one context). */
int dbsrg_assemble_to_host(dbsrg_ctx *ctx, int nlists, const dbsrg_list *lists,
                           int nwin, double *hch_host, double *acf_host);

/* The same assembly streamed through a caller's staging area instead of a
 * whole host matrix, for matrices larger than the host memory set aside
 * for them: stage holds two windows (2*nwin blocks of ms x ms; one window
 * when nwin >= iicc), host memory (pinned, for the overlap) or device
 * memory.  Window w is copied into half w % 2 of stage while window w+1 is
 * assembled; once that copy is complete, fn(user, 0, blo, nblocks, half)
 * runs on the calling thread with the window's blocks blo .. blo+nblocks-1
 * (hch layout) and may read them until it returns, the device meanwhile
 * assembling the next window.  Windows, their sizes (first and last
 * window short), nwin <= 0, the allocation rule, acf_host and the zeroed
 * parts are as for dbsrg_assemble_to_host.  No counterpart in DBSR_MAT3,
 * which holds the whole matrix (updates.f90:2-76) and writes it with
 * Record_matrix. */
int dbsrg_assemble_streamed_host(dbsrg_ctx *ctx, int nlists,
                                 const dbsrg_list *lists, int nwin,
                                 double *stage, dbsrg_window_fn fn,
                                 void *user, double *acf_host);

/* A whole assembly captured as one CUDA graph, for matrices rebuilt many
 * times from the same lists with new orbitals (SCF iterations, scans over
 * orbital parameters).  dbsrg_graph_capture plans every list (segments and
 * chunks, which read the lists back to the host), drops the cached tables,
 * captures the zeroing of the matrix, acf and the perturber and target
 * parts, every table, pair-potential and digit build and every
 * contraction and scatter into one graph, and runs it once: the matrix
 * then equals the one dbsrg_gen_matrix gives for the same lists.  The
 * lists' arrays are read during the call only.  dbsrg_graph_launch(ctx,
 * pq) runs the graph again, after copying pq(ns,2,nbf) (host or device,
 * the orbitals' count and ipbs unchanged; NULL: the orbitals held) into
 * the context: every table and orbital product is rebuilt and the matrix
 * assembled anew, equal to what dbsrg_set_orbitals and dbsrg_gen_matrix
 * would give.  A replay repeats the capture's precision, tuning and
 * matrix parts.  The whole matrix must be allocated (no window).  The
 * graph is dropped by dbsrg_graph_release and by every call that frees
 * or replaces memory it names: dbsrg_set_orbitals, dbsrg_alloc_matrix*,
 * dbsrg_alloc_perturbers, dbsrg_set_targets, dbsrg_set_dhl,
 * dbsrg_invalidate_tables, dbsrg_release_tables, dbsrg_destroy; after
 * that dbsrg_graph_launch returns DBSRG_ESTATE.  No counterpart in
 * DBSR_MAT3, which builds each matrix once. */
int dbsrg_graph_capture(dbsrg_ctx *ctx, int nlists, const dbsrg_list *lists);
int dbsrg_graph_launch(dbsrg_ctx *ctx, const double *pq);
int dbsrg_graph_release(dbsrg_ctx *ctx);

/* Page-locked host memory for a matrix that the device writes (the hch_host
 * of dbsrg_assemble_to_host, the stage of dbsrg_assemble_streamed_host):
 * an anonymous mapping aligned to the kernel's transparent huge page size
 * with huge pages requested, zeroed by several host threads and registered
 * with the CUDA driver.  Copies from the device into 64 KB pages of a
 * matrix of tens of GB ran at two speeds from one run to the next; into
 * huge pages they run at the link's rate.  *out receives the address;
 * DBSRG_ENOMEM when the mapping or the registration fails.  Free with
 * dbsrg_host_free.  No counterpart in DBSR_MAT3. */
int dbsrg_host_alloc(size_t bytes, void **out);
int dbsrg_host_free(void *p);

/* UPDATE_HX(ich,jch,d,C) (updates.f90:79-106): add C*d (d is ms x ms,
 * host or device) to the block of channel pair (ich,jch). */
int dbsrg_update_hx(dbsrg_ctx *ctx, int ich, int jch, const double *d,
                    double c);
/* UPDATE_HW(ich,jch,v,w,C) (updates.f90:183-216): the rank-1 term C v w^T
 * (v, w of length ms, host or device) into the block of (ich,jch),
 * transposed for ich < jch and symmetrised with C/2 for ich = jch. */
int dbsrg_update_hw(dbsrg_ctx *ctx, int ich, int jch, const double *v,
                    const double *w, double c);
/* UPDATE_HV(ich,ip,v,C) (updates.f90:220-242): C v into the channel-
 * perturber vector hcp(:,icb(ich,ip)).  UPDATE_HB(ic,jc,C) (:245-264): C
 * into the perturber scalar hp(ibb(ic,jc)). */
int dbsrg_update_hv(dbsrg_ctx *ctx, int ich, int ip, const double *v,
                    double c);
int dbsrg_update_hb(dbsrg_ctx *ctx, int ic, int jc, double c);

/* Perturber part of the matrix (Alloc_dbsr_matrix, updates.f90:47-72):
 * hcp(ms,iicb) channel-perturber vectors numbered by icb(nch,npert) and
 * hp(iibb) perturber-perturber scalars numbered by ibb(npert,npert)
 * (1-based, 0 = not held; host or device arrays), on the device, zeroed
 * here and by dbsrg_zero_matrix.  npert = 0 frees them.  A new
 * dbsrg_alloc_matrix drops them.  dbsrg_get_perturbers copies them out
 * (either pointer may be NULL). */
int dbsrg_alloc_perturbers(dbsrg_ctx *ctx, int npert, const int *icb,
                           int iicb, const int *ibb, int iibb);
int dbsrg_get_perturbers(dbsrg_ctx *ctx, double *hcp, double *hp);

/* Target interaction and overlap matrices of Target_h (target_subs.f90:
 * 2-31): htarg and otarg of ntarg(ntarg+1)/2 elements, iptar(nch) the
 * target of each channel, and the switches iitar (UPDATE_HX of the target
 * structures for iitar > 0 or > 1, as R/S/L_data and O_data test them) and
 * check_target (L_data itype 3) of mod_dbsr_mat.f90:72-76 (defaults 0 and
 * 1).  Zeroed here and by dbsrg_zero_matrix; a new dbsrg_alloc_matrix drops
 * them.  Without targets (ntarg = 0, the default) Target_h adds nothing. */
int dbsrg_set_targets(dbsrg_ctx *ctx, int ntarg, const int *iptar, int iitar,
                      int check_target);
int dbsrg_get_targets(dbsrg_ctx *ctx, double *htarg, double *otarg);

/* One-electron Dirac matrices for L_data (module dhl_core of the external
 * library, Gen_dhl_core sub1.f90:23): hd(ms,ms,nkap) for the kappas
 * kap_list(nkap), and kbs(nbf) the kappa of every orbital of
 * dbsrg_set_orbitals (call it after that).  L_data's Lval(i,j) is taken as
 * p_i^T hd(kappa_i) p_j and Gen_Lvec(i) as hd(kappa_i) p_i with p = (P; Q),
 * and itype 3 adds hd(kappa) itself. */
int dbsrg_set_dhl(dbsrg_ctx *ctx, int nkap, const int *kap_list,
                  const double *hd, const int *kbs);
/* hch (the current window), hcp and hp multiplied by s: the core-energy
 * shifts of SUB1 between the overlap and the Hamiltonian passes
 * (sub1.f90:96, 222-223, hch = hch * Ecore and the same for hcp, hp). */
int dbsrg_scale_matrix(dbsrg_ctx *ctx, double s);
/* eps_c of the O and L lists (mod_dbsr_mat.f90:50, default 1e-10):
 * coefficients below it are skipped (O_data.f90:35, L_data.f90:48). */
int dbsrg_set_eps_c(dbsrg_ctx *ctx, double eps_c);

/* Energy functional and its gradient (the SCF potentials of DBSR_HF /
 * DBSR_MCHF, hf_matrix.f90:2-163): E = sum_e coef[e] *
 * R^k[e](i1[e], i2[e]; i3[e], i4[e]) with R^k as rk (dbsr_lib_dbs.f90:
 * 3981-4022) over the orbitals of dbsrg_set_orbitals (1-based, bound:
 * ipbs = 0), and, when grad != NULL, dE/dpq in the layout pq(ns,2,nbf)
 * (zero for orbitals that appear in no entry).  Host or device arrays;
 * *energy is written on the host.  No counterpart in DBSR_MAT3 itself: the
 * backward of the assembly's R^k contraction. */
int dbsrg_backward(dbsrg_ctx *ctx, int n, const int *k, const int *i1,
                   const int *i2, const int *i3, const int *i4,
                   const double *coef, double *energy, double *grad);

/* Copies of results (host or device destination).  With a window, the
 * block of dbsrg_get_block must lie in it and dbsrg_get_matrix copies the
 * window's blocks. */
int dbsrg_get_block(dbsrg_ctx *ctx, int ich, int jch, double *out);
int dbsrg_get_matrix(dbsrg_ctx *ctx, double *hch);
int dbsrg_get_acf(dbsrg_ctx *ctx, double *acf);
/* Device pointer to hch, the window's first block (valid until the next
 * alloc/destroy). */
int dbsrg_matrix_device_ptr(dbsrg_ctx *ctx, double **hch_dev);

/* The channel basis of the write-out, on the
 * device-resident whole matrix (no window).
 * dbsrg_diag_channels -- Diag_channels (diag.f90:2-81): for every channel
 * ich with a diagonal block, the generalized problem H c = E B c on the
 * B-splines kept by the zero conditions (iprm(j,ich) != 0, j = 1..ms,
 * zero_cond.f90), H the current diagonal block of hch and B = bdiag(:,:,ich)
 * (the overlap diagonal blocks, ms x ms x nch, host or device); the
 * solutions with emin <= E <= emax and |E| >= egap, ascending, restored to
 * the full net with their largest component positive, go to
 * sol(:, 1:nsol(ich), ich) (ms x ms x nch, host or device; the rest zero),
 * their energies to eval(1:nsol(ich), ich) (ms x nch).  iprm, eval and nsol
 * are host arrays.
 * dbsrg_channel_basis -- the block transformation of Record_matrix
 * (record_matrix.f90:14-26): every block of a channel pair ich > jch becomes
 * c = D_ich^T H D_jch (nsol(ich) x nsol(jch) in its top-left corner, zero
 * elsewhere; D = sol), in place; diagonal blocks stay.  out, when not NULL,
 * receives a copy of the transformed hch.  In the split form
 * (DBSRG_SPLIT_BF16) the products are split-BF16 tensor-core products
 * (within 1e-10 of each block's largest element), in the FP64 forms cuBLAS
 * DGEMM.  Both load cuSOLVER and cuBLAS on first use. */
int dbsrg_diag_channels(dbsrg_ctx *ctx, const double *bdiag, const int *iprm,
                        double emin, double emax, double egap, double *sol,
                        double *eval, int *nsol);
int dbsrg_channel_basis(dbsrg_ctx *ctx, const double *sol, const int *nsol,
                        double *out);

/* The dbsr_mat.nnn write-out, as Fortran sequential unformatted records
 * (gfortran's layout: a 4-byte record length before and after each record,
 * machine byte order).
 * dbsrg_record_header -- SUB1's records after Diag_channels
 * (sub1.f90:164-168), written to a new file at path (truncated, as the
 * rewind of nui does): (ns, nch, npert, nsp, nsq), (nsol), (jpsol(0:nch)),
 * (eval(1:nsol)), (diag(1:ms, 1:ipsol(ich), ich) of every channel); sol,
 * eval and nsol as dbsrg_diag_channels returns them (eval, nsol host).
 * dbsrg_record_matrix -- Record_matrix (record_matrix.f90:2-60), appended
 * to path: (ich, jch) and c = D_ich^T H D_jch (nsol(ich) x nsol(jch)) for
 * every channel pair ich > jch whose block has an element of at least
 * 1e-20 (the test on the block before the transformation), (nch+ip, ich)
 * and D_ich^T hcp(:,k) for every such channel-perturber vector,
 * (nch+ip, nch+jp) and hp(k) for every nonzero perturber element, then
 * (0, 0).  With icase = 0 and overlaps != NULL (host, (nch+npert)^2,
 * column-major) the largest modulus of each written record goes to
 * overlaps(ich, jch), overlaps(nch+ip, ich), overlaps(nch+ip, nch+jp)
 * (the input of Check_mat); other elements are left as they are.  The
 * blocks are transformed in place on the device (dbsrg_channel_basis):
 * hch holds the transformed blocks afterwards.
 * dbsrg_record_acf -- the closing records (mk) and (bcf(nch,nch,0:mk))
 * (sub1.f90:286-287), appended; bcf (host) as SUB1 collects it.
 * A file that cannot be opened or written gives DBSRG_EIO. */
int dbsrg_record_header(dbsrg_ctx *ctx, const char *path, int nsp, int nsq,
                        const double *sol, const double *eval, const int *nsol);
int dbsrg_record_matrix(dbsrg_ctx *ctx, const double *sol, const int *nsol,
                        int icase, const char *path, double *overlaps);
int dbsrg_record_acf(dbsrg_ctx *ctx, const char *path, const double *bcf);

/* Orthogonality of the channels to bound orbitals,
 * in place on the device-resident whole matrix: DBS_ORTH
 * (DBSR_MAT3/dbs_orth.f90:2-84), Bentley's projection
 *     H(ich,jch) -> (1 - A_ich) H(ich,jch) (1 - A_jch^T),
 *     A_c = sum_{j: iort(j,c) != 0} (B v_j) v_j^T,
 * v_j = (P_j; Q_j) from the orbitals of dbsrg_set_orbitals and B the
 * B-spline overlap blockdiag(fpbs, fqbs) (Get_pv/Get_qv, bpq of
 * read_data.f90:144-145).  iort(nbf,nch) (host, Fortran order): nonzero
 * where channel ich is made orthogonal to orbital j -- the reference's
 * selection is ipbs(j) = 0, kbs(j) = kbs(ipch(ich)) and IBORT = 0
 * (dbs_orth.f90:39-43).  Orbitals with ipbs != 0 give DBSRG_EINVAL, more
 * than 32 orbitals for one channel DBSRG_ERANGE.  Channel-perturber blocks
 * (hcp) are not held by this library. */
int dbsrg_orth_channels(dbsrg_ctx *ctx, const int *iort);

/* SCF potential matrix of one orbital: DBSR_HF's
 * hf_matrix (hf_matrix.f90:2-70; the Breit part of hf_matrix_breit when
 * dbsrg_hf_breit_list holds entries)
 *   hfm = (qsum dhl + sum_{ii,jj,k} [direct + exchange]) / qsum
 * for orbital iorb (1-based) of dbsrg_set_orbitals, with a(nbf,0:kmax) and
 * b(nbf,0:kmax) (host, Fortran order) the values of the energy
 * expression's a(iorb,j,k) and b(iorb,j,k) (hf_MOD_energy.f90:20-57), dhl
 * the one-electron matrix (ms x ms, MAT_dhl_pq, host or device) or NULL,
 * and hfm (ms x ms, host or device) the result.  The context must hold a
 * one-channel matrix (dbsrg_alloc_matrix with nch = iicc = 1, mk >= kmax);
 * it is the work area and is overwritten.  Runs in the precision the
 * context selected.  2 qsum hfm p_iorb (without dhl) is the gradient of the
 * two-electron energy with respect to p_iorb, the quantity dbsrg_backward
 * returns for the same energy. */
int dbsrg_hf_matrix(dbsrg_ctx *ctx, int iorb, int kmax, const double *a,
                    const double *b, double qsum, const double *dhl,
                    double *hfm);
/* The Breit part of dbsrg_hf_matrix (hf_matrix_breit, hf_matrix.f90:91-163,
 * DBSR_HF's mbreit = 2): the rk4 entries of the Breit energy (module
 * rk4_data, dbsr_lib_zcom.f90:2984-3003) -- kr1 = k + 1000*itype (itype 0
 * S^k ppqq, 1 pqqp), kr2 = int 1..4, kr3, kr4 orbitals (1-based), crk the
 * coefficient; host arrays, copied.  Every later dbsrg_hf_matrix adds, per
 * itype, k <= kmax and int, convol_sk case int of the coefficient-weighted
 * densities of the orbital's partners into its quadrant, before the
 * division by qsum.  As in the reference, the exchange forms int 3 and 4
 * add nothing: hf_matrix_breit hands convol_sk the storage 'x','x', which
 * convol_sk does not contract (dbsr_lib_dbs.f90:2610-2700).  nrk = 0
 * removes the Breit part. */
int dbsrg_hf_breit_list(dbsrg_ctx *ctx, int nrk, const int *kr1,
                        const int *kr2, const int *kr3, const int *kr4,
                        const double *crk);

/* DBSR_MCHF's SCF potential matrices on a one-channel matrix (as for
 * dbsrg_hf_matrix), in the precision form selected.
 * dbsrg_mchf_matrix -- mchf_matrix (DBSR_MCHF/mchf_matrix.f90:2-251) of
 * orbital iorb outside the core: the one-electron entries (li1, li2, lc;
 * nl of them) and the R^k entries (rk, ri1..ri4, rcoef; nr) with the
 * expansion weights already applied (WW(ic,jc) L_coef and WW(ic,jc)
 * Rk_coef, mchf_matrix.f90:65, 95), k ascending; dhl (ms x ms) the
 * one-electron matrix of Get_hd_core; irhs, newton and eps_c as in the
 * reference.  Out: hfm (ms x ms), rhs (ms), hx (ms x ms, written when
 * newton != 0), e = e(i) and qsum = qsum(i) (host scalars).  The
 * Add_id4_data classification (mchf_matrix.f90:98-135) is applied with
 * entries appended in order; the Newton term convolves the last -3 density
 * of each k unweighted, as the reference's Convol(ns,ks,xx,x,4,..) does.
 * dbsrg_mchf_core -- core_matrix (mchf_matrix.f90:255-346) of a core
 * orbital: a, b (nbf x (kmax+1), host) the angular coefficients a(i,j,k),
 * b(i,j,k), qsum (nbf, host), hd (ms x ms) of Get_hd; out hfm and, when
 * newton != 0, hx.
 * Lists, e and qsum are host arrays; dhl/hd and the outputs host or device. */
int dbsrg_mchf_matrix(dbsrg_ctx *ctx, int iorb, int kmax, int nl, const int *li1,
                      const int *li2, const double *lc, int nr, const int *rk,
                      const int *ri1, const int *ri2, const int *ri3, const int *ri4,
                      const double *rcoef, const double *dhl, int irhs, int newton,
                      double eps_c, double *hfm, double *rhs, double *hx, double *e,
                      double *qsum);
int dbsrg_mchf_core(dbsrg_ctx *ctx, int iorb, int kmax, const double *a, const double *b,
                    const double *qsum, const double *hd, int newton, double *hfm,
                    double *hx);

/* List producer between the decoded angular bank and Gen_matrix (the part
 * after the bank's records are read; the records, state tables and overlap
 * factors of State_res / Det_fact come from the caller).  Replaces Add_integral (add_integral.f90:2-57: parity filter,
 * Breit expansion over v = k-1..k+1 by SMU, hf_energy_BR.f90:58-121), the
 * classification Idef_Otype/Ltype/Rtype/itype (idef_type.f90:1-437) and the
 * sorted, merged lists of Add_coef/Add_cdata/Merge_cdata/Add_matrix
 * (MOD_c_data.f90:117-368): coefficients are appended in arrival order and
 * each (kpol, itype) list is sorted once by (K1,K2,K3,K4) on host threads,
 * equal keys summed in arrival order, sums with |c| <= eps_c dropped,
 * instead of the reference's insertion by binary search and shifting.
 * icase 0 (O), 1 (L), 2 (R), 3 (S) as DBSR_MAT3's icase; ipbs, lbs (l of each
 * orbital, icase 2) and kbs (kappa, icase 3) are nbf host arrays; mk the
 * largest multipole; eps_c and check_target as in mod_dbsr_mat.f90 (1e-10,
 * 1).  Host code only; no device is needed except by
 * dbsrg_lists_gen_matrix. */
typedef struct dbsrg_lists dbsrg_lists;
int dbsrg_lists_create(dbsrg_lists **lists, int icase, int nbf,
                       const int *ipbs, const int *lbs, const int *kbs,
                       int mk, double eps_c, int check_target);
int dbsrg_lists_destroy(dbsrg_lists *lists);
/* The integral code of a bank record (state_res.f90:83-96): jcase (2 bits),
 * kpol (10), and the positions i4, i3, i2, i1 (5 bits each) from the
 * bottom. */
int dbsrg_lists_decode(int n, const int *code, int *jcase, int *kpol,
                       int *i1, int *i2, int *i3, int *i4);
/* Add_integral for n coefficients: multipole kpol, orbitals i1..i4
 * (1-based), coefficient c, and the reference's ic, jc, io, jo. */
int dbsrg_lists_add(dbsrg_lists *lists, int n, const int *kpol, const int *i1,
                    const int *i2, const int *i3, const int *i4,
                    const double *c, const int *ic, const int *jc,
                    const int *io, const int *jo);
/* Length of the merged list (kpol, itype), and its entries in
 * (K1,K2,K3,K4) order (host arrays of that length). */
int dbsrg_lists_count(dbsrg_lists *lists, int kpol, int itype);
int dbsrg_lists_get(dbsrg_lists *lists, int kpol, int itype, int *k1,
                    int *k2, int *k3, int *k4, double *cdata);
/* Add_matrix for every non-empty list, kpol outer and itype inner as
 * State_res calls it (state_res.f90:187-191): dbsrg_gen_matrix on ctx. */
int dbsrg_lists_gen_matrix(dbsrg_lists *lists, dbsrg_ctx *ctx);

/* One assembled B-spline integral table, in the reference layout
 * rkb(ns,ns,ks,ks) for R (type 0 pppp,1 qqqq,2 pqpq,3 qpqp; mrk_*,
 * dbsr_lib_dbs.f90:2898-3492) or rkb(ns,ns,2ks-1,2ks-1) for S (type 0
 * ppqq, 1 pqqp; msk_*, :3601-3833). */
int dbsrg_get_table(dbsrg_ctx *ctx, int family, int type, int k,
                    double *out);
/* Cell moments (moment_pp/qq/pq/qp, :1401-1564) as rkm(ks*ks,nv) and
 * diagonal-cell integrals (triang_*, :2979-3936) as rkd(ks*ks,ks*ks,nv). */
int dbsrg_get_moments(dbsrg_ctx *ctx, int which, int k, double *out);
int dbsrg_get_diag_cells(dbsrg_ctx *ctx, int type, int k, double *out);
/* Grid arrays: name is one of "gr","grw","grm","pbsp","qbsp","pbsd",
 * "qbsd","fpbs","fqbs","fppqq" (reference shapes). */
int dbsrg_get_grid_array(dbsrg_ctx *ctx, const char *name, double *out);

/* Free the cached R^k/S^k tables and everything derived from them (cell
 * data, far fields, pair potentials), returning the memory to the device
 * (the reference keeps its tables for the whole run,
 * dbsr_lib_dbs.f90:1595-1624). */
int dbsrg_release_tables(dbsrg_ctx *ctx);
/* Mark the same caches stale: the next assembly rebuilds every table in
 * the memory they occupied (no reference counterpart). */
int dbsrg_invalidate_tables(dbsrg_ctx *ctx);

/* Number of this library's kernels launched by the context so far. */
long long dbsrg_kernel_launches(const dbsrg_ctx *ctx);
/* Wait for every queued kernel of the context and report a failure of any
 * of them (DBSRG_ETIMEOUT: a bounded wait of a tensor-core kernel ran out). */
int dbsrg_sync(dbsrg_ctx *ctx);

/* Tuning parameters (no reference counterpart), picked per device and grid
 * size by dbsr_gb300/autotune.py:
 *   "xchunk"  segments per pass of the factored exchange (default 256; the
 *             batch of the Z-digit and tensor-core exchange kernels)
 *   "dchunk"  segments per pass of the factored direct contraction (4096)
 *   "windows" windows of dbsrg_assemble_to_host when nwin <= 0 (8)
 * Results do not depend on them (every block sums the same terms in the
 * same order). */
int dbsrg_set_tuning(dbsrg_ctx *ctx, const char *name, int value);
int dbsrg_get_tuning(const dbsrg_ctx *ctx, const char *name, int *value);

/* Failure detection of the tensor-core exchange: every wait of its
 * pipeline gives up after a limit (2 s by default; 1 us .. 60 s here), the
 * kernel then drains its own copies and MMAs, frees its TMEM and returns,
 * and the call reports DBSRG_ETIMEOUT with the context usable.
 * dbsrg_inject_wait_timeout(ctx, 1) makes the epilogue warps first wait on a
 * barrier that nothing completes (a test of that path, no reference
 * counterpart). */
int dbsrg_set_wait_limit(dbsrg_ctx *ctx, long long ns);
int dbsrg_inject_wait_timeout(dbsrg_ctx *ctx, int enable);

/* Asynchronous mode (off by default; no reference counterpart -- Gen_matrix
 * returns with the matrix updated, gen_matrix.f90:2-17).  When on,
 * dbsrg_gen_matrix returns once the list's kernels are queued: the host-side
 * set-up of the next R/S list (segments, chunks, quadrant records) then
 * overlaps the kernels of this one.  The lists may be reused or freed on
 * return (they are copied during the call).  A failure of a queued kernel is
 * reported by the next call that waits: dbsrg_sync, the read-outs
 * (dbsrg_get_*), dbsrg_matrix_device_ptr and the state changes
 * (dbsrg_set_orbitals, dbsrg_alloc_matrix, dbsrg_zero_matrix,
 * dbsrg_set_precision, dbsrg_update_hx, dbsrg_release_tables, dbsrg_backward).
 * dbsrg_gen_batch pipelines every context this way and waits at its end. */
int dbsrg_set_async(dbsrg_ctx *ctx, int enable);

/* Per-kernel device timing (no reference counterpart; it replaces the
 * CPU_time counters time_convol/time_density of dbsr_lib_dbs.f90:1106-1116
 * and t_rdata/t_sdata of mod_dbsr_mat.f90:114).  enable=1 clears the record
 * and brackets every kernel launch with CUDA events on the context stream;
 * dbsrg_timing_report writes a JSON object {"kernel": [launches, ms], ...}
 * into buf (synchronising the stream first). */
int dbsrg_timing(dbsrg_ctx *ctx, int enable);
int dbsrg_timing_report(dbsrg_ctx *ctx, char *buf, size_t len);

/* Allocation-free exchange contraction of one channel-pair segment.  This
 * entry point has no counterpart in the reference; it exists for callers
 * that cannot call cudaMalloc: MPI ranks that share one GPU under a device
 * memory split agreed at start-up, host programs whose device memory is
 * owned by another allocator (a pool reserved up front), and loops that
 * cannot afford the device-wide synchronisation an allocation or free may
 * bring.  It needs no context.
 *
 * For the n list entries (k2,k3,cdata) of one segment it forms the 'x'
 * density xx = sum_e cdata(e)*pq(:,jp1,k2(e)) pq(:,jp2,k3(e))^T and writes
 * out(ns,ns) = convol(xx, case 3, 's','s') with the R^k table rkb
 * (ns,ns,ks,ks) -- the block R_data adds for itype 4 (R_data.f90:250-262).
 * All pointers are device pointers owned by the caller; stream may be NULL.
 * The density lives in a fixed static device array: ns is limited to 512
 * (larger ns returns DBSRG_ERANGE, as do orbital indices outside 1..nbf).
 * The array is shared by all calls on a device: calls that overlap on the
 * GPU race and must be ordered by the caller.  The first call on a device
 * sets up the array's address (cudaGetSymbolAddress); that address belongs
 * to the device's context of the moment, so the entry point must not be
 * used after a cudaDeviceReset of the device in the same process.  The call is synchronous: it waits on
 * its stream for its own kernels and the read-back of its error word. */
int dbsrg_exchange_segment_noalloc(int ns, int ks, const double *rkb,
                                   const double *pq, int nbf, int jp1,
                                   int jp2, int n, const int *k2,
                                   const int *k3, const double *cdata,
                                   double *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif
