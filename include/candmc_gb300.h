/*
 * candmc_gb300.h -- C ABI of the GB300 (sm_103a) implementation of CANDMC's
 * QR hot path: binary-tree TSQR, Householder reconstruction (TSQR-HR) and the
 * CAQR trailing update A -= Y*T^T*(Y^T*A).
 *
 * Every function returns a status code (CANDMC_OK on success) and never
 * throws.  Matrices are column-major float64 with a leading dimension, as in
 * the reference.  Functions without a suffix take DEVICE pointers and run on
 * the given CUDA stream (a cudaStream_t passed as void*, NULL = legacy default
 * stream); they return once the work is enqueued.  Functions with the _host
 * suffix take HOST pointers, copy in, compute and copy out, and return after
 * the result is on the host.
 *
 * The reference's process grid (CommData_t / pview) collapses to one GPU: the
 * entry points below are the reference functions at numPes == 1 (a 1 x 1
 * grid), with the MPI arguments dropped.  The C++ drop-in with the reference's
 * exact signatures (include/candmc/*.h) sits on top of these.
 */
#ifndef CANDMC_GB300_H
#define CANDMC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define CANDMC_OK 0
#define CANDMC_ERR_ARG 1      /* invalid size, leading dimension or pointer */
#define CANDMC_ERR_ALLOC 2    /* device or host allocation failed */
#define CANDMC_ERR_CUDA 3     /* a CUDA runtime call or kernel launch failed */
#define CANDMC_ERR_TIMEOUT 4  /* a bounded device-side wait ran out */
#define CANDMC_ERR_NUMERIC 5  /* non-finite value or zero pivot detected */
#define CANDMC_ERR_NODEV 6    /* no usable sm_103 device */

/* arithmetic forms of the trailing-update contractions */
#define CANDMC_PREC_FP64 0    /* plain FP64 (SIMT DFMA) */
#define CANDMC_PREC_OZAKI 1   /* emulated FP64: BF16 Ozaki slices on tcgen05, FP32 accumulation */
#define CANDMC_PREC_FP32 2    /* FP32 contraction (inputs rounded to FP32) */

const char* candmc_status_string(int status);
int candmc_version(void);
/* last CUDA error text recorded by a failing call (thread-local) */
const char* candmc_last_error(void);

/* ---- launch accounting (no counterpart in the reference, which times phases
 * with CTF timers, alg/shared/timer.h:21-35) ---------------------------------
 * candmc_launch_count: kernels this library has launched since load.
 * candmc_profile_begin(mask): from now on, bracket every launch of a kernel
 * class whose bit is set in mask with CUDA events on its launching stream.
 * candmc_profile_end: synchronises those events, writes per class (index <
 * ncls) the summed kernel milliseconds, the summed algorithmic work (flops
 * for contractions, bytes for memory-bound kernels) and the launch count, and
 * stops recording. */
#define CANDMC_KCLASS_GEMM_TN 0     /* FP64 split-K Z = Y^T A partials */
#define CANDMC_KCLASS_GEMM_NN 1     /* FP64 A -= Y Z */
#define CANDMC_KCLASS_REDUCE 2      /* split-K reduction + T^T */
#define CANDMC_KCLASS_PANEL_LEAF 3  /* TSQR leaves + tree + reconstruction */
#define CANDMC_KCLASS_PANEL_Y 4     /* Y = Q_leaf * (chain * U^-1) */
#define CANDMC_KCLASS_SMALL 5       /* b x b products, inverses, copies */
#define CANDMC_KCLASS_OZ_SLICE 6    /* Ozaki: FP64 -> BF16 slices */
#define CANDMC_KCLASS_OZ_TN 7       /* Ozaki: Z = Y^T A on tcgen05 */
#define CANDMC_KCLASS_OZ_NN 8       /* Ozaki: A -= Y Z on tcgen05 */
#define CANDMC_KCLASS_F32 9         /* FP32-form contractions (3 BF16 slices on tcgen05) */
#define CANDMC_KCLASS_OZ_PANEL 10   /* emulated-FP64 contractions inside a panel (half-panel updates) */
long long candmc_launch_count(void);
int candmc_profile_begin(unsigned mask);
int candmc_profile_end(int ncls, double* ms, double* work, long long* launches);

/* ---- TSQR-HR panel ------------------------------------------------------
 * hh_recon_qr: alg/QR/hh_recon/hh_recon.h:66-75 (hh_recon.cxx:129-321).
 * In: A (m x b, lda >= m, m >= b >= 1).  Out: A = Y\(S*R) -- Y strictly below
 * the diagonal (unit diagonal implicit), S*R on and above it; W (b x b, ld b,
 * upper) = U*S = -T*Y1^T.  T (b x b, ld b, upper, nullable) receives the
 * compact-WY factor with Q = I - Y*T*Y^T.  Scratch is stream-ordered device
 * memory released before return.
 */
int candmc_hh_recon_qr(double* A, int64_t lda, int64_t m, int64_t b, double* W, double* T,
                       void* stream);
int candmc_hh_recon_qr_host(double* A, int64_t lda, int64_t m, int64_t b, double* W, double* T);

/* candmc_hh_recon_qr_noalloc: no counterpart in the reference.  The same
 * TSQR-HR as candmc_hh_recon_qr (same arguments; W and T required), for
 * callers that cannot let a library allocate device memory during their run,
 * e.g. a server that budgets all GPU memory at start-up or a framework whose
 * own allocator must own every device buffer.  It allocates nothing: its
 * scratch is a fixed array of about 3.7 MB inside the library, held on every
 * GPU that loads the library until exit.  Limits: 1 <= b <= 32 and
 * b <= m <= 8192; larger sizes return CANDMC_ERR_ARG.  All calls share that
 * array, so calls that overlap on the GPU race: serialize them.  The first
 * call on a device sets up that device (looks up the array's address, under
 * a mutex); make it before any stream capture begins.  A numeric failure in
 * the kernels (non-finite U^-1) is not reported by the return code: the call
 * does not read its device status back, so check W and T for non-finite
 * values where that matters. */
int candmc_hh_recon_qr_noalloc(double* A, int64_t lda, int64_t m, int64_t b, double* W, double* T,
                               void* stream);

/* bitree_tsqr at numPes == 1: alg/QR/tsqr/bitree_tsqr.h:58-70 (bitree_tsqr.cxx:91-248).
 * The single-rank tree is the leaf dgeqrf (bitree_tsqr.cxx:129-146): A becomes
 * the LAPACK-form Householder QR Y\R (when output_Y), R (b x b, ld b, zero
 * below the diagonal) and tau (b).  Computed by TSQR + reconstruction, so the
 * reflectors are LAPACK's up to rounding (the last one of a square panel is
 * the reconstruction's sign-choice reflector with tau = 2, as the reference's
 * own tests note, test/QR/test_qr_2d.cxx:135-138). */
int candmc_bitree_tsqr(double* A, int64_t lda, double* R, double* tau, int64_t m, int64_t b,
                       int output_Y, void* stream);

/* tree_tsqr: alg/QR/tsqr/bitree_tsqr.h:16-19 (bitree_tsqr.cxx:20-34, LAPACK
 * dtpqrt(b, b, b, min(b,16)) on the stacked [R1; R2]).  A (2b x b, ld 2b, device)
 * holds R1 over R2; only their upper triangles are read.  On return R1's upper
 * triangle holds R, R2's upper triangle holds the reflector block V (the
 * reflectors are [e_j; V(:,j)]), and every strictly-lower entry of A is as it
 * was.  T (nullable; min(b,16) x b, ld min(b,16)) receives dtpqrt's
 * block-diagonal factor: for each min(b,16)-wide group of columns, the upper
 * triangle of that group's compact-WY T; entries below it are not written.
 * The reference's buf workspace argument is not needed. */
int candmc_tree_tsqr(double* A, int64_t b, double* T, void* stream);

/* construct_Q1 at numPes == 1: alg/QR/tsqr/bitree_tsqr.h:91-104
 * (construct_tsqr_Q.cxx:87-108, dorgqr): Q1 (m x k, ld ldq) = first k columns
 * of Q = H_0...H_{b-1} from the reflectors in Y (lower part of a Y\R buffer)
 * and tau.  k <= b. */
int candmc_construct_Q1(const double* Y, int64_t ldy, const double* tau, double* Q1, int64_t ldq,
                        int64_t m, int64_t b, int64_t k, void* stream);

/* apply_tsqr_QT at numPes == 1: alg/QR/tsqr/bitree_tsqr.h:126-138
 * (apply_tsqr_QT.cxx:31-163 on one rank: dlarft + dlarfb, i.e. dormqr 'L','T').
 * B (m x k, ld ldb) <- Q^T B with Q = H_0...H_{b-1} from the reflectors in Y
 * (lower part of a Y\R buffer, m x b) and tau. */
int candmc_apply_tsqr_QT(const double* Y, int64_t ldy, const double* tau, double* B, int64_t ldb,
                         int64_t m, int64_t b, int64_t k, void* stream);

/* tau_recon: alg/shared/util.h:675-680 (util.cxx:437-466).  tau (ncol) from
 * the Householder vectors in Y (nrow x ncol, ld lda): tau_i = 2/(1 + ||y_i||^2),
 * the norm over column i's part given by structure -- 'R' all nrow rows, 'L'
 * rows below the diagonal (unit diagonal implicit), 'U' rows 0..i -- and 0 where
 * that gives 2 (an empty reflector), as the reference does.  Valid for the
 * exact reflectors of a Householder reconstruction (tau = 2/(y^T y)). */
int candmc_tau_recon(char structure, int64_t ncol, int64_t nrow, int64_t lda, const double* Y, double* tau,
                     void* stream);

/* compute_invT_from_W: alg/QR/hh_recon/hh_recon.h:13-15 (hh_recon.cxx:26-31).
 * invT (b x b, ld b) holds Y1 on entry and T^-T = -W^-T*Y1 on return. */
int candmc_compute_invT_from_W(const double* W, int64_t b, double* invT, void* stream);

/* signed_NLU / recursive_NLU: alg/QR/hh_recon/hh_recon.h:27-49
 * (hh_recon.cxx:43-110).  Sign-choice unpivoted LU of (A - S), S_ii =
 * -sign(A_ii); A (b x b, lda) becomes L\U, rows i of R (ldr) with S_ii = -1
 * are negated, signs (int64, b, device) receives S_ii.  Both compute the same
 * factorization (the recursion only reorders the arithmetic). */
int candmc_signed_NLU(double* A, double* R, int64_t b, int64_t lda, int64_t ldr, int64_t* signs,
                      void* stream);
int candmc_recursive_NLU(double* A, double* R, int64_t b, int64_t lda, int64_t ldr,
                         int64_t* signs, void* stream);

/* ---- T factor ------------------------------------------------------------
 * compute_invT_from_Y: alg/QR/qr_2d/qr_2d.h:25-31 (qr_2d.cxx:22-60).
 * T (ldt) = stril(Y^T*Y) with the diagonal halved = T^-T, Y explicit mb x b. */
int candmc_compute_invT_from_Y(const double* Y, int64_t ldy, double* T, int64_t ldt, int64_t mb,
                               int64_t b, void* stream);
/* rectangular form: alg/QR/qr_2d/qr_2d.h:47-56 (qr_2d.cxx:76-106): T = Y1^T*Y2 (b1 x b2). */
int candmc_compute_invT_from_Y2(const double* Y1, int64_t ldy1, const double* Y2, int64_t ldy2,
                                double* T, int64_t ldt, int64_t mb, int64_t b1, int64_t b2,
                                void* stream);

/* ---- CAQR trailing update -------------------------------------------------
 * upd_A: alg/QR/qr_2d/qr_2d.h:99-108 (qr_2d.cxx:224-282).
 * A (mb x kb, lda) <- (I - Y*T*Y^T)^T * A with Y explicit (mb x b, ldy: unit
 * diagonal and zeros above it stored, as update_A packs it).  W selects T as
 * in the reference: NULL -> T^-T from Y^T*Y; W_is_T == 0 -> W = -T*Y1^T;
 * W_is_T != 0 -> W holds T^-T (lower).  precision: CANDMC_PREC_*. */
int candmc_upd_A(const double* Y, int64_t ldy, double* A, int64_t lda, int64_t mb, int64_t kb,
                 int64_t b, const double* W, int W_is_T, int precision, void* stream);

/* update_A: alg/QR/qr_2d/qr_2d.h:74-85 (qr_2d.cxx:124-177).  Y is read from
 * a Y\R buffer (strict lower part; unit diagonal implied).  A is m x k.
 * aggreg_Y (nullable, lda_aY) receives the explicit Y (m x b). */
int candmc_update_A(const double* Y, int64_t ldy, double* A, int64_t lda, int64_t m, int64_t k,
                    int64_t b, const double* W, double* aggreg_Y, int64_t lda_aY, int W_is_T,
                    int precision, void* stream);

/* ---- full CAQR --------------------------------------------------------------
 * QR_2D: alg/QR/qr_2d/qr_2d.h:124-131 (qr_2d.cxx:299-363) on a 1 x 1 grid.
 * A (m x k, lda) becomes Y\R of all panels.  aggreg_Y (nullable, lda_aY)
 * receives the explicit Y of every panel.  precision: CANDMC_PREC_*. */
int candmc_QR_2D(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, double* aggreg_Y,
                 int64_t lda_aY, int precision, void* stream);
int candmc_QR_2D_host(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int precision);

/* QR_2D_2D: alg/QR/qr_2d/qr_2d.h:176-188 (qr_2d.cxx:772-897): two-level
 * blocking, b a multiple of b_sub; each b-wide block is factored by QR_2D with
 * panel width b_sub and the rest of the matrix is updated once per block with
 * the aggregated Y and T = (T^-T from Y^T*Y)^-T. */
int candmc_QR_2D_2D(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int64_t b_sub,
                    double* aggreg_Y, int64_t lda_aY, int precision, void* stream);

/* QR_2D_pipe: alg/QR/qr_2d/qr_2d.h:293-302 (qr_2d.cxx:378-635).  On one GPU
 * the lookahead pipeline computes the same factorization as QR_2D; the
 * lookahead is realised by stream ordering. */
int candmc_QR_2D_pipe(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int precision,
                      void* stream);

/* ---- Yamamoto's basis-kernel representation ----------------------------------
 * alg/QR/hh_recon/yamamoto.h:21-32, alg/QR/qr_2d/qr_y2d.h (qr_y2d.cxx:13-393),
 * device pointers.  The representation: Q^T = I + Qm W Qm^T with
 * Qm = [Q1 - S; Q2] (m x b) and W = (Q1 - S)^-1 S (b x b, ld b) for the first
 * b columns [Q1; Q2] of a TSQR basis and the sign choice S.  The returned
 * pair is the reference's up to the reference's own sign matrix S_ref
 * (Qm_ref = Qm S_ref, W_ref = S_ref W S_ref): it is built from the
 * Householder reconstruction with the basis whose S is the identity.
 * Qm W Qm^T, the updates and S*R are the reference's.
 *
 * Yamamoto: A (m x b, lda) becomes Y\(S*R) (Householder Y below the
 * diagonal); Qm (ldq >= m) and W are written. */
int candmc_Yamamoto(double* A, int64_t lda, double* Qm, int64_t ldq, int64_t m, int64_t b, double* W,
                    void* stream);

/* upd_Yamamoto_A (qr_y2d.h:79-99): A (mb x kb, lda) += Qm (W (Qm^T A)),
 * b <= 256 (<= 128 for the ozaki and fp32 forms). */
int candmc_upd_Yamamoto_A(const double* Qm, int64_t ldq, double* A, int64_t lda, int64_t mb, int64_t kb,
                          int64_t b, const double* W, int precision, void* stream);

/* aggregator::append (qr_y2d.h:30-43): appends the mb x b Qm at rows
 * [shift, shift + mb) and columns [n, n + b) of aQm (ld_aqm rows, ld_at
 * columns) and the block row [T (Qm^T aQm) aT, T] to aT (ld_at x ld_at).
 * The caller adds b to its n.  CANDMC_ERR_ARG if the block does not fit. */
int candmc_yamamoto_append(double* aQm, int64_t ld_aqm, double* aT, int64_t ld_at, int64_t n, int64_t shift,
                           int64_t mb, int64_t b, const double* Qm, int64_t ldq, const double* T, void* stream);

/* QR_Yamamoto_2D (qr_y2d.h:102-119) and QR_Yamamoto_2D_2D (qr_y2d.h:122-139)
 * on a 1 x 1 grid.  A (m x k) becomes Y\(S*R) of all panels; Y is the
 * Householder Y for either value of compute_Y.  aQm/aT (both null, or the
 * aggregator's buffers with *agg_n and *agg_shift its counters, updated on
 * return) receive the panels' representation as the reference's aggregator
 * does. */
int candmc_QR_Yamamoto_2D(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int compute_Y, double* aQm,
                          int64_t ld_aqm, double* aT, int64_t ld_at, int64_t* agg_n, int64_t* agg_shift,
                          int precision, void* stream);
int candmc_QR_Yamamoto_2D_2D(double* A, int64_t lda, int64_t m, int64_t k, int64_t b, int64_t b_sub,
                             int compute_Y, double* aQm, int64_t ld_aqm, double* aT, int64_t ld_at,
                             int64_t* agg_n, int64_t* agg_shift, int precision, void* stream);

/* ---- symmetric full -> band reduction: alg/SE/CANSE.h:17-22
 * (alg/SE/full_to_band.cxx:27-295), the eigensolver's caller of QR_2D_pipe and
 * compute_invT_from_Y, on a 1 x 1 grid.  A (n x n, ld lda, symmetric, stored
 * in full, as the reference stores it) becomes Q^T A Q in band form with
 * bandwidth b: for every
 * band step the (n - r0 - b) x b block below the band is factored by CAQR in
 * panels of b_sub (b a multiple of b_sub, b <= 256) and the trailing block
 * receives the two-sided update A22 -= U V' + (U V')^T (U = Y T^T,
 * V' = Y^T A22 - (Y^T A22 Y) U^T / 2).  On return the lower triangle holds
 * the band (diagonal blocks and the R blocks below them) with the reflectors
 * Y below the band, as the reference leaves them; entries above the diagonal
 * are not kept up to date.  precision: the form of the panel CAQR's own
 * trailing updates (the two-sided updates are FP64).  Waits for the stream and
 * returns the device status. */
int candmc_sym_full2band(double* A, int64_t lda, int64_t n, int64_t b, int64_t b_sub, int precision,
                         void* stream);

/* ---- least squares (no counterpart in the reference, which stops at the
 * factorization; built from QR_2D_pipe and update_A) ---------------------------
 * min ||A X - B||_F for A m x n (m >= n, full column rank), B m x nrhs, device
 * pointers.  A is factored in the requested form (a copy; A itself stays
 * resident for the residuals), X0 = R^-1 (Q^T B)[0:n] with Q applied in FP64,
 * then up to max_refine FP64 refinement steps of the corrected semi-normal
 * equations (r = B - A X, X += R^-1 R^-T A^T r), or, with the tuning knob
 * "ls_refine" = 1, of the augmented system [I A; A^T 0][r; X] = [B; 0]
 * (Bjorck 1967: f = B - r - A X, g = -A^T r, h = R^-T g, d = Q^T f,
 * dX = R^-1 (d[0:n] - h), dr = Q [h; d[n:m]]), until the largest per-column max|dX| / max|X| is <= tol.  With R from A's
 * own QR the iteration contracts by about kappa(A) * u_R per step (u_R: the
 * unit roundoff of R's form) and stops at the FP64 data's forward-error level,
 * about kappa(A) * u; a correction that is not smaller than the one before is
 * not applied and ends the refinement.  stats (nullable, 4 doubles):
 * corrections applied, last and first relative correction, device status. */
int candmc_ls_solve(const double* A, int64_t lda, int64_t m, int64_t n, const double* B, int64_t ldb,
                    int64_t nrhs, double* X, int64_t ldx, int64_t b, int precision, int max_refine,
                    double tol, double* stats, void* stream);

/* ---- batched least squares (no counterpart in the reference) ----------------
 * nprob independent problems min ||A_i x_i - b_i|| with 1 <= n_i <= 128 and
 * m_i >= n_i; host arrays of sizes and DEVICE pointers.  A_i (ld lda[i])
 * becomes Y\R of its TSQR-HR; b_i (m_i x 1) becomes Q^T b_i with x_i in its
 * first n_i entries (the dgels convention).  Problems are sorted by cost and
 * dealt onto nstreams streams; use_graph != 0 captures the schedule into a
 * CUDA graph on first use (keyed by sizes, pointers, nstreams and tuning) and
 * replays it afterwards. */
int candmc_batched_ls(int64_t nprob, const int64_t* m, const int64_t* n, double* const* A,
                      const int64_t* lda, double* const* B, int nstreams, int use_graph, void* stream);

/* candmc_batched_ls_f32: the float32-input variant (no counterpart in the
 * reference): A_i (ld lda_i) and b_i are float32; they are widened into an
 * FP64 work area on the device (one per device, grown on demand and held until
 * the process exits), solved by candmc_batched_ls in FP64, and x_i is rounded
 * into the first n_i entries of b_i (A_i is left as it was).  At most 65535
 * problems per call.  Calls from several host threads run one at a time; the
 * host waits for the previous call on this device to finish (the work area is
 * shared) and synchronises the stream once to upload the problem tables. */
int candmc_batched_ls_f32(int64_t nprob, const int64_t* m, const int64_t* n, float* const* A,
                          const int64_t* lda, float* const* B, int nstreams, int use_graph, void* stream);

/* candmc_batched_status: waits for the stream, then returns in *status the
 * first failure any batched call's kernels recorded on this device since the
 * last call (CANDMC_OK if none: e.g. CANDMC_ERR_TIMEOUT, CANDMC_ERR_NUMERIC)
 * and clears it.  Batched calls return once their work is enqueued, so their
 * device-side failures surface here. */
int candmc_batched_status(void* stream, int* status);

/* tuning knobs: "leaf_rows" (target rows per TSQR leaf, 32..256, default 64);
 * "pipe_tree" (1, the default: the levels of the TSQR tree overlap column by
 * column; 0: level by level); "oz_reserve_sms" (SMs kept free of the
 * persistent emulated-FP64 update kernel during QR_2D_pipe, for the panel
 * stream; default 32); "pipe_leaf_rows" (leaf height of the panels QR_2D_pipe
 * factors, 32..256, default 128; panels of 32768 rows or more take at least
 * 256); "panel_oz_min_rows" (in the emulated-FP64
 * and FP32 forms, panels with at least this many rows apply each half's Q^T to
 * the other half of the panel in emulated FP64 on the tensor cores instead of
 * the FP64 pipe; default 8192, 0 disables); "ls_refine" (candmc_ls_solve's refinement: 0, the
 * default, the corrected semi-normal equations; 1 the augmented system
 * [I A; A^T 0] refining x and r); "batched_form" (CANDMC_PREC_OZAKI, the
 * default: candmc_batched_ls's panels apply each half-panel's Q^T to the
 * other half on the tensor cores from "panel_oz_min_rows" rows on, in
 * emulated FP64 on FP64 storage; CANDMC_PREC_FP64: on the FP64 pipe) */
int candmc_set_tuning(const char* key, int64_t value);

/* ---- least-squares request server (no counterpart in the reference) ---------
 * Continuous batching of single-RHS least-squares requests on one GPU.
 * nworkers host threads, each with its own CUDA stream, take requests in
 * arrival order; a request is admitted once its arrival time has come, a
 * worker is idle and its device-memory estimate (candmc_ls_request_bytes)
 * fits beside the admitted ones within budget_bytes.  Each admitted request is
 * copied in from HOST memory, solved by candmc_ls_solve (A, Y\R, T and R stay
 * resident across the refinement steps) and x is copied back out.  Requests
 * run concurrently on the workers' streams; the kernels of one request do not
 * depend on what else runs, so each result is the same alone and in a mix.
 *
 * candmc_server_create: precision form, panel width b and the refinement
 *   controls of candmc_ls_solve; *out receives the handle.
 * candmc_server_submit: A (m x n, ld lda), bvec (m) and x (n) are host
 *   pointers that must stay valid until the request completes; arrival_s is
 *   the earliest admission time on the server clock (candmc_server_now; pass
 *   a time <= now for "at once").  A request whose estimate exceeds the whole
 *   budget fails with CANDMC_ERR_ALLOC at once.  *ticket identifies it.
 * candmc_server_wait: waits up to timeout_s seconds (< 0: no limit) for the
 *   request; returns CANDMC_ERR_TIMEOUT if it has not completed, else the
 *   request's own status.  info (nullable, 8 doubles): status, arrival, admit
 *   and completion times (s, server clock), refinement steps, last relative
 *   correction, device bytes reserved, worker index.
 * candmc_server_stats (8 doubles): bytes reserved now, peak bytes reserved,
 *   requests completed, requests in flight now, peak in flight, requests
 *   pending, budget, workers.
 * candmc_server_destroy: lets running requests finish, cancels pending ones
 *   (status CANDMC_ERR_CANCELLED) and joins the workers. */
#define CANDMC_ERR_CANCELLED 7   /* request dropped when the server shut down */
int candmc_server_create(double budget_bytes, int nworkers, int precision, int64_t b, int max_refine,
                         double tol, void** out);
int candmc_server_submit(void* server, const double* A, int64_t lda, int64_t m, int64_t n,
                         const double* bvec, double* x, double arrival_s, int64_t* ticket);
int candmc_server_wait(void* server, int64_t ticket, double timeout_s, double* info);
double candmc_server_now(void* server);
int candmc_server_stats(void* server, double* out);
int candmc_server_destroy(void* server);
/* device bytes a candmc_ls_solve of an m x n problem with one right-hand side
 * reserves at most (inputs, factor, T factors, residual vectors and the
 * largest transient workspace of the panel and trailing-update kernels) */
int64_t candmc_ls_request_bytes(int64_t m, int64_t n, int64_t b, int precision);
/* high-water mark of the device's default memory pool (bytes in use); reset
 * != 0 restarts it from the current use */
int candmc_mem_high_water(int reset, uint64_t* bytes);

#ifdef __cplusplus
}
#endif

#endif /* CANDMC_GB300_H */
