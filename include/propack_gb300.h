/*
 * propack_gb300.h -- C ABI of the GB300 Lanczos-bidiagonalisation library.
 *
 * The two drivers keep PROPACK 2.1's Fortran argument lists and gfortran's
 * calling convention (lower-case name + trailing underscore, every scalar by
 * reference, one hidden size_t length per CHARACTER argument appended after
 * the last argument, column-major arrays), so a Fortran program that links
 * against libpropack_gb300.so instead of libdpropack runs unchanged.
 *
 * All arithmetic between APROD calls runs in CUDA kernels on the current
 * device; the library keeps device mirrors of U, V and B and copies the
 * results back into the caller's arrays on exit.  There is no CPU path: if
 * no CUDA device is usable the drivers return INFO = PROPACK_ERR_CUDA.
 */
#ifndef PROPACK_GB300_H
#define PROPACK_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The user operator, exactly the reference's APROD (double/dlansvd.F:20-33):
 *   SUBROUTINE APROD(TRANSA, M, N, X, Y, DPARM, IPARM)
 * TRANSA = 'n': Y(1:M) = A X(1:N);  TRANSA = 't': Y(1:N) = A' X(1:M).
 * X and Y are HOST arrays when the library calls a user APROD. */
typedef void (*propack_aprod_t)(const char *transa, const int *m, const int *n,
                                const double *x, double *y, double *dparm,
                                int *iparm, size_t transa_len);

/* Negative INFO codes added by this library (the reference's own codes are
 * INFO = 0, INFO = J > 0 (invariant subspace of dimension J) and INFO = -1
 * (not converged); double/dlansvd.F:79-83, double/dlansvd_irl.F:93-99). */
#define PROPACK_ERR_ARG   (-2) /* an argument is out of range            */
#define PROPACK_ERR_CUDA  (-3) /* a CUDA call failed (no device, OOM, ..) */
#define PROPACK_ERR_HANDLE (-4) /* iparm does not hold a live operator   */
#define PROPACK_ERR_WAIT  (-5) /* a bounded device-side wait gave up     */

/* DLANSVD: k largest singular triplets, Krylov dimension grown up to kmax.
 * Replaces double/dlansvd.F:1-3 (argument meaning: dlansvd.F:10-83).
 * On exit *k holds the number of converged triplets and doption[2] the
 * estimate of ||A|| (double/dlanbpro.F:547). */
void dlansvd_(const char *jobu, const char *jobv, const int *m, const int *n,
              int *k, const int *kmax, propack_aprod_t aprod,
              double *U, const int *ldu, double *sigma, double *bnd,
              double *V, const int *ldv, const double *tolin,
              double *work, const int *lwork, int *iwork, const int *liwork,
              double *doption, const int *ioption, int *info,
              double *dparm, int *iparm, size_t jobu_len, size_t jobv_len);

/* DLANSVD_IRL: neig triplets by implicitly restarted Lanczos
 * bidiagonalisation with fixed dimension dim and p shifts per restart.
 * Replaces double/dlansvd_irl.F:1-3 (argument meaning: :10-99).
 * On exit *neig holds the number of converged triplets. */
void dlansvd_irl_(const char *which, const char *jobu, const char *jobv,
                  const int *m, const int *n, const int *dim, const int *p,
                  int *neig, const int *maxiter, propack_aprod_t aprod,
                  double *U, const int *ldu, double *sigma, double *bnd,
                  double *V, const int *ldv, const double *tolin,
                  double *work, const int *lwork, int *iwork,
                  const int *liwork, double *doption, const int *ioption,
                  int *info, double *dparm, int *iparm, size_t which_len,
                  size_t jobu_len, size_t jobv_len);

/* The counters of double/stat.h:6-15 for the calling host thread:
 * clearstat replaces double/printstat.F:4-32, printstat :35-75. */
void clearstat_(void);
void printstat_(void);

/* ---------------------------------------------------------------------
 * Device-resident sparse operator (the library's own APROD).
 *
 * A = S + L diag(w) R'   with S (m x n), L (m x r), R (n x r) given as
 * host CSR arrays (0-based, int64 row pointers, int32 column indices,
 * float64 values); r = 0 for a plain CSR matrix.  The library copies them
 * to the device and builds A' there.  A Lanczos driver that receives
 * propack_gpu_csr_aprod_ as its APROD argument recognises it by address
 * and applies the operator on the device with no host traffic; the
 * operator's handle travels in iparm[0..1] (low, high 32 bits).  No
 * counterpart exists in the reference: it supplies the APROD that the
 * reference leaves to the user (double/dlanbpro.F:288, :420).
 * Returns 0 and writes the handle, or a negative PROPACK_ERR_* code. */
int propack_csr_create(int m, int n, const int64_t *s_rowptr,
                       const int32_t *s_colidx, const double *s_val,
                       int r, const int64_t *l_rowptr, const int32_t *l_colidx,
                       const double *l_val, const int64_t *r_rowptr,
                       const int32_t *r_colidx, const double *r_val,
                       const double *w, int64_t *handle);
int propack_csr_destroy(int64_t handle);
/* SpMV schedule of the operators built after the call (per host process),
 * per direction: 0 (default) a rule on the mean row length -- chunked
 * below 128 nonzeros per row, staged above -- so that a matrix always gets
 * the same schedule and the same summation order; 1 always chunked;
 * 2 always staged; 3 a timed choice -- propack_csr_create builds the
 * run-interleaved copy of any matrix with fewer than 512 nonzeros per row
 * on average, times both schedules on the device and keeps the faster
 * (the rule's choice unless the other is more than 5 % faster; a near-tie
 * can go either way between builds).  Results depend only on the matrix
 * and the schedule.  Returns 0 or PROPACK_ERR_ARG. */
int propack_set_spmv_schedule(int mode);
/* The schedules chosen for A (sched[0]) and A' (sched[1]): 1 chunked,
 * 0 staged; tuned_ms (optional, 4 floats): the timed chunked / staged ms
 * per product of A, then of A' (0 where not timed). */
int propack_csr_schedule(int64_t handle, int *sched, float *tuned_ms);
/* Store a handle in iparm[0..1] (helper for C callers). */
void propack_handle_to_iparm(int64_t handle, int *iparm);

/* APROD-compatible entry: with HOST x, y it copies x in, applies the
 * device operator named by iparm[0..1] and copies y out.  Passed as the
 * APROD argument of dlansvd_/dlansvd_irl_ it is never called through the
 * pointer: the drivers apply the operator on device vectors directly. */
void propack_gpu_csr_aprod_(const char *transa, const int *m, const int *n,
                            const double *x, double *y, double *dparm,
                            int *iparm, size_t transa_len);

/* Apply the device operator to DEVICE vectors without allocating any
 * device memory: y = A x (trans = 0; x has n entries, y has m) or
 * y = A' x (trans != 0; x has m, y has n), enqueued on `stream` (a
 * cudaStream_t; NULL for the default stream) and not synchronised.
 * For callers that must not call cudaMalloc/cudaFree while they run.
 * The only scratch is a fixed array of PROPACK_NOALLOC_MAX_DOUBLES
 * doubles (512 KiB) in device memory, held by every GPU that loads the
 * library until the process exits; an operator whose low-rank term needs
 * r*(1+segments)+1 > PROPACK_NOALLOC_MAX_DOUBLES doubles is rejected with
 * PROPACK_ERR_ARG.  All calls share that array: calls that may overlap on
 * the GPU (different streams, different host threads) race and must be
 * serialised by the caller.  The first call on each device looks up the
 * array's device address (no allocation); make that first call before
 * any stream capture.  That first call (on each device, and the first on
 * each host thread) may also make the CUDA runtime load the library's
 * kernels onto the device (lazy module loading), which takes device
 * memory: callers should make one warm-up call before the section that
 * must not allocate.  x and y must be memory the operator's device can
 * address (device memory of that device, managed memory, or mapped host
 * memory); anything else is refused with PROPACK_ERR_ARG before any
 * launch.  A complex operator (propack_zcsr_create, either form): x
 * holds n (trans: m) complex entries as interleaved (re, im) doubles, 2n
 * doubles, and y receives 2m (trans: 2n) doubles; trans != 0 applies A^H.
 * For the native form x and y must be 16-byte aligned (PROPACK_ERR_ARG
 * otherwise).  No counterpart exists in the reference.  Returns 0 or a
 * negative PROPACK_ERR_* code. */
#define PROPACK_NOALLOC_MAX_DOUBLES 65536
int propack_csr_apply_noalloc(int64_t handle, int trans, const double *x,
                              double *y, void *stream);

/* ---------------------------------------------------------------------
 * Per-thread call statistics of the last driver call on this host thread
 * (the reference keeps these in COMMON /timing/; here they are
 * thread-local so the library is reentrant).  No reference counterpart. */
typedef struct {
    int64_t nopx;      /* operator applications (matvecs)       */
    int64_t nreorth;   /* reorthogonalisations                  */
    int64_t ndot;      /* inner products in reorthogonalisation */
    int64_t nrestart;  /* implicit restarts                     */
    int64_t nbsvd;     /* bidiagonal SVDs                       */
    int64_t nlandim;   /* final Lanczos dimension               */
    double device_ms;  /* device time between entry and exit    */
    double lanczos_ms; /* of which inside Lanczos steps         */
    double bsvd_ms;    /* of which bidiagonal SVD + shifts      */
    double gemm_ms;    /* of which restart / Ritz products      */
    int64_t kernel_launches; /* kernels this library launched   */
    double solve_ms;   /* device time from the start vector in HBM
                          to the Ritz vectors in HBM (no host copies) */
    int64_t nopx_low;  /* mixed form: matvecs of the FP32 phase        */
    double low_ms;     /* mixed form: device ms of the FP32 phase      */
    int64_t cgs_cols_u; /* basis columns (length m) read by Gram-Schmidt passes */
    int64_t cgs_cols_v; /* basis columns (length n) read by Gram-Schmidt passes */
} propack_stats_t;
void propack_get_stats(propack_stats_t *out);

/* Precision of dlansvd_irl_ for the calling host thread.  mode 0 (the
 * default) is the reference's FP64 method.  mode 1 is the mixed form:
 * Lanczos vectors, SpMV (on an FP32 copy of the values) and Gram-Schmidt
 * in FP32 with compensated (two-sum / two-product) reductions, while
 * alpha, beta, the omega recurrences (with FP32 unit roundoff), the
 * bidiagonal SVD and the shifts stay FP64; the FP32 run stops at
 * max(tol, 1e-6) (or after 8 restarts without a new converged value) and
 * an FP64 run with the same dim and p, started from the sum of the top
 * neig FP32 Ritz vectors, refines the triplets to the requested tol.
 * which = 'S' always runs in FP64.  Mode 2 is the FP32 form alone (no FP64
 * refinement; tol no finer than 16 * 2^-24), the form of slansvd_ and
 * slansvd_irl_.
 * Returns 0, or PROPACK_ERR_ARG for another mode.  No reference
 * counterpart. */
int propack_set_precision(int mode);
int propack_get_precision(void);

/* Per-kernel device timing: with profiling on, CUDA events are recorded
 * on the launching stream around every launch of the main kernels and
 * propack_get_profile returns, per kernel class, the summed milliseconds
 * and launch counts accumulated since propack_set_profiling(1).  Classes
 * in order: SpMV A'u (fused), SpMV Av (fused), ELR pass, CGS projection,
 * CGS update, low-rank prepass, bidiagonal analysis, IRL sweeps, GEMM,
 * then the FP32 (mixed form) SpMV A'u, SpMV Av, CGS projection, CGS update,
 * then the Ritz preparation (SVD of the final bidiagonal).
 * Returns the number of classes.  No reference counterpart. */
void propack_set_profiling(int on);
int propack_get_profile(double *total_ms, int64_t *launches, int n);

/* Arithmetic of the FP64 form's Gram-Schmidt passes for the calling host
 * thread: 0 FP64 FMAs (dgemv as in dreorth.F:85-95, :174); 1 each FP64
 * value split exactly into three FP32 pieces and the products summed at
 * three levels on the FP32 pipe (error ~2^-53 of sum |w x|, like an FP64
 * dot product's own rounding), then one FP64 FMA per row; 2 (the default)
 * each basis column split once into FP32 (hi, lo) planes kept beside the
 * FP64 basis (one more basis-sized array of device memory), the products
 * summed on the FP32 pipe as compensated FP32 pairs (error a few 2^-48 of
 * sum |w x|), then one FP64 FMA per row.  The complex*16 drivers run
 * mode 2 on planes of the real and imaginary parts and mode 1 as mode 0.
 * Mode 2 applies to solves whose kmax is at most ~2800 (complex drivers:
 * ~1500) and falls back to mode 0 above that.  Returns 0 or
 * PROPACK_ERR_ARG. */
int propack_set_cgs_arith(int mode);

/* The binary (SASS) version of the library's kernels as the CUDA runtime
 * loaded them on the current device: 103 for sm_103a.  Returns it, or
 * PROPACK_ERR_CUDA when no device is usable.  No reference counterpart. */
int propack_kernel_binary_version(void);

/* ---- Single-precision drivers ------------------------------------------
 * SLANSVD / SLANSVD_IRL: the argument lists of single/slansvd.F:1-3 and
 * single/slansvd_irl.F:1-3 (REAL arrays, REAL tolin/doption/dparm, a REAL
 * APROD).  They run the FP32 form: FP32 Lanczos vectors, SpMV on the FP32
 * copy of the values and Gram-Schmidt with compensated reductions, FP64
 * scalars, tol no finer than 16 * 2^-24.  which = 'S' runs in FP64.  A user
 * APROD receives REAL host vectors; propack_gpu_csr_saprod_ is recognised by
 * address like the double version. */
typedef void (*propack_saprod_t)(const char *transa, const int *m, const int *n,
                                 const float *x, float *y, float *dparm,
                                 int *iparm, size_t transa_len);
void slansvd_(const char *jobu, const char *jobv, const int *m, const int *n,
              int *k, const int *kmax, propack_saprod_t aprod,
              float *U, const int *ldu, float *sigma, float *bnd,
              float *V, const int *ldv, const float *tolin,
              float *work, const int *lwork, int *iwork, const int *liwork,
              float *doption, const int *ioption, int *info,
              float *dparm, int *iparm, size_t jobu_len, size_t jobv_len);
void slansvd_irl_(const char *which, const char *jobu, const char *jobv,
                  const int *m, const int *n, const int *dim, const int *p,
                  int *neig, const int *maxiter, propack_saprod_t aprod,
                  float *U, const int *ldu, float *sigma, float *bnd,
                  float *V, const int *ldv, const float *tolin,
                  float *work, const int *lwork, int *iwork, const int *liwork,
                  float *doption, const int *ioption, int *info,
                  float *dparm, int *iparm,
                  size_t which_len, size_t jobu_len, size_t jobv_len);
/* The device operator as a REAL APROD (host REAL vectors in and out). */
void propack_gpu_csr_saprod_(const char *transa, const int *m, const int *n,
                             const float *x, float *y, float *dparm, int *iparm,
                             size_t transa_len);

/* ---- Complex*16 drivers ------------------------------------------------
 * ZLANSVD / ZLANSVD_IRL: the argument lists of complex16/zlansvd.F:1-3 and
 * complex16/zlansvd_irl.F:1-3.  U, V, ZWORK and ZPARM are COMPLEX*16 (a
 * propack_z16 has the same layout: real part, then imaginary part);
 * Sigma, bnd, WORK and DOPTION stay DOUBLE PRECISION.  The APROD is the
 * reference's complex one (complex16/zlanbpro.F:297, :442):
 *   SUBROUTINE APROD(TRANSA, M, N, X, Y, ZPARM, IPARM)
 * TRANSA = 'n': Y(1:M) = A X(1:N);  TRANSA = 'c': Y(1:N) = A^H X(1:M).
 * Always FP64 arithmetic (propack_set_precision does not apply).  ZWORK,
 * WORK and IWORK are not used. */
typedef struct {
    double re, im;
} propack_z16;
typedef void (*propack_zaprod_t)(const char *transa, const int *m, const int *n,
                                 const propack_z16 *x, propack_z16 *y,
                                 propack_z16 *zparm, int *iparm, size_t transa_len);
void zlansvd_(const char *jobu, const char *jobv, const int *m, const int *n,
              int *k, const int *kmax, propack_zaprod_t aprod,
              propack_z16 *U, const int *ldu, double *sigma, double *bnd,
              propack_z16 *V, const int *ldv, const double *tolin,
              double *work, const int *lwork, propack_z16 *zwork,
              const int *lzwrk, int *iwork, const int *liwork,
              double *doption, const int *ioption, int *info,
              propack_z16 *zparm, int *iparm, size_t jobu_len, size_t jobv_len);
void zlansvd_irl_(const char *which, const char *jobu, const char *jobv,
                  const int *m, const int *n, const int *dim, const int *p,
                  int *neig, const int *maxiter, propack_zaprod_t aprod,
                  propack_z16 *U, const int *ldu, double *sigma, double *bnd,
                  propack_z16 *V, const int *ldv, const double *tolin,
                  double *work, const int *lwork, propack_z16 *zwork,
                  const int *lzwrk, int *iwork, const int *liwork,
                  double *doption, const int *ioption, int *info,
                  propack_z16 *zparm, int *iparm,
                  size_t which_len, size_t jobu_len, size_t jobv_len);

/* Upload a complex m x n CSR matrix (0-based int64 row pointers, int32
 * column indices, complex*16 values) as a device operator for the complex
 * drivers.  Default (native) form: the device keeps the complex CSR (an
 * int32 index and a complex*16 value per entry, 20 bytes) and its
 * conjugate transpose, built on the device; the complex SpMV accumulates
 * in complex arithmetic and, inside the Lanczos steps, also forms the
 * complex projection that the local reorthogonalisation subtracts.  Block
 * form (propack_set_zcsr_form(1)): the device holds the real 2m x 2n
 * matrix in which each entry b + ic becomes the 2x2 block [b -c; c b] on
 * the (re, im) pairs (48 bytes per complex entry), applied by the real
 * kernels.  Both give A x and A^H x to rounding.  Same checks and error
 * codes as propack_csr_create (native: fewer than 2^31 entries; block
 * form: 4 nnz < 2^31); the handle is freed with propack_csr_destroy. */
int propack_zcsr_create(int m, int n, const int64_t *rowptr, const int32_t *colidx, const propack_z16 *val,
                        int64_t *handle);
/* The form of complex operators created afterwards (process-wide): 0
 * native complex CSR (default), 1 the real 2x2-block form.  Returns 0, or
 * PROPACK_ERR_ARG for another value. */
int propack_set_zcsr_form(int form);
/* The 2x2-block form itself, on the host (used by propack_zcsr_create):
 * rowptr2 has 2m+1 entries, colidx2 and val2 4 nnz(A) entries.  Returns 0,
 * or PROPACK_ERR_ARG for a negative size or 4 nnz(A) >= 2^31. */
int propack_zcsr_expand(int m, int n, const int64_t *rowptr, const int32_t *colidx, const propack_z16 *val,
                        int64_t *rowptr2, int32_t *colidx2, double *val2);
/* The complex device operator as a ZAPROD (host complex*16 vectors in and
 * out); the complex drivers recognise it by address and then keep every
 * product on the device. */
void propack_gpu_csr_zaprod_(const char *transa, const int *m, const int *n,
                             const propack_z16 *x, propack_z16 *y, propack_z16 *zparm,
                             int *iparm, size_t transa_len);

/* ---- Learned start vector (no reference counterpart) ----------------
 * A row-wise MLP (18 -> 256 -> 256 -> 1, ReLU; BF16 weights, FP32
 * accumulation) that proposes the start vector U(:,1) in place of dgetu0's
 * random one (double/dgetu0.F:11-89) for a family of related matrices.
 * Features of row i: log1p(nnz)/4, ||y_i||/rho and 2 y_i/rho for the
 * 16-column Gaussian sketch y = A*Omega (Omega drawn from `seed` by a
 * counter-based generator; rho = RMS of ||y_i||).  Training minimises
 * -(1/k) sum_j log(c_j^2 + 1e-4 ||u0||^2/k) + log ||u0||^2, c = U'u0, for
 * the leading k left singular vectors U of a training matrix (column-major,
 * ldu >= m).  The operator is a propack_csr_create handle.  All functions
 * return 0 or a negative PROPACK_ERR_*; the model runs on the device that
 * was current at creation. */
int propack_mlp_create(uint64_t seed, int64_t *handle);
int propack_mlp_destroy(int64_t handle);
/* number of parameters; flat FP32 order W1[256][18], b1[256], W2[256][256]
 * ([out][in]), b2[256], w3[256], b3[1] */
int propack_mlp_nparams(void);
/* copy the parameters out (get) and/or in (set); either may be NULL */
int propack_mlp_params(int64_t handle, float *get, const float *set);
/* the m x 18 feature matrix of the operator's rows (row-major), host */
int propack_mlp_features(int64_t handle, int64_t op_handle, uint64_t seed, float *F);
/* the proposed start vector (m entries, host; not normalised) */
int propack_mlp_start(int64_t handle, int64_t op_handle, uint64_t seed, double *u0);
/* loss and its gradient (nparams floats, host) for (operator, U); no update */
int propack_mlp_grad(int64_t handle, int64_t op_handle, uint64_t seed, const double *U, int ldu, int k,
                     float *grad, double *loss);
/* one Adam step (beta 0.9 / 0.999) with learning rate lr on (operator, U) */
int propack_mlp_train_step(int64_t handle, int64_t op_handle, uint64_t seed, const double *U, int ldu, int k,
                           double lr, double *loss);
/* the kernel of the 256 x 256 layer, process-wide: 1 (default) tcgen05.mma
 * with FP32 accumulators in tensor memory, 0 the mma.sync kernel (the
 * reference implementation; results differ only in the FP32 accumulation
 * order).  Returns 0 or PROPACK_ERR_ARG. */
int propack_mlp_set_impl(int impl);

/* ---- Batched solver (no reference counterpart) -----------------------
 * nprob independent CSR matrices with FP32 values, solved by dlansvd_irl
 * (double/dlansvd_irl.F) with full reorthogonalisation (iterated classical
 * Gram-Schmidt on every step), FP64 vectors, p = dim - neig exact shifts,
 * one persistent kernel (a CTA per problem, work queue by decreasing size)
 * whose restart cycles are replayed as a CUDA graph.
 * Problem p: m[p] x n[p]; its m[p]+1 row pointers (0-based, its own
 * nonzeros) follow those of problem p-1 in `rowptr`; its column indices
 * and values are colidx/val[nnz_off[p] .. nnz_off[p+1]).  Total nonzeros
 * below 2^31. */
int propack_batch_create(int nprob, const int *m, const int *n, const int *rowptr, const int64_t *nnz_off,
                         const int *colidx, const float *val, int64_t *handle);
int propack_batch_destroy(int64_t handle);
/* u0: the start vectors (U(:,1) of every problem, concatenated, sum(m)
 * entries).  sigma, bnd: nprob x neig (row p = problem p).  info[p]: 0
 * converged, -1 not converged within maxiter (dlansvd_irl's INFO=-1), 1
 * the problem met an invariant subspace or clustered Ritz values that the
 * batched kernel leaves to the single-problem driver.  U, V (optional):
 * the neig left / right singular vectors of every converged problem,
 * concatenated (m[p] x neig, n[p] x neig, column-major each).
 * Requires 1 <= neig < dim <= min(64, m[p], n[p]). */
int propack_batch_solve(int64_t handle, int dim, int neig, int maxiter, double tol, const double *u0,
                        double *sigma, double *bnd, int *info, double *U, double *V);
typedef struct {
    int64_t nopx;            /* matvecs of all problems */
    int64_t nreorth;         /* Gram-Schmidt reorthogonalisations */
    int64_t converged;       /* problems with info 0 */
    int64_t fallback;        /* problems with info 1 */
    double device_ms;        /* device time of the solve (start vectors to results) */
    int64_t cycles;          /* CUDA-graph replays of the restart cycle */
    int64_t grid;            /* CTAs of the persistent kernel */
    int64_t kernel_launches;
    double tune_ms;          /* host ms of the autotuner in this call (0: the batch was tuned before) */
} propack_batch_stats_t;
int propack_batch_get_stats(propack_batch_stats_t *out);

/* The batched kernel's autotuner.  The problems fall into
 * PROPACK_BATCH_CLASSES size classes (quarters of the batch by decreasing
 * nonzeros + 8 (m + n)).  Before the first solve of a batch, every
 * candidate pair (g, dc) -- g lanes per row in the sparse products (1, 4, 8
 * or 32: the row split), dc columns per warp in the Gram-Schmidt
 * projections (1, 2 or 4: the tile) -- is timed on a sample of each class
 * (one CTA per sampled problem: both products and one set of projections,
 * CUDA events), and the fastest is kept; the defaults (1, 1) stay unless a
 * candidate is more than 3 % faster.  dc does not change any result; g
 * changes the summation order of the products (results differ at rounding
 * level between choices), so a caller who needs the same bits across
 * batches pins the table with propack_batch_set_tuning.
 * propack_batch_get_tuning writes per class g, dc and the probe's ms with
 * them and with (1, 1) (0 when the table was set by the caller) and returns
 * 0 (not tuned yet), 1 (timed) or 2 (set by the caller), or
 * PROPACK_ERR_HANDLE.  propack_batch_set_tuning(h, NULL, NULL) asks for a
 * new timing at the next solve.  No reference counterpart. */
#define PROPACK_BATCH_CLASSES 4
int propack_batch_get_tuning(int64_t handle, int *g, int *dc, float *ms_tuned, float *ms_default);
int propack_batch_set_tuning(int64_t handle, const int *g, const int *dc);
/* Arithmetic of a batch's products and Gram-Schmidt passes: 0 FP64 FMAs on
 * the FP64 bases (default), 2 FP32 (hi, lo) planes of every basis column,
 * split once per final column, summed as compensated FP32 pairs (results
 * agree with the FP64 ones to rounding; on a GB300 the batched workload
 * measured slower with planes).  A timed autotuner table is redone when the
 * arithmetic changes.  Returns 0, PROPACK_ERR_ARG or PROPACK_ERR_HANDLE. */
int propack_batch_set_arith(int64_t handle, int arith);

/* ---- FP64 product on the tensor cores --------------------------------
 * C (mr x nc, column-major ldc) = A (mr x kk, column-major lda) op(B), with
 * op(B)(l, j) = B[j * ldb + l] (tb = 0) or B[l * ldb + j] (tb = 1); all
 * pointers are device memory.  This is the restart / Ritz product of
 * dlansvd_irl.F:371-398 and dritzvec.F:130-198 (dgemm_ovwr.F:56-87) as the
 * drivers run it: an error-free split of both operands into seven BF16
 * digits, exact FP32 level sums, int64 recombination.  impl 1 is the
 * tcgen05 kernel (every thread splits digits, one issues the MMAs between
 * CTA barriers), impl 2 the warp-specialised tcgen05 kernel (sixteen
 * splitting warps and one MMA warp meeting on mbarriers), impl 0 the
 * mma.sync kernel; all give the same bits.  The drivers use the kernel set
 * by propack_set_gemm_impl (1 or 2).  Requires mr >= 1, 1 <= kk <= 256,
 * lda, ldc >= mr. */
int propack_gemm_f64_tc(int impl, int mr, int nc, int kk, const double *A, int lda, const double *B, int ldb,
                        int tb, double *C, int ldc);
/* The tcgen05 kernel of the drivers' restart and Ritz products (1 or 2,
 * default 2; process-wide).  Returns 0 or PROPACK_ERR_ARG. */
int propack_set_gemm_impl(int impl);

/* Device memory of the library's operators and solves comes from its own
 * stream-ordered pool, which keeps freed memory for the next call instead
 * of returning it to the driver (repeated solves skip the mapping of GBs
 * of device memory).  This returns all of it that is not in use, and frees
 * the idle pinned host buffers through which results are copied into
 * pageable (ordinary) host arrays (two 64 MiB halves per copy that ran
 * concurrently; kept between calls for the same reason).
 * Returns 0 or PROPACK_ERR_CUDA. */
int propack_release_memory(void);

/* Roofline calibration of the sparse products: the device ms of one pass of
 * nnz random 8-byte reads from an n-entry FP64 vector (which stays in L2 for
 * n up to ~16 M) with their 12-byte (int32 index, FP64 value) stream, flat,
 * four independent entries in flight per thread -- the fastest a product
 * with uniformly random columns can run on this GPU, whatever its rows.
 * Median of five passes after three.  Returns 0 or a negative
 * PROPACK_ERR_*.  No reference counterpart. */
int propack_gather_ceiling(int n, int64_t nnz, float *ms);

/* Last error message for the calling thread ("" if none). */
const char *propack_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* PROPACK_GB300_H */
