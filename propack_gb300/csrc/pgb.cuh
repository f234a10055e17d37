// pgb.cuh -- shared definitions of the GB300 Lanczos-bidiagonalisation
// library: error handling, the device-resident Lanczos state, the device
// CSR operator, and warp/CTA reduction helpers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

namespace pgb {

// ---------------------------------------------------------------- errors
void set_error(const std::string &msg);
#define PGB_CUDA(call)                                                              \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            ::pgb::set_error(std::string(#call " failed: ") + cudaGetErrorString(e_)); \
            throw ::pgb::CudaFailure();                                             \
        }                                                                           \
    } while (0)
struct CudaFailure {};
struct ArgFailure {};
struct WaitFailure {};

// kernel launch accounting (for the stats struct)
extern thread_local int64_t g_launches;
#define PGB_LAUNCHED() (++::pgb::g_launches)

// Optional per-kernel timing with CUDA events recorded on the launching
// stream (propack_set_profiling); off by default.
enum ProfKind { PK_SPMV_ADJ, PK_SPMV_FWD, PK_ELR, PK_CGS_DOTS, PK_CGS_UPD, PK_THIN, PK_ANALYSE, PK_SWEEPS,
                PK_GEMM, PK_SPMV_ADJ32, PK_SPMV_FWD32, PK_CGS_DOTS32, PK_CGS_UPD32, PK_RITZ, PK_N };
extern thread_local int g_prof_on;
void prof_mark(int kind, cudaStream_t s, bool begin);
void prof_collect();
#define PGB_PROF(kind, s, ...)                                     \
    do {                                                           \
        if (::pgb::g_prof_on) ::pgb::prof_mark((kind), (s), true); \
        __VA_ARGS__;                                               \
        if (::pgb::g_prof_on) ::pgb::prof_mark((kind), (s), false);\
    } while (0)

// ------------------------------------------------------------- constants
constexpr double EPS = 1.1102230246251565e-16;      // dlamch('e') = 2^-53
constexpr double SFMIN = 2.2250738585072014e-308;   // dlamch('s')
constexpr double KAPPA = 0.717;                     // dlanbpro.F:118
constexpr double KAPPA_GETU0 = (double)0.717f;      // dgetu0.F:30 (REAL literal)
constexpr double FUDGE = 1.01;                      // dlanbpro.F:117
constexpr int NTRY = 5;                             // dreorth.F:64
constexpr int BS = 256;                             // threads per CTA of the vector kernels
constexpr int NNZ_PB = 2048;                        // nnz per CTA segment of the low-rank prepass
constexpr int NNZ_W = 256;                          // nnz staged per warp in the SpMV (multiple of 32)
constexpr int ROWS_W = 32;                          // rows per SpMV row block (<= 32)

// ------------------------------------------------------- device operator
// CSR with int32 row pointers (nnz < 2^31) and CSR-adaptive row blocks.
struct Csr {
    int rows = 0, cols = 0;   // cols counts the low-rank tail columns too
    int ncol0 = 0;            // columns < ncol0 gather x; the rest gather z
    int64_t nnz = 0;
    int *ptr = nullptr;       // rows+1
    int *idx = nullptr;       // nnz
    double *val = nullptr;    // nnz
    float *valf = nullptr;    // nnz (FP32 copy for the mixed-precision path)
    int nblk = 0;             // row blocks
    int *blk = nullptr;       // nblk+1 row boundaries
    int segs = 0;             // thin matrices: segments per row for the split reduction
    int short_rows = 0;       // 1: the chunked schedule, 0: the staged one
    float tuned_ms[2] = {0.f, 0.f};  // timed choice: chunked, staged ms per product (0: not timed)
    // chunked schedule: the entries of each 32-row tile re-laid so that lane
    // l's run of C consecutive entries is read with coalesced loads
    int *tbase = nullptr;     // tiles+1: first 32-entry unit of each tile
    int *cidx = nullptr;      // 32 * tbase[tiles] (padding: column 0, value 0)
    double *cval = nullptr;
    float *cvalf = nullptr;
    // a native complex matrix (Operator::cplx == 2): (re, im) values in CSR
    // order and run-interleaved for the chunked schedule, which it always
    // uses; val, valf and cval stay null
    double2 *zval = nullptr;  // nnz
    double2 *czval = nullptr; // 32 * tbase[tiles]
};

// A = S + L diag(w) R'.  fwd = [S | L] (m x (n+r)), adj = [S' | R]
// (n x (m+r)); thin_r = R' (r x n), thin_l = L' (r x m).
struct Operator {
    int m = 0, n = 0, r = 0;
    Csr fwd, adj, thin_r, thin_l;
    double *w = nullptr;
    double *zbuf = nullptr;      // r: the low-rank coefficients of the current product
    double *zpart = nullptr;     // r * segs partials
    unsigned int *zticket = nullptr;
    int64_t id = 0;
    int device = 0;
    // 1: a complex m/2 x n/2 matrix held as its real 2x2-block form (fwd
    // computes A x and adj computes A^H x on (re, im) pairs); 2: a complex
    // m x n matrix held natively (index + complex value per entry, adj its
    // conjugate transpose)
    int cplx = 0;
};
Operator *lookup_operator(int64_t handle);

// ------------------------------------------------- Lanczos device state
// Deferred scaling of a Lanczos vector (dsafescal, dsafescal.F:49-53):
// mode 0 = none, 1 = multiply by val (= 1/alpha), 2 = divide by val
// (|alpha| < sfmin), 3 = zero the vector (reorthogonalisation collapse,
// dreorth.F:96-98).
struct Pend {
    int mode;
    double val;
};

struct LbCtl {
    // parameters of the current dlanbpro call
    int m, n, k;            // rows, cols, target dimension
    int ldu, ldv;
    int icgs, ielr;
    double delta, eta, epsn, epsn2;
    double eps_vec;         // unit roundoff of the Lanczos vectors (2^-53 FP64, 2^-24 FP32)
    // recurrence state (dlanbpro.F:123-126)
    int j;                  // current step, 1-based
    int full_reorth, force_reorth;
    int ierr;
    double alpha, beta, anorm, amax, numax, mumax, rnorm;
    // per half-step phase state
    int elr_active, elr_iter;
    double elr_s;           // ELR inner product for the coming iteration
    // complex*16 vectors (zlanbpro): stored as (re, im) pairs of doubles; the
    // ELR projection is complex and leaves B alone (zlanbpro.F:318-331),
    // and its first inner product is formed by the first ELR kernel
    int cplx;
    int elr_need_dot;
    double elr_s_im;
    int reorth_active, reorth_iter, reorth_count;
    int cgs_phase;          // 0: the next CGS kernel forms the projections, 1: it applies them
    double reorth_nrm0;
    int nsel;               // columns selected for reorthogonalisation
    int collapsed;          // the last reorthogonalisation zeroed the vector
    int ndot_iter;          // inner products counted per CGS pass (dreorth.F:91, :164)
    Pend pend_u, pend_v;    // deferred scaling of the newest u / v column
    int pend_u_col, pend_v_col;
    // suspension: the device met a case the enqueued sequence cannot finish
    int status;             // 0 running, 1 suspended, 2 finished early (invariant subspace)
    int susp_reason;        // 1 = getu0 needed (invariant subspace test), 2 = reorth iterations
    int susp_side;          // 0 = V half, 1 = U half
    int susp_j;
    // statistics (double/stat.h)
    long long nopx, nreorth, ndot;
    long long cgs_cols_u, cgs_cols_v;  // basis columns streamed by Gram-Schmidt passes, per side
    // last-CTA tickets
    unsigned int ticket;
};

// Everything a Lanczos kernel needs, passed by value.
struct LbArgs {
    LbCtl *ctl;
    void *U, *V;            // device Lanczos vectors (double or float), column-major
    int ldu, ldv;
    double *balpha, *bbeta; // B(:,1), B(:,2)
    double *mu, *nu;
    int *index;             // reorthogonalisation intervals (1-based)
    int *sel;               // expanded column list (0-based)
    double *h;              // CGS coefficients (complex: (re, im) pairs)
    double *part_sq, *part_dot;   // per-CTA partial sums (nb)
    double *part_cols;            // (kmax+1) * nb partial CGS dots, column c at c*nb
                                  // (complex: 2 (kmax+1) * nb, re at 2c*nb, im at (2c+1)*nb)
    int nb;                 // CTAs of the vector kernels
    int nb_spmv;            // CTAs the fused SpMV may use (>= nb; the partial-sum arrays hold it)
    int kmax;               // capacity of the column arrays
    Csr fwd, adj;           // device operator (fwd = [S|L], adj = [S'|R])
    Csr zfwd, zadj;         // a native complex operator (A, A^H; rows = 0 otherwise)
    const double *z;        // low-rank coefficients of the current product
    // FP64 form, Gram-Schmidt on the FP32 pipe (null when off): the
    // basis columns as FP32 (hi, lo) planes with the leading dimensions of
    // U and V, a flag per column (1: its planes hold the column's current
    // value), and the planes of the vector being reorthogonalised
    float2 *Up, *Vp;
    int *okU, *okV;
    float2 *xpl;
};
// real scalars per element of a Lanczos vector: 1 for double and float, 2
// for complex*16, held as double2 = (re, im).  LbArgs' ldu, ldv and the
// rows of its operators count real scalars.
template <typename T>
struct VecW {
    static constexpr int w = 1;
};
template <>
struct VecW<double2> {
    static constexpr int w = 2;
};
template <typename T>
__host__ __device__ __forceinline__ T *ucol(const LbArgs &a, int c) { return (T *)a.U + (size_t)c * a.ldu; }
template <typename T>
__host__ __device__ __forceinline__ T *vcol(const LbArgs &a, int c) { return (T *)a.V + (size_t)c * a.ldv; }

// FP64 accumulation, or FP32 with compensated (two-sum / two-product)
// accumulation; value() returns the sum in double.
template <typename T>
struct Acc;
template <>
struct Acc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add_prod(double a, double b) { s = fma(a, b, s); }
    __device__ __forceinline__ void add(double a) { s += a; }
    __device__ __forceinline__ double value() const { return s; }
};
template <>
struct Acc<float> {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float p)
    {
        const float t = s + p;
        const float bp = t - s;
        c += (s - (t - bp)) + (p - bp);
        s = t;
    }
    __device__ __forceinline__ void add_prod(float a, float b)
    {
        const float p = a * b;
        const float pe = fmaf(a, b, -p);
        const float t = s + p;
        const float bp = t - s;
        c += ((s - (t - bp)) + (p - bp)) + pe;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// --------------------------------------------------------- helpers
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
// Deterministic CTA sum (fixed tree); all threads get the result.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double *sh)
{
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    if (w == 0) {
        t = (lane < NT / 32) ? sh[lane] : 0.0;
        t = warp_sum(t);
        if (lane == 0) sh[0] = t;
    }
    __syncthreads();
    t = sh[0];
    __syncthreads();
    return t;
}
template <int NT>
__device__ __forceinline__ double block_max(double v, double *sh)
{
    v = warp_max(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    if (w == 0) {
        t = (lane < NT / 32) ? sh[lane] : 0.0;
        t = warp_max(t);
        if (lane == 0) sh[0] = t;
    }
    __syncthreads();
    t = sh[0];
    __syncthreads();
    return t;
}

// Last-CTA election after every CTA has published its partials.
__device__ __forceinline__ bool last_cta(unsigned int *ticket)
{
    __shared__ bool amlast;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int t = atomicAdd(ticket, 1u);
        amlast = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (amlast) {
        __threadfence();
        if (threadIdx.x == 0) *ticket = 0u;
    }
    return amlast;
}

__device__ __forceinline__ double apply_pend(double x, Pend p)
{
    switch (p.mode) {
    case 1: return x * p.val;
    case 2: return x / p.val;
    case 3: return 0.0;
    default: return x;
    }
}
__device__ __forceinline__ float apply_pend(float x, Pend p)
{
    switch (p.mode) {
    case 1: return x * (float)p.val;
    case 2: return (float)((double)x / p.val);
    case 3: return 0.f;
    default: return x;
    }
}


// ------------------------------------------------ small dense kernels
struct AnaArgs {
    const double *balpha, *bbeta;  // B of the Lanczos run
    double *a1, *b1, *bnd;         // scratch: sigma(B), bounds (dim+1)
    double *w;                     // 4*(dim+1) scratch
    const LbCtl *ctl;              // rnorm of the run
    double *sigma_out, *bnd_out;   // neig / k
    int *nconv_out;
    double *anorm_drv;             // the driver's local anorm
    int dim, m, n, neig, kk;       // kk: k = dim - p (IRL) or k (lansvd)
    int irl, small_side;
    double tol;
    double *wz;                    // bidiag_scratch(dim) doubles (lane-parallel path)
};

struct SweepArgs {
    double *balpha, *bbeta;   // modified in place
    const double *a1, *bnd;   // from k_analyse
    double *P, *Q;            // (dim+1)^2, dim^2
    double *shifts;           // dim
    double *w;                // 4*(dim+1)
    LbCtl *ctl;               // rnorm <- beta_k, nrestart counted by the host
    int dim, k, neig, small_side;
    double min_relgap;
    double *wz;               // bidiag_scratch(dim) doubles: the sweeps' rotations
};

struct RitzArgs {
    const double *balpha, *bbeta;
    double *D, *E;      // dim+1 scratch copies
    double *Mt;         // (dim+1)^2 : Q' of dbdqr
    double *P;          // dim^2 : left vectors of R
    double *Qt;         // dim^2 : right vectors' transpose
    double *w;          // 4*(dim+1)
    int dim, m, n;
    double *wz;         // bidiag_scratch(dim) doubles (lane-parallel path)
    int *flag;          // set to 1 when the lane-parallel vectors are not trusted
    int k, mstart;      // the wanted vectors: indices mstart-1 .. mstart+k-2
};

// scratch of the lane-parallel bidiagonal kernels for dimension dim
inline size_t bidiag_scratch(int dim) { return 8 * (size_t)(dim + 1) * (dim + 1) + 64; }

// analysis: nconv_out < 0 signals that the lane-parallel path declined and
// launch_analyse_qr must be run instead
void launch_analyse(const AnaArgs &a, cudaStream_t s);
void launch_analyse_qr(const AnaArgs &a, cudaStream_t s);
void launch_sweeps(const SweepArgs &a, cudaStream_t s);
// Ritz preparation: returns false when only the QR path applies; otherwise
// *a.flag != 0 afterwards asks for launch_ritz_prep_qr
bool launch_ritz_prep(const RitzArgs &a, cudaStream_t s);
void launch_ritz_prep_qr(const RitzArgs &a, cudaStream_t s);
template <typename T>
void gemm(int mr, int nc, int kk, const T *A, int lda, bool ta, const double *B, int ldb, bool tb, T *C, int ldc,
          cudaStream_t s);
// FP64 C = A op(B) on the BF16 tensor cores (error-free digit split); false
// when the shape is outside its range (then the caller uses the FP64 kernel)
bool gemm_f64_tc(int mr, int nc, int kk, const double *A, int lda, const double *B, int ldb, bool tb, double *C,
                 int ldc, cudaStream_t s);
template <typename T>
void copy_cols(const T *src, int lds, T *dst, int ldd, int rows, int cols, cudaStream_t s);

// ------------------------------------------------ Lanczos step enqueue
void lb_set_smem_limits(int kmax);
bool lb_planes_fit(int kmax, bool cplx);
// Gram-Schmidt arithmetic of the FP64 form: 0 FP64 FMAs, 1 three-way
// splits on the FP32 pipe (pgb_f3.cuh), 2 split-once planes (the default)
enum CgsArith { CGS_FP64 = 0, CGS_F3 = 1, CGS_PLANES = 2 };
extern thread_local int g_cgs_arith;
template <typename T>
void lb_enqueue_half(const LbArgs &a, const Operator *op, int side, int j, int ielr, int ntry_spec,
                     bool host_product, cudaStream_t s);
template <typename T>
void lb_enqueue_cgs_more(const LbArgs &a, int side, int j, int passes, cudaStream_t s);
template <typename T>
void lb_enqueue_flush(const LbArgs &a, cudaStream_t s);
template <typename T>
void op_thin(const Operator &op, bool trans, const T *x, cudaStream_t s);
int64_t handle_from_iparm(const int *iparm);
const char *last_error();

// --------------------------------------------------------- host helpers
struct Dev {
    int device = 0;
    int sms = 0;
    int nb = 0;            // CTAs for the streaming kernels
};
const Dev &device_info();

// The library's own stream-ordered device memory pool (one per device).  It
// keeps memory that is freed for the next allocation instead of returning
// it to the driver, so that repeated solves and operator builds do not pay
// for mapping GBs of device memory each time; propack_release_memory()
// gives it back.
cudaMemPool_t lib_pool();
void release_bounce_buffers();  // the idle pinned bounce buffers of pageable result copies
// host -> device copy on s; pageable sources go through the bounce buffers
void h2d_bytes(void *dst, const void *src, size_t bytes, cudaStream_t s);
void *pool_alloc(size_t bytes, cudaStream_t s);  // zero bytes allowed; never returns null
inline void pool_free(void *p, cudaStream_t s)
{
    if (p) cudaFreeAsync(p, s);
}

// exclusive scan of n ints into out[0..n] (out[n] = total, also returned)
int scan_excl(const int *in, int *out, int n, cudaStream_t s);

// operator application on device vectors (no Lanczos fusion)
template <typename T>
void op_apply(const Operator &op, bool trans, const T *x, T *y, cudaStream_t s);
// y = A x (trans: A^H x) for a complex operator of either form, on complex
// device vectors
void op_zapply(const Operator &op, bool trans, const double2 *x, double2 *y, cudaStream_t s);
// the plain complex product of one side of a native complex operator
void op_zspmv_plain_launch(const Csr &A, const double2 *x, double2 *y, cudaStream_t s);

}  // namespace pgb
