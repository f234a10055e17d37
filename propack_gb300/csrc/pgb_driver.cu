// pgb_driver.cu -- the DLANSVD / DLANSVD_IRL drivers behind the C ABI.
//
// Control flow follows double/dlansvd_irl.F:160-419 and double/dlansvd.F:
// 131-291; the Lanczos recurrence follows double/dlanbpro.F:146-549.  The
// host only orchestrates: the Lanczos vectors, B, the omega recurrences, the
// bidiagonal SVD, the shifts and the restart/Ritz products all live and run
// on the device.  One host/device round trip per restart reads the number of
// converged values.  Rare cases (a random restart vector after an
// invariant subspace, dgetu0.F; the resume prologue of dlanbpro.F:231-275)
// are driven from the host with device kernels.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <type_traits>
#include <vector>

#include "../../include/propack_gb300.h"
#include "pgb.cuh"

namespace pgb {

// ------------------------------------------------------------- statistics
struct Stats {
    int64_t nopx = 0, nreorth = 0, ndot = 0, nrestart = 0, nbsvd = 0, nlandim = 0, nsing = 0;
    double device_ms = 0, lanczos_ms = 0, bsvd_ms = 0, gemm_ms = 0;
    int64_t launches = 0;
    double solve_ms = 0;
    int64_t nopx_low = 0;   // matvecs of the FP32 phase (mixed form)
    double low_ms = 0;      // device ms of the FP32 phase (mixed form)
    int64_t cgs_cols_u = 0, cgs_cols_v = 0;  // basis columns streamed by Gram-Schmidt
};
static thread_local Stats g_stat;       // cumulative (clearstat_/printstat_)
static thread_local Stats g_last;       // last driver call (propack_get_stats)

// PROPACK_GB300_TRACE=1 prints the driver's decisions (suspensions of the
// Lanczos step sequence, restarts, phases of the mixed form) to stderr
static bool trace_on()
{
    static const bool on = [] {
        const char *e = getenv("PROPACK_GB300_TRACE");
        return e && e[0] && e[0] != '0';
    }();
    return on;
}

// steps enqueued between two looks at the device status word
constexpr int LB_WINDOW = 8;

// ------------------------------------------------------------ small kernels
#define LCG_A 33952834046453ULL
#define LCG_MASK ((1ULL << 48) - 1ULL)

__device__ __forceinline__ unsigned long long mulmod48(unsigned long long a, unsigned long long b)
{
    return (a * b) & LCG_MASK;
}
// x[i] = 2 * (seed * a^(offset+i+1) mod 2^48) / 2^48 - 1: dlarnv(2, ...) with
// dlaruv's generator (Lapack_Util/dlarnv.f, dlaruv.f), 64 values per thread.
template <typename T>
__global__ void k_rng_pm1(T *x, int n, unsigned long long seed, long long offset)
{
    const double r48 = 1.0 / 281474976710656.0;
    const long long nchunk = (n + 63) / 64;
    for (long long cidx = blockIdx.x * (long long)blockDim.x + threadIdx.x; cidx < nchunk;
         cidx += (long long)gridDim.x * blockDim.x) {
        unsigned long long e = (unsigned long long)(offset + cidx * 64 + 1), p = 1, b = LCG_A;
        while (e) {
            if (e & 1) p = mulmod48(p, b);
            b = mulmod48(b, b);
            e >>= 1;
        }
        unsigned long long s = mulmod48(seed, p);
        const int i0 = (int)(cidx * 64);
        for (int q = 0; q < 64 && i0 + q < n; q++) {
            x[i0 + q] = (T)(2.0 * ((double)s * r48) - 1.0);
            s = mulmod48(s, LCG_A);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(BS) k_sumsq_part(const T *x, int n, double *part)
{
    __shared__ double red[32];
    Acc<T> a;
    for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) a.add_prod(x[i], x[i]);
    const double s = block_sum<BS>(a.value(), red);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}
__global__ void __launch_bounds__(BS) k_sum_final(const double *part, int nb, double *out)
{
    __shared__ double red[32];
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += BS) s += part[b];
    s = block_sum<BS>(s, red);
    if (threadIdx.x == 0) *out = s;
}
// partial W(:,0:kk)' x per CTA (contiguous row chunks), column c at c*nb
template <typename T>
__global__ void __launch_bounds__(BS) k_gemvt_part(const T *W, size_t ld, int len, int kk, const T *x, double *part)
{
    const int chunk = (len + gridDim.x - 1) / gridDim.x;
    const int r0 = blockIdx.x * chunk, r1 = min(len, r0 + chunk);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int c = w; c < kk; c += BS / 32) {
        const T *col = W + (size_t)c * ld;
        Acc<T> acc;
        for (int r = r0 + lane; r < r1; r += 32) acc.add_prod(col[r], x[r]);
        const double v = warp_sum(acc.value());
        if (lane == 0) part[(size_t)c * gridDim.x + blockIdx.x] = v;
    }
}
__global__ void __launch_bounds__(BS) k_gemvt_final(const double *part, int nb, int kk, double *h)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int c = w; c < kk; c += BS / 32) {
        double s = 0.0;
        for (int b = lane; b < nb; b += 32) s += part[(size_t)c * nb + b];
        s = warp_sum(s);
        if (lane == 0) h[c] = s;
    }
}
template <typename T>
__global__ void __launch_bounds__(BS) k_gemvn_upd(const T *W, size_t ld, int len, int kk, const double *h, T *x)
{
    for (int r = blockIdx.x * BS + threadIdx.x; r < len; r += gridDim.x * BS) {
        T acc = 0;
        for (int c = 0; c < kk; c++) acc = fma(W[(size_t)c * ld + r], (T)h[c], acc);
        x[r] -= acc;
    }
}
// complex*16 forms of the two above (zgemv 'C' and 'N' of zcgs): column c's
// partial (re, im) at rows 2c, 2c+1 of part; h as (re, im) pairs
__global__ void __launch_bounds__(BS) k_zgemvt_part(const double2 *W, size_t ld, int len, int kk, const double2 *x,
                                                    double *part)
{
    const int chunk = (len + gridDim.x - 1) / gridDim.x;
    const int r0 = blockIdx.x * chunk, r1 = min(len, r0 + chunk);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int c = w; c < kk; c += BS / 32) {
        const double2 *col = W + (size_t)c * ld;
        double re = 0.0, im = 0.0;
        for (int r = r0 + lane; r < r1; r += 32) {
            const double2 a = col[r], b = x[r];
            re = fma(a.x, b.x, re);
            re = fma(a.y, b.y, re);
            im = fma(a.x, b.y, im);
            im = fma(-a.y, b.x, im);
        }
        re = warp_sum(re);
        im = warp_sum(im);
        if (lane == 0) {
            part[(size_t)(2 * c) * gridDim.x + blockIdx.x] = re;
            part[(size_t)(2 * c + 1) * gridDim.x + blockIdx.x] = im;
        }
    }
}
__global__ void __launch_bounds__(BS) k_zgemvn_upd(const double2 *W, size_t ld, int len, int kk, const double *h,
                                                   double2 *x)
{
    for (int r = blockIdx.x * BS + threadIdx.x; r < len; r += gridDim.x * BS) {
        double ar = 0.0, ai = 0.0;
        for (int c = 0; c < kk; c++) {
            const double2 w = W[(size_t)c * ld + r];
            const double hr = h[2 * c], hi = h[2 * c + 1];
            ar = fma(w.x, hr, ar);
            ar = fma(-w.y, hi, ar);
            ai = fma(w.x, hi, ai);
            ai = fma(w.y, hr, ai);
        }
        double2 v = x[r];
        v.x -= ar;
        v.y -= ai;
        x[r] = v;
    }
}
template <typename T>
__global__ void k_scale(T *x, int n, int mode, double val)
{
    Pend p;
    p.mode = mode;
    p.val = val;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = apply_pend(x[i], p);
}
// apply the deferred scale of u (which=0) or v (which=1) to its column now
template <typename T>
__global__ void k_apply_pend_col(LbCtl *ctl, T *U, int ldu, T *V, int ldv, int m, int n, int which, int *ok)
{
    const Pend p = which == 0 ? ctl->pend_u : ctl->pend_v;
    const int col = which == 0 ? ctl->pend_u_col : ctl->pend_v_col;
    if (p.mode != 0 && col >= 0) {
        if (ok && blockIdx.x == 0 && threadIdx.x == 0) ok[col] = 0;  // its FP32 planes are stale
        T *x = which == 0 ? U + (size_t)col * ldu : V + (size_t)col * ldv;
        const int len = which == 0 ? m : n;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x)
            x[i] = apply_pend(x[i], p);
    }
}
__global__ void k_clear_pend(LbCtl *ctl, int which)
{
    if (which == 0) ctl->pend_u.mode = 0;
    else ctl->pend_v.mode = 0;
}
template <typename TS, typename TD>
__global__ void k_convert(const TS *src, TD *dst, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = (TD)src[i];
}
// out[r] = sum over the first ncols columns of U (the warm start of the
// FP64 refinement: a vector in the span of the FP32 Ritz vectors)
template <typename T>
__global__ void k_sum_cols(const T *U, size_t ldu, int m, int ncols, double *out)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < ncols; c++) s += (double)U[(size_t)c * ldu + r];
        out[r] = s;
    }
}

// ------------------------------------------------------------- context
// The Ritz products for page-locked host arrays run in row chunks of about
// RITZ_CHUNK_ROWS (each far above the tensor-core GEMM's 4096-row minimum,
// so every chunk takes the same kernel and gives the same bits), so that
// the copy of a finished chunk to the host overlaps the next products.
constexpr int RITZ_CHUNK_ROWS = 1 << 19;
constexpr int RITZ_MAX_CHUNKS = 8;

struct Ctx {
    int m = 0, n = 0, kmax = 0, ldu = 0, ldv = 0, es = 8;
    int vw = 1;                             // real scalars per vector element (2: complex*16)
    cudaStream_t s = nullptr;
    void *U = nullptr, *V = nullptr;        // Lanczos vectors (double or float)
    LbCtl *ctl = nullptr;
    LbCtl *hctl = nullptr;  // pinned host copy
    double *balpha = nullptr, *bbeta = nullptr, *mu = nullptr, *nu = nullptr, *h = nullptr;
    double *part_sq = nullptr, *part_dot = nullptr, *part_cols = nullptr;
    int nb_spmv = 0;  // grid bound of the fused SpMV (spmv_grid_bound)
    int *index = nullptr, *sel = nullptr;
    void *xr = nullptr, *yr = nullptr;      // max(m,n) scratch of the vector type
    double *dx = nullptr, *dy = nullptr;    // max(m,n) FP64 scratch
    double *scal = nullptr;                 // device scalar slots
    double *hscal = nullptr;                // pinned host scalars
    // dense
    double *a1 = nullptr, *b1 = nullptr, *bnd = nullptr, *w = nullptr, *P = nullptr, *Q = nullptr;
    double *shifts = nullptr, *sig_out = nullptr, *bnd_out = nullptr, *anorm_drv = nullptr;
    int *nconv = nullptr;
    double *D = nullptr, *E = nullptr, *Mt = nullptr, *Pr = nullptr, *Qt = nullptr, *X = nullptr;
    double *wz = nullptr;                   // scratch of the lane-parallel bidiagonal kernels
    int *dflag = nullptr;
    void *gout = nullptr;                   // GEMM output scratch (vector type)
    // FP32 (hi, lo) planes of the FP64 bases for the Gram-Schmidt passes,
    // their per-column flags and the planes of the vector being
    // reorthogonalised (null: the FP64 or three-way-split kernels)
    float2 *Up = nullptr, *Vp = nullptr, *xpl = nullptr;
    int *okU = nullptr, *okV = nullptr;
    // operator
    const Operator *op = nullptr;
    propack_aprod_t aprod = nullptr;
    double *dparm = nullptr;
    int *iparm = nullptr;
    propack_zaprod_t zaprod = nullptr;      // complex*16 host APROD and its ZPARM
    propack_z16 *zparm = nullptr;
    double *hx = nullptr, *hy = nullptr;    // pinned host vectors for a host APROD
    int nb = 0;
    int ntry_spec = 2;
    int *hstat = nullptr;                   // pinned status words of the enqueue windows
    cudaEvent_t wev[2] = {nullptr, nullptr};
    std::vector<void *> allocs;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evs0 = nullptr, evs1 = nullptr;
    // the caller's page-locked U and V (set_host_out): dev_ritzvec forms
    // the Ritz vectors in row chunks and copies each finished chunk there on
    // s2 while the next chunks are formed on s; done[side] = columns copied
    char *hout[2] = {nullptr, nullptr};
    size_t hpitch[2] = {0, 0};
    int done[2] = {0, 0};
    cudaStream_t s2 = nullptr;
    cudaEvent_t ev_chunk[2][RITZ_MAX_CHUNKS] = {};
    cudaEvent_t ev_s2 = nullptr;

    // zero-filled device memory from the library's pool
    void *dbytes(size_t bytes)
    {
        void *p = dbytes_raw(bytes);
        PGB_CUDA(cudaMemsetAsync(p, 0, std::max<size_t>(bytes, 16), s));
        return p;
    }
    // device memory left as it is: only for arrays that are always written
    // before they are read
    void *dbytes_raw(size_t bytes)
    {
        bytes = std::max<size_t>(bytes, 16);
        void *p = pool_alloc(bytes, s);
        allocs.push_back(p);
        return p;
    }
    template <typename T>
    T *dalloc(size_t count) { return (T *)dbytes(sizeof(T) * count); }
    ~Ctx()
    {
        if (s2) cudaStreamSynchronize(s2);  // copies of Ritz chunks read pool memory
        if (s) {
            for (void *p : allocs) pool_free(p, s);
            cudaStreamSynchronize(s);
        }
        if (hctl) cudaFreeHost(hctl);
        if (hscal) cudaFreeHost(hscal);
        if (hstat) cudaFreeHost(hstat);
        for (cudaEvent_t e : wev)
            if (e) cudaEventDestroy(e);
        if (hx) cudaFreeHost(hx);
        if (hy) cudaFreeHost(hy);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (evs0) cudaEventDestroy(evs0);
        if (evs1) cudaEventDestroy(evs1);
        for (auto &side : ev_chunk)
            for (cudaEvent_t e : side)
                if (e) cudaEventDestroy(e);
        if (ev_s2) cudaEventDestroy(ev_s2);
        if (s2) cudaStreamDestroy(s2);
        if (s) cudaStreamDestroy(s);
    }
    LbArgs args() const
    {
        LbArgs a;
        a.ctl = ctl; a.U = U; a.V = V; a.ldu = ldu * vw; a.ldv = ldv * vw;
        a.balpha = balpha; a.bbeta = bbeta; a.mu = mu; a.nu = nu;
        a.index = index; a.sel = sel; a.h = h;
        a.part_sq = part_sq; a.part_dot = part_dot; a.part_cols = part_cols;
        a.nb = nb; a.kmax = kmax;
        a.nb_spmv = std::max(nb, nb_spmv);
        if (op && op->cplx == 2) {
            // a native complex operator: its own kernels read zfwd / zadj;
            // fwd and adj carry only the vector lengths in real scalars
            a.zfwd = op->fwd; a.zadj = op->adj;
            a.fwd.rows = m * vw; a.adj.rows = n * vw; a.z = nullptr;
        } else if (op) {
            a.fwd = op->fwd; a.adj = op->adj; a.z = op->zbuf;
        } else {
            a.fwd.rows = m * vw; a.adj.rows = n * vw; a.z = nullptr;
        }
        a.Up = Up; a.Vp = Vp; a.okU = okU; a.okV = okV; a.xpl = xpl;
        return a;
    }
    template <typename T>
    T *Ucol(int c) const { return (T *)U + (size_t)c * ldu; }
    template <typename T>
    T *Vcol(int c) const { return (T *)V + (size_t)c * ldv; }
    void sync() { PGB_CUDA(cudaStreamSynchronize(s)); }
    void get_ctl()
    {
        PGB_CUDA(cudaMemcpyAsync(hctl, ctl, sizeof(LbCtl), cudaMemcpyDeviceToHost, s));
        sync();
    }
    void put_ctl() { PGB_CUDA(cudaMemcpyAsync(ctl, hctl, sizeof(LbCtl), cudaMemcpyHostToDevice, s)); }
};

// CTAs of the vector kernels: about 2048 vector elements or 16384 nonzeros
// each, at most the four per SM that the partial-sum arrays hold.  A small
// problem then runs its many short kernels on a few CTAs instead of
// launching four per SM that mostly find no work.
static int vec_grid(int64_t elems, int64_t nnz)
{
    const int64_t cap = device_info().nb;
    const int64_t want = std::max((elems + 2047) / 2048, (nnz + 16383) / 16384);
    return (int)std::max<int64_t>(1, std::min(cap, want));
}
// CTAs the fused SpMV may use: one per 256 rows (a 32-row tile per warp),
// at most the four per SM that the partial-sum arrays hold.  The SpMV's
// latency chain (row bounds, indices, gathers) runs once per tile, so a
// small matrix wants its tiles spread over warps rather than its nonzeros
// over few CTAs.
static int spmv_grid_bound(int64_t rows)
{
    const int64_t cap = device_info().nb;
    return (int)std::max<int64_t>(1, std::min(cap, (rows + 255) / 256));
}

template <typename T>
static void init_ctx(Ctx &c, int m, int n, int kmax)
{
    const Dev &d = device_info();
    c.m = m; c.n = n; c.kmax = kmax; c.es = (int)sizeof(T);
    c.vw = VecW<T>::w;
    c.ldu = (m + 31) / 32 * 32;
    c.ldv = (n + 31) / 32 * 32;
    c.nb = d.nb;
    PGB_CUDA(cudaStreamCreateWithFlags(&c.s, cudaStreamNonBlocking));
    PGB_CUDA(cudaEventCreate(&c.ev0));
    PGB_CUDA(cudaEventCreate(&c.ev1));
    PGB_CUDA(cudaEventCreate(&c.evs0));
    PGB_CUDA(cudaEventCreate(&c.evs1));
    c.U = c.dalloc<T>((size_t)c.ldu * (kmax + 1));
    c.V = c.dalloc<T>((size_t)c.ldv * (kmax + 1));
    c.ctl = c.dalloc<LbCtl>(1);
    PGB_CUDA(cudaMallocHost(&c.hctl, sizeof(LbCtl)));
    memset(c.hctl, 0, sizeof(LbCtl));
    c.balpha = c.dalloc<double>(kmax + 2);
    c.bbeta = c.dalloc<double>(kmax + 2);
    c.mu = c.dalloc<double>(kmax + 2);
    c.nu = c.dalloc<double>(kmax + 2);
    c.h = c.dalloc<double>((size_t)(kmax + 2) * c.vw);
    c.part_sq = c.dalloc<double>(c.nb);
    c.part_dot = c.dalloc<double>(c.nb);
    c.part_cols = c.dalloc<double>((size_t)c.nb * (kmax + 2) * c.vw);
    c.index = c.dalloc<int>(2 * (size_t)kmax + 8);
    c.sel = c.dalloc<int>(kmax + 2);
    const int mn = std::max(m, n);
    c.xr = c.dalloc<T>(mn);
    c.yr = c.dalloc<T>(mn);
    c.dx = c.dalloc<double>(mn);
    c.dy = c.dalloc<double>(mn);
    c.scal = c.dalloc<double>(8);
    PGB_CUDA(cudaMallocHost(&c.hscal, sizeof(double) * 8));
    PGB_CUDA(cudaMallocHost(&c.hstat, sizeof(int) * 2));
    c.hstat[0] = c.hstat[1] = 0;
    for (cudaEvent_t &e : c.wev) PGB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    const size_t d1 = kmax + 2;
    c.a1 = c.dalloc<double>(d1); c.b1 = c.dalloc<double>(d1); c.bnd = c.dalloc<double>(d1);
    c.w = c.dalloc<double>(4 * d1);
    c.wz = c.dalloc<double>(bidiag_scratch(kmax));
    c.dflag = c.dalloc<int>(4);
    c.P = c.dalloc<double>(d1 * d1); c.Q = c.dalloc<double>(d1 * d1);
    c.shifts = c.dalloc<double>(d1);
    c.sig_out = c.dalloc<double>(d1); c.bnd_out = c.dalloc<double>(d1);
    c.anorm_drv = c.dalloc<double>(1);
    c.nconv = c.dalloc<int>(1);
    c.D = c.dalloc<double>(d1); c.E = c.dalloc<double>(d1);
    c.Mt = c.dalloc<double>(d1 * d1); c.Pr = c.dalloc<double>(d1 * d1); c.Qt = c.dalloc<double>(d1 * d1);
    c.X = c.dalloc<double>(d1 * d1);
    // the restart/Ritz product's output: written by the GEMM before it is read
    c.gout = c.dbytes_raw(sizeof(T) * (size_t)std::max(c.ldu, c.ldv) * (kmax + 1));
    // the partial-sum arrays above hold d.nb CTAs; the grid follows the size
    c.nb = vec_grid((int64_t)std::max(m, n) * c.vw, 0);
    constexpr bool fp64 = std::is_same<T, double>::value || std::is_same<T, double2>::value;
    if (fp64 && g_cgs_arith == CGS_PLANES && lb_planes_fit(kmax, c.vw == 2)) {
        // planes of every real scalar (complex: of re and im); written (flag
        // set) before any kernel reads them
        c.Up = (float2 *)c.dbytes_raw(sizeof(float2) * (size_t)c.ldu * c.vw * (kmax + 1));
        c.Vp = (float2 *)c.dbytes_raw(sizeof(float2) * (size_t)c.ldv * c.vw * (kmax + 1));
        c.xpl = c.dalloc<float2>((size_t)mn * c.vw);
        c.okU = c.dalloc<int>(kmax + 2);
        c.okV = c.dalloc<int>(kmax + 2);
    }
    lb_set_smem_limits(kmax);
}

// ----------------------------------------------------- device utilities
template <typename T>
static double dev_nrm2(Ctx &c, const T *x, int n)
{
    if constexpr (VecW<T>::w == 2) {
        return dev_nrm2<double>(c, (const double *)x, 2 * n);
    } else {
        k_sumsq_part<T><<<c.nb, BS, 0, c.s>>>(x, n, c.part_sq);
        PGB_LAUNCHED();
        k_sum_final<<<1, BS, 0, c.s>>>(c.part_sq, c.nb, c.scal);
        PGB_LAUNCHED();
        PGB_CUDA(cudaMemcpyAsync(c.hscal, c.scal, sizeof(double), cudaMemcpyDeviceToHost, c.s));
        c.sync();
        return std::sqrt(c.hscal[0]);
    }
}
template <typename T>
static void dev_scale(Ctx &c, T *x, int n, int mode, double val)
{
    if constexpr (VecW<T>::w == 2) {
        dev_scale<double>(c, (double *)x, 2 * n, mode, val);
    } else {
        if (mode == 0 || n <= 0) return;
        k_scale<T><<<c.nb, 256, 0, c.s>>>(x, n, mode, val);
        PGB_LAUNCHED();
    }
}
// dsafescal on the device
template <typename T>
static void dev_safescal(Ctx &c, T *x, int n, double alpha)
{
    if (std::fabs(alpha) >= SFMIN) dev_scale<T>(c, x, n, 1, 1.0 / alpha);
    else dev_scale<T>(c, x, n, 2, alpha);
}
template <typename TS, typename TD>
static void dev_convert(Ctx &c, const TS *src, TD *dst, int n)
{
    k_convert<TS, TD><<<c.nb, 256, 0, c.s>>>(src, dst, n);
    PGB_LAUNCHED();
}

// y = op(A) x on device vectors, through the device operator or the
// caller's host APROD (which sees FP64 host vectors)
template <typename T>
static void dev_aprod(Ctx &c, bool trans, const T *x, T *y)
{
    const int nin = trans ? c.m : c.n, nout = trans ? c.n : c.m;
    if constexpr (VecW<T>::w == 2) {
        // the device operator (native, or the real 2x2-block form); a host
        // ZAPROD sees complex*16 vectors with TRANSA 'n' or 'c'
        // (zlanbpro.F:297, :442)
        if (c.op) {
            op_zapply(*c.op, trans, (const double2 *)x, (double2 *)y, c.s);
            return;
        }
        PGB_CUDA(cudaMemcpyAsync(c.hx, x, sizeof(T) * nin, cudaMemcpyDeviceToHost, c.s));
        c.sync();
        const char ta = trans ? 'c' : 'n';
        c.zaprod(&ta, &c.m, &c.n, (const propack_z16 *)c.hx, (propack_z16 *)c.hy, c.zparm, c.iparm, 1);
        PGB_CUDA(cudaMemcpyAsync(y, c.hy, sizeof(T) * nout, cudaMemcpyHostToDevice, c.s));
    } else {
        if (c.op) {
            op_apply<T>(*c.op, trans, x, y, c.s);
            return;
        }
        const double *xd = (const double *)x;
        if (sizeof(T) != sizeof(double)) {
            dev_convert<T, double>(c, x, c.dx, nin);
            xd = c.dx;
        }
        PGB_CUDA(cudaMemcpyAsync(c.hx, xd, sizeof(double) * nin, cudaMemcpyDeviceToHost, c.s));
        c.sync();
        const char ta = trans ? 't' : 'n';
        c.aprod(&ta, &c.m, &c.n, c.hx, c.hy, c.dparm, c.iparm, 1);
        if (sizeof(T) != sizeof(double)) {
            PGB_CUDA(cudaMemcpyAsync(c.dy, c.hy, sizeof(double) * nout, cudaMemcpyHostToDevice, c.s));
            dev_convert<double, T>(c, c.dy, y, nout);
        } else {
            PGB_CUDA(cudaMemcpyAsync((double *)y, c.hy, sizeof(double) * nout, cudaMemcpyHostToDevice, c.s));
        }
    }
}

// dreorth against all of W(:,0:kk) (index = [1, kk, kk+1]), iterated CGS;
// host-driven (resume prologue and dgetu0 only)
template <typename T>
static void dev_reorth_full(Ctx &c, const T *W, size_t ld, int len, int kk, T *x, double *nrm, double kappa)
{
    if (kk <= 0 || len <= 0) return;
    for (int itry = 0; itry < NTRY; itry++) {
        const double nrm0 = *nrm;
        if constexpr (VecW<T>::w == 2) {
            k_zgemvt_part<<<c.nb, BS, 0, c.s>>>(W, ld, len, kk, x, c.part_cols);
            PGB_LAUNCHED();
            k_gemvt_final<<<1, BS, 0, c.s>>>(c.part_cols, c.nb, 2 * kk, c.h);
            PGB_LAUNCHED();
            k_zgemvn_upd<<<c.nb, BS, 0, c.s>>>(W, ld, len, kk, c.h, x);
            PGB_LAUNCHED();
        } else {
            k_gemvt_part<T><<<c.nb, BS, 0, c.s>>>(W, ld, len, kk, x, c.part_cols);
            PGB_LAUNCHED();
            k_gemvt_final<<<1, BS, 0, c.s>>>(c.part_cols, c.nb, kk, c.h);
            PGB_LAUNCHED();
            k_gemvn_upd<T><<<c.nb, BS, 0, c.s>>>(W, ld, len, kk, c.h, x);
            PGB_LAUNCHED();
        }
        g_last.ndot += 2 * (int64_t)kk;
        *nrm = dev_nrm2<T>(c, x, len);
        if (*nrm > kappa * nrm0) { g_last.nreorth++; return; }
    }
    *nrm = 0.0;
    dev_scale<T>(c, x, len, 3, 0.0);
    g_last.nreorth++;
}

// dgetu0 (double/dgetu0.F:11-89): a random vector in span(op(A)) orthogonal
// to the first j columns of W; returns u0norm, anormest, ierr.
template <typename T>
static int dev_getu0(Ctx &c, bool trans, int j, int ntry, T *u0, double *u0norm, const T *W, size_t ld,
                     double *anormest)
{
    const unsigned long long seed = (1ull << 36) | (3ull << 24) | (5ull << 12) | 7ull;
    const int rsize = trans ? c.m : c.n, usize = trans ? c.n : c.m;
    T *xr = (T *)c.xr;
    for (int itry = 0; itry < ntry; itry++) {
        // complex: zlarnv(2) draws the real and imaginary parts as 2 rsize
        // consecutive values of the same stream
        const int nval = rsize * VecW<T>::w;
        const int nch = (nval + 63) / 64;
        using E = typename std::conditional<VecW<T>::w == 2, double, T>::type;
        k_rng_pm1<E><<<std::max(1, std::min(c.nb, (nch + 255) / 256)), 256, 0, c.s>>>((E *)xr, nval, seed,
                                                                                      (long long)itry * nval);
        PGB_LAUNCHED();
        const double nrm = dev_nrm2<T>(c, xr, rsize);
        dev_aprod<T>(c, trans, xr, u0);
        g_last.nopx++;
        *u0norm = dev_nrm2<T>(c, u0, usize);
        *anormest = *u0norm / nrm;
        // dgetu0.F:30 has a REAL literal, zgetu0.F:30 a DOUBLE one
        if (j >= 1) dev_reorth_full<T>(c, W, ld, usize, j, u0, u0norm, VecW<T>::w == 2 ? KAPPA : KAPPA_GETU0);
        if (*u0norm > 0) return 0;
    }
    return -1;
}

// the deferred scale of u (which=0) or v (which=1) applied to its column
template <typename T>
static void apply_pend_col(Ctx &c, int which)
{
    using E = typename std::conditional<VecW<T>::w == 2, double, T>::type;
    const int w = VecW<T>::w;
    k_apply_pend_col<E><<<c.nb, 256, 0, c.s>>>(c.ctl, (E *)c.U, c.ldu * w, (E *)c.V, c.ldv * w, c.m * w, c.n * w,
                                               which, which == 0 ? c.okU : c.okV);
    PGB_LAUNCHED();
}

// ------------------------------------------------------------ dlanbpro
struct LbResult {
    int ierr;
};

// Run dlanbpro (double/dlanbpro.F:1-549) from k0 to *kp on the device.
template <typename T>
static void dev_lanbpro(Ctx &c, int k0, int *kp, double *rnorm, double *doption, const int *ioption, int *ierr)
{
    const int m = c.m, n = c.n;
    int k = *kp;
    LbCtl &h = *c.hctl;
    // the device holds the authoritative control block between calls;
    // refresh the host copy (counters, pending scales)
    c.get_ctl();
    const int mn = std::max(m, n);
    h.m = m; h.n = n; h.k = k; h.ldu = c.ldu * c.vw; h.ldv = c.ldv * c.vw;
    h.icgs = ioption[0]; h.ielr = ioption[1];
    h.cplx = VecW<T>::w == 2;
    h.elr_need_dot = 0;
    // machine constants of the Lanczos vectors (FP32 vectors: eps = 2^-24)
    constexpr bool f32 = std::is_same<T, float>::value;
    const double eps = !f32 ? EPS : 5.9604644775390625e-08;
    h.eps_vec = eps;
    // the breakdown level of alpha/beta: max(m,n)*eps in FP64 (as the
    // reference); with FP32 vectors that worst-case bound reaches ~0.2*||A||
    // at a few million rows, so the FP32 level is the statistical
    // sqrt(max(m,n))*eps (2^-24), which still sits far above the rounding noise
    // of an FP32 product with compensated norms
    h.epsn = !f32 ? (double)mn * eps : std::sqrt((double)mn) * eps;
    h.epsn2 = std::sqrt((double)mn) * eps;
    h.delta = doption[0] < 0 ? std::sqrt(eps / k) : doption[0];
    h.eta = doption[1] < 0 ? std::pow(eps, 0.75) / std::sqrt((double)k) : doption[1];
    h.full_reorth = (h.delta <= h.eta || h.delta == 0.0);
    h.status = 0;
    h.elr_active = 0;
    h.reorth_active = 0;
    h.collapsed = 0;
    double anorm;
    std::vector<double> hb(2 * (size_t)(k + 2), 0.0);
    if (k0 > 0) {
        PGB_CUDA(cudaMemcpyAsync(hb.data(), c.balpha, sizeof(double) * k0, cudaMemcpyDeviceToHost, c.s));
        PGB_CUDA(cudaMemcpyAsync(hb.data() + k + 2, c.bbeta, sizeof(double) * k0, cudaMemcpyDeviceToHost, c.s));
        c.sync();
    }
    double *ba = hb.data(), *bb = hb.data() + k + 2;
    if (doption[2] > 0) {
        anorm = doption[2];
    } else if (k0 > 0) {
        anorm = std::hypot(ba[0], bb[0]);
        if (anorm <= 0) { *ierr = -1; doption[2] = anorm; return; }
    } else {
        anorm = 0.0;
    }
    *ierr = 0;
    PGB_CUDA(cudaMemsetAsync(c.mu, 0, sizeof(double) * (k + 2), c.s));
    PGB_CUDA(cudaMemsetAsync(c.nu, 0, sizeof(double) * (k + 2), c.s));
    PGB_CUDA(cudaMemsetAsync(c.index, 0, sizeof(int) * (2 * (size_t)k + 4), c.s));
    double anormest = 0.0;
    if (*rnorm == 0.0) {
        int e = dev_getu0<T>(c, false, k0, 3, c.Ucol<T>(k0), rnorm, (T *)c.U, c.ldu, &anormest);
        *ierr = e;
        anorm = std::max(anorm, anormest);
    }
    int j0;
    h.pend_u.mode = 0; h.pend_v.mode = 0; h.pend_u_col = -1; h.pend_v_col = -1;
    if (k0 == 0) {
        h.amax = 0.0;
        h.alpha = 0.0;
        h.beta = *rnorm;
        h.force_reorth = 0;
        double s;
        int e;
        if (n > m) e = dev_getu0<T>(c, false, 0, 1, (T *)c.yr, &s, (T *)c.U, c.ldu, &anormest);
        else e = dev_getu0<T>(c, true, 0, 1, (T *)c.yr, &s, (T *)c.V, c.ldv, &anormest);
        *ierr = e;
        anorm = std::max(anorm, FUDGE * anormest);
        j0 = 1;
        if (h.beta != 0.0) {
            // deferred dsafescal of u_1
            if (std::fabs(h.beta) >= SFMIN) { h.pend_u.mode = 1; h.pend_u.val = 1.0 / h.beta; }
            else { h.pend_u.mode = 2; h.pend_u.val = h.beta; }
            h.pend_u_col = 0;
        }
        const double one = 1.0;
        PGB_CUDA(cudaMemcpyAsync(c.mu, &one, sizeof(double), cudaMemcpyHostToDevice, c.s));
        PGB_CUDA(cudaMemcpyAsync(c.nu, &one, sizeof(double), cudaMemcpyHostToDevice, c.s));
    } else {
        h.force_reorth = 1;
        h.alpha = ba[k0 - 1];
        h.beta = *rnorm;
        if (k0 < k && h.beta * h.delta < anorm * eps) { h.full_reorth = 1; *ierr = k0; }
        const int idx3[3] = {1, k0, k0 + 1};
        PGB_CUDA(cudaMemcpyAsync(c.index, idx3, sizeof(idx3), cudaMemcpyHostToDevice, c.s));
        T *uk = c.Ucol<T>(k0);
        dev_scale<T>(c, uk, m, 1, *rnorm);
        dev_reorth_full<T>(c, (T *)c.U, c.ldu, m, k0, uk, rnorm, KAPPA);
        dev_safescal<T>(c, uk, m, *rnorm);
        std::vector<double> mus(k0, h.epsn2);
        PGB_CUDA(cudaMemcpyAsync(c.mu, mus.data(), sizeof(double) * k0, cudaMemcpyHostToDevice, c.s));
        PGB_CUDA(cudaMemcpyAsync(c.nu, mus.data(), sizeof(double) * k0, cudaMemcpyHostToDevice, c.s));
        h.beta = *rnorm;
        bb[k0 - 1] = h.beta;
        PGB_CUDA(cudaMemcpyAsync(c.bbeta + k0 - 1, &bb[k0 - 1], sizeof(double), cudaMemcpyHostToDevice, c.s));
        h.amax = 0.0;
        for (int j = 1; j <= k0; j++) {
            h.amax = std::max(h.amax, std::max(ba[j - 1], bb[j - 1]));
            double a1, b1;
            if (j == 1) {
                anorm = std::max(anorm, FUDGE * h.alpha);
            } else if (j == 2) {
                a1 = bb[0] / h.amax;
                a1 = FUDGE * h.amax * std::sqrt((ba[0] / h.amax) * (ba[0] / h.amax) + a1 * a1 + ba[1] / h.amax * a1);
                anorm = std::max(anorm, a1);
            } else {
                a1 = ba[j - 2] / h.amax;
                b1 = bb[j - 2] / h.amax;
                a1 = FUDGE * h.amax * std::sqrt(a1 * a1 + b1 * b1 + a1 * bb[j - 3] / h.amax + ba[j - 1] / h.amax * b1);
                anorm = std::max(anorm, a1);
            }
        }
        j0 = k0 + 1;
    }
    h.anorm = anorm;
    h.numax = 0.0;
    h.mumax = 0.0;
    h.rnorm = *rnorm;
    h.ierr = *ierr;
    h.j = j0;
    h.ticket = 0;
    c.put_ctl();

    // the step loop: enqueue everything, then look for a suspension
    const bool host_ap = (c.op == nullptr);
    int j = j0, side = 0;
    bool finished = false;
    int rounds = 0;
    while (!finished) {
        if (++rounds > 4 * (k + 2)) {
            set_error("dlanbpro: too many suspensions");
            throw WaitFailure();
        }
        LbArgs a = c.args();
        // the host may have written columns since the last round (start
        // vector, prologue, a suspension's fresh vector): no plane is trusted
        if (c.okU) {
            PGB_CUDA(cudaMemsetAsync(c.okU, 0, sizeof(int) * (c.kmax + 2), c.s));
            PGB_CUDA(cudaMemsetAsync(c.okV, 0, sizeof(int) * (c.kmax + 2), c.s));
        }
        if (!host_ap) {
            // enqueue in windows of LB_WINDOW steps; before a window goes in,
            // the status word of the window two back is read (its copy was
            // queued behind it), so at most two windows of launches are
            // wasted when a step suspends, and the device never runs dry
            int wnum = 0;
            while (j <= k) {
                if (wnum >= 2) {
                    PGB_CUDA(cudaEventSynchronize(c.wev[wnum & 1]));
                    if (c.hstat[wnum & 1] != 0) break;
                }
                const int jend = std::min(k, j + LB_WINDOW - 1);
                for (; j <= jend; j++) {
                    for (; side < 2; side++) lb_enqueue_half<T>(a, c.op, side, j, h.ielr, c.ntry_spec, false, c.s);
                    side = 0;
                }
                PGB_CUDA(cudaMemcpyAsync(&c.hstat[wnum & 1], &c.ctl->status, sizeof(int), cudaMemcpyDeviceToHost,
                                         c.s));
                PGB_CUDA(cudaEventRecord(c.wev[wnum & 1], c.s));
                wnum++;
            }
            c.get_ctl();
        } else {
            // host APROD: one synchronous product per half step
            bool susp = false;
            for (; j <= k && !susp; j++) {
                for (; side < 2 && !susp; side++) {
                    T *x = side == 0 ? c.Ucol<T>(j - 1) : c.Vcol<T>(j - 1);
                    T *y = side == 0 ? c.Vcol<T>(j - 1) : c.Ucol<T>(j);
                    // the product must see the scaled input
                    apply_pend_col<T>(c, side == 0 ? 0 : 1);
                    k_clear_pend<<<1, 1, 0, c.s>>>(c.ctl, side == 0 ? 0 : 1);
                    PGB_LAUNCHED();
                    dev_aprod<T>(c, side == 0, x, y);
                    lb_enqueue_half<T>(a, nullptr, side, j, h.ielr, c.ntry_spec, true, c.s);
                    c.get_ctl();
                    if (h.status != 0) susp = true;
                    if (susp) break;
                }
                if (susp) break;
                side = 0;
            }
            if (!susp) c.get_ctl();
        }
        if (h.status == 0) {
            finished = true;
            break;
        }
        // ---- a suspension: finish the case on the host side, then resume
        const int sj = h.susp_j, ss = h.susp_side;
        if (trace_on())
            fprintf(stderr, "[propack_gb300] lanbpro suspension: reason %d step %d side %c alpha %.3e beta %.3e anorm %.3e\n",
                    h.susp_reason, sj, ss == 0 ? 'v' : 'u', h.alpha, h.beta, h.anorm);
        if (h.susp_reason == 2) {
            h.status = 0;
            c.put_ctl();
            lb_enqueue_cgs_more<T>(c.args(), ss, sj, NTRY - c.ntry_spec, c.s);
            c.get_ctl();
            if (h.status != 0 && h.susp_reason == 2) {
                set_error("reorthogonalisation did not finish within NTRY passes");
                throw WaitFailure();
            }
            if (h.status == 0) {
                // continue after the finished half step
                if (ss == 0) { j = sj; side = 1; }
                else { j = sj + 1; side = 0; }
                continue;
            }
            // fell into an invariant-subspace suspension: handled below
        }
        if (h.susp_reason != 1) {
            set_error("device control block reports an unknown suspension");
            throw WaitFailure();
        }
        if (h.susp_reason == 1) {
            const int jj = h.susp_j;
            h.status = 0;
            if (h.susp_side == 0) {
                // dlanbpro.F:372-405: new random v_j orthogonal to V(:,1:j-1)
                // (u_j may still carry its deferred scale: apply it first)
                c.put_ctl();
                apply_pend_col<T>(c, 0);
                k_clear_pend<<<1, 1, 0, c.s>>>(c.ctl, 0);
                PGB_LAUNCHED();
                c.get_ctl();
                double alpha = 0.0;
                T *vj = c.Vcol<T>(jj - 1);
                int e = dev_getu0<T>(c, true, jj - 1, 3, vj, &alpha, (T *)c.V, c.ldv, &anormest);
                h.ierr = e;
                if (alpha == 0.0) {
                    k = jj - 1;
                    h.ierr = -jj;
                    c.put_ctl();
                    finished = true;
                    break;
                }
                dev_safescal<T>(c, vj, n, alpha);
                h.alpha = 0.0;
                h.force_reorth = 1;
                if (h.delta > 0) h.full_reorth = 0;
                const double z0 = 0.0;
                PGB_CUDA(cudaMemcpyAsync(c.balpha + jj - 1, &z0, sizeof(double), cudaMemcpyHostToDevice, c.s));
                h.pend_v.mode = 0;
                h.pend_v_col = jj - 1;
                c.put_ctl();
                j = jj; side = 1;
            } else {
                // dlanbpro.F:503-535: new random u_{j+1} orthogonal to U(:,1:j)
                c.put_ctl();
                apply_pend_col<T>(c, 1);
                k_clear_pend<<<1, 1, 0, c.s>>>(c.ctl, 1);
                PGB_LAUNCHED();
                c.get_ctl();
                double beta = 0.0;
                T *uj1 = c.Ucol<T>(jj);
                int e = dev_getu0<T>(c, false, jj, 3, uj1, &beta, (T *)c.U, c.ldu, &anormest);
                h.ierr = e;
                if (beta == 0.0) {
                    k = jj;
                    h.ierr = -jj;
                    c.put_ctl();
                    finished = true;
                    break;
                }
                dev_safescal<T>(c, uj1, m, beta);
                h.beta = 0.0;
                h.force_reorth = 1;
                if (h.delta > 0) h.full_reorth = 0;
                const double z0 = 0.0;
                PGB_CUDA(cudaMemcpyAsync(c.bbeta + jj - 1, &z0, sizeof(double), cudaMemcpyHostToDevice, c.s));
                h.pend_u.mode = 0;
                h.pend_u_col = jj;
                h.rnorm = 0.0;
                c.put_ctl();
                j = jj + 1; side = 0;
            }
            continue;
        }
    }
    // apply the deferred scaling of the newest columns
    lb_enqueue_flush<T>(c.args(), c.s);
    c.get_ctl();
    *kp = k;
    *rnorm = h.rnorm;
    *ierr = h.ierr;
    doption[2] = h.anorm;
}

// ------------------------------------------------------------- drivers
static inline bool yes(const char *c) { return c && (c[0] == 'y' || c[0] == 'Y'); }

// precision of the Lanczos vectors for this host thread: 0 = FP64 (the
// reference's method), 1 = mixed (FP32 vectors and FP64 scalars, then a
// short FP64 refinement)
static thread_local int g_precision = 0;
constexpr double EPS32 = 5.9604644775390625e-08;
constexpr double MIXED_TOL = 1e-6;  // convergence level of the FP32 phase

// ---------------------------------------- results to pageable host memory
// A caller's U and V are often ordinary (pageable) arrays: a Fortran
// program's arrays, numpy's.  A device-to-pageable cudaMemcpy goes through
// the driver's own staging and the first touch of each destination page on
// one thread; here such copies go through a pinned bounce buffer of two
// BOUNCE_BYTES halves instead: one cudaMemcpy2DAsync per chunk of whole
// columns into one half while host threads copy the previous chunk out of
// the other half in parallel.

// A small pool of host threads for the copies out of the bounce buffer.
class HostPool {
public:
    static HostPool &get()
    {
        static HostPool p;
        return p;
    }
    // run f(i) for i in [0, n) on the pool and the calling thread; returns
    // when all are done (one job at a time: concurrent callers take turns)
    void run(int n, const std::function<void(int)> &f)
    {
        if (n <= 1 || workers_.empty()) {
            for (int i = 0; i < n; i++) f(i);
            return;
        }
        std::lock_guard<std::mutex> one(run_mu_);
        std::unique_lock<std::mutex> lk(mu_);
        job_ = &f;
        njob_ = n;
        next_ = 0;
        done_ = 0;
        ++gen_;
        cv_.notify_all();
        lk.unlock();
        work();
        lk.lock();
        done_cv_.wait(lk, [&] { return done_ == njob_; });
        job_ = nullptr;
    }
    int threads() const { return (int)workers_.size() + 1; }

private:
    HostPool()
    {
        const unsigned hc = std::thread::hardware_concurrency();
        const int nt = (int)std::min(16u, std::max(1u, hc)) - 1;
        for (int i = 0; i < nt; i++) workers_.emplace_back([this] { loop(); });
    }
    ~HostPool()
    {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
            cv_.notify_all();
        }
        for (auto &t : workers_) t.join();
    }
    void work()
    {
        for (;;) {
            int i;
            const std::function<void(int)> *f;
            {
                std::lock_guard<std::mutex> lk(mu_);
                if (!job_ || next_ >= njob_) return;
                i = next_++;
                f = job_;
            }
            (*f)(i);
            std::lock_guard<std::mutex> lk(mu_);
            if (++done_ == njob_) done_cv_.notify_all();
        }
    }
    void loop()
    {
        long long seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
            }
            work();
        }
    }
    std::vector<std::thread> workers_;
    std::mutex run_mu_, mu_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(int)> *job_ = nullptr;
    int njob_ = 0, next_ = 0, done_ = 0;
    long long gen_ = 0;
    bool stop_ = false;
};

constexpr size_t BOUNCE_BYTES = (size_t)64 << 20;

// bounce buffers (two halves of BOUNCE_BYTES, pinned) and their events,
// kept in a process-wide free list: a copy takes one for its duration, so
// there are as many as copies ever ran at once; propack_release_memory()
// frees the idle ones
struct Bounce {
    char *buf = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
};
static std::mutex g_bounce_mu;
static std::vector<Bounce> g_bounce_free;
struct BounceLease {
    Bounce b;
    BounceLease()
    {
        {
            std::lock_guard<std::mutex> lk(g_bounce_mu);
            if (!g_bounce_free.empty()) {
                b = g_bounce_free.back();
                g_bounce_free.pop_back();
                return;
            }
        }
        PGB_CUDA(cudaMallocHost(&b.buf, 2 * BOUNCE_BYTES));
        for (cudaEvent_t &e : b.ev) PGB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    ~BounceLease()
    {
        std::lock_guard<std::mutex> lk(g_bounce_mu);
        g_bounce_free.push_back(b);
    }
};
void release_bounce_buffers()
{
    std::lock_guard<std::mutex> lk(g_bounce_mu);
    for (Bounce &b : g_bounce_free) {
        cudaFreeHost(b.buf);
        for (cudaEvent_t e : b.ev) cudaEventDestroy(e);
    }
    g_bounce_free.clear();
}

// host memory the GPU's copy engines can reach directly (page-locked or
// registered, or managed)
static bool host_pinned(const void *p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type != cudaMemoryTypeUnregistered;
}

// ncols columns of `colbytes` bytes from device src (pitch spitch) to host
// dst (pitch dpitch): straight when dst is pinned, through the bounce
// buffer otherwise
static void d2h_columns(char *dst, size_t dpitch, const char *src, size_t spitch, size_t colbytes, int ncols,
                        cudaStream_t s)
{
    if (ncols <= 0 || colbytes == 0) return;
    if (host_pinned(dst)) {
        PGB_CUDA(cudaMemcpy2DAsync(dst, dpitch, src, spitch, colbytes, ncols, cudaMemcpyDeviceToHost, s));
        return;
    }
    BounceLease lease;
    Bounce &b = lease.b;
    HostPool &pool = HostPool::get();
    // pieces: whole columns per chunk, or slices of one column when a column exceeds a half
    struct Piece {
        int c0, nc;
        size_t off, bytes;  // within the column (nc == 1 slices) or whole columns
    };
    std::vector<Piece> pieces;
    if (colbytes <= BOUNCE_BYTES) {
        const int per = (int)std::max<size_t>(1, BOUNCE_BYTES / colbytes);
        for (int c0 = 0; c0 < ncols; c0 += per) pieces.push_back({c0, std::min(per, ncols - c0), 0, colbytes});
    } else {
        for (int c = 0; c < ncols; c++)
            for (size_t off = 0; off < colbytes; off += BOUNCE_BYTES)
                pieces.push_back({c, 1, off, std::min(BOUNCE_BYTES, colbytes - off)});
    }
    auto issue = [&](size_t i) {
        const Piece &p = pieces[i];
        char *half = b.buf + (i & 1) * BOUNCE_BYTES;
        PGB_CUDA(cudaMemcpy2DAsync(half, p.bytes, src + (size_t)p.c0 * spitch + p.off, spitch, p.bytes, p.nc,
                                   cudaMemcpyDeviceToHost, s));
        PGB_CUDA(cudaEventRecord(b.ev[i & 1], s));
    };
    auto drain = [&](size_t i) {
        const Piece &p = pieces[i];
        PGB_CUDA(cudaEventSynchronize(b.ev[i & 1]));
        const char *half = b.buf + (i & 1) * BOUNCE_BYTES;
        const size_t total = p.bytes * p.nc;
        const int parts = (int)std::min<size_t>((size_t)pool.threads() * 2, std::max<size_t>(1, total >> 20));
        const size_t step = (total + parts - 1) / parts;
        pool.run(parts, [&](int q) {
            size_t a = (size_t)q * step, e = std::min(total, a + step);
            while (a < e) {
                const size_t col = a / p.bytes, within = a % p.bytes;
                const size_t len = std::min(e - a, p.bytes - within);
                memcpy(dst + (p.c0 + col) * dpitch + p.off + within, half + a, len);
                a += len;
            }
        });
    };
    issue(0);
    for (size_t i = 0; i < pieces.size(); i++) {
        if (i + 1 < pieces.size()) issue(i + 1);  // the other half is free: piece i-1 was drained
        drain(i);
    }
}

// bytes from host src to device dst on stream s: straight when src is
// pinned (or small); otherwise through the bounce buffer, each 64 MB piece
// copied into a half by the host pool while the other half's copy to the
// device runs.  Returns when the buffer is free again (its last copies
// done); the device copies are ordered on s.
void h2d_bytes(void *dst, const void *src, size_t bytes, cudaStream_t s)
{
    if (bytes == 0) return;
    if (bytes < ((size_t)4 << 20) || host_pinned(src)) {
        PGB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
        return;
    }
    BounceLease lease;
    Bounce &b = lease.b;
    HostPool &pool = HostPool::get();
    const size_t np = (bytes + BOUNCE_BYTES - 1) / BOUNCE_BYTES;
    for (size_t i = 0; i < np; i++) {
        const size_t off = i * BOUNCE_BYTES, len = std::min(BOUNCE_BYTES, bytes - off);
        char *half = b.buf + (i & 1) * BOUNCE_BYTES;
        if (i >= 2) PGB_CUDA(cudaEventSynchronize(b.ev[i & 1]));  // piece i-2 has left this half
        const int parts = (int)std::min<size_t>((size_t)pool.threads() * 2, std::max<size_t>(1, len >> 20));
        const size_t step = (len + parts - 1) / parts;
        const char *from = (const char *)src + off;
        pool.run(parts, [&](int q) {
            const size_t a = (size_t)q * step, e = std::min(len, a + step);
            if (a < e) memcpy(half + a, from + a, e - a);
        });
        PGB_CUDA(cudaMemcpyAsync((char *)dst + off, half, len, cudaMemcpyHostToDevice, s));
        PGB_CUDA(cudaEventRecord(b.ev[i & 1], s));
    }
    for (size_t h = 0; h < 2 && h < np; h++) PGB_CUDA(cudaEventSynchronize(b.ev[h]));
}

template <typename T>
static void copy_out(Ctx &c, double *U, int ldu, double *V, int ldv, int ncols, bool du, bool dv)
{
    if (ncols <= 0) return;
    if constexpr (std::is_same<T, float>::value) {
        // FP32 bases: widen column by column through the FP64 scratch
        for (int side = 0; side < 2; side++) {
            if (side == 0 ? !du : !dv) continue;
            const int rows = side == 0 ? c.m : c.n;
            double *H = side == 0 ? U : V;
            const int ldh = side == 0 ? ldu : ldv;
            for (int col = 0; col < ncols; col++) {
                const T *src = side == 0 ? c.Ucol<T>(col) : c.Vcol<T>(col);
                dev_convert<T, double>(c, src, c.dx, rows);
                PGB_CUDA(cudaMemcpyAsync(H + (size_t)col * ldh, c.dx, sizeof(double) * rows, cudaMemcpyDeviceToHost,
                                         c.s));
            }
        }
        return;
    } else {
    // FP64 or complex*16 (sizeof(T) = 16) bases into the caller's arrays;
    // the sides dev_ritzvec already copied chunk by chunk (on s2) are done
    // once s2 is
    if (du && c.done[0] < ncols)
        d2h_columns((char *)U, sizeof(T) * ldu, (const char *)c.U, sizeof(T) * c.ldu, sizeof(T) * c.m, ncols, c.s);
    if (dv && c.done[1] < ncols)
        d2h_columns((char *)V, sizeof(T) * ldv, (const char *)c.V, sizeof(T) * c.ldv, sizeof(T) * c.n, ncols, c.s);
    if (c.s2) {
        PGB_CUDA(cudaEventRecord(c.ev_s2, c.s2));
        PGB_CUDA(cudaStreamWaitEvent(c.s, c.ev_s2, 0));
    }
    }
}

// the caller's U and V, when page-locked, receive the Ritz vectors from
// dev_ritzvec chunk by chunk (the FP64 and complex*16 drivers)
template <typename T>
static void set_host_out(Ctx &c, double *U, int ldu, double *V, int ldv, bool du, bool dv)
{
    if (du && host_pinned(U)) { c.hout[0] = (char *)U; c.hpitch[0] = sizeof(T) * (size_t)ldu; }
    if (dv && host_pinned(V)) { c.hout[1] = (char *)V; c.hpitch[1] = sizeof(T) * (size_t)ldv; }
}

// A(:,0:nc) <- A(:,0:kk) op(B)   (dgemm_ovwr_left) on rows r0:r1
// (complex A times the real B: the real GEMM on the (re, im) rows,
// zdgemm_ovwr_left of complex16/zgemm_ovwr.F).  Row i of the product
// reads only row i of A, so a row range can be overwritten once its own
// product is formed.
template <typename T>
static void ovwr_left(Ctx &c, T *A, int lda, int rows, int nc, int kk, const double *B, int ldb, bool tb, int r0 = 0,
                      int r1 = -1)
{
    if (r1 < 0) r1 = rows;
    const int nr = r1 - r0;
    if constexpr (VecW<T>::w == 2) {
        const double *Ar = (const double *)A + 2 * (size_t)r0;
        double *Gr = (double *)c.gout + 2 * (size_t)r0;
        gemm<double>(2 * nr, nc, kk, Ar, 2 * lda, false, B, ldb, tb, Gr, 2 * lda, c.s);
        copy_cols<double>(Gr, 2 * lda, (double *)A + 2 * (size_t)r0, 2 * lda, 2 * nr, nc, c.s);
    } else {
        gemm<T>(nr, nc, kk, A + r0, lda, false, B, ldb, tb, (T *)c.gout + r0, lda, c.s);
        copy_cols<T>((T *)c.gout + r0, lda, A + r0, lda, nr, nc, c.s);
    }
}

// the Ritz product of one side; with a page-locked host array (FP64 and
// complex*16 bases) in row chunks, each copied to the host on s2 as soon as
// it is formed
template <typename T>
static void ritz_side(Ctx &c, int side, T *A, int lda, int rows, int nc, int kk, const double *B, int ldb)
{
    if (sizeof(T) < 8 || !c.hout[side] || rows < 2 * RITZ_CHUNK_ROWS) {
        ovwr_left<T>(c, A, lda, rows, nc, kk, B, ldb, true);
        return;
    }
    const int nch = std::min(RITZ_MAX_CHUNKS, (rows + RITZ_CHUNK_ROWS - 1) / RITZ_CHUNK_ROWS);
    const int per = ((rows + nch - 1) / nch + 127) / 128 * 128;
    if (!c.s2) PGB_CUDA(cudaStreamCreateWithFlags(&c.s2, cudaStreamNonBlocking));
    if (!c.ev_s2) PGB_CUDA(cudaEventCreateWithFlags(&c.ev_s2, cudaEventDisableTiming));
    for (int i = 0; i < nch; i++) {
        const int r0 = i * per, r1 = std::min(rows, r0 + per);
        if (r0 >= r1) break;
        ovwr_left<T>(c, A, lda, rows, nc, kk, B, ldb, true, r0, r1);
        cudaEvent_t &e = c.ev_chunk[side][i];
        if (!e) PGB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        PGB_CUDA(cudaEventRecord(e, c.s));
        PGB_CUDA(cudaStreamWaitEvent(c.s2, e, 0));
        PGB_CUDA(cudaMemcpy2DAsync(c.hout[side] + sizeof(T) * (size_t)r0, c.hpitch[side], A + r0,
                                   sizeof(T) * (size_t)lda, sizeof(T) * (size_t)(r1 - r0), nc,
                                   cudaMemcpyDeviceToHost, c.s2));
    }
    c.done[side] = nc;
}

// the bidiagonal analysis; returns the number of converged values
static int analyse(Ctx &c, const AnaArgs &a)
{
    launch_analyse(a, c.s);
    g_last.nbsvd++;
    int nc = 0;
    PGB_CUDA(cudaMemcpyAsync(c.hscal, c.nconv, sizeof(int), cudaMemcpyDeviceToHost, c.s));
    c.sync();
    memcpy(&nc, c.hscal, sizeof(int));
    if (nc < 0) {
        if (trace_on()) fprintf(stderr, "[propack_gb300] analysis: lane-parallel path declined, QR path\n");
        launch_analyse_qr(a, c.s);
        PGB_CUDA(cudaMemcpyAsync(c.hscal, c.nconv, sizeof(int), cudaMemcpyDeviceToHost, c.s));
        c.sync();
        memcpy(&nc, c.hscal, sizeof(int));
    }
    return nc;
}

// dritzvec (double/dritzvec.F:1-199)
template <typename T>
static void dev_ritzvec(Ctx &c, bool small_side, bool du, bool dv, int k, int dim)
{
    RitzArgs r;
    r.balpha = c.balpha; r.bbeta = c.bbeta; r.D = c.D; r.E = c.E; r.Mt = c.Mt; r.P = c.Pr; r.Qt = c.Qt;
    r.w = c.w; r.dim = dim; r.m = c.m; r.n = c.n;
    r.wz = c.wz; r.flag = c.dflag;
    r.mstart = small_side ? dim - k + 1 : 1;
    r.k = k;
    bool qr = !launch_ritz_prep(r, c.s);
    if (!qr) {
        PGB_CUDA(cudaMemcpyAsync(c.hscal, c.dflag, sizeof(int), cudaMemcpyDeviceToHost, c.s));
        c.sync();
        int f = 0;
        memcpy(&f, c.hscal, sizeof(int));
        qr = f != 0;
        if (qr && trace_on()) fprintf(stderr, "[propack_gb300] Ritz vectors: clustered values, QR path\n");
    }
    if (qr) launch_ritz_prep_qr(r, c.s);
    const int dp1 = dim + 1;
    // X = P' Mt(1:dim, 1:dim+1)   (dim x dim+1, ld dim+1)
    gemm<double>(dim, dp1, dim, c.Pr, dim, true, c.Mt, dp1, false, c.X, dp1, c.s);
    const int mstart = small_side ? dim - k + 1 : 1;
    if (du) ritz_side<T>(c, 0, (T *)c.U, c.ldu, c.m, k, dp1, c.X + (mstart - 1), dp1);
    if (dv) ritz_side<T>(c, 1, (T *)c.V, c.ldv, c.n, k, dim, c.Qt + (mstart - 1), dim);
}

struct Timer {
    Ctx &c;
    double &acc;
    cudaEvent_t a, b;
    Timer(Ctx &cc, double &ac) : c(cc), acc(ac)
    {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, c.s);
    }
    ~Timer()
    {
        cudaEventRecord(b, c.s);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        acc += ms;
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
};

static void add_ctx_counters(Ctx &c)
{
    c.get_ctl();
    g_last.nopx += c.hctl->nopx;
    g_last.nreorth += c.hctl->nreorth;
    g_last.ndot += c.hctl->ndot;
    g_last.cgs_cols_u += c.hctl->cgs_cols_u;
    g_last.cgs_cols_v += c.hctl->cgs_cols_v;
}

static void finish_stats(int64_t launches0)
{
    g_last.launches = g_launches - launches0;
    g_stat.nopx += g_last.nopx;
    g_stat.nreorth += g_last.nreorth;
    g_stat.ndot += g_last.ndot;
    g_stat.nrestart += g_last.nrestart;
    g_stat.nbsvd += g_last.nbsvd;
    g_stat.nlandim = g_last.nlandim;
    g_stat.nsing = g_last.nsing;
    g_stat.device_ms += g_last.device_ms;
    g_stat.launches += g_last.launches;
}

static void setup_operator(Ctx &c, propack_aprod_t aprod, double *dparm, int *iparm)
{
    if ((void *)aprod == (void *)propack_gpu_csr_zaprod_) {
        set_error("a complex operator needs the complex drivers");
        throw ArgFailure();
    }
    if (aprod == propack_gpu_csr_aprod_) {
        const Operator *op = lookup_operator(handle_from_iparm(iparm));
        if (!op) {
            set_error("APROD is propack_gpu_csr_aprod_ but iparm holds no live operator handle");
            throw ArgFailure();
        }
        if (op->cplx || op->m != c.m || op->n != c.n) {
            set_error(op->cplx ? "a complex operator needs the complex drivers" : "operator shape does not match m, n");
            throw ArgFailure();
        }
        c.op = op;
        c.nb = std::max(c.nb, vec_grid(0, std::max(op->fwd.nnz, op->adj.nnz)));
        c.nb_spmv = spmv_grid_bound(std::max(op->fwd.rows, op->adj.rows));
    } else {
        c.aprod = aprod;
        c.dparm = dparm;
        c.iparm = iparm;
        PGB_CUDA(cudaMallocHost(&c.hx, sizeof(double) * std::max(c.m, c.n)));
        PGB_CUDA(cudaMallocHost(&c.hy, sizeof(double) * std::max(c.m, c.n)));
    }
}

// the complex drivers: propack_gpu_csr_zaprod_ with a complex operator's
// handle, or a user ZAPROD called on pinned host complex*16 vectors
static void setup_zoperator(Ctx &c, propack_zaprod_t aprod, propack_z16 *zparm, int *iparm)
{
    if ((void *)aprod == (void *)propack_gpu_csr_aprod_ || (void *)aprod == (void *)propack_gpu_csr_saprod_) {
        set_error("a real operator needs the real drivers");
        throw ArgFailure();
    }
    if (aprod == propack_gpu_csr_zaprod_) {
        const Operator *op = lookup_operator(handle_from_iparm(iparm));
        if (!op) {
            set_error("APROD is propack_gpu_csr_zaprod_ but iparm holds no live operator handle");
            throw ArgFailure();
        }
        // the real 2x2-block form is 2m x 2n, the native form m x n
        const int f = op->cplx == 1 ? 2 : 1;
        if (!op->cplx || op->m != f * c.m || op->n != f * c.n) {
            set_error(!op->cplx ? "a real operator needs the real drivers" : "operator shape does not match m, n");
            throw ArgFailure();
        }
        c.op = op;
        c.nb = std::max(c.nb, vec_grid(0, std::max(op->fwd.nnz, op->adj.nnz)));
        c.nb_spmv = spmv_grid_bound(std::max(op->fwd.rows, op->adj.rows));
    } else {
        c.zaprod = aprod;
        c.zparm = zparm;
        c.iparm = iparm;
        PGB_CUDA(cudaMallocHost(&c.hx, sizeof(propack_z16) * std::max(c.m, c.n)));
        PGB_CUDA(cudaMallocHost(&c.hy, sizeof(propack_z16) * std::max(c.m, c.n)));
    }
}

struct IrlIn {
    bool small_side = false, du = true, dv = true;
    int m = 0, n = 0, dim = 0, p = 0, neig = 0, maxiter = 0;
    double tol = 0.0;
    // mixed form only: form the top-neig Ritz vectors even when not all
    // converged, and stop after this many restarts without a new converged
    // value (0: never; the reference's behaviour)
    bool ritz_always = false;
    int stall_limit = 0;
};
struct IrlOut {
    int nconv = 0, info = 0, dim = 0, ritz = 0;
    std::vector<double> sigma, bnd;
};

// dlansvd_irl.F:188-418 on a context whose U(:,1) holds the start vector;
// the Ritz vectors are left in the context.
template <typename T>
static void irl_loop(Ctx &c, const IrlIn &in, double *doption, const int *ioption, IrlOut &out)
{
    const int m = in.m, n = in.n, neig0 = in.neig;
    int dim = in.dim;
    const int k = dim - in.p;
    double rnorm = dev_nrm2<T>(c, c.Ucol<T>(0), m);
    int ierr = 0;
    double anorm_drv = 0.0;
    if (rnorm == 0.0) {
        double est = 0.0;
        ierr = dev_getu0<T>(c, false, 0, 1, c.Ucol<T>(0), &rnorm, (T *)c.U, c.ldu, &est);
        anorm_drv = est;
    }
    PGB_CUDA(cudaMemcpyAsync(c.anorm_drv, &anorm_drv, sizeof(double), cudaMemcpyHostToDevice, c.s));
    out.info = 0;
    int iter = 0, nconv = 0, kold = 0, best = 0, since = 0;
    while (nconv < neig0 && iter < in.maxiter) {
        {
            Timer t(c, g_last.lanczos_ms);
            dev_lanbpro<T>(c, kold, &dim, &rnorm, doption, ioption, &ierr);
        }
        kold = k;
        {
            Timer t(c, g_last.bsvd_ms);
            AnaArgs a;
            a.balpha = c.balpha; a.bbeta = c.bbeta; a.a1 = c.a1; a.b1 = c.b1; a.bnd = c.bnd; a.w = c.w;
            a.ctl = c.ctl; a.sigma_out = c.sig_out; a.bnd_out = c.bnd_out; a.nconv_out = c.nconv;
            a.anorm_drv = c.anorm_drv; a.dim = dim; a.m = m; a.n = n; a.neig = neig0; a.kk = k;
            a.irl = 1; a.small_side = in.small_side; a.tol = in.tol; a.wz = c.wz;
            nconv = analyse(c, a);
        }
        if (ierr < 0) {
            if (dim < k) out.info = dim;
            break;
        }
        if (trace_on())
            fprintf(stderr, "[propack_gb300] irl %s iter %d: dim %d nconv %d ierr %d\n",
                    VecW<T>::w == 2 ? "complex" : sizeof(T) == sizeof(double) ? "fp64" : "fp32", iter, dim, nconv,
                    ierr);
        if (in.stall_limit > 0) {
            if (nconv > best) { best = nconv; since = 0; }
            else if (++since >= in.stall_limit) break;
        }
        if (nconv < neig0) {
            {
                Timer t(c, g_last.bsvd_ms);
                SweepArgs sw;
                sw.balpha = c.balpha; sw.bbeta = c.bbeta; sw.a1 = c.a1; sw.bnd = c.bnd; sw.P = c.P; sw.Q = c.Q;
                sw.shifts = c.shifts; sw.w = c.w; sw.ctl = c.ctl; sw.dim = dim; sw.k = k; sw.neig = neig0;
                sw.small_side = in.small_side; sw.min_relgap = doption[3]; sw.wz = c.wz;
                launch_sweeps(sw, c.s);
            }
            {
                Timer t(c, g_last.gemm_ms);
                ovwr_left<T>(c, (T *)c.U, c.ldu, m, k + 1, dim + 1, c.P, dim + 1, false);
                ovwr_left<T>(c, (T *)c.V, c.ldv, n, k, dim, c.Q, dim, false);
            }
            // rnorm = beta_k after the sweeps (written into the control block)
            c.get_ctl();
            rnorm = c.hctl->rnorm;
            g_last.nrestart++;
        }
        iter++;
    }
    out.sigma.assign(std::max(nconv, 1), 0.0);
    out.bnd.assign(std::max(nconv, 1), 0.0);
    PGB_CUDA(cudaMemcpyAsync(out.sigma.data(), c.sig_out, sizeof(double) * std::max(nconv, 1), cudaMemcpyDeviceToHost,
                             c.s));
    PGB_CUDA(cudaMemcpyAsync(out.bnd.data(), c.bnd_out, sizeof(double) * std::max(nconv, 1), cudaMemcpyDeviceToHost,
                             c.s));
    c.sync();
    if ((nconv >= neig0 || out.info > 0) && (in.du || in.dv)) {
        Timer t(c, g_last.gemm_ms);
        dev_ritzvec<T>(c, in.small_side, in.du, in.dv, nconv, dim);
    } else if (in.ritz_always && (in.du || in.dv)) {
        // the restart above left B and the bases at dimension k; when the
        // loop stopped before a restart they are at dim
        Timer t(c, g_last.gemm_ms);
        const int kk = std::min(neig0, dim);
        dev_ritzvec<T>(c, in.small_side, in.du, in.dv, kk, dim);
        nconv = std::max(nconv, 0);
        out.ritz = kk;
    }
    out.nconv = nconv;
    out.dim = dim;
}

// one IRL solve in the vectors' own precision (FP64, or complex*16 through
// a ZAPROD or a complex operator); U(:,1) in, the Ritz vectors out
template <typename T>
static void irl_plain(const IrlIn &in, propack_aprod_t aprod, double *dparm, propack_zaprod_t zaprod,
                      propack_z16 *zparm, int *iparm, double *U, int ldu, double *V, int ldv, double *doption,
                      const int *ioption, IrlOut &out)
{
    Ctx c;
    init_ctx<T>(c, in.m, in.n, in.dim);
    if constexpr (VecW<T>::w == 2) setup_zoperator(c, zaprod, zparm, iparm);
    else setup_operator(c, aprod, dparm, iparm);
    set_host_out<T>(c, U, ldu, V, ldv, in.du, in.dv);
    PGB_CUDA(cudaEventRecord(c.ev0, c.s));
    PGB_CUDA(cudaMemcpyAsync(c.U, U, sizeof(T) * in.m, cudaMemcpyHostToDevice, c.s));
    PGB_CUDA(cudaEventRecord(c.evs0, c.s));
    irl_loop<T>(c, in, doption, ioption, out);
    PGB_CUDA(cudaEventRecord(c.evs1, c.s));
    copy_out<T>(c, U, ldu, V, ldv, out.nconv, in.du, in.dv);
    PGB_CUDA(cudaEventRecord(c.ev1, c.s));
    c.sync();
    float ms = 0;
    cudaEventElapsedTime(&ms, c.ev0, c.ev1);
    g_last.device_ms = ms;
    cudaEventElapsedTime(&ms, c.evs0, c.evs1);
    g_last.solve_ms = ms;
    add_ctx_counters(c);
}

static void run_irl(const char *which, const char *jobu, const char *jobv, int m, int n, int dim, int p, int *neig,
                    int maxiter, propack_aprod_t aprod, double *U, int ldu, double *sigma, double *bnd, double *V,
                    int ldv, double tolin, double *doption, const int *ioption, int *info, double *dparm, int *iparm)
{
    if (m <= 0 || n <= 0 || dim <= 0 || p < 0 || *neig < 0 || ldu < m || ldv < n || !aprod || !U || !V || !sigma ||
        !bnd || !doption || !ioption) {
        set_error("dlansvd_irl_: invalid argument");
        throw ArgFailure();
    }
    const int64_t l0 = g_launches;
    g_last = Stats();
    IrlIn in;
    in.small_side = which && (which[0] == 's' || which[0] == 'S');
    in.du = yes(jobu);
    in.dv = yes(jobv);
    in.m = m;
    in.n = n;
    in.dim = std::min(dim, std::min(n + 1, m + 1));
    in.p = p;
    in.neig = *neig;
    in.maxiter = maxiter;
    in.tol = std::min(1.0, std::max(16.0 * EPS, tolin));
    const int k = in.dim - p;
    if (k < 1 || in.neig > k) {
        set_error("dlansvd_irl_: need 1 <= neig <= dim - p");
        throw ArgFailure();
    }
    IrlOut out;
    if (g_precision == 2 && !in.small_side) {
        // FP32 only (the single-precision drivers): FP32 vectors, SpMV and
        // Gram-Schmidt, FP64 scalars; tol no finer than 16 * 2^-24
        Ctx c;
        init_ctx<float>(c, m, n, in.dim);
        setup_operator(c, aprod, dparm, iparm);
        PGB_CUDA(cudaEventRecord(c.ev0, c.s));
        PGB_CUDA(cudaMemcpyAsync(c.dx, U, sizeof(double) * m, cudaMemcpyHostToDevice, c.s));
        PGB_CUDA(cudaEventRecord(c.evs0, c.s));
        dev_convert<double, float>(c, c.dx, c.Ucol<float>(0), m);
        double dop32[4] = {doption[0], doption[1], doption[2], doption[3]};
        if (dop32[0] >= 0) dop32[0] = std::max(dop32[0], std::sqrt(EPS32));
        if (dop32[1] >= 0) dop32[1] = std::max(dop32[1], std::pow(EPS32, 0.75));
        IrlIn in32 = in;
        in32.tol = std::min(1.0, std::max(16.0 * EPS32, tolin));
        irl_loop<float>(c, in32, dop32, ioption, out);
        PGB_CUDA(cudaEventRecord(c.evs1, c.s));
        copy_out<float>(c, U, ldu, V, ldv, out.nconv, in.du, in.dv);
        PGB_CUDA(cudaEventRecord(c.ev1, c.s));
        c.sync();
        float ms = 0;
        cudaEventElapsedTime(&ms, c.ev0, c.ev1);
        g_last.device_ms = ms;
        cudaEventElapsedTime(&ms, c.evs0, c.evs1);
        g_last.solve_ms = ms;
        g_last.low_ms = ms;
        add_ctx_counters(c);
        g_last.nopx_low = g_last.nopx;
        doption[2] = dop32[2];
    } else if (g_precision == 0 || in.small_side) {
        irl_plain<double>(in, aprod, dparm, nullptr, nullptr, iparm, U, ldu, V, ldv, doption, ioption, out);
    } else {
        // mixed form: FP32 Lanczos to MIXED_TOL, then FP64 refinement
        Ctx c32;
        init_ctx<float>(c32, m, n, in.dim);
        setup_operator(c32, aprod, dparm, iparm);
        PGB_CUDA(cudaEventRecord(c32.ev0, c32.s));
        PGB_CUDA(cudaMemcpyAsync(c32.dx, U, sizeof(double) * m, cudaMemcpyHostToDevice, c32.s));
        PGB_CUDA(cudaEventRecord(c32.evs0, c32.s));
        dev_convert<double, float>(c32, c32.dx, c32.Ucol<float>(0), m);
        double dop32[4] = {doption[0], doption[1], doption[2], doption[3]};
        if (dop32[0] >= 0) dop32[0] = std::max(dop32[0], std::sqrt(EPS32));
        if (dop32[1] >= 0) dop32[1] = std::max(dop32[1], std::pow(EPS32, 0.75));
        IrlIn in32 = in;
        in32.tol = std::max(in.tol, MIXED_TOL);
        in32.du = true;
        in32.dv = false;
        in32.ritz_always = true;
        in32.stall_limit = 8;
        IrlOut out32;
        irl_loop<float>(c32, in32, dop32, ioption, out32);
        add_ctx_counters(c32);
        const int64_t nopx32 = g_last.nopx;
        PGB_CUDA(cudaEventRecord(c32.evs1, c32.s));
        c32.sync();
        float ms32 = 0;
        cudaEventElapsedTime(&ms32, c32.evs0, c32.evs1);
        // FP64 refinement: the FP64 IRL with the caller's dim and shifts,
        // started from the sum of the FP32 Ritz vectors (a vector whose
        // Krylov space holds the wanted subspace to FP32 accuracy), with the
        // FP32 run's ||A|| estimate
        IrlIn in64 = in;
        Ctx c64;
        init_ctx<double>(c64, m, n, in64.dim);
        setup_operator(c64, aprod, dparm, iparm);
        set_host_out<double>(c64, U, ldu, V, ldv, in.du, in.dv);
        const int nwarm = std::min(std::max(out32.nconv, out32.ritz), in.neig);
        if (nwarm > 0) {
            k_sum_cols<float><<<c64.nb, 256, 0, c64.s>>>(c32.Ucol<float>(0), c32.ldu, m, nwarm, c64.Ucol<double>(0));
            PGB_LAUNCHED();
        } else {
            PGB_CUDA(cudaMemcpyAsync(c64.U, U, sizeof(double) * m, cudaMemcpyHostToDevice, c64.s));
        }
        double dop64[4] = {doption[0], doption[1], dop32[2], doption[3]};
        PGB_CUDA(cudaEventRecord(c64.evs0, c64.s));
        irl_loop<double>(c64, in64, dop64, ioption, out);
        PGB_CUDA(cudaEventRecord(c64.evs1, c64.s));
        copy_out<double>(c64, U, ldu, V, ldv, out.nconv, in.du, in.dv);
        PGB_CUDA(cudaEventRecord(c64.ev1, c64.s));
        c64.sync();
        float ms64 = 0, msall = 0;
        cudaEventElapsedTime(&ms64, c64.evs0, c64.evs1);
        cudaEventElapsedTime(&msall, c32.ev0, c64.ev1);
        g_last.solve_ms = ms32 + ms64;
        g_last.device_ms = msall;
        g_last.low_ms = ms32;
        add_ctx_counters(c64);
        g_last.nopx_low = nopx32;
        doption[2] = dop64[2];
    }
    for (int i = 0; i < out.nconv && i < in.neig; i++) { sigma[i] = out.sigma[i]; bnd[i] = out.bnd[i]; }
    *info = out.info;
    *neig = out.nconv;
    g_last.nlandim = out.dim;
    prof_collect();
    finish_stats(l0);
}

// T = complex*16 (double2): U, V are the caller's complex arrays and the
// operator comes from zaprod / zparm
template <typename T>
static void run_lansvd_t(const char *jobu, const char *jobv, int m, int n, int *kp, int kmax, propack_aprod_t aprod,
                       double *U, int ldu, double *sigma, double *bnd, double *V, int ldv, double tolin,
                       double *doption, const int *ioption, int *info, double *dparm, int *iparm,
                       propack_zaprod_t zaprod = nullptr, propack_z16 *zparm = nullptr)
{
    const int k = *kp;
    constexpr bool cplx = VecW<T>::w == 2;
    if (m <= 0 || n <= 0 || k <= 0 || kmax <= 0 || ldu < m || ldv < n || !(cplx ? (void *)zaprod : (void *)aprod) ||
        !U || !V || !sigma || !bnd || !doption || !ioption) {
        set_error(cplx ? "zlansvd_: invalid argument" : "dlansvd_: invalid argument");
        throw ArgFailure();
    }
    const int64_t l0 = g_launches;
    g_last = Stats();
    const int lanmax = std::min(std::min(n + 1, m + 1), kmax);
    constexpr bool f32 = std::is_same<T, float>::value;
    const double tol = std::min(1.0, std::max(16.0 * (f32 ? EPS32 : EPS), tolin));
    // the FP32 vectors keep orthogonality at the FP32 levels sqrt(eps), eps^(3/4)
    double dop[4] = {doption[0], doption[1], doption[2], 0.0};
    if (f32 && dop[0] >= 0) dop[0] = std::max(dop[0], std::sqrt(EPS32));
    if (f32 && dop[1] >= 0) dop[1] = std::max(dop[1], std::pow(EPS32, 0.75));
    Ctx c;
    init_ctx<T>(c, m, n, lanmax);
    if constexpr (cplx) setup_zoperator(c, zaprod, zparm, iparm);
    else setup_operator(c, aprod, dparm, iparm);
    if constexpr (sizeof(T) >= 8) set_host_out<T>(c, U, ldu, V, ldv, yes(jobu), yes(jobv));
    PGB_CUDA(cudaEventRecord(c.ev0, c.s));
    if constexpr (cplx) {
        PGB_CUDA(cudaMemcpyAsync(c.U, U, sizeof(T) * m, cudaMemcpyHostToDevice, c.s));
        PGB_CUDA(cudaEventRecord(c.evs0, c.s));
    } else {
        PGB_CUDA(cudaMemcpyAsync(c.dx, U, sizeof(double) * m, cudaMemcpyHostToDevice, c.s));
        PGB_CUDA(cudaEventRecord(c.evs0, c.s));
        dev_convert<double, T>(c, c.dx, c.Ucol<T>(0), m);
    }
    double rnorm = dev_nrm2<T>(c, c.Ucol<T>(0), m);
    int ierr = 0;
    double anorm_drv = 0.0;
    if (rnorm == 0.0) {
        double est = 0.0;
        ierr = dev_getu0<T>(c, false, 0, 1, c.Ucol<T>(0), &rnorm, (T *)c.U, c.ldu, &est);
        anorm_drv = est;
    }
    PGB_CUDA(cudaMemcpyAsync(c.anorm_drv, &anorm_drv, sizeof(double), cudaMemcpyHostToDevice, c.s));
    g_last.nsing = k;
    *info = 0;
    int neig = 0, jold = 0;
    int j = std::min(k + std::max(8, k) + 1, lanmax);
    std::vector<double> hs(lanmax + 2), hb(lanmax + 2);
    while (neig < k) {
        {
            Timer t(c, g_last.lanczos_ms);
            dev_lanbpro<T>(c, jold, &j, &rnorm, dop, ioption, &ierr);
        }
        jold = j;
        {
            Timer t(c, g_last.bsvd_ms);
            AnaArgs a;
            a.balpha = c.balpha; a.bbeta = c.bbeta; a.a1 = c.a1; a.b1 = c.b1; a.bnd = c.bnd; a.w = c.w;
            a.ctl = c.ctl; a.sigma_out = c.sig_out; a.bnd_out = c.bnd_out; a.nconv_out = c.nconv;
            a.anorm_drv = c.anorm_drv; a.dim = j; a.m = m; a.n = n; a.neig = k; a.kk = k;
            a.irl = 0; a.small_side = 0; a.tol = tol; a.wz = c.wz;
            neig = analyse(c, a);
        }
        if (ierr < 0) {
            if (j < k) *info = j;
            break;
        }
        if (j >= lanmax) {
            if (neig < k) *info = -1;
            break;
        }
        int dj;
        if (neig > 1) {
            dj = std::min(j / 2, ((k - neig) * (j - 6)) / (2 * neig + 1));
            dj = std::min(100, std::max(2, dj));
        } else {
            dj = j / 2;
            dj = std::min(100, std::max(10, dj));
        }
        j = std::min(j + dj, lanmax);
    }
    const int lim = std::min(j, k);
    PGB_CUDA(cudaMemcpyAsync(hs.data(), c.sig_out, sizeof(double) * std::max(neig, 1), cudaMemcpyDeviceToHost, c.s));
    PGB_CUDA(cudaMemcpyAsync(hb.data(), c.bnd_out, sizeof(double) * std::max(lim, 1), cudaMemcpyDeviceToHost, c.s));
    c.sync();
    for (int i = 0; i < neig; i++) sigma[i] = hs[i];
    for (int i = 0; i < lim; i++) bnd[i] = hb[i];
    const bool du = yes(jobu), dv = yes(jobv);
    if ((neig >= k || *info > 0) && (du || dv)) {
        Timer t(c, g_last.gemm_ms);
        dev_ritzvec<T>(c, false, du, dv, neig, jold);
    }
    PGB_CUDA(cudaEventRecord(c.evs1, c.s));
    copy_out<T>(c, U, ldu, V, ldv, neig, du, dv);
    doption[2] = dop[2];
    PGB_CUDA(cudaEventRecord(c.ev1, c.s));
    c.sync();
    float ms = 0;
    cudaEventElapsedTime(&ms, c.ev0, c.ev1);
    g_last.device_ms = ms;
    cudaEventElapsedTime(&ms, c.evs0, c.evs1);
    g_last.solve_ms = ms;
    *kp = neig;
    g_last.nlandim = j;
    add_ctx_counters(c);
    prof_collect();
    finish_stats(l0);
}

// dlansvd (double/dlansvd.F:131-291); FP32 vectors when the precision is 2
static void run_lansvd(const char *jobu, const char *jobv, int m, int n, int *kp, int kmax, propack_aprod_t aprod,
                       double *U, int ldu, double *sigma, double *bnd, double *V, int ldv, double tolin,
                       double *doption, const int *ioption, int *info, double *dparm, int *iparm)
{
    if (g_precision == 2)
        run_lansvd_t<float>(jobu, jobv, m, n, kp, kmax, aprod, U, ldu, sigma, bnd, V, ldv, tolin, doption, ioption,
                            info, dparm, iparm);
    else
        run_lansvd_t<double>(jobu, jobv, m, n, kp, kmax, aprod, U, ldu, sigma, bnd, V, ldv, tolin, doption,
                             ioption, info, dparm, iparm);
}

// ZLANSVD_IRL (complex16/zlansvd_irl.F): the FP64 IRL on complex*16
// vectors; the precision setting does not apply
static void run_zirl(const char *which, const char *jobu, const char *jobv, int m, int n, int dim, int p, int *neig,
                     int maxiter, propack_zaprod_t aprod, propack_z16 *U, int ldu, double *sigma, double *bnd,
                     propack_z16 *V, int ldv, double tolin, double *doption, const int *ioption, int *info,
                     propack_z16 *zparm, int *iparm)
{
    if (m <= 0 || n <= 0 || dim <= 0 || p < 0 || *neig < 0 || ldu < m || ldv < n || !aprod || !U || !V || !sigma ||
        !bnd || !doption || !ioption) {
        set_error("zlansvd_irl_: invalid argument");
        throw ArgFailure();
    }
    const int64_t l0 = g_launches;
    g_last = Stats();
    IrlIn in;
    in.small_side = which && (which[0] == 's' || which[0] == 'S');
    in.du = yes(jobu);
    in.dv = yes(jobv);
    in.m = m;
    in.n = n;
    in.dim = std::min(dim, std::min(n + 1, m + 1));
    in.p = p;
    in.neig = *neig;
    in.maxiter = maxiter;
    in.tol = std::min(1.0, std::max(16.0 * EPS, tolin));
    const int k = in.dim - p;
    if (k < 1 || in.neig > k) {
        set_error("zlansvd_irl_: need 1 <= neig <= dim - p");
        throw ArgFailure();
    }
    IrlOut out;
    irl_plain<double2>(in, nullptr, nullptr, aprod, zparm, iparm, (double *)U, ldu, (double *)V, ldv, doption,
                       ioption, out);
    for (int i = 0; i < out.nconv && i < in.neig; i++) { sigma[i] = out.sigma[i]; bnd[i] = out.bnd[i]; }
    *info = out.info;
    *neig = out.nconv;
    g_last.nlandim = out.dim;
    prof_collect();
    finish_stats(l0);
}

}  // namespace pgb

// ------------------------------------------------------------------ C ABI
using namespace pgb;

// LWORK / LIWORK (/ LZWRK) as the reference's drivers use them: the leading
// part of WORK that they always clear (dzero of 8*dim+3+2*dim^2 entries,
// double/dlansvd_irl.F:177-188; 7*lanmax+2+2*lanmax^2, double/dlansvd.F:
// 151-160) plus the max(m,n) vector that dgetu0 and dlanbpro take from its
// tail; IWORK holds dlanbpro's 2*dim+1 interval bounds; ZWORK (complex
// drivers) the max(m,n) complex vector of zgetu0.  The device path keeps
// its own workspace and never reads or writes WORK, IWORK or ZWORK; a call
// that declares less than the reference would overrun is refused with
// PROPACK_ERR_ARG.
static void check_work(const char *who, bool irl, int m, int n, int dim, const int *lwork, const int *liwork,
                       const int *lzwrk, bool cplx)
{
    if (!lwork || !liwork || (cplx && !lzwrk)) {
        set_error(std::string(who) + ": LWORK, LIWORK" + (cplx ? " and LZWRK" : "") + " are required");
        throw ArgFailure();
    }
    const long long d = std::max(0, std::min(dim, std::min(m, n) + 1));
    const long long mn = std::max(m, n);
    const long long need = (irl ? 2 * d * d + 8 * d + 3 : 2 * d * d + 7 * d + 2) + mn;
    const long long needi = 2 * d + 1;
    char msg[256];
    if (*lwork < need) {
        snprintf(msg, sizeof msg, "%s: LWORK = %d is below %lld (%s + max(m,n))", who, *lwork, need,
                 irl ? "2*dim^2+8*dim+3" : "2*kmax^2+7*kmax+2");
        set_error(msg);
        throw ArgFailure();
    }
    if (*liwork < needi) {
        snprintf(msg, sizeof msg, "%s: LIWORK = %d is below 2*%s+1 = %lld", who, *liwork, irl ? "dim" : "kmax",
                 needi);
        set_error(msg);
        throw ArgFailure();
    }
    if (cplx && *lzwrk < mn) {
        snprintf(msg, sizeof msg, "%s: LZWRK = %d is below max(m,n) = %lld", who, *lzwrk, mn);
        set_error(msg);
        throw ArgFailure();
    }
}

extern "C" void dlansvd_irl_(const char *which, const char *jobu, const char *jobv, const int *m, const int *n,
                             const int *dim, const int *p, int *neig, const int *maxiter, propack_aprod_t aprod,
                             double *U, const int *ldu, double *sigma, double *bnd, double *V, const int *ldv,
                             const double *tolin, double *work, const int *lwork, int *iwork, const int *liwork,
                             double *doption, const int *ioption, int *info, double *dparm, int *iparm,
                             size_t which_len, size_t jobu_len, size_t jobv_len)
{
    (void)work; (void)iwork; (void)which_len; (void)jobu_len; (void)jobv_len;
    set_error("");
    try {
        if (m && n && dim) check_work("dlansvd_irl_", true, *m, *n, *dim, lwork, liwork, nullptr, false);
        run_irl(which, jobu, jobv, *m, *n, *dim, *p, neig, *maxiter, aprod, U, *ldu, sigma, bnd, V, *ldv, *tolin,
                doption, ioption, info, dparm, iparm);
    } catch (const CudaFailure &) {
        *info = PROPACK_ERR_CUDA;
    } catch (const ArgFailure &) {
        *info = PROPACK_ERR_ARG;
    } catch (const WaitFailure &) {
        *info = PROPACK_ERR_WAIT;
    }
}

extern "C" void dlansvd_(const char *jobu, const char *jobv, const int *m, const int *n, int *k, const int *kmax,
                         propack_aprod_t aprod, double *U, const int *ldu, double *sigma, double *bnd, double *V,
                         const int *ldv, const double *tolin, double *work, const int *lwork, int *iwork,
                         const int *liwork, double *doption, const int *ioption, int *info, double *dparm, int *iparm,
                         size_t jobu_len, size_t jobv_len)
{
    (void)work; (void)iwork; (void)jobu_len; (void)jobv_len;
    set_error("");
    try {
        if (m && n && kmax) check_work("dlansvd_", false, *m, *n, *kmax, lwork, liwork, nullptr, false);
        run_lansvd(jobu, jobv, *m, *n, k, *kmax, aprod, U, *ldu, sigma, bnd, V, *ldv, *tolin, doption, ioption, info,
                   dparm, iparm);
    } catch (const CudaFailure &) {
        *info = PROPACK_ERR_CUDA;
    } catch (const ArgFailure &) {
        *info = PROPACK_ERR_ARG;
    } catch (const WaitFailure &) {
        *info = PROPACK_ERR_WAIT;
    }
}

// ------------------------------------------------------ complex drivers
// ZLANSVD / ZLANSVD_IRL (complex16/zlansvd.F:1-3, complex16/zlansvd_irl.F:1-3):
// complex*16 U, V, ZWORK and ZPARM; DOUBLE PRECISION Sigma, bnd, WORK and
// DOPTION; the APROD takes TRANSA 'n' (y = A x) or 'c' (y = A^H x).
extern "C" void zlansvd_irl_(const char *which, const char *jobu, const char *jobv, const int *m, const int *n,
                             const int *dim, const int *p, int *neig, const int *maxiter, propack_zaprod_t aprod,
                             propack_z16 *U, const int *ldu, double *sigma, double *bnd, propack_z16 *V,
                             const int *ldv, const double *tolin, double *work, const int *lwork, propack_z16 *zwork,
                             const int *lzwrk, int *iwork, const int *liwork, double *doption, const int *ioption,
                             int *info, propack_z16 *zparm, int *iparm, size_t which_len, size_t jobu_len,
                             size_t jobv_len)
{
    (void)work; (void)zwork; (void)iwork;
    (void)which_len; (void)jobu_len; (void)jobv_len;
    set_error("");
    try {
        if (m && n && dim) check_work("zlansvd_irl_", true, *m, *n, *dim, lwork, liwork, lzwrk, true);
        run_zirl(which, jobu, jobv, *m, *n, *dim, *p, neig, *maxiter, aprod, U, *ldu, sigma, bnd, V, *ldv, *tolin,
                 doption, ioption, info, zparm, iparm);
    } catch (const CudaFailure &) {
        *info = PROPACK_ERR_CUDA;
    } catch (const ArgFailure &) {
        *info = PROPACK_ERR_ARG;
    } catch (const WaitFailure &) {
        *info = PROPACK_ERR_WAIT;
    }
}

extern "C" void zlansvd_(const char *jobu, const char *jobv, const int *m, const int *n, int *k, const int *kmax,
                         propack_zaprod_t aprod, propack_z16 *U, const int *ldu, double *sigma, double *bnd,
                         propack_z16 *V, const int *ldv, const double *tolin, double *work, const int *lwork,
                         propack_z16 *zwork, const int *lzwrk, int *iwork, const int *liwork, double *doption,
                         const int *ioption, int *info, propack_z16 *zparm, int *iparm, size_t jobu_len,
                         size_t jobv_len)
{
    (void)work; (void)zwork; (void)iwork; (void)jobu_len; (void)jobv_len;
    set_error("");
    try {
        if (m && n && kmax) check_work("zlansvd_", false, *m, *n, *kmax, lwork, liwork, lzwrk, true);
        run_lansvd_t<double2>(jobu, jobv, *m, *n, k, *kmax, nullptr, (double *)U, *ldu, sigma, bnd, (double *)V,
                              *ldv, *tolin, doption, ioption, info, nullptr, iparm, aprod, zparm);
    } catch (const CudaFailure &) {
        *info = PROPACK_ERR_CUDA;
    } catch (const ArgFailure &) {
        *info = PROPACK_ERR_ARG;
    } catch (const WaitFailure &) {
        *info = PROPACK_ERR_WAIT;
    }
}

// ---------------------------------------------- single-precision drivers
// SLANSVD / SLANSVD_IRL (single/slansvd.F:1-3, single/slansvd_irl.F:1-3):
// the same argument lists with REAL arrays and a REAL APROD.  They run the
// FP32 form (FP32 vectors, SpMV and Gram-Schmidt, FP64 scalars) and widen /
// narrow at the boundary.  A user APROD is reached through a trampoline that
// narrows the FP64 vectors of the host path to the caller's REAL arrays.
struct SAprod {
    propack_saprod_t f = nullptr;
    float *sparm = nullptr;
    std::vector<float> xf, yf;
};
static thread_local SAprod g_saprod;

static void saprod_trampoline(const char *transa, const int *m, const int *n, const double *x, double *y,
                              double *dparm, int *iparm, size_t transa_len)
{
    (void)dparm;
    const bool t = transa[0] == 't' || transa[0] == 'T';
    const int nin = t ? *m : *n, nout = t ? *n : *m;
    g_saprod.xf.resize(std::max(nin, 1));
    g_saprod.yf.resize(std::max(nout, 1));
    for (int i = 0; i < nin; i++) g_saprod.xf[i] = (float)x[i];
    g_saprod.f(transa, m, n, g_saprod.xf.data(), g_saprod.yf.data(), g_saprod.sparm, iparm, transa_len);
    for (int i = 0; i < nout; i++) y[i] = g_saprod.yf[i];
}

// widened copies of the caller's REAL arrays for the FP64-interfaced drivers
struct SArgs {
    std::vector<double> U, V, sig, bnd, opt;
    propack_aprod_t ap = nullptr;
};
static void s_prepare(SArgs &w, propack_saprod_t aprod, int m, int n, int ncols_u, int ncols_v, int ldu, int ldv,
                      const float *U, int nsig, const float *soption, int nopt, float *sparm)
{
    w.U.assign((size_t)m * ncols_u, 0.0);
    for (int i = 0; i < m; i++) w.U[i] = U[i];  // U(:,1), the start vector
    w.V.assign((size_t)n * ncols_v, 0.0);
    w.sig.assign(std::max(nsig, 1), 0.0);
    w.bnd.assign(std::max(nsig, 1), 0.0);
    w.opt.assign(4, 0.0);
    for (int i = 0; i < nopt; i++) w.opt[i] = soption[i];
    (void)ldu; (void)ldv;
    if (aprod == propack_gpu_csr_saprod_) {
        w.ap = propack_gpu_csr_aprod_;
    } else {
        g_saprod.f = aprod;
        g_saprod.sparm = sparm;
        w.ap = saprod_trampoline;
    }
}
static void s_finish(const SArgs &w, int m, int n, int ncols, bool du, bool dv, float *U, int ldu, float *V, int ldv,
                     float *sigma, float *bnd, int nsig, float *soption, int nopt)
{
    for (int c = 0; c < ncols; c++) {
        if (du)
            for (int i = 0; i < m; i++) U[(size_t)c * ldu + i] = (float)w.U[(size_t)c * m + i];
        if (dv)
            for (int i = 0; i < n; i++) V[(size_t)c * ldv + i] = (float)w.V[(size_t)c * n + i];
    }
    for (int i = 0; i < nsig; i++) { sigma[i] = (float)w.sig[i]; bnd[i] = (float)w.bnd[i]; }
    for (int i = 0; i < nopt; i++) soption[i] = (float)w.opt[i];
}

extern "C" void slansvd_irl_(const char *which, const char *jobu, const char *jobv, const int *m, const int *n,
                             const int *dim, const int *p, int *neig, const int *maxiter, propack_saprod_t aprod,
                             float *U, const int *ldu, float *sigma, float *bnd, float *V, const int *ldv,
                             const float *tolin, float *work, const int *lwork, int *iwork, const int *liwork,
                             float *soption, const int *ioption, int *info, float *sparm, int *iparm,
                             size_t which_len, size_t jobu_len, size_t jobv_len)
{
    (void)work; (void)iwork; (void)which_len; (void)jobu_len; (void)jobv_len;
    set_error("");
    const int saved = g_precision;
    try {
        if (!m || !n || !dim || !neig || !U || !V || !sigma || !bnd || !soption || !ioption || !info || !aprod ||
            *m <= 0 || *n <= 0 || *dim <= 0 || *ldu < *m || *ldv < *n) {
            set_error("slansvd_irl_: invalid argument");
            throw ArgFailure();
        }
        check_work("slansvd_irl_", true, *m, *n, *dim, lwork, liwork, nullptr, false);
        SArgs w;
        const int k0 = *neig;
        s_prepare(w, aprod, *m, *n, *dim + 1, *dim, *ldu, *ldv, U, k0, soption, 4, sparm);
        g_precision = 2;
        run_irl(which, jobu, jobv, *m, *n, *dim, *p, neig, *maxiter, w.ap, w.U.data(), *m, w.sig.data(),
                w.bnd.data(), w.V.data(), *n, (double)*tolin, w.opt.data(), ioption, info, nullptr, iparm);
        g_precision = saved;
        s_finish(w, *m, *n, std::min(*neig, k0), yes(jobu), yes(jobv), U, *ldu, V, *ldv, sigma, bnd,
                 std::min(*neig, k0), soption, 4);
    } catch (const CudaFailure &) {
        g_precision = saved;
        *info = PROPACK_ERR_CUDA;
    } catch (const ArgFailure &) {
        g_precision = saved;
        *info = PROPACK_ERR_ARG;
    } catch (const WaitFailure &) {
        g_precision = saved;
        *info = PROPACK_ERR_WAIT;
    }
}

extern "C" void slansvd_(const char *jobu, const char *jobv, const int *m, const int *n, int *k, const int *kmax,
                         propack_saprod_t aprod, float *U, const int *ldu, float *sigma, float *bnd, float *V,
                         const int *ldv, const float *tolin, float *work, const int *lwork, int *iwork,
                         const int *liwork, float *soption, const int *ioption, int *info, float *sparm, int *iparm,
                         size_t jobu_len, size_t jobv_len)
{
    (void)work; (void)iwork; (void)jobu_len; (void)jobv_len;
    set_error("");
    const int saved = g_precision;
    try {
        if (!m || !n || !k || !kmax || !U || !V || !sigma || !bnd || !soption || !ioption || !info || !aprod ||
            *m <= 0 || *n <= 0 || *kmax <= 0 || *k <= 0 || *ldu < *m || *ldv < *n) {
            set_error("slansvd_: invalid argument");
            throw ArgFailure();
        }
        check_work("slansvd_", false, *m, *n, *kmax, lwork, liwork, nullptr, false);
        SArgs w;
        const int k0 = *k;
        s_prepare(w, aprod, *m, *n, *kmax + 1, *kmax, *ldu, *ldv, U, k0, soption, 3, sparm);
        g_precision = 2;
        run_lansvd(jobu, jobv, *m, *n, k, *kmax, w.ap, w.U.data(), *m, w.sig.data(), w.bnd.data(), w.V.data(), *n,
                   (double)*tolin, w.opt.data(), ioption, info, nullptr, iparm);
        g_precision = saved;
        // dlansvd returns bounds for the first k values even when fewer converged
        s_finish(w, *m, *n, std::min(*k, k0), yes(jobu), yes(jobv), U, *ldu, V, *ldv, sigma, bnd, k0, soption, 3);
    } catch (const CudaFailure &) {
        g_precision = saved;
        *info = PROPACK_ERR_CUDA;
    } catch (const ArgFailure &) {
        g_precision = saved;
        *info = PROPACK_ERR_ARG;
    } catch (const WaitFailure &) {
        g_precision = saved;
        *info = PROPACK_ERR_WAIT;
    }
}

extern "C" void clearstat_(void) { g_stat = Stats(); }

extern "C" int propack_set_precision(int mode)
{
    if (mode != 0 && mode != 1 && mode != 2) return PROPACK_ERR_ARG;
    g_precision = mode;
    return 0;
}
extern "C" int propack_get_precision(void) { return g_precision; }

extern "C" int propack_kernel_binary_version(void)
{
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, k_sum_final) != cudaSuccess) {
        set_error("cudaFuncGetAttributes failed (no usable CUDA device?)");
        return PROPACK_ERR_CUDA;
    }
    return fa.binaryVersion;
}

extern "C" int propack_set_cgs_arith(int mode)
{
    if (mode != CGS_FP64 && mode != CGS_F3 && mode != CGS_PLANES) return PROPACK_ERR_ARG;
    g_cgs_arith = mode;
    return 0;
}

extern "C" void printstat_(void)
{
    const Stats &s = g_stat;
    printf("+-----------------------------------------------------------+\n");
    printf(" Dimension of Lanczos basis                  = %12lld\n", (long long)s.nlandim);
    printf(" Number of singular values requested         = %12lld\n", (long long)s.nsing);
    printf(" Number of restarts                          = %12lld\n", (long long)s.nrestart);
    printf(" Number of matrix-vector multiplications     = %12lld\n", (long long)s.nopx);
    printf(" Number of reorthogonalizations              = %12lld\n", (long long)s.nreorth);
    printf(" Number of inner products in reorth.         = %12lld\n", (long long)s.ndot);
    printf(" Number of bidiagonal SVDs                   = %12lld\n", (long long)s.nbsvd);
    printf(" Device time (ms)                            = %12.3f\n", s.device_ms);
    printf(" Kernel launches                             = %12lld\n", (long long)s.launches);
    printf("+-----------------------------------------------------------+\n");
}

extern "C" void propack_get_stats(propack_stats_t *out)
{
    const Stats &s = g_last;
    out->nopx = s.nopx;
    out->nreorth = s.nreorth;
    out->ndot = s.ndot;
    out->nrestart = s.nrestart;
    out->nbsvd = s.nbsvd;
    out->nlandim = s.nlandim;
    out->device_ms = s.device_ms;
    out->lanczos_ms = s.lanczos_ms;
    out->bsvd_ms = s.bsvd_ms;
    out->gemm_ms = s.gemm_ms;
    out->kernel_launches = s.launches;
    out->solve_ms = s.solve_ms;
    out->nopx_low = s.nopx_low;
    out->low_ms = s.low_ms;
    out->cgs_cols_u = s.cgs_cols_u;
    out->cgs_cols_v = s.cgs_cols_v;
}
