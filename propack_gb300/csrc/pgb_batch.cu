// pgb_batch.cu -- many independent small problems in one persistent kernel.
//
// Each problem p is an m_p x n_p CSR matrix with FP32 values; the solver
// runs dlansvd_irl (double/dlansvd_irl.F:160-419) on every problem with full
// reorthogonalisation (dlanbpro.F with delta = 0: every new Lanczos vector
// is orthogonalised against all previous ones by iterated classical
// Gram-Schmidt, dreorth.F:106-210) and FP64 vectors.  Optionally the products
// and the Gram-Schmidt passes read the bases as FP32 (hi, lo) planes, split
// once per final column (pgb_planes.cuh; propack_batch_set_arith).
//
// Execution: one CTA owns one problem at a time.  A persistent grid pulls
// problems from a work queue ordered by decreasing cost (an atomic ticket)
// and runs up to BATCH_CYCLES_PER_LAUNCH restart cycles of each active problem:
//   Lanczos extension k0 -> dim (both SpMVs, ELR, CGS) ... dlanbpro.F
//   bidiagonal analysis (lane-parallel bisection + twisted bounds,
//   drefinebounds, convergence count) ..................... dlansvd_irl.F:218-290
//   converged: Ritz vectors (dritzvec.F) | else: exact shifts, wavefront
//   bsvdstep sweeps and the restart products ............... dlansvd_irl.F:304-398
// The host captures "reset ticket, cycle kernel, read the number of active
// problems" in a CUDA graph and replays it until every problem has finished.
// A problem that meets an invariant subspace (which the reference handles
// with a fresh random vector, dgetu0.F) is marked for the single-problem
// driver.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/propack_gb300.h"
#include "pgb.cuh"
#include "pgb_bidiag.cuh"
#include "pgb_planes.cuh"
#include "pgb_scalar.cuh"

namespace pgb {

constexpr int BT = 256;  // threads per CTA
constexpr int BW = BT / 32;
constexpr int BDIM_MAX = 64;
// restart cycles a CTA runs on one problem per graph replay.  The cycle is
// FP64-pipe bound on its SM, and every replay ends at the slowest CTA, so
// problems run (nearly) to completion inside one replay: the makespan is then
// the largest problem's solve or the total work over the grid, whichever is
// longer; further replays only serve problems that need more cycles
constexpr int BATCH_CYCLES_PER_LAUNCH = 64;

enum { BS_ACTIVE = 0, BS_CONVERGED = 1, BS_MAXITER = 2, BS_FALLBACK = 3 };

struct BProb {
    int m, n;
    const int *ptr, *idx;     // A (m x n), local column indices
    const float *val;
    const int *tptr, *tidx;   // A' (n x m)
    const float *tval;
    double *U, *V;            // m x (dim+1), n x dim (leading dimensions m, n)
    float2 *Up, *Vp;          // their FP32 (hi, lo) planes, written when a column is final
    double *alpha, *beta;     // dim + 1 each
    double *sig, *bnd;        // neig each (outputs)
    double rnorm, anorm;
    int k0, iter, status, nconv, nopx, nreorth;
    int g;    // SpMV row split: lanes per row (1, 4, 8 or 32), chosen by the autotuner
    int dc;   // Gram-Schmidt projections: columns per warp (1, 2 or 4), chosen by the autotuner
};

struct BCfg {
    int dim, k, neig, maxiter, ielr;
    double tol, min_relgap;
};

// per-CTA scratch (global memory): sizes for dimension dim
struct BScrLayout {
    size_t P, Q, coef, tw, Mt, Xt, W, total;
};
__host__ __device__ inline BScrLayout bscr_layout(int dim, int maxrows)
{
    BScrLayout L;
    const size_t d1 = dim + 1;
    L.P = 0;
    L.Q = L.P + d1 * d1;
    L.coef = L.Q + (size_t)dim * dim;
    L.tw = L.coef + (size_t)dim * 4 * d1;
    L.Mt = L.tw + (size_t)dim * 6 * dim;
    L.Xt = L.Mt + d1 * d1;
    L.W = L.Xt + d1 * dim;
    L.total = L.W + (size_t)maxrows * d1;
    return L;
}

struct BShared {
    double red[32];
    double h[BDIM_MAX + 2];
    double d[BDIM_MAX + 2], e[BDIM_MAX + 2], sig[BDIM_MAX + 2], bnd[BDIM_MAX + 2];
    double b2[2 * BDIM_MAX + 2];
    double cs[BDIM_MAX + 2], sn[BDIM_MAX + 2];
    double shifts[BDIM_MAX + 2];
    double scal[8];
    float2 hp[BDIM_MAX + 2];  // Gram-Schmidt coefficients as planes
    int flag, xe;
};

// ------------------------------------------------------ CTA vector helpers
__device__ __forceinline__ double cta_sum(double v, BShared &S) { return block_sum<BT>(v, S.red); }

__device__ double cta_nrm2(const double *x, int n, BShared &S)
{
    double a = 0.0;
    for (int i = threadIdx.x; i < n; i += BT) a = fma(x[i], x[i], a);
    return sqrt(cta_sum(a, S));
}
__device__ double cta_dot(const double *x, const double *y, int n, BShared &S)
{
    double a = 0.0;
    for (int i = threadIdx.x; i < n; i += BT) a = fma(x[i], y[i], a);
    return cta_sum(a, S);
}
__device__ void cta_axpy(int n, double a, const double *x, double *y)
{
    for (int i = threadIdx.x; i < n; i += BT) y[i] = fma(a, x[i], y[i]);
    __syncthreads();
}
// dsafescal (dsafescal.F:4-55)
__device__ void cta_safescal(int n, double a, double *x)
{
    if (fabs(a) >= SFMIN) {
        const double r = 1.0 / a;
        for (int i = threadIdx.x; i < n; i += BT) x[i] *= r;
    } else {
        for (int i = threadIdx.x; i < n; i += BT) x[i] /= a;
    }
    __syncthreads();
}
// y = A x (A: rows x *, CSR with FP32 values) with g lanes per row (the row
// split, g a power of two <= 32): a group of g lanes takes a row, each lane
// every g-th nonzero with four (index, value) pairs and four gathers in
// flight, then the group adds its partial sums by a shuffle tree.  g = 1 is
// one thread per row.  The autotuner picks g per problem class: long rows
// and few of them favour wide groups, many short rows g = 1.
__device__ void cta_spmv(const int *ptr, const int *idx, const float *val, int rows, const double *x, double *y,
                         int g)
{
    const int grp = threadIdx.x / g, lig = threadIdx.x % g, ngrp = BT / g;
    for (int r0 = 0; r0 < rows; r0 += ngrp) {
        const int r = r0 + grp;
        double s = 0.0;
        if (r < rows) {
            const int e1 = ptr[r + 1];
            int e = ptr[r] + lig;
            for (; e + 3 * g < e1; e += 4 * g) {
                const int c0 = idx[e], c1 = idx[e + g], c2 = idx[e + 2 * g], c3 = idx[e + 3 * g];
                const float v0 = val[e], v1 = val[e + g], v2 = val[e + 2 * g], v3 = val[e + 3 * g];
                const double x0 = x[c0], x1 = x[c1], x2 = x[c2], x3 = x[c3];
                s = fma((double)v0, x0, s);
                s = fma((double)v1, x1, s);
                s = fma((double)v2, x2, s);
                s = fma((double)v3, x3, s);
            }
            for (; e < e1; e += g) s = fma((double)val[e], x[idx[e]], s);
        }
        // every lane of a warp takes part (rows past the end add zeros)
        for (int o = g >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, g);
        if (r < rows && lig == 0) y[r] = s;
    }
    __syncthreads();
}
// dreorth with iterated CGS (dreorth.F:106-210): x against the first ncols
// columns of W (leading dimension ld); *nrm is ||x|| on entry and exit
// projections h = W(:, 0:ncols)' x into S.h: each warp takes dc adjacent
// columns at a time and reads each x element once for all of them (the
// autotuner's choice of dc; every column's sum is formed in the same order
// whatever dc is, so the choice does not change the result)
template <int DC>
__device__ void cta_proj(const double *W, int ld, int ncols, const double *x, int len, BShared &S)
{
    const int lane = threadIdx.x & 31;
    for (int c0 = (threadIdx.x >> 5) * DC; c0 < ncols; c0 += BW * DC) {
        const int nc = min(DC, ncols - c0);
        double s[DC];
#pragma unroll
        for (int u = 0; u < DC; u++) s[u] = 0.0;
        for (int i = lane; i < len; i += 32) {
            const double xi = x[i];
#pragma unroll
            for (int u = 0; u < DC; u++)
                if (u < nc) s[u] = fma(W[(size_t)(c0 + u) * ld + i], xi, s[u]);
        }
#pragma unroll
        for (int u = 0; u < DC; u++) {
            const double t = warp_sum(s[u]);
            if (lane == 0 && u < nc) S.h[c0 + u] = t;
        }
    }
}
__device__ void cta_proj_dc(const double *W, int ld, int ncols, const double *x, int len, BShared &S, int dc)
{
    if (dc >= 4) cta_proj<4>(W, ld, ncols, x, len, S);
    else if (dc == 2) cta_proj<2>(W, ld, ncols, x, len, S);
    else cta_proj<1>(W, ld, ncols, x, len, S);
}

__device__ void cta_reorth(const double *W, int ld, int ncols, double *x, int len, double *nrm, BShared &S, int &count,
                           int dc)
{
    if (ncols <= 0) return;
    double nrm0 = *nrm;
    for (int it = 0; it < NTRY; it++) {
        cta_proj_dc(W, ld, ncols, x, len, S, dc);
        __syncthreads();
        double a = 0.0;
        for (int i = threadIdx.x; i < len; i += BT) {
            double v = x[i];
            int c = 0;
            for (; c + 3 < ncols; c += 4) {
                const double w0 = W[(size_t)c * ld + i], w1 = W[(size_t)(c + 1) * ld + i];
                const double w2 = W[(size_t)(c + 2) * ld + i], w3 = W[(size_t)(c + 3) * ld + i];
                v = fma(-w0, S.h[c], v);
                v = fma(-w1, S.h[c + 1], v);
                v = fma(-w2, S.h[c + 2], v);
                v = fma(-w3, S.h[c + 3], v);
            }
            for (; c < ncols; c++) v = fma(-W[(size_t)c * ld + i], S.h[c], v);
            x[i] = v;
            a = fma(v, v, a);
        }
        const double s = sqrt(cta_sum(a, S));
        if (s > KAPPA * nrm0) {
            *nrm = s;
            count++;
            return;
        }
        nrm0 = s;
    }
    for (int i = threadIdx.x; i < len; i += BT) x[i] = 0.0;
    __syncthreads();
    *nrm = 0.0;
    count++;
}

// ---------------------------------------------------- on the FP32 pipe
// With propack_batch_set_arith(h, 2) the cycle's products and Gram-Schmidt
// passes read the bases as FP32 (hi, lo) planes (pgb_planes.cuh): every
// basis column is split once, when it is final (normalised, or rewritten by
// a restart), and every later product or projection that reads it runs on
// the FP32 pipe instead of the FP64 pipe.  Measured on a GB300 (1024
// problems of the batched workload) it is not faster: 4899 ms and 635,328
// matvecs against 4299 ms and 581,632 with the FP64 routines above, which
// stay the default.

__device__ void cta_split_col(const double *w, float2 *wp, int len)
{
    for (int i = threadIdx.x; i < len; i += BT) wp[i] = pl_split(w[i]);
}

// y = A x with x given by its planes: each product val * (hi + lo) with the
// FP32 value exact, summed as a compensated pair, the row split g as in
// cta_spmv; y in FP64
__device__ void cta_spmv_pl(const int *ptr, const int *idx, const float *val, int rows, const float2 *xp, double *y,
                            int g)
{
    const int grp = threadIdx.x / g, lig = threadIdx.x % g, ngrp = BT / g;
    for (int r0 = 0; r0 < rows; r0 += ngrp) {
        const int r = r0 + grp;
        PlAcc acc;
        if (r < rows) {
            const int e1 = ptr[r + 1];
            int e = ptr[r] + lig;
            for (; e + 3 * g < e1; e += 4 * g) {
                const int c0 = idx[e], c1 = idx[e + g], c2 = idx[e + 2 * g], c3 = idx[e + 3 * g];
                const float v0 = val[e], v1 = val[e + g], v2 = val[e + 2 * g], v3 = val[e + 3 * g];
                const float2 x0 = xp[c0], x1 = xp[c1], x2 = xp[c2], x3 = xp[c3];
                acc.add(v0, 0.f, x0.x, x0.y);
                acc.add(v1, 0.f, x1.x, x1.y);
                acc.add(v2, 0.f, x2.x, x2.y);
                acc.add(v3, 0.f, x3.x, x3.y);
            }
            for (; e < e1; e += g) {
                const float2 xv = xp[idx[e]];
                acc.add(val[e], 0.f, xv.x, xv.y);
            }
        }
        for (int o = g >> 1; o > 0; o >>= 1)
            pl_pair_add(acc.s, acc.c, __shfl_xor_sync(0xffffffffu, acc.s, o, g),
                        __shfl_xor_sync(0xffffffffu, acc.c, o, g));
        if (r < rows && lig == 0) y[r] = acc.value_int();
    }
    __syncthreads();
}

// projections S.h = Wp(:, 0:ncols)' xq * back from the planes, dc adjacent
// columns per warp (every column's sum in the same order whatever dc is)
template <int DC>
__device__ void cta_proj_pl(const float2 *Wp, int ld, int ncols, const float2 *xq, int len, double back, BShared &S)
{
    const int lane = threadIdx.x & 31;
    for (int c0 = (threadIdx.x >> 5) * DC; c0 < ncols; c0 += BW * DC) {
        const int nc = min(DC, ncols - c0);
        PlAcc acc[DC];
        for (int i = lane; i < len; i += 32) {
            const float2 xv = xq[i];
#pragma unroll
            for (int u = 0; u < DC; u++)
                if (u < nc) {
                    const float2 wv = Wp[(size_t)(c0 + u) * ld + i];
                    acc[u].add(wv.x, wv.y, xv.x, xv.y);
                }
        }
#pragma unroll
        for (int u = 0; u < DC; u++) {
            const double t = warp_sum(acc[u].value_int());
            if (lane == 0 && u < nc) S.h[c0 + u] = t * back;
        }
    }
}
__device__ void cta_proj_pl_dc(const float2 *Wp, int ld, int ncols, const float2 *xq, int len, double back, BShared &S,
                               int dc)
{
    if (dc >= 4) cta_proj_pl<4>(Wp, ld, ncols, xq, len, back, S);
    else if (dc == 2) cta_proj_pl<2>(Wp, ld, ncols, xq, len, back, S);
    else cta_proj_pl<1>(Wp, ld, ncols, xq, len, back, S);
}

// x (len) as planes in xq, scaled by 2^-xs for the CTA's largest exponent
// (|x 2^-xs| < 2); returns 2^xs
__device__ double cta_xplanes(const double *x, int len, float2 *xq, BShared &S)
{
    if (threadIdx.x == 0) S.xe = 0;
    __syncthreads();
    int e = 0;
    for (int i = threadIdx.x; i < len; i += BT) e = max(e, f3_expo(x[i]));
    if (e) atomicMax(&S.xe, e);
    __syncthreads();
    const int xs = S.xe == 0 ? 0 : S.xe - 1023;
    for (int i = threadIdx.x; i < len; i += BT) xq[i] = pl_xsplit(x[i], xs);
    __syncthreads();
    return f3_pow2(xs);
}

// dreorth with iterated CGS on the planes of W (dreorth.F:106-210); the same
// control flow as cta_reorth.  xq: len float2 of scratch
__device__ void cta_reorth_pl(const float2 *Wp, int ld, int ncols, double *x, int len, double *nrm, BShared &S,
                              int &count, int dc, float2 *xq)
{
    if (ncols <= 0) return;
    double nrm0 = *nrm;
    for (int it = 0; it < NTRY; it++) {
        const double back = cta_xplanes(x, len, xq, S);
        cta_proj_pl_dc(Wp, ld, ncols, xq, len, back, S, dc);
        __syncthreads();
        // h as planes, scaled by the power of two of its largest entry
        if (threadIdx.x == 0) S.xe = 0;
        __syncthreads();
        int he = 0;
        for (int c = threadIdx.x; c < ncols; c += BT) he = max(he, f3_expo(S.h[c]));
        if (he) atomicMax(&S.xe, he);
        __syncthreads();
        const int hs = S.xe == 0 ? 0 : S.xe - 1023;
        for (int c = threadIdx.x; c < ncols; c += BT) S.hp[c] = pl_xsplit(S.h[c], hs);
        __syncthreads();
        const double hback = f3_pow2(hs);
        double a = 0.0;
        for (int i = threadIdx.x; i < len; i += BT) {
            PlAcc sm;
            for (int c = 0; c < ncols; c++) {
                const float2 wv = Wp[(size_t)c * ld + i];
                sm.add(wv.x, wv.y, S.hp[c].x, S.hp[c].y);
            }
            double v = x[i];
            v = fma(-pl_f2d(sm.s), hback, v);
            v = fma(-pl_f2d(sm.c), hback, v);
            x[i] = v;
            a = fma(v, v, a);
        }
        const double s = sqrt(cta_sum(a, S));
        if (s > KAPPA * nrm0) {
            *nrm = s;
            count++;
            return;
        }
        nrm0 = s;
    }
    for (int i = threadIdx.x; i < len; i += BT) x[i] = 0.0;
    __syncthreads();
    *nrm = 0.0;
    count++;
}

// ------------------------------------------------------------- Lanczos
// dlanbpro.F:146-549 with full reorthogonalisation, from k0 to dim.
// Returns false when the problem must go to the single-problem driver.
template <bool PL>
__device__ bool b_lanbpro(BProb &P, const BCfg &c, BShared &S, float2 *xq)
{
    const int m = P.m, n = P.n, dim = c.dim, k0 = P.k0;
    float2 *Up = P.Up, *Vp = P.Vp;
    int nopx = 0, nre = 0;  // counted redundantly by every thread, stored by thread 0
    bool ok = true;
    const int mn = m > n ? m : n;
    const double epsn = (double)mn * EPS;
    double *U = P.U, *V = P.V, *ba = P.alpha, *bb = P.beta;
    double anorm = P.anorm, alpha, beta, amax = 0.0, a1, b1, s;
    int j0;
    if (k0 == 0) {
        beta = P.rnorm;
        alpha = 0.0;
        cta_safescal(m, beta, U);
        if (PL) cta_split_col(U, Up, m);
        __syncthreads();
        j0 = 1;
    } else {
        alpha = ba[k0 - 1];
        beta = P.rnorm;
        // the restart rewrote U(:, 0:k0) and V(:, 0:k0): their planes
        if (PL)
            for (int q = 0; q < k0; q++) {
                cta_split_col(U + (size_t)q * m, Up + (size_t)q * m, m);
                cta_split_col(V + (size_t)q * n, Vp + (size_t)q * n, n);
            }
        __syncthreads();
        double *uk = U + (size_t)k0 * m;
        for (int i = threadIdx.x; i < m; i += BT) uk[i] *= P.rnorm;
        __syncthreads();
        double r = P.rnorm;
        if (PL) cta_reorth_pl(Up, m, k0, uk, m, &r, S, nre, P.dc, xq);
        else cta_reorth(U, m, k0, uk, m, &r, S, nre, P.dc);
        cta_safescal(m, r, uk);
        if (PL) cta_split_col(uk, Up + (size_t)k0 * m, m);
        __syncthreads();
        beta = r;
        if (threadIdx.x == 0) bb[k0 - 1] = beta;
        __syncthreads();
        for (int j = 1; j <= k0; j++) {
            amax = fmax(amax, fmax(ba[j - 1], bb[j - 1]));
            if (j == 1) {
                anorm = fmax(anorm, FUDGE * alpha);
            } else if (j == 2) {
                a1 = bb[0] / amax;
                a1 = FUDGE * amax * sqrt((ba[0] / amax) * (ba[0] / amax) + a1 * a1 + ba[1] / amax * a1);
                anorm = fmax(anorm, a1);
            } else {
                a1 = ba[j - 2] / amax;
                b1 = bb[j - 2] / amax;
                a1 = FUDGE * amax * sqrt(a1 * a1 + b1 * b1 + a1 * bb[j - 3] / amax + ba[j - 1] / amax * b1);
                anorm = fmax(anorm, a1);
            }
        }
        j0 = k0 + 1;
    }
    for (int j = j0; j <= dim; j++) {
        double *vj = V + (size_t)(j - 1) * n, *uj = U + (size_t)(j - 1) * m, *uj1 = U + (size_t)j * m;
        // alpha_j v_j = A' u_j - beta_j v_{j-1}
        if (PL) cta_spmv_pl(P.tptr, P.tidx, P.tval, n, Up + (size_t)(j - 1) * m, vj, P.g);
        else cta_spmv(P.tptr, P.tidx, P.tval, n, uj, vj, P.g);
        nopx++;
        if (j == 1) {
            alpha = cta_nrm2(vj, n, S);
            anorm = fmax(anorm, FUDGE * alpha);
        } else {
            cta_axpy(n, -beta, vj - n, vj);
            alpha = cta_nrm2(vj, n, S);
            if (c.ielr > 0 && alpha < KAPPA * beta) {
                for (int i = 1; i <= c.ielr; i++) {
                    s = cta_dot(vj - n, vj, n, S);
                    cta_axpy(n, -s, vj - n, vj);
                    if (beta != 0.0) {
                        beta = beta + s;
                        if (threadIdx.x == 0) bb[j - 2] = beta;
                    }
                    s = cta_nrm2(vj, n, S);
                    if (s >= KAPPA * alpha) break;
                    alpha = s;
                }
                alpha = s;
            }
            amax = fmax(amax, alpha);
            if (j == 2) {
                a1 = bb[0] / amax;
                a1 = FUDGE * amax * sqrt((ba[0] / amax) * (ba[0] / amax) + a1 * a1 + alpha / amax * a1);
            } else {
                a1 = ba[j - 2] / amax;
                b1 = bb[j - 2] / amax;
                a1 = FUDGE * amax * sqrt(a1 * a1 + b1 * b1 + a1 * bb[j - 3] / amax + alpha / amax * b1);
            }
            anorm = fmax(anorm, a1);
        }
        if (alpha != 0.0) {
            if (PL) cta_reorth_pl(Vp, n, j - 1, vj, n, &alpha, S, nre, P.dc, xq);
            else cta_reorth(V, n, j - 1, vj, n, &alpha, S, nre, P.dc);
        }
        if (alpha < anorm * epsn && j < dim) { ok = false; break; }
        if (threadIdx.x == 0) ba[j - 1] = alpha;
        if (alpha != 0.0) cta_safescal(n, alpha, vj);
        if (PL) {
            cta_split_col(vj, Vp + (size_t)(j - 1) * n, n);
            __syncthreads();
        }
        // beta_{j+1} u_{j+1} = A v_j - alpha_j u_j
        if (PL) cta_spmv_pl(P.ptr, P.idx, P.val, m, Vp + (size_t)(j - 1) * n, uj1, P.g);
        else cta_spmv(P.ptr, P.idx, P.val, m, vj, uj1, P.g);
        nopx++;
        cta_axpy(m, -alpha, uj, uj1);
        beta = cta_nrm2(uj1, m, S);
        if (c.ielr > 0 && beta < KAPPA * alpha) {
            for (int i = 1; i <= c.ielr; i++) {
                s = cta_dot(uj, uj1, m, S);
                cta_axpy(m, -s, uj, uj1);
                if (alpha != 0.0) {
                    alpha = alpha + s;
                    if (threadIdx.x == 0) ba[j - 1] = alpha;
                }
                s = cta_nrm2(uj1, m, S);
                if (s >= KAPPA * beta) break;
                beta = s;
            }
            beta = s;
        }
        __syncthreads();
        amax = fmax(amax, beta);
        if (j <= 1) {
            a1 = hypot(ba[0], beta);
        } else {
            a1 = ba[j - 1] / amax;
            a1 = amax * sqrt(a1 * a1 + (beta / amax) * (beta / amax) + a1 * bb[j - 2] / amax);
        }
        anorm = fmax(anorm, a1);
        if (beta != 0.0) {
            if (PL) cta_reorth_pl(Up, m, j, uj1, m, &beta, S, nre, P.dc, xq);
            else cta_reorth(U, m, j, uj1, m, &beta, S, nre, P.dc);
        }
        if (beta < anorm * epsn && j < dim) { ok = false; break; }
        if (threadIdx.x == 0) bb[j - 1] = beta;
        if (beta != 0.0) cta_safescal(m, beta, uj1);
        if (PL) {
            cta_split_col(uj1, Up + (size_t)j * m, m);
            __syncthreads();
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        P.rnorm = beta;
        P.anorm = anorm;
        P.nopx += nopx;
        P.nreorth += nre;
    }
    __syncthreads();
    return ok;
}

// ------------------------------------------------------------ analysis
// singular values of R (S.d, S.e; upper bidiagonal dim x dim) into S.sig,
// warp multisection per value
__device__ void b_sigmas(int dim, BShared &S)
{
    for (int j = threadIdx.x; j < 2 * dim - 1; j += BT) {
        const double b = tgk_b(S.d, S.e, j);
        S.b2[j] = b * b;
    }
    if (threadIdx.x == 0) tgk_bounds(S.d, S.e, dim, S.scal[0], S.scal[1]);
    __syncthreads();
    for (int t = (threadIdx.x >> 5) + 1; t <= dim; t += BW) {
        const double v = warp_sigma(dim, S.b2, t, S.scal[0], S.scal[1]);
        if ((threadIdx.x & 31) == 0) S.sig[t - 1] = v;
    }
    __syncthreads();
}

// dlansvd_irl.F:218-290: sigma, bounds, convergence count (IRL branch)
__device__ int b_analyse(BProb &P, const BCfg &c, BShared &S, double *scr, const BScrLayout &L)
{
    const int dim = c.dim, mn = P.m < P.n ? P.m : P.n;
    for (int i = threadIdx.x; i < dim; i += BT) { S.d[i] = P.alpha[i]; S.e[i] = P.beta[i]; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double c1 = 0.0, c2 = 0.0;
        bdqr_dev(dim == mn, dim, S.d, S.e, &c1, &c2, nullptr, 0);
        S.scal[2] = c1;
        S.flag = 0;
    }
    __syncthreads();
    b_sigmas(dim, S);
    const double c1 = S.scal[2];
    for (int i = threadIdx.x; i < dim; i += BT) {
        double *Dp = scr + L.tw + (size_t)i * 6 * dim, *Dm = Dp + 2 * dim;
        const double zn = tgk_twisted(S.d, S.e, dim, S.sig[i], S.scal[1], Dp, Dm, nullptr);
        const double b = fabs(P.rnorm * c1 * sqrt(2.0) * zn);
        if (!(b == b) || !(S.sig[i] == S.sig[i])) S.flag = 1;
        S.bnd[i] = b;
    }
    __syncthreads();
    if (S.flag) return -1;
    if (threadIdx.x == 0) {
        const double eps34 = pow(EPS, 0.75);
        const double epsn = (double)(P.m > P.n ? P.m : P.n) * EPS / 2.0;
        double anorm = P.anorm;
        if (dim > 5) anorm = S.sig[0];
        else anorm = fmax(anorm, S.sig[0]);
        P.anorm = anorm;
        const int lim = dim < c.neig ? dim : c.neig;
        refinebounds_dev(mn, lim, S.sig, S.bnd, epsn * anorm, eps34);
        int nconv = 0, i = 1;
        while (i <= lim) {
            if (S.bnd[i - 1] <= c.tol * S.sig[i - 1]) { nconv++; i++; }
            else i = c.k + 1;
        }
        P.nconv = nconv;
    }
    __syncthreads();
    return P.nconv;
}

// ------------------------------------------------------------- restart
// exact shifts, wavefront bsvdstep sweeps (the same step order argument as
// k_irl_chain: sweep s+1 runs step i while sweep s runs step i+3), P and Q,
// then U(:,1:k+1) <- U P(:,1:k+1), V(:,1:k) <- V Q(:,1:k)
__device__ void b_restart(BProb &P, const BCfg &c, BShared &S, double *scr, const BScrLayout &L)
{
    const int dim = c.dim, k = c.k, dp1 = dim + 1, nsw = dim - k;
    double *D = S.d, *E = S.e;  // the lower bidiagonal B of the run
    for (int i = threadIdx.x; i < dim; i += BT) { D[i] = P.alpha[i]; E[i] = P.beta[i]; }
    if (threadIdx.x == 0) {
        for (int i = dim; i >= k + 1; i--) {
            const double relgap = S.sig[k - 1] - (S.sig[i - 1] + S.bnd[i - 1]);
            S.shifts[dim - i] = (relgap > c.min_relgap * S.sig[k - 1]) ? S.sig[i - 1] : 0.0;
        }
    }
    __syncthreads();
    double *coef = scr + L.coef;
    {
        const int s = threadIdx.x;
        const int kk = dim - s;
        const bool active = s < nsw && kk > 1;
        const double sigma = active ? S.shifts[s] : 0.0;
        double *cu = coef + (size_t)(s < nsw ? s : 0) * 4 * dp1, *su = cu + dp1, *cv = cu + 2 * dp1, *sv = cu + 3 * dp1;
        double x = 0.0, y = 0.0, cc, sn, r;
        const int gend = dim + 3 * (nsw - 1);
        for (int g = 0; g <= gend; g++) {
            const int i = g - 3 * s;
            if (active && i >= 0 && i <= kk) {
                if (i == 0) {
                    x = D[0] * D[0] - sigma * sigma;
                    y = E[0] * D[0];
                } else if (i < kk) {
                    if (i > 1) lartg(x, y, cc, sn, E[i - 2]);
                    else lartg(x, y, cc, sn, r);
                    x = cc * D[i - 1] + sn * E[i - 1];
                    E[i - 1] = -sn * D[i - 1] + cc * E[i - 1];
                    D[i - 1] = x;
                    y = sn * D[i];
                    D[i] = cc * D[i];
                    cu[i - 1] = cc; su[i - 1] = sn;
                    lartg(x, y, cc, sn, D[i - 1]);
                    x = cc * E[i - 1] + sn * D[i];
                    D[i] = -sn * E[i - 1] + cc * D[i];
                    E[i - 1] = x;
                    y = sn * E[i];
                    E[i] = cc * E[i];
                    cv[i - 1] = cc; sv[i - 1] = sn;
                } else {
                    lartg(x, y, cc, sn, E[kk - 2]);
                    x = cc * D[kk - 1] + sn * E[kk - 1];
                    E[kk - 1] = -sn * D[kk - 1] + cc * E[kk - 1];
                    D[kk - 1] = x;
                    cu[kk - 1] = cc; su[kk - 1] = sn;
                }
            }
            __syncthreads();
        }
    }
    // P ((dim+1)^2) and Q (dim^2), one warp per row, waves of 32 sweeps with
    // lag 2; the row lives in the warp's slice of the scratch
    double *Pm = scr + L.P, *Qm = scr + L.Q;
    const int lane = threadIdx.x & 31;
    for (int row = threadIdx.x >> 5; row < dp1 + dim; row += BW) {
        const bool isP = row < dp1;
        const int rr = isP ? row : row - dp1, nrows = isP ? dp1 : dim;
        double *M = isP ? Pm : Qm;
        for (int t = lane; t < nrows; t += 32) M[(size_t)t * nrows + rr] = (t == rr) ? 1.0 : 0.0;
        __syncwarp();
        for (int w0 = 0; w0 < nsw; w0 += 32) {
            const int s = w0 + lane, kk = dim - s;
            const int nrot = (s < nsw && kk > 1) ? (isP ? kk : kk - 1) : -1;
            const double *cc = coef + (size_t)(s < nsw ? s : 0) * 4 * dp1 + (isP ? 0 : 2 * dp1), *ss = cc + dp1;
            const int kk0 = dim - w0;
            const int gend = (isP ? kk0 : kk0 - 1) + 2 * 31;
            double xc = 0.0;
            for (int g = 0; g <= gend; g++) {
                const int t = g - 2 * lane;
                if (nrot > 0 && t >= 0 && t <= nrot) {
                    if (t < nrot) {
                        const double cv = cc[t], sv = ss[t];
                        if (t == 0) xc = M[rr];
                        const double yc = M[(size_t)(t + 1) * nrows + rr];
                        M[(size_t)t * nrows + rr] = cv * xc + sv * yc;
                        xc = cv * yc - sv * xc;
                    } else {
                        M[(size_t)nrot * nrows + rr] = xc;
                    }
                }
                __syncwarp();
            }
        }
    }
    for (int i = threadIdx.x; i < dim; i += BT) { P.alpha[i] = D[i]; P.beta[i] = E[i]; }
    __syncthreads();
    // restart products through the W scratch (rows x (k+1))
    double *W = scr + L.W;
    for (int side = 0; side < 2; side++) {
        const int rows = side == 0 ? P.m : P.n, kin = side == 0 ? dp1 : dim, kout = side == 0 ? k + 1 : k;
        double *A = side == 0 ? P.U : P.V;
        const double *B = side == 0 ? Pm : Qm;
        const int ldb = side == 0 ? dp1 : dim;
        for (int i = threadIdx.x; i < rows; i += BT)
            for (int cc = 0; cc < kout; cc++) {
                double a = 0.0;
                for (int l = 0; l < kin; l++) a = fma(A[(size_t)l * rows + i], B[(size_t)cc * ldb + l], a);
                W[(size_t)cc * rows + i] = a;
            }
        __syncthreads();
        for (size_t t = threadIdx.x; t < (size_t)rows * kout; t += BT) A[t] = W[t];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        P.rnorm = E[k - 1];
        P.k0 = k;
    }
    __syncthreads();
}

// --------------------------------------------------------------- Ritz
// dritzvec.F:1-199 for the leading neig triplets: dbdqr with Q', the
// singular vectors of R by twisted factorizations, then the products.
// Returns false (single-problem driver) for values closer than 1e-9 sigma_1.
__device__ bool b_ritz(BProb &P, const BCfg &c, BShared &S, double *scr, const BScrLayout &L)
{
    const int dim = c.dim, dp1 = dim + 1, neig = c.neig, mn = P.m < P.n ? P.m : P.n;
    for (int i = threadIdx.x; i < dim; i += BT) { S.d[i] = P.alpha[i]; S.e[i] = P.beta[i]; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double cs, sn, r;
        double *D = S.d, *E = S.e;
        int i;
        for (i = 1; i <= dim - 1; i++) {
            lartg(D[i - 1], E[i - 1], cs, sn, r);
            D[i - 1] = r;
            E[i - 1] = sn * D[i];
            D[i] = cs * D[i];
            S.cs[i - 1] = cs; S.sn[i - 1] = sn;
        }
        int nrot = dim - 1;
        if (dim != mn) {
            lartg(D[dim - 1], E[dim - 1], cs, sn, r);
            D[dim - 1] = r;
            E[dim - 1] = 0.0;
            S.cs[dim - 1] = cs; S.sn[dim - 1] = sn;
            nrot = dim;
        }
        S.scal[3] = nrot;
        S.flag = 0;
    }
    __syncthreads();
    const int nrot = (int)S.scal[3];
    double *Mt = scr + L.Mt;
    for (int j = threadIdx.x; j < dp1; j += BT) {
        double *col = Mt + (size_t)j * dp1;
        for (int i = 0; i < dp1; i++) col[i] = 0.0;
        if (j == 0) col[0] = 1.0;
        else if (j - 1 < nrot) { col[j - 1] = S.sn[j - 1]; col[j] = S.cs[j - 1]; }
        else col[j] = 1.0;
        for (int i = (j == 0 ? 0 : j); i < nrot; i++) {
            col[i + 1] = -S.sn[i] * col[i];
            col[i] = S.cs[i] * col[i];
        }
    }
    b_sigmas(dim, S);
    // vectors x_q (dim) and y_q (dim) into the twisted scratch rows
    double *tw = scr + L.tw;
    for (int q = threadIdx.x; q < neig; q += BT) {
        const double smax = S.sig[0];
        const double gap = fmin(q > 0 ? S.sig[q - 1] - S.sig[q] : INFINITY, q + 1 < dim ? S.sig[q] - S.sig[q + 1] : INFINITY);
        if (!(gap > 1e-9 * smax) || !(S.sig[q] > 1e-9 * smax)) { S.flag = 1; continue; }
        double *Dp = tw + (size_t)q * 6 * dim, *Dm = Dp + 2 * dim, *z = Dm + 2 * dim;
        tgk_twisted(S.d, S.e, dim, S.sig[q], S.scal[1], Dp, Dm, z);
        double nx = 0.0, ny = 0.0;
        for (int t = 0; t < dim; t++) { nx += z[2 * t] * z[2 * t]; ny += z[2 * t + 1] * z[2 * t + 1]; }
        if (!(nx > 0.0) || !(ny > 0.0)) { S.flag = 1; continue; }
        const double ix = 1.0 / sqrt(nx), iy = 1.0 / sqrt(ny);
        // x_q -> Dp[0..dim), y_q -> Dm[0..dim) (the pivots are no longer needed)
        for (int t = 0; t < dim; t++) { Dp[t] = z[2 * t] * ix; Dm[t] = z[2 * t + 1] * iy; }
    }
    __syncthreads();
    if (S.flag) return false;
    // Xt(l, q) = sum_t y_q(t) Mt(t, l), l < dim + 1
    double *Xt = scr + L.Xt;
    for (int t2 = threadIdx.x; t2 < dp1 * neig; t2 += BT) {
        const int l = t2 % dp1, q = t2 / dp1;
        const double *y = tw + (size_t)q * 6 * dim + 2 * dim;
        double a = 0.0;
        for (int t = 0; t < dim; t++) a = fma(y[t], Mt[(size_t)l * dp1 + t], a);
        Xt[(size_t)q * dp1 + l] = a;
    }
    __syncthreads();
    double *W = scr + L.W;
    for (int side = 0; side < 2; side++) {
        const int rows = side == 0 ? P.m : P.n, kin = side == 0 ? dp1 : dim;
        double *A = side == 0 ? P.U : P.V;
        for (int i = threadIdx.x; i < rows; i += BT)
            for (int q = 0; q < neig; q++) {
                const double *b = side == 0 ? Xt + (size_t)q * dp1 : tw + (size_t)q * 6 * dim;
                double a = 0.0;
                for (int l = 0; l < kin; l++) a = fma(A[(size_t)l * rows + i], b[l], a);
                W[(size_t)q * rows + i] = a;
            }
        __syncthreads();
        for (size_t t = threadIdx.x; t < (size_t)rows * neig; t += BT) A[t] = W[t];
        __syncthreads();
    }
    for (int q = threadIdx.x; q < neig; q += BT) { P.sig[q] = S.sig[q]; P.bnd[q] = S.bnd[q]; }
    __syncthreads();
    return true;
}

// ------------------------------------------------------- the cycle kernel
template <bool PL>
__global__ void __launch_bounds__(BT, 2) k_batch_cycle(BProb *probs, const int *order, int nprob, BCfg c,
                                                    double *scratch, size_t scr_stride, int *ticket, int *active,
                                                    int cycles_per_launch)
{
    __shared__ BShared S;
    __shared__ int pidx;
    const BScrLayout L = bscr_layout(c.dim, 0);
    double *scr = scratch + (size_t)blockIdx.x * scr_stride;
    while (true) {
        if (threadIdx.x == 0) pidx = atomicAdd(ticket, 1);
        __syncthreads();
        const int qi = pidx;
        if (qi >= nprob) break;
        BProb &P = probs[order[qi]];
        // up to cycles_per_launch restart cycles of this problem, then it is
        // handed back to the queue of the next replay
        for (int rep = 0; rep < cycles_per_launch && P.status == BS_ACTIVE; rep++) {
            bool ok = b_lanbpro<PL>(P, c, S, reinterpret_cast<float2 *>(scr + L.W));
            int nconv = ok ? b_analyse(P, c, S, scr, L) : -1;
            if (nconv < 0) {
                if (threadIdx.x == 0) P.status = BS_FALLBACK;
            } else if (nconv >= c.neig) {
                // the bounds of the converged values are the ones reported
                for (int q = threadIdx.x; q < c.neig; q += BT) P.bnd[q] = S.bnd[q];
                if (!b_ritz(P, c, S, scr, L)) {
                    if (threadIdx.x == 0) P.status = BS_FALLBACK;
                } else if (threadIdx.x == 0) {
                    P.status = BS_CONVERGED;
                }
            } else {
                b_restart(P, c, S, scr, L);
                if (threadIdx.x == 0) {
                    P.iter++;
                    if (P.iter >= c.maxiter) {
                        P.status = BS_MAXITER;
                        for (int q = 0; q < c.neig; q++) { P.sig[q] = S.sig[q]; P.bnd[q] = S.bnd[q]; }
                    }
                }
            }
            __syncthreads();
        }
        if (threadIdx.x == 0 && P.status == BS_ACTIVE) atomicAdd(active, 1);
        __syncthreads();
    }
}

// The autotuner's probe: for each sampled problem (one CTA each) the two
// products and the Gram-Schmidt projections of one vector against ncols
// columns on both sides, with the candidate row split g and projection tile
// dc.  The operands are the problem's own basis arrays and planes, zeroed
// beforehand: U(:,0) -> V(:,0) -> U(:,1), and column ncols of each side
// against the ncols before it.
template <bool PL>
__global__ void __launch_bounds__(BT) k_batch_probe(const BProb *probs, const int *sample, int ns, int g, int dc,
                                                    int ncols)
{
    __shared__ BShared S;
    for (int q = blockIdx.x; q < ns; q += gridDim.x) {
        const BProb &P = probs[sample[q]];
        if (PL) {
            cta_spmv_pl(P.tptr, P.tidx, P.tval, P.n, P.Up, P.V, g);
            cta_spmv_pl(P.ptr, P.idx, P.val, P.m, P.Vp, P.U + P.m, g);
            cta_proj_pl_dc(P.Up, P.m, ncols, P.Up + (size_t)ncols * P.m, P.m, 1.0, S, dc);
            __syncthreads();
            cta_proj_pl_dc(P.Vp, P.n, ncols, P.Vp + (size_t)ncols * P.n, P.n, 1.0, S, dc);
        } else {
            cta_spmv(P.tptr, P.tidx, P.tval, P.n, P.U, P.V, g);
            cta_spmv(P.ptr, P.idx, P.val, P.m, P.V, P.U + P.m, g);
            cta_proj_dc(P.U, P.m, ncols, P.U + (size_t)ncols * P.m, P.m, S, dc);
            __syncthreads();
            cta_proj_dc(P.V, P.n, ncols, P.V + (size_t)ncols * P.n, P.n, S, dc);
        }
        __syncthreads();
    }
}

// per-problem start: rnorm = ||U(:,1)||
__global__ void __launch_bounds__(BT) k_batch_start(BProb *probs, int nprob)
{
    __shared__ BShared S;
    for (int p = blockIdx.x; p < nprob; p += gridDim.x) {
        BProb &P = probs[p];
        const double r = cta_nrm2(P.U, P.m, S);
        if (threadIdx.x == 0) {
            P.rnorm = r;
            P.anorm = 0.0;
            P.k0 = 0;
            P.iter = 0;
            P.nconv = 0;
            P.nopx = 0;
            P.nreorth = 0;
            P.status = r > 0.0 ? BS_ACTIVE : BS_FALLBACK;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------ transposition
// A' of the block-diagonal batch: global column gc = noff[p] + col
__global__ void k_bt_count(int nprob, const int *moff, const int *noff, const int *rowptr, const int64_t *zoff,
                           const int *colidx, int *cnt)
{
    for (int p = blockIdx.x; p < nprob; p += gridDim.x) {
        const int m = moff[p + 1] - moff[p];
        const int *rp = rowptr + moff[p] + p;  // m + 1 entries per problem
        for (int e = threadIdx.x; e < rp[m]; e += blockDim.x) atomicAdd(&cnt[noff[p] + colidx[zoff[p] + e]], 1);
    }
}
__global__ void k_bt_scatter(int nprob, const int *moff, const int *noff, const int *rowptr, const int64_t *zoff,
                             const int *colidx, const float *val, const int *tptr, int *fill, int *tidx, float *tval)
{
    for (int p = blockIdx.x; p < nprob; p += gridDim.x) {
        const int m = moff[p + 1] - moff[p];
        const int *rp = rowptr + moff[p] + p;
        for (int r = threadIdx.x; r < m; r += blockDim.x)
            for (int e = rp[r]; e < rp[r + 1]; e++) {
                const int gc = noff[p] + colidx[zoff[p] + e];
                const int pos = tptr[gc] + atomicAdd(&fill[gc], 1);
                tidx[pos] = r;  // local row
                tval[pos] = val[zoff[p] + e];
            }
    }
}
// entries of each transposed row in increasing original row (insertion sort;
// rows are short), so the transposed SpMV sums in a fixed order
__global__ void k_bt_sort(int ncols, const int *tptr, int *tidx, float *tval)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncols; c += gridDim.x * blockDim.x) {
        const int a = tptr[c], b = tptr[c + 1];
        for (int i = a + 1; i < b; i++) {
            const int key = tidx[i];
            const float v = tval[i];
            int j = i - 1;
            while (j >= a && tidx[j] > key) { tidx[j + 1] = tidx[j]; tval[j + 1] = tval[j]; j--; }
            tidx[j + 1] = key;
            tval[j + 1] = v;
        }
    }
}

// ----------------------------------------------------------- host side
struct Batch {
    int nprob = 0, device = 0;
    std::vector<int> m, n;
    std::vector<int64_t> zoff;
    int *d_moff = nullptr, *d_noff = nullptr, *d_rowptr = nullptr, *d_colidx = nullptr, *d_tptr = nullptr,
        *d_tidx = nullptr;
    int64_t *d_zoff = nullptr;
    float *d_val = nullptr, *d_tval = nullptr;
    int64_t total_m = 0, total_n = 0, total_nnz = 0;
    std::vector<int> order;  // problems by decreasing cost
    // autotuner: per size class (quarters of `order`) the row split and the
    // projection tile, the probe's ms with them and with the defaults (1, 1)
    int tuned = 0;           // 0: tune at the next solve, 1: timed, 2: set by the caller
    int tuned_pl = -1;       // the arithmetic the timed table was made for (1: planes)
    int planes = 0;          // products and Gram-Schmidt on FP32 planes (propack_batch_set_arith)
    int g[PROPACK_BATCH_CLASSES], dc[PROPACK_BATCH_CLASSES];
    float ms_best[PROPACK_BATCH_CLASSES], ms_default[PROPACK_BATCH_CLASSES];
    int cls(int pos) const { return std::min(PROPACK_BATCH_CLASSES - 1, pos * PROPACK_BATCH_CLASSES / nprob); }
};
static std::mutex g_batch_mu;
static std::map<int64_t, Batch *> g_batches;
static int64_t g_batch_next = 1;
static thread_local propack_batch_stats_t g_batch_stats;

// Time every candidate (row split g, projection tile dc) on a sample of each
// size class and keep the fastest; the defaults (1, 1) stay unless a
// candidate is more than 3 % faster, so that near-ties do not flip the
// choice (and with it the SpMV's summation order) between batches.
template <bool PL>
static void batch_tune(Batch *B, BProb *dprob, int grid, int dim, cudaStream_t s)
{
    static const int gs[] = {1, 4, 8, 32};
    static const int dcs[] = {1, 2, 4};
    const int np = B->nprob, ncols = std::max(1, dim / 2);
    int *dsample = nullptr;
    PGB_CUDA(cudaMalloc(&dsample, sizeof(int) * std::max(1, np)));
    cudaEvent_t e0, e1;
    PGB_CUDA(cudaEventCreate(&e0));
    PGB_CUDA(cudaEventCreate(&e1));
    for (int c = 0; c < PROPACK_BATCH_CLASSES; c++) {
        const int p0 = c * np / PROPACK_BATCH_CLASSES, p1 = (c + 1) * np / PROPACK_BATCH_CLASSES;
        B->g[c] = 1;
        B->dc[c] = 1;
        B->ms_best[c] = B->ms_default[c] = 0.f;
        if (p1 <= p0) continue;
        const int ns = std::min(p1 - p0, grid);
        std::vector<int> sample(ns);
        for (int q = 0; q < ns; q++) sample[q] = B->order[p0 + (int)((int64_t)q * (p1 - p0) / ns)];
        PGB_CUDA(cudaMemcpyAsync(dsample, sample.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s));
        float best = 0.f, def = 0.f;
        for (int g : gs)
            for (int dc : dcs) {
                k_batch_probe<PL><<<ns, BT, 0, s>>>(dprob, dsample, ns, g, dc, ncols);
                PGB_LAUNCHED();
                PGB_CUDA(cudaEventRecord(e0, s));
                for (int r = 0; r < 2; r++) {
                    k_batch_probe<PL><<<ns, BT, 0, s>>>(dprob, dsample, ns, g, dc, ncols);
                    PGB_LAUNCHED();
                }
                PGB_CUDA(cudaEventRecord(e1, s));
                PGB_CUDA(cudaEventSynchronize(e1));
                float ms = 0.f;
                PGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                ms *= 0.5f;
                if (g == 1 && dc == 1) def = ms;
                if (best == 0.f || ms < best) {
                    best = ms;
                    B->g[c] = g;
                    B->dc[c] = dc;
                }
            }
        if (!(best < 0.97f * def)) {
            B->g[c] = 1;
            B->dc[c] = 1;
            best = def;
        }
        B->ms_best[c] = best;
        B->ms_default[c] = def;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(dsample);
    B->tuned = 1;
    B->tuned_pl = PL ? 1 : 0;
}

}  // namespace pgb

using namespace pgb;

#define BATCH_TRY(...)                    \
    try {                                 \
        __VA_ARGS__;                      \
        return 0;                         \
    } catch (const ArgFailure &) {        \
        return PROPACK_ERR_ARG;           \
    } catch (const CudaFailure &) {       \
        return PROPACK_ERR_CUDA;          \
    } catch (const WaitFailure &) {       \
        return PROPACK_ERR_WAIT;          \
    }

extern "C" int propack_batch_create(int nprob, const int *m, const int *n, const int *rowptr, const int64_t *nnz_off,
                                    const int *colidx, const float *val, int64_t *handle)
{
    BATCH_TRY({
        if (nprob <= 0 || !m || !n || !rowptr || !nnz_off || !colidx || !val || !handle) {
            set_error("propack_batch_create: invalid argument");
            throw ArgFailure();
        }
        Batch *B = new Batch();
        B->nprob = nprob;
        B->m.assign(m, m + nprob);
        B->n.assign(n, n + nprob);
        B->zoff.assign(nnz_off, nnz_off + nprob + 1);
        std::vector<int> moff(nprob + 1, 0), noff(nprob + 1, 0);
        for (int p = 0; p < nprob; p++) {
            if (m[p] <= 0 || n[p] <= 0) { delete B; set_error("propack_batch_create: empty problem"); throw ArgFailure(); }
            moff[p + 1] = moff[p] + m[p];
            noff[p + 1] = noff[p] + n[p];
            const int *rp = rowptr + moff[p] + p;
            if (rp[0] != 0 || (int64_t)rp[m[p]] != nnz_off[p + 1] - nnz_off[p]) {
                delete B;
                set_error("propack_batch_create: row pointers do not match nnz_off");
                throw ArgFailure();
            }
            for (int64_t e = 0; e < rp[m[p]]; e++) {
                const int cidx = colidx[nnz_off[p] + e];
                if (cidx < 0 || cidx >= n[p]) { delete B; set_error("propack_batch_create: column out of range"); throw ArgFailure(); }
            }
        }
        B->total_m = moff[nprob];
        B->total_n = noff[nprob];
        B->total_nnz = nnz_off[nprob];
        if (B->total_nnz >= (1ll << 31) || B->total_n >= (1ll << 31)) {
            delete B;
            set_error("propack_batch_create: the batch needs fewer than 2^31 nonzeros");
            throw ArgFailure();
        }
        PGB_CUDA(cudaGetDevice(&B->device));
        cudaStream_t s;
        PGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        const int64_t nnz = B->total_nnz;
        PGB_CUDA(cudaMalloc(&B->d_moff, sizeof(int) * (nprob + 1)));
        PGB_CUDA(cudaMalloc(&B->d_noff, sizeof(int) * (nprob + 1)));
        PGB_CUDA(cudaMalloc(&B->d_zoff, sizeof(int64_t) * (nprob + 1)));
        PGB_CUDA(cudaMalloc(&B->d_rowptr, sizeof(int) * (B->total_m + nprob)));
        PGB_CUDA(cudaMalloc(&B->d_colidx, sizeof(int) * std::max<int64_t>(nnz, 1)));
        PGB_CUDA(cudaMalloc(&B->d_val, sizeof(float) * std::max<int64_t>(nnz, 1)));
        PGB_CUDA(cudaMalloc(&B->d_tptr, sizeof(int) * (B->total_n + 1)));
        PGB_CUDA(cudaMalloc(&B->d_tidx, sizeof(int) * std::max<int64_t>(nnz, 1)));
        PGB_CUDA(cudaMalloc(&B->d_tval, sizeof(float) * std::max<int64_t>(nnz, 1)));
        PGB_CUDA(cudaMemcpyAsync(B->d_moff, moff.data(), sizeof(int) * (nprob + 1), cudaMemcpyHostToDevice, s));
        PGB_CUDA(cudaMemcpyAsync(B->d_noff, noff.data(), sizeof(int) * (nprob + 1), cudaMemcpyHostToDevice, s));
        PGB_CUDA(cudaMemcpyAsync(B->d_zoff, nnz_off, sizeof(int64_t) * (nprob + 1), cudaMemcpyHostToDevice, s));
        PGB_CUDA(cudaMemcpyAsync(B->d_rowptr, rowptr, sizeof(int) * (B->total_m + nprob), cudaMemcpyHostToDevice, s));
        PGB_CUDA(cudaMemcpyAsync(B->d_colidx, colidx, sizeof(int) * nnz, cudaMemcpyHostToDevice, s));
        PGB_CUDA(cudaMemcpyAsync(B->d_val, val, sizeof(float) * nnz, cudaMemcpyHostToDevice, s));
        // transpose: count, scan, scatter, sort
        int *cnt = nullptr, *fill = nullptr;
        PGB_CUDA(cudaMalloc(&cnt, sizeof(int) * (B->total_n + 1)));
        PGB_CUDA(cudaMalloc(&fill, sizeof(int) * (B->total_n + 1)));
        PGB_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * (B->total_n + 1), s));
        PGB_CUDA(cudaMemsetAsync(fill, 0, sizeof(int) * (B->total_n + 1), s));
        k_bt_count<<<std::min(nprob, 65535), 256, 0, s>>>(nprob, B->d_moff, B->d_noff, B->d_rowptr, B->d_zoff,
                                                         B->d_colidx, cnt);
        PGB_LAUNCHED();
        scan_excl(cnt, B->d_tptr, (int)B->total_n, s);
        k_bt_scatter<<<std::min(nprob, 65535), 256, 0, s>>>(nprob, B->d_moff, B->d_noff, B->d_rowptr, B->d_zoff,
                                                           B->d_colidx, B->d_val, B->d_tptr, fill, B->d_tidx,
                                                           B->d_tval);
        PGB_LAUNCHED();
        k_bt_sort<<<std::min<int64_t>(4096, (B->total_n + 255) / 256), 256, 0, s>>>((int)B->total_n, B->d_tptr,
                                                                                     B->d_tidx, B->d_tval);
        PGB_LAUNCHED();
        PGB_CUDA(cudaStreamSynchronize(s));
        cudaFree(cnt);
        cudaFree(fill);
        cudaStreamDestroy(s);
        // work order: decreasing cost (nnz and row count), longest first
        B->order.resize(nprob);
        for (int p = 0; p < nprob; p++) B->order[p] = p;
        std::sort(B->order.begin(), B->order.end(), [&](int a, int b) {
            const double ca = (double)(nnz_off[a + 1] - nnz_off[a]) + 8.0 * (m[a] + n[a]);
            const double cb = (double)(nnz_off[b + 1] - nnz_off[b]) + 8.0 * (m[b] + n[b]);
            return ca > cb;
        });
        std::lock_guard<std::mutex> lk(g_batch_mu);
        *handle = g_batch_next++;
        g_batches[*handle] = B;
    })
}

extern "C" int propack_batch_destroy(int64_t handle)
{
    Batch *B = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_batch_mu);
        auto it = g_batches.find(handle);
        if (it == g_batches.end()) return PROPACK_ERR_HANDLE;
        B = it->second;
        g_batches.erase(it);
    }
    for (void *q : {(void *)B->d_moff, (void *)B->d_noff, (void *)B->d_zoff, (void *)B->d_rowptr, (void *)B->d_colidx,
                    (void *)B->d_val, (void *)B->d_tptr, (void *)B->d_tidx, (void *)B->d_tval})
        if (q) cudaFree(q);
    delete B;
    return 0;
}

extern "C" int propack_batch_solve(int64_t handle, int dim, int neig, int maxiter, double tol, const double *u0,
                                   double *sigma, double *bnd, int *info, double *U, double *V)
{
    Batch *B = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_batch_mu);
        auto it = g_batches.find(handle);
        if (it == g_batches.end()) return PROPACK_ERR_HANDLE;
        B = it->second;
    }
    BATCH_TRY({
        const int np = B->nprob;
        int maxrows = 0, minmn = 1 << 30;
        for (int p = 0; p < np; p++) {
            maxrows = std::max(maxrows, std::max(B->m[p], B->n[p]));
            minmn = std::min(minmn, std::min(B->m[p], B->n[p]));
        }
        if (dim < 2 || dim > BDIM_MAX || neig < 1 || neig >= dim || dim > minmn || maxiter < 1 || !u0 || !sigma ||
            !bnd || !info) {
            set_error("propack_batch_solve: need 1 <= neig < dim <= min(64, m, n) and maxiter >= 1");
            throw ArgFailure();
        }
        g_batch_stats = propack_batch_stats_t();
        g_batch_stats.tune_ms = 0.0;
        const int64_t l0 = g_launches;
        cudaStream_t s;
        PGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        cudaEvent_t e0, e1;
        PGB_CUDA(cudaEventCreate(&e0));
        PGB_CUDA(cudaEventCreate(&e1));
        // device memory: bases, B, outputs, problem table, per-CTA scratch
        const int d1 = dim + 1;
        double *dU = nullptr, *dV = nullptr, *dab = nullptr, *dsb = nullptr, *scratch = nullptr;
        BProb *dprob = nullptr;
        int *dorder = nullptr, *dticket = nullptr, *dactive = nullptr, *hactive = nullptr;
        std::vector<void *> allocs;
        auto alloc = [&](void **p, size_t bytes) {
            PGB_CUDA(cudaMalloc(p, std::max<size_t>(bytes, 16)));
            allocs.push_back(*p);
        };
        alloc((void **)&dU, sizeof(double) * (size_t)B->total_m * d1);
        alloc((void **)&dV, sizeof(double) * (size_t)B->total_n * dim);
        // the plane arithmetic (propack_batch_set_arith(h, 2)) keeps FP32
        // (hi, lo) planes of both bases; the default uses the FP64 bases
        const bool pl = B->planes != 0;
        float2 *dUp = nullptr, *dVp = nullptr;
        if (pl) {
            alloc((void **)&dUp, sizeof(float2) * (size_t)B->total_m * d1);
            alloc((void **)&dVp, sizeof(float2) * (size_t)B->total_n * dim);
        }
        alloc((void **)&dab, sizeof(double) * (size_t)np * 2 * (d1 + 1));
        alloc((void **)&dsb, sizeof(double) * (size_t)np * 2 * neig);
        alloc((void **)&dprob, sizeof(BProb) * np);
        alloc((void **)&dorder, sizeof(int) * np);
        alloc((void **)&dticket, sizeof(int));
        alloc((void **)&dactive, sizeof(int));
        PGB_CUDA(cudaMallocHost(&hactive, sizeof(int)));
        int occ = 0;
        PGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pl ? k_batch_cycle<true> : k_batch_cycle<false>,
                                                               BT, 0));
        const int grid = std::max(1, std::min(np, std::max(1, occ) * device_info().sms));
        const BScrLayout L = bscr_layout(dim, maxrows);
        const size_t stride = (L.total + 31) / 32 * 32;
        alloc((void **)&scratch, sizeof(double) * stride * grid);
        // problem table
        std::vector<BProb> hp(np);
        int64_t mo = 0, no = 0;
        std::vector<int> moff(np + 1, 0);
        for (int p = 0; p < np; p++) moff[p + 1] = moff[p] + B->m[p];
        for (int p = 0; p < np; p++) {
            BProb &P = hp[p];
            memset(&P, 0, sizeof(BProb));
            P.m = B->m[p];
            P.n = B->n[p];
            P.ptr = B->d_rowptr + moff[p] + p;
            P.idx = B->d_colidx + B->zoff[p];
            P.val = B->d_val + B->zoff[p];
            P.tptr = B->d_tptr + no;  // global offsets: the transposed pointers are absolute
            P.tidx = B->d_tidx;
            P.tval = B->d_tval;
            P.U = dU + mo * d1;
            P.V = dV + no * dim;
            P.Up = pl ? dUp + mo * d1 : nullptr;
            P.Vp = pl ? dVp + no * dim : nullptr;
            P.alpha = dab + (size_t)p * 2 * (d1 + 1);
            P.beta = P.alpha + (d1 + 1);
            P.sig = dsb + (size_t)p * 2 * neig;
            P.bnd = P.sig + neig;
            mo += B->m[p];
            no += B->n[p];
        }
        // the tuning (once per batch, before its first solve's timing) and
        // every problem's choice by its size class
        for (int p = 0; p < np; p++) hp[p].g = hp[p].dc = 1;
        // a timed table is redone when the arithmetic changed since
        if (!B->tuned || (B->tuned == 1 && B->tuned_pl != (pl ? 1 : 0))) {
            const auto t0 = std::chrono::steady_clock::now();
            PGB_CUDA(cudaMemcpyAsync(dprob, hp.data(), sizeof(BProb) * np, cudaMemcpyHostToDevice, s));
            PGB_CUDA(cudaMemsetAsync(dU, 0, sizeof(double) * (size_t)B->total_m * d1, s));
            PGB_CUDA(cudaMemsetAsync(dV, 0, sizeof(double) * (size_t)B->total_n * dim, s));
            if (pl) {
                PGB_CUDA(cudaMemsetAsync(dUp, 0, sizeof(float2) * (size_t)B->total_m * d1, s));
                PGB_CUDA(cudaMemsetAsync(dVp, 0, sizeof(float2) * (size_t)B->total_n * dim, s));
                batch_tune<true>(B, dprob, grid, dim, s);
            } else {
                batch_tune<false>(B, dprob, grid, dim, s);
            }
            g_batch_stats.tune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
                                        .count();
        }
        for (int pos = 0; pos < np; pos++) {
            const int c = B->cls(pos);
            hp[B->order[pos]].g = B->g[c];
            hp[B->order[pos]].dc = B->dc[c];
        }
        PGB_CUDA(cudaMemcpyAsync(dprob, hp.data(), sizeof(BProb) * np, cudaMemcpyHostToDevice, s));
        PGB_CUDA(cudaMemcpyAsync(dorder, B->order.data(), sizeof(int) * np, cudaMemcpyHostToDevice, s));
        PGB_CUDA(cudaMemsetAsync(dab, 0, sizeof(double) * (size_t)np * 2 * (d1 + 1), s));
        PGB_CUDA(cudaEventRecord(e0, s));
        // start vectors: U(:,1) of problem p = u0[moff[p] .. moff[p+1])
        mo = 0;
        for (int p = 0; p < np; p++) {
            PGB_CUDA(cudaMemcpyAsync(hp[p].U, u0 + mo, sizeof(double) * B->m[p], cudaMemcpyHostToDevice, s));
            mo += B->m[p];
        }
        k_batch_start<<<std::min(np, 4096), BT, 0, s>>>(dprob, np);
        PGB_LAUNCHED();
        BCfg cfg;
        cfg.dim = dim;
        cfg.k = neig;
        cfg.neig = neig;
        cfg.maxiter = maxiter;
        cfg.ielr = 1;
        cfg.tol = std::min(1.0, std::max(16.0 * EPS, tol));
        cfg.min_relgap = 0.002;
        // one restart cycle as a CUDA graph
        cudaGraph_t graph;
        cudaGraphExec_t exec;
        PGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        PGB_CUDA(cudaMemsetAsync(dticket, 0, sizeof(int), s));
        PGB_CUDA(cudaMemsetAsync(dactive, 0, sizeof(int), s));
        if (pl)
            k_batch_cycle<true><<<grid, BT, 0, s>>>(dprob, dorder, np, cfg, scratch, stride, dticket, dactive,
                                                    BATCH_CYCLES_PER_LAUNCH);
        else
            k_batch_cycle<false><<<grid, BT, 0, s>>>(dprob, dorder, np, cfg, scratch, stride, dticket, dactive,
                                                     BATCH_CYCLES_PER_LAUNCH);
        PGB_CUDA(cudaMemcpyAsync(hactive, dactive, sizeof(int), cudaMemcpyDeviceToHost, s));
        PGB_CUDA(cudaStreamEndCapture(s, &graph));
        PGB_CUDA(cudaGraphInstantiate(&exec, graph, 0));
        int cycles = 0;
        while (cycles * BATCH_CYCLES_PER_LAUNCH < maxiter) {
            PGB_CUDA(cudaGraphLaunch(exec, s));
            PGB_LAUNCHED();
            PGB_CUDA(cudaStreamSynchronize(s));
            cycles++;
            if (*hactive == 0) break;
        }
        PGB_CUDA(cudaEventRecord(e1, s));
        PGB_CUDA(cudaMemcpyAsync(hp.data(), dprob, sizeof(BProb) * np, cudaMemcpyDeviceToHost, s));
        std::vector<double> hsb((size_t)np * 2 * neig);
        PGB_CUDA(cudaMemcpyAsync(hsb.data(), dsb, sizeof(double) * hsb.size(), cudaMemcpyDeviceToHost, s));
        PGB_CUDA(cudaStreamSynchronize(s));
        mo = 0;
        no = 0;
        for (int p = 0; p < np; p++) {
            const BProb &P = hp[p];
            for (int q = 0; q < neig; q++) {
                sigma[(size_t)p * neig + q] = hsb[(size_t)p * 2 * neig + q];
                bnd[(size_t)p * neig + q] = hsb[(size_t)p * 2 * neig + neig + q];
            }
            info[p] = P.status == BS_CONVERGED ? 0 : (P.status == BS_MAXITER ? -1 : 1);
            if (P.status == BS_CONVERGED) {
                if (U)
                    PGB_CUDA(cudaMemcpyAsync(U + mo * neig, P.U, sizeof(double) * (size_t)P.m * neig,
                                             cudaMemcpyDeviceToHost, s));
                if (V)
                    PGB_CUDA(cudaMemcpyAsync(V + no * neig, P.V, sizeof(double) * (size_t)P.n * neig,
                                             cudaMemcpyDeviceToHost, s));
            }
            g_batch_stats.nopx += P.nopx;
            g_batch_stats.nreorth += P.nreorth;
            g_batch_stats.converged += P.status == BS_CONVERGED;
            g_batch_stats.fallback += P.status == BS_FALLBACK;
            mo += P.m;
            no += P.n;
        }
        PGB_CUDA(cudaStreamSynchronize(s));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        g_batch_stats.device_ms = ms;
        g_batch_stats.cycles = cycles;
        g_batch_stats.grid = grid;
        g_batch_stats.kernel_launches = g_launches - l0;
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        for (void *q : allocs) cudaFree(q);
        cudaFreeHost(hactive);
        cudaStreamDestroy(s);
    })
}

extern "C" int propack_batch_set_arith(int64_t handle, int arith)
{
    if (arith != 0 && arith != 2) return PROPACK_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_batch_mu);
    auto it = g_batches.find(handle);
    if (it == g_batches.end()) return PROPACK_ERR_HANDLE;
    it->second->planes = arith == 2 ? 1 : 0;
    return 0;
}

extern "C" int propack_batch_get_tuning(int64_t handle, int *g, int *dc, float *ms_tuned, float *ms_default)
{
    std::lock_guard<std::mutex> lk(g_batch_mu);
    auto it = g_batches.find(handle);
    if (it == g_batches.end()) return PROPACK_ERR_HANDLE;
    const Batch *B = it->second;
    for (int c = 0; c < PROPACK_BATCH_CLASSES; c++) {
        if (g) g[c] = B->tuned ? B->g[c] : 0;
        if (dc) dc[c] = B->tuned ? B->dc[c] : 0;
        if (ms_tuned) ms_tuned[c] = B->tuned == 1 ? B->ms_best[c] : 0.f;
        if (ms_default) ms_default[c] = B->tuned == 1 ? B->ms_default[c] : 0.f;
    }
    return B->tuned;
}

extern "C" int propack_batch_set_tuning(int64_t handle, const int *g, const int *dc)
{
    std::lock_guard<std::mutex> lk(g_batch_mu);
    auto it = g_batches.find(handle);
    if (it == g_batches.end()) return PROPACK_ERR_HANDLE;
    Batch *B = it->second;
    if (!g || !dc) {
        B->tuned = 0;  // time again at the next solve
        return 0;
    }
    for (int c = 0; c < PROPACK_BATCH_CLASSES; c++) {
        const bool okg = g[c] == 1 || g[c] == 2 || g[c] == 4 || g[c] == 8 || g[c] == 16 || g[c] == 32;
        const bool okd = dc[c] == 1 || dc[c] == 2 || dc[c] == 4;
        if (!okg || !okd) {
            set_error("propack_batch_set_tuning: g must be 1, 2, 4, 8, 16 or 32 and dc 1, 2 or 4");
            return PROPACK_ERR_ARG;
        }
    }
    for (int c = 0; c < PROPACK_BATCH_CLASSES; c++) {
        B->g[c] = g[c];
        B->dc[c] = dc[c];
        B->ms_best[c] = B->ms_default[c] = 0.f;
    }
    B->tuned = 2;
    return 0;
}

extern "C" int propack_batch_get_stats(propack_batch_stats_t *out)
{
    if (!out) return PROPACK_ERR_ARG;
    *out = g_batch_stats;
    return 0;
}
