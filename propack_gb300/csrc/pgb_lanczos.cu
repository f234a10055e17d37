// pgb_lanczos.cu -- device-resident steps of dlanbpro (double/dlanbpro.F:283-546).
//
// One Lanczos step is a fixed sequence of kernels per half step (V half:
// alpha_j v_j = A' u_j - beta_j v_{j-1}; U half: beta_{j+1} u_{j+1} =
// A v_j - alpha_j u_j):
//
//   k_lb_spmv     fused SpMV + axpy with the previous vector + partial
//                 sums of ||y||^2 and <prev, y>  (dlanbpro.F:288-296, :420-424)
//   k_lb_elr      one extended-local-reorthogonalisation pass (:301-316, :429-443)
//   k_lb_cgs_dots projections of one classical Gram-Schmidt pass
//                 (dreorth.F:174)
//   k_lb_cgs_upd  v -= W h and ||v||^2 (dreorth.F:85-95, dcgs :199);
//                 a second pass (the iterated refinement) repeats the pair
//
// Every kernel ends with a last-CTA tail that reduces the partial sums in a
// fixed order and runs the scalar logic of dlanbpro on the device: the
// alpha/beta bookkeeping, the ||A|| estimate, the omega recurrences
// (dupdate_nu/mu, parallel over k), dcompute_int, the reorthogonalisation
// decision and the invariant-subspace test.  The host never reads a scalar
// between kernels: a kernel whose phase is not needed (no ELR, no
// reorthogonalisation) sees that in the control block and returns at once.
// Cases that the fixed sequence cannot finish (an invariant subspace that
// needs a fresh random vector, more Gram-Schmidt passes than were enqueued)
// set status = 1 and every later kernel of the sequence returns; the host
// finishes the case and resumes.
//
// dsafescal (dsafescal.F:4-55) is deferred: the new vector is left
// unscaled, the product that reads it through the operator is scaled
// instead (A(v/a) = (Av)/a), and the next same-side SpMV, which reads it
// row by row, writes the scaled value back.
#include <type_traits>

#include "pgb.cuh"
#include "pgb_f3.cuh"
#include "pgb_planes.cuh"
#include "pgb_spmv.cuh"

namespace pgb {

struct Tail {
    LbCtl c;
    int go;
    double red[32];
};

__device__ __forceinline__ Pend make_scale(double a)
{
    Pend p;
    if (fabs(a) >= SFMIN) { p.mode = 1; p.val = 1.0 / a; }
    else { p.mode = 2; p.val = a; }
    return p;
}

// ---------------------------------------------------------------- tails
__device__ void tail_load(const LbArgs &a, Tail &t)
{
    if (threadIdx.x == 0) t.c = *a.ctl;
    __syncthreads();
}
__device__ void tail_store(const LbArgs &a, Tail &t)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        *a.ctl = t.c;
        __threadfence();
    }
}
// fixed-order sum of the per-CTA partials
__device__ double sum_parts(const double *p, int nb, double *red)
{
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += BS) s += p[b];
    return block_sum<BS>(s, red);
}
// the same for two (three) arrays, their loads issued together: one round
// trip instead of two (three), the same sums
__device__ void sum_parts2(const double *p, const double *q, int nb, double *red, double &sp, double &sq)
{
    double s = 0.0, u = 0.0;
    for (int b = threadIdx.x; b < nb; b += BS) {
        s += p[b];
        u += q[b];
    }
    sp = block_sum<BS>(s, red);
    sq = block_sum<BS>(u, red);
}
__device__ void sum_parts3(const double *p, const double *q, const double *r, int nb, double *red, double &sp,
                           double &sq, double &sr)
{
    double s = 0.0, u = 0.0, v = 0.0;
    for (int b = threadIdx.x; b < nb; b += BS) {
        s += p[b];
        u += q[b];
        v += r[b];
    }
    sp = block_sum<BS>(s, red);
    sq = block_sum<BS>(u, red);
    sr = block_sum<BS>(v, red);
}

// dset_mu (dlanbpro.F:555-577), thread 0
__device__ void set_mu(int k, double *mu, const int *index, double val)
{
    int i = 0;
    while (index[i] <= k && index[i] > 0) {
        const int p = index[i], q = index[i + 1];
        for (int j = p; j <= q; j++) mu[j - 1] = val;
        i += 2;
    }
}

// dcompute_int (dlanbpro.F:581-624), thread 0.  Fortran DO-variable exit
// values are reproduced (s = lo-1 and i = j+1 when a search runs out).
__device__ void compute_int(const double *mu, int j, double delta, double eta, int *index)
{
    if (delta < eta) return;
    int ip = 0, i = 0, k, s;
    index[0] = 0;
    while (i < j) {
        for (k = i + 1; k <= j; k++)
            if (fabs(mu[k - 1]) > delta) break;
        if (k > j) break;
        const int lo = i > 1 ? i : 1;
        for (s = k; s >= lo; s--)
            if (fabs(mu[s - 1]) < eta) break;
        index[ip++] = s + 1;
        for (i = s + 1; i <= j; i++)
            if (fabs(mu[i - 1]) < eta) break;
        index[ip++] = i - 1;
    }
    index[ip] = j + 1;
}

// expand index[] into the 0-based column list walked by dcgs (CGS) or
// dmgs (MGS stops at an empty range); thread 0.  Returns the ndot count
// of one pass.
__device__ int build_sel(const int *index, int kk, int icgs, int *sel, int *nsel)
{
    int ns = 0, nd = 0, i = 0;
    if (icgs) {
        while (index[i] <= kk && index[i] > 0) {
            const int p = index[i], q = index[i + 1];
            nd += q - p + 1;
            for (int c = p; c <= q; c++) sel[ns++] = c - 1;
            i += 2;
        }
    } else {
        int p = index[0], q = index[1];
        while (p <= kk && p > 0 && p <= q) {
            nd += q - p + 1;
            for (int c = p; c <= q; c++) sel[ns++] = c - 1;
            i += 2;
            p = index[i];
            q = index[i + 1];
        }
    }
    *nsel = ns;
    return nd + kk;
}

// dupdate_nu (dlanbpro.F:684-723), all threads; j > 1
__device__ void update_nu_par(Tail &t, const LbArgs &a, int j)
{
    const double *ba = a.balpha, *bb = a.bbeta;
    double *mu = a.mu, *nu = a.nu;
    const double e1 = t.c.epsn2, an = t.c.anorm;
    const double aj = ba[j - 1], bjm = bb[j - 2];
    const double hj = hypot(aj, bjm);
    double loc = 0.0;
    for (int k = 1 + threadIdx.x; k <= j - 1; k += BS) {
        double v = bb[k - 1] * mu[k] + ba[k - 1] * mu[k - 1] - bjm * nu[k - 1];
        const double d = e1 * (hypot(ba[k - 1], bb[k - 1]) + hj) + e1 * an;
        v = (v + copysign(d, v)) / aj;
        nu[k - 1] = v;
        loc = fmax(loc, fabs(v));
    }
    const double mx = block_max<BS>(loc, t.red);
    if (threadIdx.x == 0) {
        nu[j - 1] = 1.0;
        t.c.numax = mx;
    }
    __syncthreads();
}

// dupdate_mu (dlanbpro.F:628-679), all threads
__device__ void update_mu_par(Tail &t, const LbArgs &a, int j)
{
    const double *ba = a.balpha, *bb = a.bbeta;
    double *mu = a.mu;
    const double *nu = a.nu;
    const double e1 = t.c.epsn2, an = t.c.anorm;
    double loc = 0.0;
    if (j == 1) {
        if (threadIdx.x == 0) {
            mu[0] = e1 / bb[0];
            loc = fabs(mu[0]);
        }
    } else {
        const double aj = ba[j - 1], bj = bb[j - 1];
        const double hj = hypot(aj, bj);
        for (int k = 1 + threadIdx.x; k <= j; k += BS) {
            double v, d;
            if (k == 1) {
                v = ba[0] * nu[0] - aj * mu[0];
                d = e1 * (hj + ba[0]) + e1 * an;
            } else if (k < j) {
                v = ba[k - 1] * nu[k - 1] + bb[k - 2] * nu[k - 2] - aj * mu[k - 1];
                d = e1 * (hj + hypot(ba[k - 1], bb[k - 2])) + e1 * an;
            } else {
                v = bb[j - 2] * nu[j - 2];
                d = e1 * (hj + hypot(aj, bb[j - 2])) + e1 * an;
            }
            v = (v + copysign(d, v)) / bj;
            mu[k - 1] = v;
            loc = fmax(loc, fabs(v));
        }
    }
    const double mx = block_max<BS>(loc, t.red);
    if (threadIdx.x == 0) {
        mu[j] = 1.0;
        t.c.mumax = mx;
    }
    __syncthreads();
}

// ---------------------------------------------------------- V half logic
__device__ void v_post(Tail &t, const LbArgs &a, int j)
{
    if (threadIdx.x != 0) return;
    LbCtl &c = t.c;
    if (c.alpha < c.anorm * c.epsn && j < c.k) {
        c.rnorm = c.alpha;
        c.alpha = 0.0;
        c.status = 1;
        c.susp_reason = 1;
        c.susp_side = 0;
        c.susp_j = j;
        return;
    } else if (j > 1 && !c.full_reorth && j < c.k && (c.delta * c.alpha < c.anorm * c.eps_vec)) {
        c.ierr = j;
    }
    a.balpha[j - 1] = c.alpha;
    if (c.alpha != 0.0) c.pend_v = make_scale(c.alpha);
    else { c.pend_v.mode = c.collapsed ? 3 : 0; c.pend_v.val = 0.0; }
    c.pend_v_col = j - 1;
}
__device__ void v_post_reorth(Tail &t, const LbArgs &a, int j)
{
    if (threadIdx.x != 0) return;
    set_mu(j - 1, a.nu, a.index, t.c.eps_vec);
    t.c.numax = t.c.eta;
    t.c.force_reorth = !t.c.force_reorth;
}
// dlanbpro.F:340-367: nu recurrence and the reorthogonalisation decision
__device__ void v_reorth_decide(Tail &t, const LbArgs &a, int j)
{
    __syncthreads();
    const bool do_nu = !t.c.full_reorth && t.c.alpha != 0.0;
    if (do_nu && j > 1) update_nu_par(t, a, j);
    if (threadIdx.x == 0) {
        LbCtl &c = t.c;
        t.go = 4;
        c.collapsed = 0;
        if ((c.full_reorth || c.numax > c.delta || c.force_reorth) && c.alpha != 0.0) {
            if (c.full_reorth || c.eta == 0.0) {
                a.index[0] = 1; a.index[1] = j - 1; a.index[2] = j;
            } else if (!c.force_reorth) {
                compute_int(a.nu, j - 1, c.delta, c.eta, a.index);
            }
            if (j - 1 <= 0) {
                t.go = 3;  // dreorth returns at once for k <= 0
            } else {
                c.ndot_iter = build_sel(a.index, j - 1, c.icgs, a.sel, &c.nsel);
                c.reorth_active = 1;
                c.reorth_iter = 0;
                c.reorth_nrm0 = c.alpha;
                c.cgs_phase = 0;
                t.go = 0;
            }
        }
    }
    __syncthreads();
    if (t.go == 3) { v_post_reorth(t, a, j); v_post(t, a, j); }
    else if (t.go == 4) v_post(t, a, j);
}
// B(j,1), amax and the ||A|| estimate (dlanbpro.F:318-334), then the decision
__device__ void v_finish_alpha(Tail &t, const LbArgs &a, int j)
{
    if (threadIdx.x == 0) {
        LbCtl &c = t.c;
        const double *ba = a.balpha, *bb = a.bbeta;
        a.balpha[j - 1] = c.alpha;
        c.amax = fmax(c.amax, c.alpha);
        double a1, b1;
        if (j == 2) {
            a1 = bb[0] / c.amax;
            a1 = FUDGE * c.amax * sqrt((ba[0] / c.amax) * (ba[0] / c.amax) + a1 * a1 + ba[1] / c.amax * a1);
        } else {
            a1 = ba[j - 2] / c.amax;
            b1 = bb[j - 2] / c.amax;
            a1 = FUDGE * c.amax * sqrt(a1 * a1 + b1 * b1 + a1 * bb[j - 3] / c.amax + ba[j - 1] / c.amax * b1);
        }
        c.anorm = fmax(c.anorm, a1);
    }
    v_reorth_decide(t, a, j);
}

// ---------------------------------------------------------- U half logic
__device__ void u_post(Tail &t, const LbArgs &a, int j)
{
    if (threadIdx.x != 0) return;
    LbCtl &c = t.c;
    if (c.beta < c.anorm * c.epsn && j < c.k) {
        c.rnorm = c.beta;
        c.beta = 0.0;
        c.status = 1;
        c.susp_reason = 1;
        c.susp_side = 1;
        c.susp_j = j;
        return;
    } else if (!c.full_reorth && j < c.k && (c.delta * c.beta < c.anorm * c.eps_vec)) {
        c.ierr = j;
    }
    a.bbeta[j - 1] = c.beta;
    if (c.beta != 0.0 && c.beta != 1.0) c.pend_u = make_scale(c.beta);
    else { c.pend_u.mode = c.collapsed ? 3 : 0; c.pend_u.val = 0.0; }
    c.pend_u_col = j;
    c.rnorm = c.beta;
    c.j = j + 1;
}
__device__ void u_post_reorth(Tail &t, const LbArgs &a, int j)
{
    if (threadIdx.x != 0) return;
    set_mu(j, a.mu, a.index, t.c.eps_vec);
    t.c.mumax = t.c.eta;
    t.c.force_reorth = !t.c.force_reorth;
}
// dlanbpro.F:463-498
__device__ void u_reorth_decide(Tail &t, const LbArgs &a, int j)
{
    __syncthreads();
    const bool do_mu = !t.c.full_reorth && t.c.beta != 0.0;
    if (do_mu) update_mu_par(t, a, j);
    if (threadIdx.x == 0) {
        LbCtl &c = t.c;
        t.go = 4;
        c.collapsed = 0;
        if ((c.full_reorth || c.mumax > c.delta || c.force_reorth) && c.beta != 0.0) {
            if (c.full_reorth || c.eta == 0.0) {
                a.index[0] = 1; a.index[1] = j; a.index[2] = j + 1;
            } else if (!c.force_reorth) {
                compute_int(a.mu, j, c.delta, c.eta, a.index);
            } else {
                for (int i = 0; i < 2 * j + 1; i++)
                    if (a.index[i] == j) { a.index[i] = j + 1; break; }
            }
            c.ndot_iter = build_sel(a.index, j, c.icgs, a.sel, &c.nsel);
            c.reorth_active = 1;
            c.reorth_iter = 0;
            c.reorth_nrm0 = c.beta;
            c.cgs_phase = 0;
            t.go = 0;
        }
    }
    __syncthreads();
    if (t.go == 4) u_post(t, a, j);
}
// B(j,2), amax and the ||A|| estimate (dlanbpro.F:445-458)
__device__ void u_finish_beta(Tail &t, const LbArgs &a, int j)
{
    if (threadIdx.x == 0) {
        LbCtl &c = t.c;
        const double *ba = a.balpha, *bb = a.bbeta;
        a.bbeta[j - 1] = c.beta;
        c.amax = fmax(c.amax, c.beta);
        double a1;
        if (j <= 1) {
            a1 = hypot(ba[0], bb[0]);
        } else {
            a1 = ba[j - 1] / c.amax;
            a1 = c.amax * sqrt(a1 * a1 + (bb[j - 1] / c.amax) * (bb[j - 1] / c.amax) + a1 * bb[j - 2] / c.amax);
        }
        c.anorm = fmax(c.anorm, a1);
    }
    u_reorth_decide(t, a, j);
}

// ------------------------------------------------ continuations by phase
// cdot: the launch formed the complex projection <prev, y> = (dotp,
// dotp_im) (the native complex SpMV), so the ELR needs no pass to form it
template <int SIDE>
__device__ void after_spmv(Tail &t, const LbArgs &a, int j, double nrm, double dotp, double dotp_im = 0.0,
                           bool cdot = false)
{
    if (threadIdx.x == 0) {
        LbCtl &c = t.c;
        c.nopx++;
        t.go = 1;
        if (SIDE == 0) {
            if (j > 1) c.pend_v.mode = 0;  // v_{j-1} was scaled in place by the SpMV
            c.alpha = nrm;
            if (j == 1) {
                c.anorm = fmax(c.anorm, FUDGE * c.alpha);
                t.go = 2;
            } else if (c.ielr > 0 && c.alpha < KAPPA * c.beta) {
                c.elr_active = 1;
                c.elr_iter = 1;
                if (c.cplx) {
                    c.elr_need_dot = cdot ? 0 : 1;
                    c.elr_s = dotp;
                    c.elr_s_im = dotp_im;
                } else {
                    c.elr_s = dotp;
                    if (c.beta != 0.0) { c.beta += dotp; a.bbeta[j - 2] = c.beta; }
                }
                t.go = 0;
            }
        } else {
            c.pend_u.mode = 0;  // u_j was scaled in place by the SpMV
            c.beta = nrm;
            if (c.ielr > 0 && c.beta < KAPPA * c.alpha) {
                c.elr_active = 1;
                c.elr_iter = 1;
                if (c.cplx) {
                    c.elr_need_dot = cdot ? 0 : 1;
                    c.elr_s = dotp;
                    c.elr_s_im = dotp_im;
                } else {
                    c.elr_s = dotp;
                    if (c.alpha != 0.0) { c.alpha += dotp; a.balpha[j - 1] = c.alpha; }
                }
                t.go = 0;
            }
        }
    }
    __syncthreads();
    if (SIDE == 0) {
        if (t.go == 1) v_finish_alpha(t, a, j);
        else if (t.go == 2) v_reorth_decide(t, a, j);
    } else {
        if (t.go == 1) u_finish_beta(t, a, j);
    }
}

// dotp_im: the imaginary part of the next projection (complex vectors)
template <int SIDE>
__device__ void after_elr(Tail &t, const LbArgs &a, int j, double snrm, double dotp, double dotp_im = 0.0)
{
    if (threadIdx.x == 0) {
        LbCtl &c = t.c;
        double &cur = SIDE == 0 ? c.alpha : c.beta;
        double &oth = SIDE == 0 ? c.beta : c.alpha;
        t.go = 0;
        if (snrm >= KAPPA * cur || c.elr_iter >= c.ielr) {
            if (SIDE == 0) a.nu[j - 2] = c.eps_vec;
            else a.mu[j - 1] = c.eps_vec;
            cur = snrm;
            c.elr_active = 0;
            t.go = 1;
        } else {
            cur = snrm;
            c.elr_iter++;
            c.elr_s = dotp;
            if (c.cplx) c.elr_s_im = dotp_im;
            else if (oth != 0.0) {
                oth += dotp;
                if (SIDE == 0) a.bbeta[j - 2] = oth;
                else a.balpha[j - 1] = oth;
            }
        }
    }
    __syncthreads();
    if (t.go == 1) {
        if (SIDE == 0) v_finish_alpha(t, a, j);
        else u_finish_beta(t, a, j);
    }
}

// h[c] = sum over CTAs of part_cols[c*nb + b] (one warp per column)
// (nparts partials per column, stored with stride nb; nparts <= nb)
__device__ void reduce_cols(const LbArgs &a, int L, int nparts = -1)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (nparts < 0) nparts = a.nb;
    for (int c = w; c < L; c += BS / 32) {
        const double *p = a.part_cols + (size_t)c * a.nb;
        double s = 0.0;
        for (int b = lane; b < nparts; b += 32) s += p[b];
        s = warp_sum(s);
        if (lane == 0) a.h[c] = s;
    }
    __syncthreads();
}

template <int SIDE>
__device__ void after_cgs(Tail &t, const LbArgs &a, int j, double nrm, int last)
{
    if (threadIdx.x == 0) {
        LbCtl &c = t.c;
        double &cur = SIDE == 0 ? c.alpha : c.beta;
        c.ndot += c.ndot_iter;
        (SIDE == 1 ? c.cgs_cols_u : c.cgs_cols_v) += c.nsel;
        t.go = 0;
        if (nrm > KAPPA * c.reorth_nrm0) {
            cur = nrm;
            c.nreorth++;
            c.reorth_active = 0;
            t.go = 1;
        } else {
            c.reorth_nrm0 = nrm;
            c.reorth_iter++;
            if (c.reorth_iter >= NTRY) {
                cur = 0.0;
                c.collapsed = 1;
                c.nreorth++;
                c.reorth_active = 0;
                t.go = 1;
            } else if (last) {
                c.status = 1;
                c.susp_reason = 2;
                c.susp_side = SIDE;
                c.susp_j = j;
                cur = nrm;
                t.go = 2;
            } else {
                cur = nrm;
                t.go = 2;
            }
        }
    }
    __syncthreads();
    if (t.go == 1) {
        if (SIDE == 0) { v_post_reorth(t, a, j); v_post(t, a, j); }
        else { u_post_reorth(t, a, j); u_post(t, a, j); }
    } else if (t.go == 2) {
        if (threadIdx.x == 0) t.c.cgs_phase = 0;  // the next pass starts with its projections
    }
}

// ----------------------------------------------------------------- kernels
// T is the type of the Lanczos vectors: double (the reference's FP64
// method) or float (the mixed form: FP32 vectors, FP32 SpMV on the FP32
// copy of the values, compensated FP32 reductions; all scalars FP64).
template <typename T>
__device__ __forceinline__ const T *csr_vals(const Csr &A);
template <>
__device__ __forceinline__ const double *csr_vals<double>(const Csr &A) { return A.val; }
template <>
__device__ __forceinline__ const float *csr_vals<float>(const Csr &A) { return A.valf; }

// SHORT: the matrix of this side uses the chunked schedule (compiled
// separately so that it carries neither the staged schedule's shared memory
// nor its registers, and fits more CTAs per SM)
constexpr int SPMV_SHORT_MINB = 4;  // CTAs per SM the chunked instance is compiled for
template <int SIDE, typename T, int SHORT>
__global__ void __launch_bounds__(BS, SHORT ? SPMV_SHORT_MINB : 3) k_lb_spmv(LbArgs a, int j, int host_product)
{
    __shared__ SpmvStage<T, T> st[SHORT ? 1 : SPMV_WARPS];
    __shared__ ChunkStage<T> cst[SHORT ? SPMV_WARPS : 1];
    __shared__ double sred[32];
    __shared__ Tail t;
    const Csr &A = SIDE == 0 ? a.adj : a.fwd;
    // the control words are loaded first and the chunked schedule's tile
    // search runs while they arrive (neither depends on the other)
    const int status = a.ctl->status;
    const Pend pin = SIDE == 0 ? a.ctl->pend_u : a.ctl->pend_v;
    const Pend pprev = SIDE == 0 ? a.ctl->pend_v : a.ctl->pend_u;
    const T coef = (T)(SIDE == 0 ? a.ctl->beta : a.ctl->alpha);
    int tb0 = -1, tb1 = -1;
    if (SHORT && !host_product) chunk_warp_tiles(A.tbase, A.rows, tb0, tb1);
    if (status != 0) return;
    const bool has_prev = SIDE == 1 || j > 1;
    const T *x = SIDE == 0 ? ucol<T>(a, j - 1) : vcol<T>(a, j - 1);
    T *out = SIDE == 0 ? vcol<T>(a, j - 1) : ucol<T>(a, j);
    T *prev = SIDE == 0 ? (j > 1 ? vcol<T>(a, j - 2) : nullptr) : ucol<T>(a, j - 1);
    const double *z = a.z;
    const int n0 = A.ncol0;
    // this launch rewrites the output column and (deferred scale) the
    // previous one: their FP32 planes no longer hold them
    if (a.okU && blockIdx.x == 0 && threadIdx.x == 0) {
        int *ok = SIDE == 0 ? a.okV : a.okU;
        ok[SIDE == 0 ? j - 1 : j] = 0;
        if (has_prev) ok[SIDE == 0 ? j - 2 : j - 1] = 0;
    }
    Acc<T> sq, dt;
    auto epi = [&](int r, double acc, double pvd) {
        T y = apply_pend((T)acc, pin);
        if (has_prev) {
            T pv = (T)pvd;
            if (pprev.mode) {
                pv = apply_pend(pv, pprev);
                prev[r] = pv;
            }
            y = fma(-coef, pv, y);
            dt.add_prod(pv, y);
        }
        out[r] = y;
        sq.add_prod(y, y);
    };
    auto pre = [&](int r) -> double { return has_prev ? (double)prev[r] : 0.0; };
    if (!host_product) {
        auto xl = [&](int c) -> T { return c < n0 ? x[c] : (T)z[c - n0]; };
        if (SHORT)
            csr_rows_chunked<T, T>(A.ptr, A.tbase, A.cidx, chunk_vals<T>(A), A.rows, xl, pre, epi, cst, tb0, tb1);
        else csr_rows_staged<T, T>(A.ptr, A.idx, csr_vals<T>(A), A.blk, A.nblk, xl, pre, epi, st);
    } else {
        // the caller's APROD already wrote the product into out
        for (int r = blockIdx.x * BS + threadIdx.x; r < A.rows; r += gridDim.x * BS) epi(r, (double)out[r], pre(r));
    }
    const double sq2 = block_sum<BS>(sq.value(), sred);
    const double dt2 = block_sum<BS>(dt.value(), sred);
    if (threadIdx.x == 0) {
        a.part_sq[blockIdx.x] = sq2;
        a.part_dot[blockIdx.x] = dt2;
    }
    if (last_cta(&a.ctl->ticket)) {
        tail_load(a, t);
        double s2, d2;
        sum_parts2(a.part_sq, a.part_dot, gridDim.x, t.red, s2, d2);
        after_spmv<SIDE>(t, a, j, sqrt(s2), d2);
        tail_store(a, t);
    }
}

template <int SIDE, typename T>
__global__ void __launch_bounds__(BS) k_lb_elr(LbArgs a, int j)
{
    __shared__ double sred[32];
    __shared__ Tail t;
    if (a.ctl->status != 0 || !a.ctl->elr_active) return;
    const T s = (T)a.ctl->elr_s;
    const int len = SIDE == 0 ? a.adj.rows : a.fwd.rows;
    T *x = SIDE == 0 ? vcol<T>(a, j - 1) : ucol<T>(a, j);
    const T *p = SIDE == 0 ? vcol<T>(a, j - 2) : ucol<T>(a, j - 1);
    Acc<T> sq, dt;
    for (int r = blockIdx.x * BS + threadIdx.x; r < len; r += gridDim.x * BS) {
        const T pv = p[r];
        const T y = fma(-s, pv, x[r]);
        x[r] = y;
        sq.add_prod(y, y);
        dt.add_prod(pv, y);
    }
    const double sq2 = block_sum<BS>(sq.value(), sred);
    const double dt2 = block_sum<BS>(dt.value(), sred);
    if (threadIdx.x == 0) {
        a.part_sq[blockIdx.x] = sq2;
        a.part_dot[blockIdx.x] = dt2;
    }
    if (last_cta(&a.ctl->ticket)) {
        tail_load(a, t);
        double s2, d2;
        sum_parts2(a.part_sq, a.part_dot, gridDim.x, t.red, s2, d2);
        after_elr<SIDE>(t, a, j, sqrt(s2), d2);
        tail_store(a, t);
    }
}

// 16-byte vectors of the Lanczos type: 4 floats or 2 doubles
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    using V = float4;
    static constexpr int W = 4;
    __device__ static __forceinline__ float get(const V &v, int i)
    {
        return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
    }
    __device__ static __forceinline__ void fms(V &x, const V &w, float h)
    {
        x.x = fmaf(-w.x, h, x.x);
        x.y = fmaf(-w.y, h, x.y);
        x.z = fmaf(-w.z, h, x.z);
        x.w = fmaf(-w.w, h, x.w);
    }
};
template <>
struct Vec16<double> {
    using V = double2;
    static constexpr int W = 2;
    __device__ static __forceinline__ double get(const V &v, int i) { return i == 0 ? v.x : v.y; }
    __device__ static __forceinline__ void fms(V &x, const V &w, double h)
    {
        x.x = fma(-w.x, h, x.x);
        x.y = fma(-w.y, h, x.y);
    }
};

// projections h = W(:,sel)' x (dreorth.F:174, the dgemv('T') of dcgs):
// each CTA owns a contiguous chunk of 16-byte row vectors; each warp takes
// four columns at a time and streams the chunk once for them, so every x
// vector it loads serves four columns (ten 16-byte loads in flight per
// lane).  The last CTA also takes the rows past the last whole vector.
constexpr int DOT_COLS = 4;
template <int SIDE, typename T>
__global__ void __launch_bounds__(BS) k_lb_cgs_dots(LbArgs a, int j)
{
    using VT = Vec16<T>;
    using V = typename VT::V;
    __shared__ Tail t;
    if (a.ctl->status != 0 || !a.ctl->reorth_active || a.ctl->cgs_phase != 0) return;
    const int L = a.ctl->nsel;
    const int len = SIDE == 0 ? a.adj.rows : a.fwd.rows;
    const size_t ld = SIDE == 0 ? a.ldv : a.ldu;
    const T *W = (const T *)(SIDE == 0 ? a.V : a.U);
    const T *x = SIDE == 0 ? vcol<T>(a, j - 1) : ucol<T>(a, j);
    const int nvec = len / VT::W;
    const int chunk = (nvec + gridDim.x - 1) / gridDim.x;
    const int v0 = blockIdx.x * chunk, v1 = min(nvec, v0 + chunk);
    const bool tail_rows = blockIdx.x == gridDim.x - 1;
    const V *xv = reinterpret_cast<const V *>(x);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int c0 = w * DOT_COLS; c0 < L; c0 += (BS / 32) * DOT_COLS) {
        const int nc = min(DOT_COLS, L - c0);
        const T *col[DOT_COLS];
#pragma unroll
        for (int u = 0; u < DOT_COLS; u++) col[u] = W + (size_t)a.sel[c0 + (u < nc ? u : 0)] * ld;
        Acc<T> acc[DOT_COLS][2];
        int v = v0 + lane;
        for (; v + 32 < v1; v += 64) {
            const V x0 = xv[v], x1 = xv[v + 32];
            V w0[DOT_COLS], w1[DOT_COLS];
#pragma unroll
            for (int u = 0; u < DOT_COLS; u++) {
                w0[u] = reinterpret_cast<const V *>(col[u])[v];
                w1[u] = reinterpret_cast<const V *>(col[u])[v + 32];
            }
#pragma unroll
            for (int u = 0; u < DOT_COLS; u++)
#pragma unroll
                for (int q = 0; q < VT::W; q++) {
                    acc[u][0].add_prod(VT::get(w0[u], q), VT::get(x0, q));
                    acc[u][1].add_prod(VT::get(w1[u], q), VT::get(x1, q));
                }
        }
        if (v < v1) {
            const V x0 = xv[v];
#pragma unroll
            for (int u = 0; u < DOT_COLS; u++) {
                const V w0 = reinterpret_cast<const V *>(col[u])[v];
#pragma unroll
                for (int q = 0; q < VT::W; q++) acc[u][0].add_prod(VT::get(w0, q), VT::get(x0, q));
            }
        }
        if (tail_rows)
            for (int r = nvec * VT::W + lane; r < len; r += 32)
#pragma unroll
                for (int u = 0; u < DOT_COLS; u++) acc[u][1].add_prod(col[u][r], x[r]);
#pragma unroll
        for (int u = 0; u < DOT_COLS; u++) {
            const double sum = warp_sum(acc[u][0].value() + acc[u][1].value());
            if (lane == 0 && u < nc) a.part_cols[(size_t)(c0 + u) * a.nb + blockIdx.x] = sum;
        }
    }
    if (last_cta(&a.ctl->ticket)) {
        tail_load(a, t);
        reduce_cols(a, L);
        if (threadIdx.x == 0) t.c.cgs_phase = 1;
        tail_store(a, t);
    }
}

// x -= W(:,sel) h (dreorth.F:85-95, the dgemv('N') of dcgs) and ||x||^2:
// one 16-byte row vector per thread and step, the selected columns streamed
// with CGS_UNROLL loads in flight; h and the selection sit in shared memory.
constexpr int CGS_UNROLL = 8;
template <int SIDE, typename T>
__global__ void __launch_bounds__(BS) k_lb_cgs_upd(LbArgs a, int j, int last)
{
    using VT = Vec16<T>;
    using V = typename VT::V;
    extern __shared__ double dyn[];  // h[L] (as T, one double slot each) | sel[L]
    __shared__ double sred[32];
    __shared__ Tail t;
    if (a.ctl->status != 0 || !a.ctl->reorth_active || a.ctl->cgs_phase != 1) return;
    const int L = a.ctl->nsel;
    T *hs = reinterpret_cast<T *>(dyn);
    int *ssel = reinterpret_cast<int *>(dyn + L);
    for (int c = threadIdx.x; c < L; c += BS) {
        hs[c] = (T)a.h[c];
        ssel[c] = a.sel[c];
    }
    __syncthreads();
    const int len = SIDE == 0 ? a.adj.rows : a.fwd.rows;
    const size_t ld = SIDE == 0 ? a.ldv : a.ldu;
    const T *W = (const T *)(SIDE == 0 ? a.V : a.U);
    T *x = SIDE == 0 ? vcol<T>(a, j - 1) : ucol<T>(a, j);
    V *xv = reinterpret_cast<V *>(x);
    const int nvec = len / VT::W;
    Acc<T> sq;
    for (int v = blockIdx.x * BS + threadIdx.x; v < nvec; v += gridDim.x * BS) {
        V acc = xv[v];
        int c = 0;
        for (; c + CGS_UNROLL <= L; c += CGS_UNROLL) {
            V wv[CGS_UNROLL];
#pragma unroll
            for (int u = 0; u < CGS_UNROLL; u++) wv[u] = reinterpret_cast<const V *>(W + (size_t)ssel[c + u] * ld)[v];
#pragma unroll
            for (int u = 0; u < CGS_UNROLL; u++) VT::fms(acc, wv[u], hs[c + u]);
        }
        for (; c < L; c++) VT::fms(acc, reinterpret_cast<const V *>(W + (size_t)ssel[c] * ld)[v], hs[c]);
        xv[v] = acc;
#pragma unroll
        for (int q = 0; q < VT::W; q++) sq.add_prod(VT::get(acc, q), VT::get(acc, q));
    }
    if (blockIdx.x == gridDim.x - 1) {
        for (int r = nvec * VT::W + threadIdx.x; r < len; r += BS) {
            T y = x[r];
            for (int c = 0; c < L; c++) y = fma(-W[(size_t)ssel[c] * ld + r], hs[c], y);
            x[r] = y;
            sq.add_prod(y, y);
        }
    }
    const double sq2 = block_sum<BS>(sq.value(), sred);
    if (threadIdx.x == 0) a.part_sq[blockIdx.x] = sq2;
    if (last_cta(&a.ctl->ticket)) {
        tail_load(a, t);
        const double s2 = sum_parts(a.part_sq, gridDim.x, t.red);
        after_cgs<SIDE>(t, a, j, sqrt(s2), last);
        tail_store(a, t);
    }
}

// The FP64 form's projections on the FP32 pipe (pgb_f3.cuh): same layout
// of work and partial sums as k_lb_cgs_dots; each thread scales its own x
// values by a power of two (its largest exponent) and its partial sums
// back before the warp sum.
template <int SIDE>
__global__ void __launch_bounds__(BS) k_lb_cgs_dots_f3(LbArgs a, int j)
{
    using V = double2;
    __shared__ Tail t;
    if (a.ctl->status != 0 || !a.ctl->reorth_active || a.ctl->cgs_phase != 0) return;
    const int L = a.ctl->nsel;
    const int len = SIDE == 0 ? a.adj.rows : a.fwd.rows;
    const size_t ld = SIDE == 0 ? a.ldv : a.ldu;
    const double *W = (const double *)(SIDE == 0 ? a.V : a.U);
    const double *x = SIDE == 0 ? vcol<double>(a, j - 1) : ucol<double>(a, j);
    const int nvec = len / 2;
    const int chunk = (nvec + gridDim.x - 1) / gridDim.x;
    const int v0 = blockIdx.x * chunk, v1 = min(nvec, v0 + chunk);
    const bool tail_rows = blockIdx.x == gridDim.x - 1;
    const V *xv = reinterpret_cast<const V *>(x);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // this thread's scale: |x 2^-xs| < 2
    int xe = 0;
    for (int v = v0 + lane; v < v1; v += 32) {
        const V xx = xv[v];
        xe = max(xe, max(f3_expo(xx.x), f3_expo(xx.y)));
    }
    if (tail_rows)
        for (int r = nvec * 2 + lane; r < len; r += 32) xe = max(xe, f3_expo(x[r]));
    const int xs = xe == 0 ? 0 : xe - 1023;
    const double back = f3_pow2(xs);
    for (int c0 = w * DOT_COLS; c0 < L; c0 += (BS / 32) * DOT_COLS) {
        const int nc = min(DOT_COLS, L - c0);
        const double *col[DOT_COLS];
#pragma unroll
        for (int u = 0; u < DOT_COLS; u++) col[u] = W + (size_t)a.sel[c0 + (u < nc ? u : 0)] * ld;
        F3Acc acc[DOT_COLS];
        for (int v = v0 + lane; v < v1; v += 32) {
            const V xx = xv[v];
            V wv[DOT_COLS];
#pragma unroll
            for (int u = 0; u < DOT_COLS; u++) wv[u] = reinterpret_cast<const V *>(col[u])[v];
            const F3 x0 = f3_split(xx.x, xs), x1 = f3_split(xx.y, xs);
#pragma unroll
            for (int u = 0; u < DOT_COLS; u++) {
                acc[u].add(f3_split(wv[u].x, 0), x0);
                acc[u].add(f3_split(wv[u].y, 0), x1);
            }
        }
        if (tail_rows)
            for (int r = nvec * 2 + lane; r < len; r += 32) {
                const F3 xr = f3_split(x[r], xs);
#pragma unroll
                for (int u = 0; u < DOT_COLS; u++) acc[u].add(f3_split(col[u][r], 0), xr);
            }
#pragma unroll
        for (int u = 0; u < DOT_COLS; u++) {
            const double sum = warp_sum(acc[u].value() * back);
            if (lane == 0 && u < nc) a.part_cols[(size_t)(c0 + u) * a.nb + blockIdx.x] = sum;
        }
    }
    if (last_cta(&a.ctl->ticket)) {
        tail_load(a, t);
        reduce_cols(a, L);
        if (threadIdx.x == 0) t.c.cgs_phase = 1;
        tail_store(a, t);
    }
}

// The FP64 form's update on the FP32 pipe: sum_c W(i, c) h_c at three
// levels per row (h scaled by the power of two of its largest entry),
// then one FP64 FMA per row applies it to x.
template <int SIDE>
__global__ void __launch_bounds__(BS) k_lb_cgs_upd_f3(LbArgs a, int j, int last)
{
    using V = double2;
    extern __shared__ double dyn[];  // h[L] as F3 (one double2 slot each) | sel[L]
    __shared__ double sred[32];
    __shared__ int hsh;
    __shared__ Tail t;
    if (a.ctl->status != 0 || !a.ctl->reorth_active || a.ctl->cgs_phase != 1) return;
    const int L = a.ctl->nsel;
    F3 *h3 = reinterpret_cast<F3 *>(dyn);
    int *ssel = reinterpret_cast<int *>(dyn + 2 * (size_t)L);
    if (threadIdx.x == 0) hsh = 0;
    __syncthreads();
    int he = 0;
    for (int c = threadIdx.x; c < L; c += BS) he = max(he, f3_expo(a.h[c]));
    if (he) atomicMax(&hsh, he);
    __syncthreads();
    const int hs = hsh == 0 ? 0 : hsh - 1023;  // |h 2^-hs| < 2
    for (int c = threadIdx.x; c < L; c += BS) {
        h3[c] = f3_split(a.h[c], hs);
        ssel[c] = a.sel[c];
    }
    __syncthreads();
    const double back = f3_pow2(hs);
    const int len = SIDE == 0 ? a.adj.rows : a.fwd.rows;
    const size_t ld = SIDE == 0 ? a.ldv : a.ldu;
    const double *W = (const double *)(SIDE == 0 ? a.V : a.U);
    double *x = SIDE == 0 ? vcol<double>(a, j - 1) : ucol<double>(a, j);
    V *xv = reinterpret_cast<V *>(x);
    const int nvec = len / 2;
    Acc<double> sq;
    for (int v = blockIdx.x * BS + threadIdx.x; v < nvec; v += gridDim.x * BS) {
        F3Acc s0, s1;
        int c = 0;
        for (; c + CGS_UNROLL <= L; c += CGS_UNROLL) {
            V wv[CGS_UNROLL];
#pragma unroll
            for (int u = 0; u < CGS_UNROLL; u++) wv[u] = reinterpret_cast<const V *>(W + (size_t)ssel[c + u] * ld)[v];
#pragma unroll
            for (int u = 0; u < CGS_UNROLL; u++) {
                const F3 hc = h3[c + u];
                s0.add(f3_split(wv[u].x, 0), hc);
                s1.add(f3_split(wv[u].y, 0), hc);
            }
        }
        for (; c < L; c++) {
            const V wc = reinterpret_cast<const V *>(W + (size_t)ssel[c] * ld)[v];
            s0.add(f3_split(wc.x, 0), h3[c]);
            s1.add(f3_split(wc.y, 0), h3[c]);
        }
        V acc = xv[v];
        acc.x = fma(-s0.value(), back, acc.x);
        acc.y = fma(-s1.value(), back, acc.y);
        xv[v] = acc;
        sq.add_prod(acc.x, acc.x);
        sq.add_prod(acc.y, acc.y);
    }
    if (blockIdx.x == gridDim.x - 1) {
        for (int r = nvec * 2 + threadIdx.x; r < len; r += BS) {
            F3Acc sr;
            for (int c = 0; c < L; c++) sr.add(f3_split(W[(size_t)ssel[c] * ld + r], 0), h3[c]);
            const double y = fma(-sr.value(), back, x[r]);
            x[r] = y;
            sq.add_prod(y, y);
        }
    }
    const double sq2 = block_sum<BS>(sq.value(), sred);
    if (threadIdx.x == 0) a.part_sq[blockIdx.x] = sq2;
    if (last_cta(&a.ctl->ticket)) {
        tail_load(a, t);
        const double s2 = sum_parts(a.part_sq, gridDim.x, t.red);
        after_cgs<SIDE>(t, a, j, sqrt(s2), last);
        tail_store(a, t);
    }
}

// ------------------------------------------------ split-once planes
// The FP64 form's Gram-Schmidt on the FP32 pipe, reading each basis element
// as 8 bytes of FP32 planes: hi = the leading 24 bits of w, lo = the next
// 23, so that hi + lo holds w to 2^-47 relative (a Lanczos column has
// |w| <= 1; parts below 2^-74 are dropped, far below the column's unit norm).  A column is
// split by the first projection that selects it while its flag is clear;
// the update of the same pass and every later pass read its planes until
// the column is rewritten (the SpMV that writes a column, the flush and the
// deferred-scale kernel clear its flag; the host clears all flags whenever
// it writes columns itself).  One product w x costs 12 FP32 operations --
// hi*hi as an exact two-product folded into a two-sum, the cross terms
// hi*lo and lo*hi into the compensation -- for an error of a few 2^-48 of
// sum |w_i x_i|, the size of an FP64 dot product's own rounding over a
// few thousand terms.  A pass streams 8 bytes per element either way; on
// GB300 the FP64 pipe (2 lanes per clock per SM) holds one FMA per element
// below the HBM rate, 12 FP32 operations (128 lanes per clock) do not.

// projections h = W(:,sel)' x from the planes.  Each CTA owns a contiguous
// chunk of 2-element row vectors and each of its warps one eighth of the
// chunk.  A warp first splits its x values (scaled by a power of two per
// warp) into the x planes scratch and the rows of its slice of every
// selected column whose planes are stale (read in FP64, written as planes);
// it then streams its slice once per group of DOT_COLS columns, reading the
// planes only, so every warp has the same work whatever the column count.
// Each lane reads back only the vectors it wrote itself.  A group's sums
// are reduced over the warp as compensated FP32 pairs (no FP64 operation
// per group), then added over the warps in a fixed order, then over the
// CTAs by the last CTA.  The grid is one wave at the kernel's occupancy (<= nb CTAs).
constexpr int PL_WARPS = BS / 32;
constexpr size_t PL_SMEM_MAX = 200 * 1024;  // per-warp partials + selection of the projections
constexpr int PL_MINB = 4;                  // CTAs per SM the projection kernel is compiled for
constexpr int PL_SPLIT_UNROLL = 4;          // FP64 loads in flight per lane when a column is split
template <int SIDE>
__global__ void __launch_bounds__(BS, PL_MINB) k_lb_cgs_dots_pl(LbArgs a, int j)
{
    // [PL_WARPS][kmax + 1] per-warp partial projections | sel[kmax + 1] | fresh[kmax + 1]
    extern __shared__ double wpart[];
    __shared__ Tail t;
    if (a.ctl->status != 0 || !a.ctl->reorth_active || a.ctl->cgs_phase != 0) return;
    const int L = a.ctl->nsel;
    const int K1 = a.kmax + 1;
    int *ssel = reinterpret_cast<int *>(wpart + (size_t)PL_WARPS * K1);
    int *sfresh = ssel + K1;
    int *ok = SIDE == 0 ? a.okV : a.okU;
    for (int c = threadIdx.x; c < L; c += BS) {
        const int col = a.sel[c];
        ssel[c] = col;
        sfresh[c] = ok[col] == 0;
    }
    __syncthreads();
    const int len = SIDE == 0 ? a.adj.rows : a.fwd.rows;
    const size_t ld = SIDE == 0 ? a.ldv : a.ldu;
    const size_t ldq = ld / 2;  // leading dimension in float4 (two elements)
    const double *W = (const double *)(SIDE == 0 ? a.V : a.U);
    float2 *Wp = SIDE == 0 ? a.Vp : a.Up;
    const double *x = SIDE == 0 ? vcol<double>(a, j - 1) : ucol<double>(a, j);
    const double2 *xv = reinterpret_cast<const double2 *>(x);
    float4 *xq = reinterpret_cast<float4 *>(a.xpl);
    const int nvec = len / 2;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int chunk = (nvec + gridDim.x - 1) / gridDim.x;
    const int cb0 = min(nvec, blockIdx.x * chunk), cb1 = min(nvec, cb0 + chunk);
    const int sl = (cb1 - cb0 + PL_WARPS - 1) / PL_WARPS;
    const int v0 = min(cb1, cb0 + w * sl), v1 = min(cb1, v0 + sl);
    // the row past the last whole vector (odd lengths): lane 0 of the last warp of the last CTA
    const bool tail_row = (len & 1) && blockIdx.x == gridDim.x - 1 && w == PL_WARPS - 1 && lane == 0;
    // this warp's scale (|x 2^-xs| < 2), then its x planes
    int xe = 0;
    for (int v = v0 + lane; v < v1; v += 32) {
        const double2 xx = xv[v];
        xe = max(xe, max(f3_expo(xx.x), f3_expo(xx.y)));
    }
    if (tail_row) xe = max(xe, f3_expo(x[len - 1]));
    xe = __reduce_max_sync(0xffffffffu, xe);
    const int xs = xe == 0 ? 0 : xe - 1023;
    const double back = f3_pow2(xs);
    for (int v = v0 + lane; v < v1; v += 32) {
        const double2 xx = xv[v];
        const float2 p = pl_xsplit(xx.x, xs), q = pl_xsplit(xx.y, xs);
        xq[v] = make_float4(p.x, p.y, q.x, q.y);
    }
    float2 xr = make_float2(0.f, 0.f);
    if (tail_row) xr = pl_xsplit(x[len - 1], xs);
    // planes of the stale selected columns, on this lane's rows
    for (int c = 0; c < L; c++) {
        if (!sfresh[c]) continue;
        const int col = ssel[c];
        float4 *Wq = reinterpret_cast<float4 *>(Wp) + (size_t)col * ldq;
        const double2 *Wd = reinterpret_cast<const double2 *>(W + (size_t)col * ld);
        int v = v0 + lane;
        for (; v + 32 * (PL_SPLIT_UNROLL - 1) < v1; v += 32 * PL_SPLIT_UNROLL) {
            double2 d[PL_SPLIT_UNROLL];
#pragma unroll
            for (int u = 0; u < PL_SPLIT_UNROLL; u++) d[u] = Wd[v + 32 * u];
#pragma unroll
            for (int u = 0; u < PL_SPLIT_UNROLL; u++) Wq[v + 32 * u] = pl_split2(d[u]);
        }
        for (; v < v1; v += 32) Wq[v] = pl_split2(Wd[v]);
        if (tail_row) Wp[(size_t)col * ld + len - 1] = pl_split(W[(size_t)col * ld + len - 1]);
    }
    for (int cb = 0; cb < L; cb += DOT_COLS) {
        const int nc = min(DOT_COLS, L - cb);
        const float4 *Wq[DOT_COLS];
#pragma unroll
        for (int u = 0; u < DOT_COLS; u++)
            Wq[u] = reinterpret_cast<const float4 *>(Wp) + (size_t)ssel[cb + (u < nc ? u : 0)] * ldq;
        PlAcc acc[DOT_COLS];
        int v = v0 + lane;
        // the planes stream through once (evict-first), so that the x
        // planes, read again by every group, stay in L2
        for (; v + 32 < v1; v += 64) {
            float4 w0[DOT_COLS], w1[DOT_COLS];
#pragma unroll
            for (int u = 0; u < DOT_COLS; u++) {
                w0[u] = __ldcs(Wq[u] + v);
                w1[u] = __ldcs(Wq[u] + v + 32);
            }
            const float4 x0 = xq[v], x1 = xq[v + 32];
#pragma unroll
            for (int u = 0; u < DOT_COLS; u++) {
                acc[u].add(w0[u].x, w0[u].y, x0.x, x0.y);
                acc[u].add(w0[u].z, w0[u].w, x0.z, x0.w);
                acc[u].add(w1[u].x, w1[u].y, x1.x, x1.y);
                acc[u].add(w1[u].z, w1[u].w, x1.z, x1.w);
            }
        }
        if (v < v1) {
            const float4 x0 = xq[v];
#pragma unroll
            for (int u = 0; u < DOT_COLS; u++) {
                const float4 w0 = __ldcs(Wq[u] + v);
                acc[u].add(w0.x, w0.y, x0.x, x0.y);
                acc[u].add(w0.z, w0.w, x0.z, x0.w);
            }
        }
        if (tail_row) {
#pragma unroll
            for (int u = 0; u < DOT_COLS; u++) {
                if (u >= nc) break;
                const float2 wr = Wp[(size_t)ssel[cb + u] * ld + len - 1];
                acc[u].add(wr.x, wr.y, xr.x, xr.y);
            }
        }
        static_assert(DOT_COLS == 4, "pl_warp_sum4 sums four columns");
        const PlAcc tot = pl_warp_sum4(acc);
        if ((lane & 7) == 0 && (lane >> 3) < nc) wpart[(size_t)w * K1 + cb + (lane >> 3)] = tot.value() * back;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < L; c += BS) {
        double s = 0.0;
#pragma unroll
        for (int ww = 0; ww < PL_WARPS; ww++) s += wpart[(size_t)ww * K1 + c];
        a.part_cols[(size_t)c * a.nb + blockIdx.x] = s;
    }
    if (last_cta(&a.ctl->ticket)) {
        tail_load(a, t);
        reduce_cols(a, L, gridDim.x);
        for (int c = threadIdx.x; c < L; c += BS) ok[ssel[c]] = 1;
        if (threadIdx.x == 0) t.c.cgs_phase = 1;
        tail_store(a, t);
    }
}

// x -= W(:,sel) h from the planes, and ||x||^2: one 2-element row vector
// per thread and step, the selected columns streamed with CGS_UNROLL
// 16-byte loads in flight.  h (scaled by the power of two of its largest
// entry) sits in shared memory as (hi, lo) planes; each row's sum of
// products is formed on the FP32 pipe and applied with one FP64 FMA.
template <int SIDE>
__global__ void __launch_bounds__(BS) k_lb_cgs_upd_pl(LbArgs a, int j, int last)
{
    extern __shared__ double dyn[];  // h[L] as float2 planes (one double slot each) | sel[L]
    __shared__ double sred[32];
    __shared__ int hsh;
    __shared__ Tail t;
    if (a.ctl->status != 0 || !a.ctl->reorth_active || a.ctl->cgs_phase != 1) return;
    const int L = a.ctl->nsel;
    float2 *hp = reinterpret_cast<float2 *>(dyn);
    int *ssel = reinterpret_cast<int *>(dyn + L);
    if (threadIdx.x == 0) hsh = 0;
    __syncthreads();
    int he = 0;
    for (int c = threadIdx.x; c < L; c += BS) he = max(he, f3_expo(a.h[c]));
    if (he) atomicMax(&hsh, he);
    __syncthreads();
    const int hs = hsh == 0 ? 0 : hsh - 1023;  // |h 2^-hs| < 2
    const double hscale = f3_pow2(-hs), back = f3_pow2(hs);
    for (int c = threadIdx.x; c < L; c += BS) {
        hp[c] = pl_split(a.h[c] * hscale);
        ssel[c] = a.sel[c];
    }
    __syncthreads();
    const int len = SIDE == 0 ? a.adj.rows : a.fwd.rows;
    const size_t ld = SIDE == 0 ? a.ldv : a.ldu;
    const size_t ldq = ld / 2;
    const float4 *Wq = reinterpret_cast<const float4 *>(SIDE == 0 ? a.Vp : a.Up);
    const float2 *Wp = SIDE == 0 ? a.Vp : a.Up;
    double *x = SIDE == 0 ? vcol<double>(a, j - 1) : ucol<double>(a, j);
    double2 *xv = reinterpret_cast<double2 *>(x);
    const int nvec = len / 2;
    double sq = 0.0;
    for (int v = blockIdx.x * BS + threadIdx.x; v < nvec; v += gridDim.x * BS) {
        const double2 x0 = xv[v];
        PlAcc s0, s1;
        int c = 0;
        for (; c + CGS_UNROLL <= L; c += CGS_UNROLL) {
            float4 wv[CGS_UNROLL];
#pragma unroll
            for (int u = 0; u < CGS_UNROLL; u++) wv[u] = Wq[(size_t)ssel[c + u] * ldq + v];
#pragma unroll
            for (int u = 0; u < CGS_UNROLL; u++) {
                const float2 hc = hp[c + u];
                s0.add(wv[u].x, wv[u].y, hc.x, hc.y);
                s1.add(wv[u].z, wv[u].w, hc.x, hc.y);
            }
        }
        for (; c < L; c++) {
            const float4 wc = Wq[(size_t)ssel[c] * ldq + v];
            const float2 hc = hp[c];
            s0.add(wc.x, wc.y, hc.x, hc.y);
            s1.add(wc.z, wc.w, hc.x, hc.y);
        }
        double2 y;
        y.x = fma(-pl_f2d(s0.c), back, fma(-pl_f2d(s0.s), back, x0.x));
        y.y = fma(-pl_f2d(s1.c), back, fma(-pl_f2d(s1.s), back, x0.y));
        xv[v] = y;
        sq = fma(y.x, y.x, sq);
        sq = fma(y.y, y.y, sq);
    }
    if (blockIdx.x == gridDim.x - 1 && (len & 1) && threadIdx.x == 0) {
        const int r = len - 1;
        PlAcc sr;
        for (int c = 0; c < L; c++) {
            const float2 wc = Wp[(size_t)ssel[c] * ld + r];
            sr.add(wc.x, wc.y, hp[c].x, hp[c].y);
        }
        const double y = fma(-sr.value(), back, x[r]);
        x[r] = y;
        sq = fma(y, y, sq);
    }
    const double sq2 = block_sum<BS>(sq, sred);
    if (threadIdx.x == 0) a.part_sq[blockIdx.x] = sq2;
    if (last_cta(&a.ctl->ticket)) {
        tail_load(a, t);
        const double s2 = sum_parts(a.part_sq, gridDim.x, t.red);
        after_cgs<SIDE>(t, a, j, sqrt(s2), last);
        tail_store(a, t);
    }
}

// ------------------------------------------------- complex*16 vectors
// The complex form (complex16/zlanbpro.F) keeps alpha, beta and the omega
// recurrences real.  Its vectors are (re, im) pairs of doubles and its
// operator is the real 2x2-block form of A (pgb_operator.cu), so the fused
// SpMV, the norms, the deferred scaling and the flush above serve it as
// they are.  What differs are the inner products, which are conjugated and
// complex: in the ELR (zlanbpro.F:318-331, :451-464) and in Gram-Schmidt
// (zreorth.F, zcgs: zgemv 'C' then 'N').

// conj(w) x added to (re, im)
__device__ __forceinline__ void zdot_acc(double &re, double &im, const double2 &w, const double2 &x)
{
    re = fma(w.x, x.x, re);
    re = fma(w.y, x.y, re);
    im = fma(w.x, x.y, im);
    im = fma(-w.y, x.x, im);
}
// acc -= w h
__device__ __forceinline__ void zfms(double2 &acc, const double2 &w, const double2 &h)
{
    acc.x = fma(-w.x, h.x, acc.x);
    acc.x = fma(w.y, h.y, acc.x);
    acc.y = fma(-w.x, h.y, acc.y);
    acc.y = fma(-w.y, h.x, acc.y);
}

// One complex ELR pass: x -= s p, ||x||^2 and the next projection <p, x>.
// The fused SpMV cannot form the complex <p, x> (the real and imaginary
// rows of an element are different rows of the 2x2-block operator), so the
// first pass after it (elr_need_dot set) forms <p, x> alone.
template <int SIDE>
__global__ void __launch_bounds__(BS) k_lb_zelr(LbArgs a, int j)
{
    __shared__ double sred[32];
    __shared__ Tail t;
    if (a.ctl->status != 0 || !a.ctl->elr_active) return;
    const bool dot_only = a.ctl->elr_need_dot != 0;
    const double sr = a.ctl->elr_s, si = a.ctl->elr_s_im;
    const int len = (SIDE == 0 ? a.adj.rows : a.fwd.rows) / 2;
    double2 *x = reinterpret_cast<double2 *>(SIDE == 0 ? vcol<double>(a, j - 1) : ucol<double>(a, j));
    const double2 *p =
        reinterpret_cast<const double2 *>(SIDE == 0 ? vcol<double>(a, j - 2) : ucol<double>(a, j - 1));
    double sq = 0.0, dr = 0.0, di = 0.0;
    for (int r = blockIdx.x * BS + threadIdx.x; r < len; r += gridDim.x * BS) {
        const double2 pv = p[r];
        double2 y = x[r];
        if (!dot_only) {
            y.x = fma(-sr, pv.x, y.x);
            y.x = fma(si, pv.y, y.x);
            y.y = fma(-sr, pv.y, y.y);
            y.y = fma(-si, pv.x, y.y);
            x[r] = y;
            sq = fma(y.x, y.x, sq);
            sq = fma(y.y, y.y, sq);
        }
        zdot_acc(dr, di, pv, y);
    }
    const double sq2 = block_sum<BS>(sq, sred);
    const double dr2 = block_sum<BS>(dr, sred);
    const double di2 = block_sum<BS>(di, sred);
    if (threadIdx.x == 0) {
        a.part_sq[blockIdx.x] = sq2;
        a.part_dot[blockIdx.x] = dr2;
        a.part_cols[blockIdx.x] = di2;  // Gram-Schmidt is idle while the ELR runs
    }
    if (last_cta(&a.ctl->ticket)) {
        tail_load(a, t);
        double s2, d2, e2;
        sum_parts3(a.part_sq, a.part_dot, a.part_cols, gridDim.x, t.red, s2, d2, e2);
        if (dot_only) {
            if (threadIdx.x == 0) {
                t.c.elr_s = d2;
                t.c.elr_s_im = e2;
                t.c.elr_need_dot = 0;
            }
        } else {
            after_elr<SIDE>(t, a, j, sqrt(s2), d2, e2);
        }
        tail_store(a, t);
    }
}

// The fused complex SpMV of one half step on a native complex operator
// (zlanbpro.F:297-311 and :442-450): y = op(A) x with complex
// accumulation (one index and one 16-byte value per entry, 16-byte gathers),
// the deferred scale of x and of the previous vector, y -= coef prev (coef
// real), and the partial sums of ||y||^2 and of the complex projection
// <prev, y> = sum conj(prev) y that the first ELR pass subtracts
// (pzdotc), in the same launch.  host_product: the caller's ZAPROD already
// wrote y.
constexpr int ZSPMV_MINB = 3;    // CTAs per SM the complex SpMV is compiled for (wider values and gathers)
constexpr int ZSPMV_UNROLL = 4;  // its (index, value) pairs and gathers in flight per lane
template <int SIDE>
__global__ void __launch_bounds__(BS, ZSPMV_MINB) k_lb_zspmv(LbArgs a, int j, int host_product)
{
    __shared__ ChunkStage<double2> cst[SPMV_WARPS];
    __shared__ double sred[32];
    __shared__ Tail t;
    const Csr &A = SIDE == 0 ? a.zadj : a.zfwd;
    // control words first; the tile search runs while they arrive
    const int status = a.ctl->status;
    const Pend pin = SIDE == 0 ? a.ctl->pend_u : a.ctl->pend_v;
    const Pend pprev = SIDE == 0 ? a.ctl->pend_v : a.ctl->pend_u;
    const double coef = SIDE == 0 ? a.ctl->beta : a.ctl->alpha;
    int tb0 = -1, tb1 = -1;
    if (!host_product) chunk_warp_tiles(A.tbase, A.rows, tb0, tb1);
    if (status != 0) return;
    const bool has_prev = SIDE == 1 || j > 1;
    const double2 *x = reinterpret_cast<const double2 *>(SIDE == 0 ? ucol<double>(a, j - 1) : vcol<double>(a, j - 1));
    double2 *out = reinterpret_cast<double2 *>(SIDE == 0 ? vcol<double>(a, j - 1) : ucol<double>(a, j));
    double2 *prev = has_prev ? reinterpret_cast<double2 *>(SIDE == 0 ? vcol<double>(a, j - 2) : ucol<double>(a, j - 1))
                             : nullptr;
    // this launch rewrites the output column and (deferred scale) the
    // previous one: their planes no longer hold them
    if (a.okU && blockIdx.x == 0 && threadIdx.x == 0) {
        int *ok = SIDE == 0 ? a.okV : a.okU;
        ok[SIDE == 0 ? j - 1 : j] = 0;
        if (has_prev) ok[SIDE == 0 ? j - 2 : j - 1] = 0;
    }
    double sq = 0.0, dr = 0.0, di = 0.0;
    auto scale = [](double2 v, const Pend &p) { return make_double2(apply_pend(v.x, p), apply_pend(v.y, p)); };
    auto epi = [&](int r, double2 acc, double2 pv) {
        double2 y = scale(acc, pin);
        if (has_prev) {
            if (pprev.mode) {
                pv = scale(pv, pprev);
                prev[r] = pv;
            }
            y.x = fma(-coef, pv.x, y.x);
            y.y = fma(-coef, pv.y, y.y);
            zdot_acc(dr, di, pv, y);
        }
        out[r] = y;
        sq = fma(y.x, y.x, sq);
        sq = fma(y.y, y.y, sq);
    };
    auto pre = [&](int r) -> double2 { return has_prev ? prev[r] : make_double2(0.0, 0.0); };
    if (!host_product) {
        auto xl = [&](int c) -> double2 { return x[c]; };
        csr_rows_chunked<double2, double2, ZSPMV_UNROLL>(A.ptr, A.tbase, A.cidx, A.czval, A.rows, xl, pre, epi, cst,
                                                         tb0, tb1);
    } else {
        const int rows = (SIDE == 0 ? a.adj.rows : a.fwd.rows) / 2;
        for (int r = blockIdx.x * BS + threadIdx.x; r < rows; r += gridDim.x * BS) epi(r, out[r], pre(r));
    }
    const double sq2 = block_sum<BS>(sq, sred);
    const double dr2 = block_sum<BS>(dr, sred);
    const double di2 = block_sum<BS>(di, sred);
    if (threadIdx.x == 0) {
        a.part_sq[blockIdx.x] = sq2;
        a.part_dot[blockIdx.x] = dr2;
        a.part_cols[blockIdx.x] = di2;  // Gram-Schmidt is idle while the SpMV runs
    }
    if (last_cta(&a.ctl->ticket)) {
        tail_load(a, t);
        double s2, d2, e2;
        sum_parts3(a.part_sq, a.part_dot, a.part_cols, gridDim.x, t.red, s2, d2, e2);
        after_spmv<SIDE>(t, a, j, sqrt(s2), d2, e2, true);
        tail_store(a, t);
    }
}

// projections h = W(:,sel)^H x (the zgemv('C') of zcgs): the work layout of
// k_lb_cgs_dots with one complex element per 16-byte vector; column c's
// partials go to part_cols rows 2c (re) and 2c+1 (im), and h comes out as
// (re, im) pairs
template <int SIDE>
__global__ void __launch_bounds__(BS) k_lb_zcgs_dots(LbArgs a, int j)
{
    __shared__ Tail t;
    if (a.ctl->status != 0 || !a.ctl->reorth_active || a.ctl->cgs_phase != 0) return;
    const int L = a.ctl->nsel;
    const int len = (SIDE == 0 ? a.adj.rows : a.fwd.rows) / 2;
    const size_t ld = (size_t)(SIDE == 0 ? a.ldv : a.ldu) / 2;
    const double2 *W = reinterpret_cast<const double2 *>(SIDE == 0 ? a.V : a.U);
    const double2 *x =
        reinterpret_cast<const double2 *>(SIDE == 0 ? vcol<double>(a, j - 1) : ucol<double>(a, j));
    const int chunk = (len + gridDim.x - 1) / gridDim.x;
    const int v0 = blockIdx.x * chunk, v1 = min(len, v0 + chunk);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int c0 = w * DOT_COLS; c0 < L; c0 += (BS / 32) * DOT_COLS) {
        const int nc = min(DOT_COLS, L - c0);
        const double2 *col[DOT_COLS];
#pragma unroll
        for (int u = 0; u < DOT_COLS; u++) col[u] = W + (size_t)a.sel[c0 + (u < nc ? u : 0)] * ld;
        double re[DOT_COLS][2], im[DOT_COLS][2];
#pragma unroll
        for (int u = 0; u < DOT_COLS; u++) re[u][0] = re[u][1] = im[u][0] = im[u][1] = 0.0;
        int v = v0 + lane;
        for (; v + 32 < v1; v += 64) {
            const double2 x0 = x[v], x1 = x[v + 32];
            double2 w0[DOT_COLS], w1[DOT_COLS];
#pragma unroll
            for (int u = 0; u < DOT_COLS; u++) {
                w0[u] = col[u][v];
                w1[u] = col[u][v + 32];
            }
#pragma unroll
            for (int u = 0; u < DOT_COLS; u++) {
                zdot_acc(re[u][0], im[u][0], w0[u], x0);
                zdot_acc(re[u][1], im[u][1], w1[u], x1);
            }
        }
        if (v < v1) {
            const double2 x0 = x[v];
#pragma unroll
            for (int u = 0; u < DOT_COLS; u++) zdot_acc(re[u][0], im[u][0], col[u][v], x0);
        }
#pragma unroll
        for (int u = 0; u < DOT_COLS; u++) {
            const double sr = warp_sum(re[u][0] + re[u][1]);
            const double si = warp_sum(im[u][0] + im[u][1]);
            if (lane == 0 && u < nc) {
                a.part_cols[(size_t)(2 * (c0 + u)) * a.nb + blockIdx.x] = sr;
                a.part_cols[(size_t)(2 * (c0 + u) + 1) * a.nb + blockIdx.x] = si;
            }
        }
    }
    if (last_cta(&a.ctl->ticket)) {
        tail_load(a, t);
        reduce_cols(a, 2 * L);
        if (threadIdx.x == 0) t.c.cgs_phase = 1;
        tail_store(a, t);
    }
}

// x -= W(:,sel) h (the zgemv('N') of zcgs) and ||x||^2, one complex element
// per thread and step; h (as double2) and the selection in shared memory
template <int SIDE>
__global__ void __launch_bounds__(BS) k_lb_zcgs_upd(LbArgs a, int j, int last)
{
    extern __shared__ double dyn[];  // h[L] as (re, im) | sel[L]
    __shared__ double sred[32];
    __shared__ Tail t;
    if (a.ctl->status != 0 || !a.ctl->reorth_active || a.ctl->cgs_phase != 1) return;
    const int L = a.ctl->nsel;
    double2 *hs = reinterpret_cast<double2 *>(dyn);
    int *ssel = reinterpret_cast<int *>(dyn + 2 * (size_t)L);
    for (int c = threadIdx.x; c < L; c += BS) {
        hs[c] = make_double2(a.h[2 * c], a.h[2 * c + 1]);
        ssel[c] = a.sel[c];
    }
    __syncthreads();
    const int len = (SIDE == 0 ? a.adj.rows : a.fwd.rows) / 2;
    const size_t ld = (size_t)(SIDE == 0 ? a.ldv : a.ldu) / 2;
    const double2 *W = reinterpret_cast<const double2 *>(SIDE == 0 ? a.V : a.U);
    double2 *x = reinterpret_cast<double2 *>(SIDE == 0 ? vcol<double>(a, j - 1) : ucol<double>(a, j));
    double sq = 0.0;
    for (int v = blockIdx.x * BS + threadIdx.x; v < len; v += gridDim.x * BS) {
        double2 acc = x[v];
        int c = 0;
        for (; c + CGS_UNROLL <= L; c += CGS_UNROLL) {
            double2 wv[CGS_UNROLL];
#pragma unroll
            for (int u = 0; u < CGS_UNROLL; u++) wv[u] = W[(size_t)ssel[c + u] * ld + v];
#pragma unroll
            for (int u = 0; u < CGS_UNROLL; u++) zfms(acc, wv[u], hs[c + u]);
        }
        for (; c < L; c++) zfms(acc, W[(size_t)ssel[c] * ld + v], hs[c]);
        x[v] = acc;
        sq = fma(acc.x, acc.x, sq);
        sq = fma(acc.y, acc.y, sq);
    }
    const double sq2 = block_sum<BS>(sq, sred);
    if (threadIdx.x == 0) a.part_sq[blockIdx.x] = sq2;
    if (last_cta(&a.ctl->ticket)) {
        tail_load(a, t);
        const double s2 = sum_parts(a.part_sq, gridDim.x, t.red);
        after_cgs<SIDE>(t, a, j, sqrt(s2), last);
        tail_store(a, t);
    }
}

// ------------------------------------ complex Gram-Schmidt on the planes
// The complex basis read as its real (re, im) arrays: one complex element is
// one float4 of planes (re hi, re lo, im hi, im lo), split, flagged and
// scaled exactly as in the real kernels above.  The projection
// h = sum conj(w) x has Re h = sum (w.re x.re + w.im x.im), the real dot of
// the two arrays, and Im h = sum (w.re x.im - w.im x.re), the same loaded
// values with the parts of x swapped and one negated: two compensated sums
// per column, four plane products per element, on the FP32 pipe where the
// FP64 kernels spend four FP64 FMAs per 16 bytes.

// projections h = W(:,sel)^H x (zgemv 'C' of zcgs, zreorth.F) from the
// planes: the work layout of k_lb_cgs_dots_pl with two columns per group
// (their re and im sums are the four sums of pl_warp_sum4); partials of
// column c go to part_cols rows 2c (re) and 2c+1 (im), h comes out as
// (re, im) pairs
constexpr int ZPL_COLS = 2;
template <int SIDE>
__global__ void __launch_bounds__(BS, PL_MINB) k_lb_zcgs_dots_pl(LbArgs a, int j)
{
    // [PL_WARPS][2 (kmax + 1)] per-warp partials | sel[kmax + 1] | fresh[kmax + 1]
    extern __shared__ double wpart[];
    __shared__ Tail t;
    if (a.ctl->status != 0 || !a.ctl->reorth_active || a.ctl->cgs_phase != 0) return;
    const int L = a.ctl->nsel;
    const int K1 = a.kmax + 1, K2 = 2 * K1;
    int *ssel = reinterpret_cast<int *>(wpart + (size_t)PL_WARPS * K2);
    int *sfresh = ssel + K1;
    int *ok = SIDE == 0 ? a.okV : a.okU;
    for (int c = threadIdx.x; c < L; c += BS) {
        const int col = a.sel[c];
        ssel[c] = col;
        sfresh[c] = ok[col] == 0;
    }
    __syncthreads();
    const int len = SIDE == 0 ? a.adj.rows : a.fwd.rows;  // real scalars: twice the complex length
    const size_t ld = SIDE == 0 ? a.ldv : a.ldu;
    const size_t ldq = ld / 2;  // leading dimension in float4 (one complex element)
    const double *W = (const double *)(SIDE == 0 ? a.V : a.U);
    float2 *Wp = SIDE == 0 ? a.Vp : a.Up;
    const double *x = SIDE == 0 ? vcol<double>(a, j - 1) : ucol<double>(a, j);
    const double2 *xv = reinterpret_cast<const double2 *>(x);
    float4 *xq = reinterpret_cast<float4 *>(a.xpl);
    const int nvec = len / 2;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int chunk = (nvec + gridDim.x - 1) / gridDim.x;
    const int cb0 = min(nvec, blockIdx.x * chunk), cb1 = min(nvec, cb0 + chunk);
    const int sl = (cb1 - cb0 + PL_WARPS - 1) / PL_WARPS;
    const int v0 = min(cb1, cb0 + w * sl), v1 = min(cb1, v0 + sl);
    int xe = 0;
    for (int v = v0 + lane; v < v1; v += 32) {
        const double2 xx = xv[v];
        xe = max(xe, max(f3_expo(xx.x), f3_expo(xx.y)));
    }
    xe = __reduce_max_sync(0xffffffffu, xe);
    const int xs = xe == 0 ? 0 : xe - 1023;
    const double back = f3_pow2(xs);
    for (int v = v0 + lane; v < v1; v += 32) {
        const double2 xx = xv[v];
        const float2 p = pl_xsplit(xx.x, xs), q = pl_xsplit(xx.y, xs);
        xq[v] = make_float4(p.x, p.y, q.x, q.y);
    }
    for (int c = 0; c < L; c++) {
        if (!sfresh[c]) continue;
        const int col = ssel[c];
        float4 *Wq = reinterpret_cast<float4 *>(Wp) + (size_t)col * ldq;
        const double2 *Wd = reinterpret_cast<const double2 *>(W + (size_t)col * ld);
        int v = v0 + lane;
        for (; v + 32 * (PL_SPLIT_UNROLL - 1) < v1; v += 32 * PL_SPLIT_UNROLL) {
            double2 d[PL_SPLIT_UNROLL];
#pragma unroll
            for (int u = 0; u < PL_SPLIT_UNROLL; u++) d[u] = Wd[v + 32 * u];
#pragma unroll
            for (int u = 0; u < PL_SPLIT_UNROLL; u++) Wq[v + 32 * u] = pl_split2(d[u]);
        }
        for (; v < v1; v += 32) Wq[v] = pl_split2(Wd[v]);
    }
    // conj(w) x into (re, im): w = (w.x + w.y, w.z + w.w), x likewise
    auto zacc = [](PlAcc &re, PlAcc &im, const float4 &wv, const float4 &xq4) {
        re.add(wv.x, wv.y, xq4.x, xq4.y);
        re.add(wv.z, wv.w, xq4.z, xq4.w);
        im.add(wv.x, wv.y, xq4.z, xq4.w);
        im.add(wv.z, wv.w, -xq4.x, -xq4.y);
    };
    for (int cb = 0; cb < L; cb += ZPL_COLS) {
        const int nc = min(ZPL_COLS, L - cb);
        const float4 *Wq[ZPL_COLS];
#pragma unroll
        for (int u = 0; u < ZPL_COLS; u++)
            Wq[u] = reinterpret_cast<const float4 *>(Wp) + (size_t)ssel[cb + (u < nc ? u : 0)] * ldq;
        PlAcc acc[2 * ZPL_COLS];  // re, im of column cb, then of column cb + 1
        int v = v0 + lane;
        for (; v + 32 < v1; v += 64) {
            float4 w0[ZPL_COLS], w1[ZPL_COLS];
#pragma unroll
            for (int u = 0; u < ZPL_COLS; u++) {
                w0[u] = __ldcs(Wq[u] + v);
                w1[u] = __ldcs(Wq[u] + v + 32);
            }
            const float4 x0 = xq[v], x1 = xq[v + 32];
#pragma unroll
            for (int u = 0; u < ZPL_COLS; u++) {
                zacc(acc[2 * u], acc[2 * u + 1], w0[u], x0);
                zacc(acc[2 * u], acc[2 * u + 1], w1[u], x1);
            }
        }
        if (v < v1) {
            const float4 x0 = xq[v];
#pragma unroll
            for (int u = 0; u < ZPL_COLS; u++) zacc(acc[2 * u], acc[2 * u + 1], __ldcs(Wq[u] + v), x0);
        }
        static_assert(2 * ZPL_COLS == 4, "pl_warp_sum4 sums four accumulators");
        const PlAcc tot = pl_warp_sum4(acc);
        const int q = lane >> 3;  // accumulator q: column cb + q / 2, part q % 2
        if ((lane & 7) == 0 && (q >> 1) < nc) wpart[(size_t)w * K2 + 2 * cb + q] = tot.value() * back;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < 2 * L; c += BS) {
        double s = 0.0;
#pragma unroll
        for (int ww = 0; ww < PL_WARPS; ww++) s += wpart[(size_t)ww * K2 + c];
        a.part_cols[(size_t)c * a.nb + blockIdx.x] = s;
    }
    if (last_cta(&a.ctl->ticket)) {
        tail_load(a, t);
        reduce_cols(a, 2 * L, gridDim.x);
        for (int c = threadIdx.x; c < L; c += BS) ok[ssel[c]] = 1;
        if (threadIdx.x == 0) t.c.cgs_phase = 1;
        tail_store(a, t);
    }
}

// x -= W(:,sel) h (zgemv 'N' of zcgs) from the planes, and ||x||^2: one
// complex element per thread and step; h (scaled by the power of two of its
// largest part) in shared memory as float4 planes (re hi, re lo, im hi,
// im lo); Re and Im of each row's sum formed on the FP32 pipe and applied
// with FP64 FMAs
template <int SIDE>
__global__ void __launch_bounds__(BS) k_lb_zcgs_upd_pl(LbArgs a, int j, int last)
{
    extern __shared__ double dyn[];  // h[L] as float4 planes (two double slots each) | sel[L]
    __shared__ double sred[32];
    __shared__ int hsh;
    __shared__ Tail t;
    if (a.ctl->status != 0 || !a.ctl->reorth_active || a.ctl->cgs_phase != 1) return;
    const int L = a.ctl->nsel;
    float4 *hp = reinterpret_cast<float4 *>(dyn);
    int *ssel = reinterpret_cast<int *>(dyn + 2 * (size_t)L);
    if (threadIdx.x == 0) hsh = 0;
    __syncthreads();
    int he = 0;
    for (int c = threadIdx.x; c < 2 * L; c += BS) he = max(he, f3_expo(a.h[c]));
    if (he) atomicMax(&hsh, he);
    __syncthreads();
    const int hs = hsh == 0 ? 0 : hsh - 1023;  // |h 2^-hs| < 2
    const double hscale = f3_pow2(-hs), back = f3_pow2(hs);
    for (int c = threadIdx.x; c < L; c += BS) {
        const float2 hr = pl_split(a.h[2 * c] * hscale), hi = pl_split(a.h[2 * c + 1] * hscale);
        hp[c] = make_float4(hr.x, hr.y, hi.x, hi.y);
        ssel[c] = a.sel[c];
    }
    __syncthreads();
    const int len = SIDE == 0 ? a.adj.rows : a.fwd.rows;
    const size_t ldq = (size_t)(SIDE == 0 ? a.ldv : a.ldu) / 2;
    const float4 *Wq = reinterpret_cast<const float4 *>(SIDE == 0 ? a.Vp : a.Up);
    double2 *xv = reinterpret_cast<double2 *>(SIDE == 0 ? vcol<double>(a, j - 1) : ucol<double>(a, j));
    const int nvec = len / 2;
    // w h into (re, im)
    auto zmul = [](PlAcc &re, PlAcc &im, const float4 &wv, const float4 &h) {
        re.add(wv.x, wv.y, h.x, h.y);
        re.add(wv.z, wv.w, -h.z, -h.w);
        im.add(wv.x, wv.y, h.z, h.w);
        im.add(wv.z, wv.w, h.x, h.y);
    };
    double sq = 0.0;
    for (int v = blockIdx.x * BS + threadIdx.x; v < nvec; v += gridDim.x * BS) {
        const double2 x0 = xv[v];
        PlAcc sr, si;
        int c = 0;
        for (; c + CGS_UNROLL <= L; c += CGS_UNROLL) {
            float4 wv[CGS_UNROLL];
#pragma unroll
            for (int u = 0; u < CGS_UNROLL; u++) wv[u] = Wq[(size_t)ssel[c + u] * ldq + v];
#pragma unroll
            for (int u = 0; u < CGS_UNROLL; u++) zmul(sr, si, wv[u], hp[c + u]);
        }
        for (; c < L; c++) zmul(sr, si, Wq[(size_t)ssel[c] * ldq + v], hp[c]);
        double2 y;
        y.x = fma(-pl_f2d(sr.c), back, fma(-pl_f2d(sr.s), back, x0.x));
        y.y = fma(-pl_f2d(si.c), back, fma(-pl_f2d(si.s), back, x0.y));
        xv[v] = y;
        sq = fma(y.x, y.x, sq);
        sq = fma(y.y, y.y, sq);
    }
    const double sq2 = block_sum<BS>(sq, sred);
    if (threadIdx.x == 0) a.part_sq[blockIdx.x] = sq2;
    if (last_cta(&a.ctl->ticket)) {
        tail_load(a, t);
        const double s2 = sum_parts(a.part_sq, gridDim.x, t.red);
        after_cgs<SIDE>(t, a, j, sqrt(s2), last);
        tail_store(a, t);
    }
}

// apply the deferred scaling of the newest u and v columns
template <typename T>
__global__ void __launch_bounds__(BS) k_lb_flush(LbArgs a)
{
    if (a.ctl->status != 0) return;
    const Pend pu = a.ctl->pend_u, pv = a.ctl->pend_v;
    const int cu = a.ctl->pend_u_col, cv = a.ctl->pend_v_col;
    const int m = a.fwd.rows, n = a.adj.rows;
    const int len = m > n ? m : n;
    T *uc = cu >= 0 ? ucol<T>(a, cu) : nullptr;
    T *vc = cv >= 0 ? vcol<T>(a, cv) : nullptr;
    if (a.okU && blockIdx.x == 0 && threadIdx.x == 0) {
        if (pu.mode && cu >= 0) a.okU[cu] = 0;
        if (pv.mode && cv >= 0) a.okV[cv] = 0;
    }
    for (int r = blockIdx.x * BS + threadIdx.x; r < len; r += gridDim.x * BS) {
        if (pu.mode && uc && r < m) uc[r] = apply_pend(uc[r], pu);
        if (pv.mode && vc && r < n) vc[r] = apply_pend(vc[r], pv);
    }
    if (last_cta(&a.ctl->ticket)) {
        if (threadIdx.x == 0) {
            a.ctl->pend_u.mode = 0;
            a.ctl->pend_v.mode = 0;
            __threadfence();
        }
    }
}

// ------------------------------------------------------------ host side
template <typename T>
static size_t cgs_smem(const LbArgs &a) { return (sizeof(double) + sizeof(int)) * (size_t)(a.kmax + 1) + 16; }
static size_t cgs_smem_f3(const LbArgs &a) { return (2 * sizeof(double) + sizeof(int)) * (size_t)(a.kmax + 1) + 16; }

// Gram-Schmidt arithmetic of the FP64 form (propack_set_cgs_arith)
thread_local int g_cgs_arith = CGS_PLANES;
static size_t pl_smem(int kmax) { return (sizeof(double) * PL_WARPS + 2 * sizeof(int)) * (size_t)(kmax + 1); }
// the complex projections keep (re, im) partials per warp
static size_t zpl_smem(int kmax) { return (2 * sizeof(double) * PL_WARPS + 2 * sizeof(int)) * (size_t)(kmax + 1); }
static size_t cgs_smem_pl(const LbArgs &a) { return pl_smem(a.kmax); }

template <int SIDE, typename T>
static void set_upd_limits(size_t need)
{
    PGB_CUDA(cudaFuncSetAttribute(k_lb_cgs_upd<SIDE, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need));
}
void lb_set_smem_limits(int kmax)
{
    const size_t need3 = (2 * sizeof(double) + sizeof(int)) * (size_t)(kmax + 1) + 16;
    if (need3 > 48 * 1024) {
        PGB_CUDA(cudaFuncSetAttribute(k_lb_cgs_upd_f3<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need3));
        PGB_CUDA(cudaFuncSetAttribute(k_lb_cgs_upd_f3<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need3));
    }
    if (need3 > 48 * 1024) {
        // the complex updates keep h as (re, im) or its planes: the same shared memory as the f3 update
        PGB_CUDA(cudaFuncSetAttribute(k_lb_zcgs_upd<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need3));
        PGB_CUDA(cudaFuncSetAttribute(k_lb_zcgs_upd<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need3));
        PGB_CUDA(cudaFuncSetAttribute(k_lb_zcgs_upd_pl<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need3));
        PGB_CUDA(cudaFuncSetAttribute(k_lb_zcgs_upd_pl<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need3));
    }
    const size_t needz = zpl_smem(kmax);
    if (needz > 48 * 1024 && needz <= PL_SMEM_MAX) {
        PGB_CUDA(cudaFuncSetAttribute(k_lb_zcgs_dots_pl<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)needz));
        PGB_CUDA(cudaFuncSetAttribute(k_lb_zcgs_dots_pl<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)needz));
    }
    const size_t need = (sizeof(double) + sizeof(int)) * (size_t)(kmax + 1) + 16;
    if (need > 48 * 1024) {
        set_upd_limits<0, double>(need);
        set_upd_limits<1, double>(need);
        set_upd_limits<0, float>(need);
        set_upd_limits<1, float>(need);
        PGB_CUDA(cudaFuncSetAttribute(k_lb_cgs_upd_pl<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need));
        PGB_CUDA(cudaFuncSetAttribute(k_lb_cgs_upd_pl<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need));
    }
    const size_t needp = pl_smem(kmax);
    if (needp > 48 * 1024 && needp <= PL_SMEM_MAX) {
        PGB_CUDA(cudaFuncSetAttribute(k_lb_cgs_dots_pl<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)needp));
        PGB_CUDA(cudaFuncSetAttribute(k_lb_cgs_dots_pl<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)needp));
    }
}

// the planes are used when the driver allocated them (FP64 form, kmax small
// enough for the projections' per-warp partials in shared memory; complex
// vectors keep twice the partials)
bool lb_planes_fit(int kmax, bool cplx) { return (cplx ? zpl_smem(kmax) : pl_smem(kmax)) <= PL_SMEM_MAX; }

// one wave of the plane projections at their occupancy (at most nb CTAs;
// their partials are summed over gridDim)
template <int SIDE>
static int dots_pl_grid(const LbArgs &a)
{
    static thread_local int g = 0, dev = -1;
    static thread_local size_t smem = 0;
    const Dev &d = device_info();
    const size_t need = cgs_smem_pl(a);
    if (g == 0 || dev != d.device || smem != need) {
        int per = 0;
        PGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_lb_cgs_dots_pl<SIDE>, BS, need));
        g = std::max(1, per) * d.sms;
        dev = d.device;
        smem = need;
    }
    return std::min(g, a.nb);
}

// one CGS pass: the projections, then the update (each kernel returns at
// once when the control block says that its half of the pass is not due)
template <int SIDE, typename T>
static void launch_cgs_pass(const LbArgs &a, int j, int last, cudaStream_t s)
{
    if (sizeof(T) == 8 && a.Up) {
        PGB_PROF(PK_CGS_DOTS, s, k_lb_cgs_dots_pl<SIDE><<<dots_pl_grid<SIDE>(a), BS, cgs_smem_pl(a), s>>>(a, j));
        PGB_LAUNCHED();
        PGB_PROF(PK_CGS_UPD, s, k_lb_cgs_upd_pl<SIDE><<<a.nb, BS, cgs_smem<T>(a), s>>>(a, j, last));
        PGB_LAUNCHED();
        return;
    }
    if (sizeof(T) == 8 && g_cgs_arith == CGS_F3) {
        PGB_PROF(PK_CGS_DOTS, s, k_lb_cgs_dots_f3<SIDE><<<a.nb, BS, 0, s>>>(a, j));
        PGB_LAUNCHED();
        PGB_PROF(PK_CGS_UPD, s, k_lb_cgs_upd_f3<SIDE><<<a.nb, BS, cgs_smem_f3(a), s>>>(a, j, last));
        PGB_LAUNCHED();
        return;
    }
    PGB_PROF(sizeof(T) == 8 ? PK_CGS_DOTS : PK_CGS_DOTS32, s, k_lb_cgs_dots<SIDE, T><<<a.nb, BS, 0, s>>>(a, j));
    PGB_LAUNCHED();
    PGB_PROF(sizeof(T) == 8 ? PK_CGS_UPD : PK_CGS_UPD32, s,
             k_lb_cgs_upd<SIDE, T><<<a.nb, BS, cgs_smem<T>(a), s>>>(a, j, last));
    PGB_LAUNCHED();
}

template <int SIDE>
static int zdots_pl_grid(const LbArgs &a)
{
    static thread_local int g = 0, dev = -1;
    static thread_local size_t smem = 0;
    const Dev &d = device_info();
    const size_t need = zpl_smem(a.kmax);
    if (g == 0 || dev != d.device || smem != need) {
        int per = 0;
        PGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_lb_zcgs_dots_pl<SIDE>, BS, need));
        g = std::max(1, per) * d.sms;
        dev = d.device;
        smem = need;
    }
    return std::min(g, a.nb);
}

// one complex Gram-Schmidt pass (on the planes when the driver keeps them)
template <int SIDE>
static void launch_zcgs_pass(const LbArgs &a, int j, int last, cudaStream_t s)
{
    if (a.Up) {
        PGB_PROF(PK_CGS_DOTS, s,
                 k_lb_zcgs_dots_pl<SIDE><<<zdots_pl_grid<SIDE>(a), BS, zpl_smem(a.kmax), s>>>(a, j));
        PGB_LAUNCHED();
        PGB_PROF(PK_CGS_UPD, s, k_lb_zcgs_upd_pl<SIDE><<<a.nb, BS, cgs_smem_f3(a), s>>>(a, j, last));
        PGB_LAUNCHED();
        return;
    }
    PGB_PROF(PK_CGS_DOTS, s, k_lb_zcgs_dots<SIDE><<<a.nb, BS, 0, s>>>(a, j));
    PGB_LAUNCHED();
    PGB_PROF(PK_CGS_UPD, s, k_lb_zcgs_upd<SIDE><<<a.nb, BS, cgs_smem_f3(a), s>>>(a, j, last));
    PGB_LAUNCHED();
}

// one wave of CTAs at the fused SpMV's occupancy (partials are summed over gridDim)
template <int SIDE, typename T, int SHORT>
static int spmv_grid(int nb)
{
    static thread_local int g = 0, dev = -1;
    const Dev &d = device_info();
    if (g == 0 || dev != d.device) {
        int per = 0;
        PGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_lb_spmv<SIDE, T, SHORT>, BS, 0));
        g = std::max(1, per) * d.sms;
        dev = d.device;
    }
    return std::min(g, nb);
}
template <int SIDE, typename T>
static void launch_spmv(const LbArgs &a, const Csr &A, int j, bool host_product, cudaStream_t s)
{
    if (host_product || A.short_rows)
        k_lb_spmv<SIDE, T, 1><<<spmv_grid<SIDE, T, 1>(a.nb_spmv), BS, 0, s>>>(a, j, host_product ? 1 : 0);
    else
        k_lb_spmv<SIDE, T, 0><<<spmv_grid<SIDE, T, 0>(a.nb_spmv), BS, 0, s>>>(a, j, host_product ? 1 : 0);
}

template <int SIDE>
static void launch_zspmv(const LbArgs &a, int j, bool host_product, cudaStream_t s)
{
    static thread_local int g = 0, dev = -1;
    const Dev &d = device_info();
    if (g == 0 || dev != d.device) {
        int per = 0;
        PGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_lb_zspmv<SIDE>, BS, 0));
        g = std::max(1, per) * d.sms;
        dev = d.device;
    }
    k_lb_zspmv<SIDE><<<std::min(g, a.nb_spmv), BS, 0, s>>>(a, j, host_product ? 1 : 0);
}

// Enqueue the kernels of one half step.  host_product: the product was
// written into the output column by a host APROD call.
// the half step of the complex form: the real fused SpMV on the 2x2-block
// operator, then one more ELR launch than ielr (the first forms the complex
// projection), then the complex Gram-Schmidt passes
static void zenqueue_half(const LbArgs &a, int side, int j, int ielr, int ntry_spec, bool host_product,
                          cudaStream_t s)
{
    const int nb = a.nb;
    // the native complex SpMV (and the host-product epilogue, which shares
    // it) forms the complex projection itself: ielr ELR launches suffice
    const bool native = host_product || a.zfwd.rows > 0;
    const int nelr = ielr > 0 ? ielr + (native ? 0 : 1) : 0;
    if (native) {
        if (side == 0) PGB_PROF(PK_SPMV_ADJ, s, launch_zspmv<0>(a, j, host_product, s));
        else PGB_PROF(PK_SPMV_FWD, s, launch_zspmv<1>(a, j, host_product, s));
        PGB_LAUNCHED();
        if (side == 1 || j > 1)
            for (int i = 0; i < nelr; i++) {
                if (side == 0) PGB_PROF(PK_ELR, s, k_lb_zelr<0><<<nb, BS, 0, s>>>(a, j));
                else PGB_PROF(PK_ELR, s, k_lb_zelr<1><<<nb, BS, 0, s>>>(a, j));
                PGB_LAUNCHED();
            }
        for (int i = 0; i < ntry_spec; i++) {
            if (side == 0) launch_zcgs_pass<0>(a, j, i == ntry_spec - 1, s);
            else launch_zcgs_pass<1>(a, j, i == ntry_spec - 1, s);
        }
        return;
    }
    if (side == 0) {
        PGB_PROF(PK_SPMV_ADJ, s, launch_spmv<0, double>(a, a.adj, j, host_product, s));
        PGB_LAUNCHED();
        if (j > 1)
            for (int i = 0; i < nelr; i++) {
                PGB_PROF(PK_ELR, s, k_lb_zelr<0><<<nb, BS, 0, s>>>(a, j));
                PGB_LAUNCHED();
            }
        for (int i = 0; i < ntry_spec; i++) launch_zcgs_pass<0>(a, j, i == ntry_spec - 1, s);
    } else {
        PGB_PROF(PK_SPMV_FWD, s, launch_spmv<1, double>(a, a.fwd, j, host_product, s));
        PGB_LAUNCHED();
        for (int i = 0; i < nelr; i++) {
            PGB_PROF(PK_ELR, s, k_lb_zelr<1><<<nb, BS, 0, s>>>(a, j));
            PGB_LAUNCHED();
        }
        for (int i = 0; i < ntry_spec; i++) launch_zcgs_pass<1>(a, j, i == ntry_spec - 1, s);
    }
}

template <typename T>
void lb_enqueue_half(const LbArgs &a, const Operator *op, int side, int j, int ielr, int ntry_spec,
                     bool host_product, cudaStream_t s)
{
    if constexpr (VecW<T>::w == 2) {
        (void)op;
        zenqueue_half(a, side, j, ielr, ntry_spec, host_product, s);
        return;
    } else {
    const int nb = a.nb;
    if (side == 0) {
        if (!host_product && op && op->r > 0)
            PGB_PROF(PK_THIN, s, op_thin<T>(*op, true, ucol<T>(a, j - 1), s));
        PGB_PROF(sizeof(T) == 8 ? PK_SPMV_ADJ : PK_SPMV_ADJ32, s,
                 launch_spmv<0, T>(a, a.adj, j, host_product, s));
        PGB_LAUNCHED();
        if (j > 1)
            for (int i = 0; i < ielr; i++) {
                PGB_PROF(PK_ELR, s, k_lb_elr<0, T><<<nb, BS, 0, s>>>(a, j));
                PGB_LAUNCHED();
            }
        for (int i = 0; i < ntry_spec; i++) launch_cgs_pass<0, T>(a, j, i == ntry_spec - 1, s);
    } else {
        if (!host_product && op && op->r > 0)
            PGB_PROF(PK_THIN, s, op_thin<T>(*op, false, vcol<T>(a, j - 1), s));
        PGB_PROF(sizeof(T) == 8 ? PK_SPMV_FWD : PK_SPMV_FWD32, s,
                 launch_spmv<1, T>(a, a.fwd, j, host_product, s));
        PGB_LAUNCHED();
        for (int i = 0; i < ielr; i++) {
            PGB_PROF(PK_ELR, s, k_lb_elr<1, T><<<nb, BS, 0, s>>>(a, j));
            PGB_LAUNCHED();
        }
        for (int i = 0; i < ntry_spec; i++) launch_cgs_pass<1, T>(a, j, i == ntry_spec - 1, s);
    }
    }
}

// more Gram-Schmidt passes after a suspension with reason 2
template <typename T>
void lb_enqueue_cgs_more(const LbArgs &a, int side, int j, int passes, cudaStream_t s)
{
    for (int i = 0; i < passes; i++) {
        if constexpr (VecW<T>::w == 2) {
            if (side == 0) launch_zcgs_pass<0>(a, j, i == passes - 1, s);
            else launch_zcgs_pass<1>(a, j, i == passes - 1, s);
        } else {
            if (side == 0) launch_cgs_pass<0, T>(a, j, i == passes - 1, s);
            else launch_cgs_pass<1, T>(a, j, i == passes - 1, s);
        }
    }
}

// (complex: the flush of the real scalars, whose lengths LbArgs counts)
template <typename T>
void lb_enqueue_flush(const LbArgs &a, cudaStream_t s)
{
    using E = typename std::conditional<VecW<T>::w == 2, double, T>::type;
    k_lb_flush<E><<<a.nb, BS, 0, s>>>(a);
    PGB_LAUNCHED();
}

template void lb_enqueue_half<double>(const LbArgs &, const Operator *, int, int, int, int, bool, cudaStream_t);
template void lb_enqueue_half<float>(const LbArgs &, const Operator *, int, int, int, int, bool, cudaStream_t);
template void lb_enqueue_cgs_more<double>(const LbArgs &, int, int, int, cudaStream_t);
template void lb_enqueue_cgs_more<float>(const LbArgs &, int, int, int, cudaStream_t);
template void lb_enqueue_flush<double>(const LbArgs &, cudaStream_t);
template void lb_enqueue_flush<float>(const LbArgs &, cudaStream_t);
template void lb_enqueue_half<double2>(const LbArgs &, const Operator *, int, int, int, int, bool, cudaStream_t);
template void lb_enqueue_cgs_more<double2>(const LbArgs &, int, int, int, cudaStream_t);
template void lb_enqueue_flush<double2>(const LbArgs &, cudaStream_t);

}  // namespace pgb
