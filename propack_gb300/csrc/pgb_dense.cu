// pgb_dense.cu -- the small dense part of the IRL/Ritz machinery, on device:
//
//   k_analyse      dbdqr + bidiagonal QR SVD (values + last row of the left
//                  vectors) + error bounds + drefinebounds + convergence
//                  count (double/dlansvd_irl.F:218-290, dlansvd.F:192-236)
//   k_irl_sweeps   exact-shift selection and dbsvdstep sweeps accumulating
//                  P and Q (dlansvd_irl.F:304-363)
//   k_ritz_prep    dbdqr with Q' + full SVD of R (the role of dbdsdc in
//                  double/dritzvec.F:116-124)
//   k_gemm         C = op(A) op(B) in FP64 for the restart and Ritz
//                  products (dlansvd_irl.F:371-398, dritzvec.F:130-198)
//
// The bidiagonal SVD is one CTA: thread 0 runs the implicit zero-shift /
// shifted QR iteration (Demmel & Kahan 1990; the algorithm of LAPACK
// dbdsqr) and records each sweep's rotation chain in shared memory; the
// whole CTA then applies the chain to the singular-vector matrices, one row
// (or column) per thread.
#include "pgb.cuh"
#include "pgb_bidiag.cuh"
#include "pgb_scalar.cuh"

namespace pgb {

// ---------------------------------------------------- CTA bidiagonal SVD
struct QrShared {
    int ll, cnt, vt_fwd, u_fwd, apply, done, info;
};

// apply a recorded chain: VT rows (pair i: rows lo+i, lo+i+1), U columns
__device__ void apply_chain(int ncvt, double *vt, int ldvt, int nru, double *u, int ldu, int lo, int cnt,
                            const double *cv, const double *sv, int vfwd, const double *cu, const double *su, int ufwd)
{
    for (int col = threadIdx.x; col < ncvt; col += blockDim.x) {
        double *A = vt + (size_t)col * ldvt + lo;
        for (int t = 0; t < cnt; t++) {
            const int i = vfwd ? t : cnt - 1 - t;
            const double c = cv[i], s = sv[i];
            const double x = A[i], y = A[i + 1];
            A[i + 1] = c * y - s * x;
            A[i] = s * y + c * x;
        }
    }
    for (int row = threadIdx.x; row < nru; row += blockDim.x) {
        for (int t = 0; t < cnt; t++) {
            const int i = ufwd ? t : cnt - 1 - t;
            const double c = cu[i], s = su[i];
            double *x = u + (size_t)(lo + i) * ldu + row, *y = x + ldu;
            const double xv = *x, yv = *y;
            *y = c * yv - s * xv;
            *x = s * yv + c * xv;
        }
    }
}

// Upper bidiagonal SVD by implicit QR, executed by the whole CTA.  d[n],
// e[n] (e[n-1] unused); VT n x ncvt (ldvt), U nru x n (ldu).  w: 4n doubles
// of shared or global scratch.  Singular values end up non-negative and
// sorted decreasingly.  Returns 0 or >0 (no convergence).
__device__ int bdsqr_cta(int n, double *d, double *e, int ncvt, double *vt, int ldvt, int nru, double *u, int ldu,
                         double *w, QrShared &q)
{
    double *c1 = w, *s1 = w + n, *c2 = w + 2 * n, *s2 = w + 3 * n;
    const int tid = threadIdx.x;
    // per-thread-0 state
    double tol = 0, thresh = 0, sminl = 0, smax = 0;
    long maxit = 0, iter = 0;
    int oldll = -1, oldm = -1, idir = 0, m = n - 1;
    if (tid == 0) {
        q.info = 0;
        q.done = (n <= 1);
        if (n > 1) {
            const double tolmul = fmax(10.0, fmin(100.0, pow(EPS, -0.125)));
            tol = tolmul * EPS;
            for (int i = 0; i < n; i++) smax = fmax(smax, fabs(d[i]));
            for (int i = 0; i < n - 1; i++) smax = fmax(smax, fabs(e[i]));
            double sminoa = fabs(d[0]);
            if (sminoa != 0.0) {
                double mu = sminoa;
                for (int i = 1; i < n; i++) {
                    mu = fabs(d[i]) * (mu / (mu + fabs(e[i - 1])));
                    sminoa = fmin(sminoa, mu);
                    if (sminoa == 0.0) break;
                }
            }
            sminoa = sminoa / sqrt((double)n);
            thresh = fmax(tol * sminoa, 6.0 * (double)n * (double)n * SFMIN);
            maxit = 6L * n * n;
        }
    }
    __syncthreads();
    while (true) {
        if (tid == 0) {
            q.apply = 0;
            while (!q.done && !q.apply) {
                if (m <= 0) { q.done = 1; break; }
                if (iter > maxit) { q.info = 1; q.done = 1; break; }
                int ll, split = -1;
                smax = fabs(d[m]);
                for (ll = m - 1; ll >= 0; ll--) {
                    const double abss = fabs(d[ll]), abse = fabs(e[ll]);
                    if (abse <= thresh) { split = ll; break; }
                    smax = fmax(smax, fmax(abss, abse));
                }
                if (split >= 0) {
                    e[split] = 0.0;
                    if (split == m - 1) { m -= 1; continue; }
                    ll = split + 1;
                } else {
                    ll = 0;
                }
                if (ll > oldm || m < oldll) idir = (fabs(d[ll]) >= fabs(d[m])) ? 1 : 2;
                bool defl = false;
                if (idir == 1) {
                    if (fabs(e[m - 1]) <= tol * fabs(d[m])) { e[m - 1] = 0.0; continue; }
                    double mu = fabs(d[ll]);
                    sminl = mu;
                    for (int l3 = ll; l3 <= m - 1; l3++) {
                        if (fabs(e[l3]) <= tol * mu) { e[l3] = 0.0; defl = true; break; }
                        mu = fabs(d[l3 + 1]) * (mu / (mu + fabs(e[l3])));
                        sminl = fmin(sminl, mu);
                    }
                } else {
                    if (fabs(e[ll]) <= tol * fabs(d[ll])) { e[ll] = 0.0; continue; }
                    double mu = fabs(d[m]);
                    sminl = mu;
                    for (int l3 = m - 1; l3 >= ll; l3--) {
                        if (fabs(e[l3]) <= tol * mu) { e[l3] = 0.0; defl = true; break; }
                        mu = fabs(d[l3]) * (mu / (mu + fabs(e[l3])));
                        sminl = fmin(sminl, mu);
                    }
                }
                if (defl) continue;
                oldll = ll;
                oldm = m;
                double shift, sll, rdum;
                if ((double)n * tol * (sminl / smax) <= fmax(EPS, 0.01 * tol)) {
                    shift = 0.0;
                } else {
                    if (idir == 1) { sll = fabs(d[ll]); sv2x2(d[m - 1], e[m - 1], d[m], shift, rdum); }
                    else { sll = fabs(d[m]); sv2x2(d[ll], e[ll], d[ll + 1], shift, rdum); }
                    if (sll > 0.0 && (shift / sll) * (shift / sll) < EPS) shift = 0.0;
                }
                iter += m - ll;
                const int cnt = m - ll;
                double cs, sn, r, oldcs, oldsn, f, g, h;
                if (shift == 0.0) {
                    if (idir == 1) {
                        cs = 1.0; oldcs = 1.0; oldsn = 0.0;
                        for (int i = ll; i <= m - 1; i++) {
                            lartg(d[i] * cs, e[i], cs, sn, r);
                            if (i > ll) e[i - 1] = oldsn * r;
                            lartg(oldcs * r, d[i + 1] * sn, oldcs, oldsn, d[i]);
                            c1[i - ll] = cs; s1[i - ll] = sn; c2[i - ll] = oldcs; s2[i - ll] = oldsn;
                        }
                        h = d[m] * cs;
                        d[m] = h * oldcs;
                        e[m - 1] = h * oldsn;
                        q.vt_fwd = 1; q.u_fwd = 1;
                        if (fabs(e[m - 1]) <= thresh) e[m - 1] = 0.0;
                        // VT gets (c1,s1), U gets (c2,s2)
                    } else {
                        cs = 1.0; oldcs = 1.0; oldsn = 0.0;
                        for (int i = m; i >= ll + 1; i--) {
                            lartg(d[i] * cs, e[i - 1], cs, sn, r);
                            if (i < m) e[i] = oldsn * r;
                            lartg(oldcs * r, d[i - 1] * sn, oldcs, oldsn, d[i]);
                            // U gets (cs,-sn) -> stored in (c2,s2); VT gets (oldcs,-oldsn) -> (c1,s1)
                            c2[i - ll - 1] = cs; s2[i - ll - 1] = -sn;
                            c1[i - ll - 1] = oldcs; s1[i - ll - 1] = -oldsn;
                        }
                        h = d[ll] * cs;
                        d[ll] = h * oldcs;
                        e[ll] = h * oldsn;
                        q.vt_fwd = 0; q.u_fwd = 0;
                        if (fabs(e[ll]) <= thresh) e[ll] = 0.0;
                    }
                } else {
                    double cosr, sinr, cosl, sinl;
                    if (idir == 1) {
                        f = (fabs(d[ll]) - shift) * (copysign(1.0, d[ll]) + shift / d[ll]);
                        g = e[ll];
                        for (int i = ll; i <= m - 1; i++) {
                            lartg(f, g, cosr, sinr, r);
                            if (i > ll) e[i - 1] = r;
                            f = cosr * d[i] + sinr * e[i];
                            e[i] = cosr * e[i] - sinr * d[i];
                            g = sinr * d[i + 1];
                            d[i + 1] = cosr * d[i + 1];
                            lartg(f, g, cosl, sinl, r);
                            d[i] = r;
                            f = cosl * e[i] + sinl * d[i + 1];
                            d[i + 1] = cosl * d[i + 1] - sinl * e[i];
                            if (i < m - 1) { g = sinl * e[i + 1]; e[i + 1] = cosl * e[i + 1]; }
                            c1[i - ll] = cosr; s1[i - ll] = sinr; c2[i - ll] = cosl; s2[i - ll] = sinl;
                        }
                        e[m - 1] = f;
                        q.vt_fwd = 1; q.u_fwd = 1;
                        if (fabs(e[m - 1]) <= thresh) e[m - 1] = 0.0;
                    } else {
                        f = (fabs(d[m]) - shift) * (copysign(1.0, d[m]) + shift / d[m]);
                        g = e[m - 1];
                        for (int i = m; i >= ll + 1; i--) {
                            lartg(f, g, cosr, sinr, r);
                            if (i < m) e[i] = r;
                            f = cosr * d[i] + sinr * e[i - 1];
                            e[i - 1] = cosr * e[i - 1] - sinr * d[i];
                            g = sinr * d[i - 1];
                            d[i - 1] = cosr * d[i - 1];
                            lartg(f, g, cosl, sinl, r);
                            d[i] = r;
                            f = cosl * e[i - 1] + sinl * d[i - 1];
                            d[i - 1] = cosl * d[i - 1] - sinl * e[i - 1];
                            if (i > ll + 1) { g = sinl * e[i - 2]; e[i - 2] = cosl * e[i - 2]; }
                            // U gets (cosr,-sinr) -> (c2,s2); VT gets (cosl,-sinl) -> (c1,s1)
                            c2[i - ll - 1] = cosr; s2[i - ll - 1] = -sinr;
                            c1[i - ll - 1] = cosl; s1[i - ll - 1] = -sinl;
                        }
                        e[ll] = f;
                        q.vt_fwd = 0; q.u_fwd = 0;
                        if (fabs(e[ll]) <= thresh) e[ll] = 0.0;
                    }
                }
                q.ll = ll;
                q.cnt = cnt;
                q.apply = (ncvt > 0 || nru > 0);
            }
        }
        __syncthreads();
        if (q.done && !q.apply) break;
        if (q.apply) apply_chain(ncvt, vt, ldvt, nru, u, ldu, q.ll, q.cnt, c1, s1, q.vt_fwd, c2, s2, q.u_fwd);
        __syncthreads();
    }
    // non-negative values
    for (int i = 0; i < n; i++) {
        if (d[i] < 0.0) {
            __syncthreads();
            for (int c = tid; c < ncvt; c += blockDim.x) vt[(size_t)c * ldvt + i] = -vt[(size_t)c * ldvt + i];
            __syncthreads();
            if (tid == 0) d[i] = -d[i];
            __syncthreads();
        }
    }
    // sort decreasingly
    __shared__ int isub_s;
    for (int i = 0; i < n - 1; i++) {
        if (tid == 0) {
            int isub = i;
            double smx = d[i];
            for (int j = i + 1; j < n; j++)
                if (d[j] > smx) { smx = d[j]; isub = j; }
            isub_s = isub;
            if (isub != i) { d[isub] = d[i]; d[i] = smx; }
        }
        __syncthreads();
        const int isub = isub_s;
        if (isub != i) {
            for (int c = tid; c < ncvt; c += blockDim.x) {
                const double t = vt[(size_t)c * ldvt + i];
                vt[(size_t)c * ldvt + i] = vt[(size_t)c * ldvt + isub];
                vt[(size_t)c * ldvt + isub] = t;
            }
            for (int r = tid; r < nru; r += blockDim.x) {
                const double t = u[(size_t)i * ldu + r];
                u[(size_t)i * ldu + r] = u[(size_t)isub * ldu + r];
                u[(size_t)isub * ldu + r] = t;
            }
        }
        __syncthreads();
    }
    return q.info;
}

// ----------------------------------------------------------------- analysis

// IRL: dlansvd_irl.F:218-290.  lansvd: dlansvd.F:192-236.  The bidiagonal,
// the bound row and the rotation chains live in shared memory when they
// fit (use_smem), so the sequential QR iteration of thread 0 runs at
// shared-memory latency.
__global__ void k_analyse(AnaArgs a, int use_smem)
{
    __shared__ QrShared q;
    extern __shared__ double dsm[];
    const int dim = a.dim;
    double *d = use_smem ? dsm : a.a1;
    double *e = use_smem ? dsm + (dim + 1) : a.b1;
    double *bnd = use_smem ? dsm + 2 * (dim + 1) : a.bnd;
    double *w = use_smem ? dsm + 3 * (dim + 1) + 1 : a.w;
    for (int i = threadIdx.x; i < dim; i += blockDim.x) { d[i] = a.balpha[i]; e[i] = a.bbeta[i]; }
    for (int i = threadIdx.x; i <= dim; i += blockDim.x) bnd[i] = 0.0;
    __syncthreads();
    const int mn = a.m < a.n ? a.m : a.n;
    if (threadIdx.x == 0) bdqr_dev(dim == mn, dim, d, e, &bnd[dim - 1], &bnd[dim], nullptr, 0);
    __syncthreads();
    bdsqr_cta(dim, d, e, 0, nullptr, 1, 1, bnd, 1, w, q);
    __syncthreads();
    if (threadIdx.x == 0) {
        const double eps34 = pow(EPS, 0.75);
        const double epsn = (double)(a.m > a.n ? a.m : a.n) * EPS / 2.0;
        double anorm = *a.anorm_drv;
        if (dim > 5) anorm = d[0];
        else anorm = fmax(anorm, d[0]);
        *a.anorm_drv = anorm;
        const double rnorm = a.ctl->rnorm;
        for (int i = 0; i < dim; i++) bnd[i] = fabs(rnorm * bnd[i]);
        int nconv = 0;
        if (a.irl) {
            const int neig = a.neig;
            if (a.small_side) refinebounds_dev(mn, dim, d, bnd, epsn * anorm, eps34);
            else refinebounds_dev(mn, dim < neig ? dim : neig, d, bnd, epsn * anorm, eps34);
            if (a.small_side) {
                for (int i = dim - neig + 1; i <= dim; i++) {
                    if (bnd[i - 1] <= a.tol * d[0]) {
                        a.sigma_out[nconv] = d[i - 1];
                        a.bnd_out[nconv] = bnd[i - 1];
                        nconv++;
                    }
                }
            } else {
                int i = 1;
                const int lim = dim < neig ? dim : neig;
                while (i <= lim) {
                    if (bnd[i - 1] <= a.tol * d[i - 1]) {
                        a.sigma_out[nconv] = d[i - 1];
                        a.bnd_out[nconv] = bnd[i - 1];
                        nconv++;
                        i++;
                    } else {
                        i = a.kk + 1;
                    }
                }
            }
        } else {
            // dlansvd: k = a.kk
            refinebounds_dev(mn, dim, d, bnd, epsn * anorm, eps34);
            const int lim = dim < a.kk ? dim : a.kk;
            for (int i = 0; i < lim; i++) a.bnd_out[i] = bnd[i];
            int i = 0;
            while (i < lim) {
                if (bnd[i] <= a.tol * d[i]) { a.sigma_out[nconv] = d[i]; nconv++; i++; }
                else i = a.kk;
            }
        }
        *a.nconv_out = nconv;
    }
    __syncthreads();
    if (use_smem) {
        // the sweeps read the Ritz values and bounds from global memory
        for (int i = threadIdx.x; i < dim; i += blockDim.x) { a.a1[i] = d[i]; a.bnd[i] = bnd[i]; }
        if (threadIdx.x == 0) a.bnd[dim] = bnd[dim];
    }
}

// ------------------------------------------------------------ IRL sweeps

// dbsvdstep chain (double/dbsvd.F:5-82) for sweep length kk: thread 0
// computes the rotations (U side in cu/su, V side in cv/sv).
__device__ void bsvdstep_chain(int kk, double sigma, double *D, double *E, double *cu, double *su, double *cv,
                               double *sv)
{
    double c, s, x, y, r;
    x = D[0] * D[0] - sigma * sigma;
    y = E[0] * D[0];
    for (int i = 1; i <= kk - 1; i++) {
        if (i > 1) lartg(x, y, c, s, E[i - 2]);
        else lartg(x, y, c, s, r);
        x = c * D[i - 1] + s * E[i - 1];
        E[i - 1] = -s * D[i - 1] + c * E[i - 1];
        D[i - 1] = x;
        y = s * D[i];
        D[i] = c * D[i];
        cu[i - 1] = c; su[i - 1] = s;
        lartg(x, y, c, s, D[i - 1]);
        x = c * E[i - 1] + s * D[i];
        D[i] = -s * E[i - 1] + c * D[i];
        E[i - 1] = x;
        y = s * E[i];
        E[i] = c * E[i];
        cv[i - 1] = c; sv[i - 1] = s;
    }
    lartg(x, y, c, s, E[kk - 2]);
    x = c * D[kk - 1] + s * E[kk - 1];
    E[kk - 1] = -s * D[kk - 1] + c * E[kk - 1];
    D[kk - 1] = x;
    cu[kk - 1] = c; su[kk - 1] = s;
}

__global__ void k_irl_sweeps(SweepArgs a, int use_smem)
{
    extern __shared__ double dsm[];
    const int dim = a.dim, k = a.k, dp1 = dim + 1;
    double *cu = use_smem ? dsm : a.w, *su = cu + dp1, *cv = cu + 2 * dp1, *sv = cu + 3 * dp1;
    double *D = use_smem ? dsm + 4 * dp1 : a.balpha;
    double *E = use_smem ? dsm + 5 * dp1 : a.bbeta;
    if (use_smem) {
        for (int i = threadIdx.x; i < dim; i += blockDim.x) { D[i] = a.balpha[i]; E[i] = a.bbeta[i]; }
    }
    // shifts (dlansvd_irl.F:304-344)
    if (threadIdx.x == 0) {
        for (int i = 0; i < dim - k; i++) a.shifts[i] = 0.0;
        int nshft = 0;
        if (a.small_side) {
            const double ref = a.a1[dim - a.neig - 1];
            for (int i = 1; i <= k; i++) {
                const double relgap = a.a1[i - 1] - a.bnd[i - 1] - ref;
                a.shifts[nshft++] = (relgap > a.min_relgap * ref) ? a.a1[i - 1] : a.a1[0];
            }
        } else {
            for (int i = dim; i >= k + 1; i--) {
                const double relgap = a.a1[k - 1] - (a.a1[i - 1] + a.bnd[i - 1]);
                a.shifts[nshft++] = (relgap > a.min_relgap * a.a1[k - 1]) ? a.a1[i - 1] : 0.0;
            }
        }
    }
    // P = I, Q = I
    for (size_t t = threadIdx.x; t < (size_t)dp1 * dp1; t += blockDim.x) a.P[t] = (t % (dp1 + 1) == 0) ? 1.0 : 0.0;
    for (size_t t = threadIdx.x; t < (size_t)dim * dim; t += blockDim.x) a.Q[t] = (t % (dim + 1) == 0) ? 1.0 : 0.0;
    __syncthreads();
    for (int i = dim; i >= k + 1; i--) {
        const double shift = a.shifts[dim - i];
        if (i <= 1) continue;  // dbsvdstep returns for k <= 1
        if (threadIdx.x == 0) bsvdstep_chain(i, shift, D, E, cu, su, cv, sv);
        __syncthreads();
        // the U rotations act on columns (t, t+1) of P, t = 0..i-1; the V
        // rotations on columns (t, t+1) of Q, t = 0..i-2; one row per thread
        for (int row = threadIdx.x; row < dp1; row += blockDim.x) {
            double *Pr = a.P + row;
            double xc = Pr[0];
            for (int t = 0; t < i; t++) {
                const double c = cu[t], s = su[t];
                const double yc = Pr[(size_t)(t + 1) * dp1];
                Pr[(size_t)t * dp1] = c * xc + s * yc;
                xc = c * yc - s * xc;
            }
            Pr[(size_t)i * dp1] = xc;
        }
        for (int row = threadIdx.x; row < dim; row += blockDim.x) {
            double *Qr = a.Q + row;
            double xc = Qr[0];
            for (int t = 0; t < i - 1; t++) {
                const double c = cv[t], s = sv[t];
                const double yc = Qr[(size_t)(t + 1) * dim];
                Qr[(size_t)t * dim] = c * xc + s * yc;
                xc = c * yc - s * xc;
            }
            Qr[(size_t)(i - 1) * dim] = xc;
        }
        __syncthreads();
    }
    if (use_smem) {
        for (int i = threadIdx.x; i < dim; i += blockDim.x) { a.balpha[i] = D[i]; a.bbeta[i] = E[i]; }
    }
    if (threadIdx.x == 0) a.ctl->rnorm = E[k - 1];
}

// -------------------------------------------------------------- Ritz prep
__global__ void k_ritz_prep(RitzArgs a, int use_smem)
{
    __shared__ QrShared q;
    extern __shared__ double dsm[];
    const int dim = a.dim;
    double *D = use_smem ? dsm : a.D;
    double *E = use_smem ? dsm + (dim + 1) : a.E;
    double *w = use_smem ? dsm + 2 * (dim + 1) : a.w;
    for (int i = threadIdx.x; i < dim; i += blockDim.x) { D[i] = a.balpha[i]; E[i] = a.bbeta[i]; }
    for (size_t t = threadIdx.x; t < (size_t)dim * dim; t += blockDim.x) {
        const double v = (t % (dim + 1) == 0) ? 1.0 : 0.0;
        a.P[t] = v;
        a.Qt[t] = v;
    }
    __syncthreads();
    const int mn = a.m < a.n ? a.m : a.n;
    if (threadIdx.x == 0) {
        double c1 = 0, c2 = 0;
        bdqr_dev(dim == mn, dim, D, E, &c1, &c2, a.Mt, dim + 1);
    }
    __syncthreads();
    bdsqr_cta(dim, D, E, dim, a.Qt, dim, dim, a.P, dim, w, q);
}

// ------------------------------------------------- lane-parallel analysis
// (the same outputs as k_analyse; see pgb_bidiag.cuh for the methods)

// bidiagonal size up to which the lane-parallel kernels are used
constexpr int PAR_DIM_MAX = 2048;

// dbdqr of B into a1 (d) / b1 (e), c1 -> bnd[dim-1], c2 -> bnd[dim]
__global__ void k_ana_qr(AnaArgs a)
{
    const int dim = a.dim;
    for (int i = threadIdx.x; i < dim; i += blockDim.x) { a.a1[i] = a.balpha[i]; a.b1[i] = a.bbeta[i]; }
    for (int i = threadIdx.x; i <= dim; i += blockDim.x) a.bnd[i] = 0.0;
    __syncthreads();
    const int mn = a.m < a.n ? a.m : a.n;
    if (threadIdx.x == 0) bdqr_dev(dim == mn, dim, a.a1, a.b1, &a.bnd[dim - 1], &a.bnd[dim], nullptr, 0);
}

// sigma_t of the upper bidiagonal (d, e), one warp per t; sig[t-1]
__global__ void __launch_bounds__(256) k_bisect(const double *d, const double *e, int n, double *sig)
{
    extern __shared__ double b2[];
    const int N = 2 * n;
    for (int j = threadIdx.x; j < N - 1; j += blockDim.x) {
        const double b = tgk_b(d, e, j);
        b2[j] = b * b;
    }
    __shared__ double gs, ps;
    if (threadIdx.x == 0) tgk_bounds(d, e, n, gs, ps);
    __syncthreads();
    const int t = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5) + 1;
    if (t > n) return;
    const double s = warp_sigma(n, b2, t, gs, ps);
    if ((threadIdx.x & 31) == 0) sig[t - 1] = s;
}

// bounds from the last components of the left vectors: one thread per
// singular value, one warp per CTA (each twisted factorisation divides at
// every step, and the FP64 pipe is the SM's); into w[dim + 1 + i]
__global__ void k_ana_twisted(AnaArgs a)
{
    const int dim = a.dim, N = 2 * dim;
    const double *sig = a.w;
    __shared__ double gs, ps;
    if (threadIdx.x == 0) tgk_bounds(a.a1, a.b1, dim, gs, ps);
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= dim) return;
    double *Dp = a.wz + (size_t)i * 2 * N, *Dm = Dp + N;
    const double zn = tgk_twisted(a.a1, a.b1, dim, sig[i], ps, Dp, Dm, nullptr);
    a.w[dim + 1 + i] = a.bnd[dim - 1] * (sqrt(2.0) * zn);
}

// the same bookkeeping as k_analyse (anorm, refinebounds, convergence
// count) on the bounds of k_ana_twisted
__global__ void k_ana_finish(AnaArgs a)
{
    const int dim = a.dim;
    const double *sig = a.w;
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    double bi = 0.0;
    if (threadIdx.x < dim) {
        const int i = threadIdx.x;
        bi = a.w[dim + 1 + i];
        if (!(bi == bi) || !(sig[i] == sig[i])) bad = 1;
    }
    __syncthreads();
    if (bad) {
        if (threadIdx.x == 0) *a.nconv_out = -1;
        return;
    }
    if (threadIdx.x < dim) {
        a.bnd[threadIdx.x] = bi;
        a.a1[threadIdx.x] = sig[threadIdx.x];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double *d = a.a1, *bnd = a.bnd;
        const int mn = a.m < a.n ? a.m : a.n;
        const double eps34 = pow(EPS, 0.75);
        const double epsn = (double)(a.m > a.n ? a.m : a.n) * EPS / 2.0;
        double anorm = *a.anorm_drv;
        if (dim > 5) anorm = d[0];
        else anorm = fmax(anorm, d[0]);
        *a.anorm_drv = anorm;
        const double rnorm = a.ctl->rnorm;
        for (int i = 0; i < dim; i++) bnd[i] = fabs(rnorm * bnd[i]);
        int nconv = 0;
        if (a.irl) {
            const int neig = a.neig;
            refinebounds_dev(mn, dim < neig ? dim : neig, d, bnd, epsn * anorm, eps34);
            int i = 1;
            const int lim = dim < neig ? dim : neig;
            while (i <= lim) {
                if (bnd[i - 1] <= a.tol * d[i - 1]) {
                    a.sigma_out[nconv] = d[i - 1];
                    a.bnd_out[nconv] = bnd[i - 1];
                    nconv++;
                    i++;
                } else {
                    i = a.kk + 1;
                }
            }
        } else {
            refinebounds_dev(mn, dim, d, bnd, epsn * anorm, eps34);
            const int lim = dim < a.kk ? dim : a.kk;
            for (int i = 0; i < lim; i++) a.bnd_out[i] = bnd[i];
            int i = 0;
            while (i < lim) {
                if (bnd[i] <= a.tol * d[i]) { a.sigma_out[nconv] = d[i]; nconv++; i++; }
                else i = a.kk;
            }
        }
        *a.nconv_out = nconv;
    }
}

// ----------------------------------------------- wavefront IRL sweeps
// The p sweeps of dlansvd_irl.F:346-363 (dbsvdstep, double/dbsvd.F:5-82)
// with their exact shifts known in advance.  Step i of a sweep touches
// D[i-1..i] and E[i-2..i] only, so sweep s+1 may run its step i while sweep
// s runs step i+3: one thread per sweep, one CTA barrier per step.  Every
// value is produced by the same operations in the same order as in the
// sequential sweeps, so B, P and Q are identical to theirs.  The rotations
// go to wz as [sweep][4][dim+1] (cu, su, cv, sv).
__global__ void k_irl_chain(SweepArgs a)
{
    extern __shared__ double dsm[];
    const int dim = a.dim, k = a.k, dp1 = dim + 1, nsw = dim - k;
    double *D = dsm, *E = dsm + dp1;
    for (int i = threadIdx.x; i < dim; i += blockDim.x) { D[i] = a.balpha[i]; E[i] = a.bbeta[i]; }
    if (threadIdx.x == 0) {
        for (int i = 0; i < dim - k; i++) a.shifts[i] = 0.0;
        int nshft = 0;
        for (int i = dim; i >= k + 1; i--) {
            const double relgap = a.a1[k - 1] - (a.a1[i - 1] + a.bnd[i - 1]);
            a.shifts[nshft++] = (relgap > a.min_relgap * a.a1[k - 1]) ? a.a1[i - 1] : 0.0;
        }
    }
    __syncthreads();
    const int s = threadIdx.x;  // this thread's sweep (blockDim >= nsw)
    const int kk = dim - s;     // dbsvdstep size of sweep s
    const bool active = s < nsw && kk > 1;
    const double sigma = active ? a.shifts[s] : 0.0;
    double *cu = a.wz + (size_t)s * 4 * dp1, *su = cu + dp1, *cv = cu + 2 * dp1, *sv = cu + 3 * dp1;
    double x = 0.0, y = 0.0, c, sn, r;
    const int gend = dim + 3 * (nsw - 1);
    for (int g = 0; g <= gend; g++) {
        const int i = g - 3 * s;
        if (active && i >= 0 && i <= kk) {
            if (i == 0) {
                x = D[0] * D[0] - sigma * sigma;
                y = E[0] * D[0];
            } else if (i < kk) {
                if (i > 1) lartg(x, y, c, sn, E[i - 2]);
                else lartg(x, y, c, sn, r);
                x = c * D[i - 1] + sn * E[i - 1];
                E[i - 1] = -sn * D[i - 1] + c * E[i - 1];
                D[i - 1] = x;
                y = sn * D[i];
                D[i] = c * D[i];
                cu[i - 1] = c; su[i - 1] = sn;
                lartg(x, y, c, sn, D[i - 1]);
                x = c * E[i - 1] + sn * D[i];
                D[i] = -sn * E[i - 1] + c * D[i];
                E[i - 1] = x;
                y = sn * E[i];
                E[i] = c * E[i];
                cv[i - 1] = c; sv[i - 1] = sn;
            } else {
                lartg(x, y, c, sn, E[kk - 2]);
                x = c * D[kk - 1] + sn * E[kk - 1];
                E[kk - 1] = -sn * D[kk - 1] + c * E[kk - 1];
                D[kk - 1] = x;
                cu[kk - 1] = c; su[kk - 1] = sn;
            }
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < dim; i += blockDim.x) { a.balpha[i] = D[i]; a.bbeta[i] = E[i]; }
    if (threadIdx.x == 0) a.ctl->rnorm = E[k - 1];
}

// P (dim+1)^2 and Q dim^2 from the recorded rotations: one warp per row,
// lane l applying sweep 32w+l two columns behind sweep 32w+l-1 (a sweep's
// rotation t reads column t+1 and finishes column t), waves of 32 sweeps.
constexpr int APPLY_WARPS = 8;
__global__ void __launch_bounds__(APPLY_WARPS * 32) k_irl_apply(SweepArgs a, int prow_blocks)
{
    extern __shared__ double rows[];
    const int dim = a.dim, k = a.k, dp1 = dim + 1, nsw = dim - k;
    const bool isP = blockIdx.x < prow_blocks;
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = (isP ? blockIdx.x : blockIdx.x - prow_blocks) * APPLY_WARPS + wid;
    const int nrows = isP ? dp1 : dim, ncols = nrows;
    if (row >= nrows) return;
    double *rw = rows + (size_t)wid * dp1;
    for (int t = lane; t < ncols; t += 32) rw[t] = (t == row) ? 1.0 : 0.0;
    __syncwarp();
    for (int w0 = 0; w0 < nsw; w0 += 32) {
        const int s = w0 + lane;
        const int kk = dim - s;
        // rotations of this sweep on this matrix: P gets kk (cu, su), Q kk-1 (cv, sv)
        const int nrot = (s < nsw && kk > 1) ? (isP ? kk : kk - 1) : -1;
        const double *cc = a.wz + (size_t)s * 4 * dp1 + (isP ? 0 : 2 * dp1), *ss = cc + dp1;
        const int kk0 = dim - w0;
        const int gend = (isP ? kk0 : kk0 - 1) + 2 * 31;
        double xc = 0.0;
        double cn = 0.0, sn = 0.0;
        if (nrot > 0) { cn = cc[0]; sn = ss[0]; }
        for (int g = 0; g <= gend; g++) {
            const int t = g - 2 * lane;
            if (nrot > 0 && t >= 0 && t <= nrot) {
                if (t < nrot) {
                    const double c = cn, s_ = sn;
                    if (t + 1 < nrot) { cn = cc[t + 1]; sn = ss[t + 1]; }
                    if (t == 0) xc = rw[0];
                    const double yc = rw[t + 1];
                    rw[t] = c * xc + s_ * yc;
                    xc = c * yc - s_ * xc;
                } else {
                    rw[nrot] = xc;
                }
            }
            __syncwarp();
        }
    }
    double *M = isP ? a.P : a.Q;
    for (int t = lane; t < ncols; t += 32) M[(size_t)t * nrows + row] = rw[t];
}

// ----------------------------------------------- lane-parallel Ritz prep
// dbdqr with Q' (dritzvec.F:112-114): thread 0 runs the rotation chain on
// R, then one thread per column of Mt replays it (the same operations as
// bdqr_dev's Q' update, column by column).
__global__ void k_ritz_qr(RitzArgs a)
{
    const int dim = a.dim, n1 = dim + 1;
    double *cs = a.w, *sn = a.w + n1;
    for (int i = threadIdx.x; i < dim; i += blockDim.x) { a.D[i] = a.balpha[i]; a.E[i] = a.bbeta[i]; }
    if (threadIdx.x == 0) *a.flag = 0;
    __syncthreads();
    const int mn = a.m < a.n ? a.m : a.n;
    __shared__ int nrot_s;
    if (threadIdx.x == 0) {
        double c, s, r;
        double *D = a.D, *E = a.E;
        int i;
        for (i = 1; i <= dim - 1; i++) {
            lartg(D[i - 1], E[i - 1], c, s, r);
            D[i - 1] = r;
            E[i - 1] = s * D[i];
            D[i] = c * D[i];
            cs[i - 1] = c; sn[i - 1] = s;
        }
        int nrot = dim - 1;
        if (dim != mn) {
            lartg(D[dim - 1], E[dim - 1], c, s, r);
            D[dim - 1] = r;
            E[dim - 1] = 0.0;
            cs[dim - 1] = c; sn[dim - 1] = s;
            nrot = dim;
        }
        nrot_s = nrot;
    }
    __syncthreads();
    const int nrot = nrot_s;
    // column j (0-based) of Q': created by rotation j-1 (for j >= 1), then
    // rotated by rotations j, j+1, ..., nrot-1 on rows (i, i+1)
    for (int j = threadIdx.x; j < n1; j += blockDim.x) {
        double *col = a.Mt + (size_t)j * n1;
        for (int i = 0; i < n1; i++) col[i] = 0.0;
        if (j == 0) col[0] = 1.0;
        else if (j - 1 < nrot) { col[j - 1] = sn[j - 1]; col[j] = cs[j - 1]; }
        else col[j] = 1.0;
        for (int i = (j == 0 ? 0 : j); i < nrot; i++) {
            col[i + 1] = -sn[i] * col[i];
            col[i] = cs[i] * col[i];
        }
    }
}

// The wanted singular vector pairs of R (indices mstart-1 .. mstart+k-2 of
// the decreasing order), one lane each: P(:, i) = y_i, Qt(i, :) = x_i'.
// Values closer than 1e-9 sigma_max to a neighbour are left to the QR path
// (flag), since single twisted vectors are only accurate to eps/gap.
__global__ void k_ritz_vecs(RitzArgs a)
{
    const int dim = a.dim, N = 2 * dim;
    const double *sig = a.w + 2 * (dim + 1);
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.k) return;
    const int i = a.mstart - 1 + q;
    const double smax = sig[0];
    const double gap = fmin(i > 0 ? sig[i - 1] - sig[i] : INFINITY, i + 1 < dim ? sig[i] - sig[i + 1] : INFINITY);
    double gs, ps;
    tgk_bounds(a.D, a.E, dim, gs, ps);
    if (!(gap > 1e-9 * smax) || !(sig[i] > 1e-9 * smax)) { *a.flag = 1; return; }
    double *Dp = a.wz + (size_t)q * 3 * N, *Dm = Dp + N, *z = Dm + N;
    tgk_twisted(a.D, a.E, dim, sig[i], ps, Dp, Dm, z);
    double nx = 0.0, ny = 0.0;
    for (int t = 0; t < dim; t++) { nx += z[2 * t] * z[2 * t]; ny += z[2 * t + 1] * z[2 * t + 1]; }
    if (!(nx > 0.0) || !(ny > 0.0) || !(nx < INFINITY) || !(ny < INFINITY)) { *a.flag = 1; return; }
    const double ix = 1.0 / sqrt(nx), iy = 1.0 / sqrt(ny);
    for (int t = 0; t < dim; t++) {
        a.Qt[(size_t)t * dim + i] = z[2 * t] * ix;
        a.P[(size_t)i * dim + t] = z[2 * t + 1] * iy;
    }
}

// ------------------------------------------------------------------ GEMM
// C(mr x nc) = op(A) op(B), 64 x 64 tiles, 256 threads x 4 x 4.  A and C
// hold T (the Lanczos vector type), B is FP64 (the small restart / Ritz
// factors); the product is formed in T.
// op(A)(i,l) = ta ? A[i*lda + l] : A[l*lda + i]; same for B with (l, j).
template <typename T>
__global__ void __launch_bounds__(256) k_gemm(int mr, int nc, int kk, const T *__restrict__ A, int lda, int ta,
                                             const double *__restrict__ B, int ldb, int tb, T *__restrict__ C,
                                             int ldc)
{
    __shared__ T As[16][64 + 1];
    __shared__ T Bs[16][64 + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int i0 = blockIdx.x * 64, j0 = blockIdx.y * 64;
    T acc[4][4] = {};
    for (int l0 = 0; l0 < kk; l0 += 16) {
        for (int t = threadIdx.x; t < 16 * 64; t += 256) {
            const int l = t / 64, i = t % 64;
            const int gi = i0 + i, gl = l0 + l;
            T v = 0;
            if (gi < mr && gl < kk) v = ta ? A[(size_t)gi * lda + gl] : A[(size_t)gl * lda + gi];
            As[l][i] = v;
            const int gj = j0 + i;
            T u = 0;
            if (gj < nc && gl < kk) u = (T)(tb ? B[(size_t)gl * ldb + gj] : B[(size_t)gj * ldb + gl]);
            Bs[l][i] = u;
        }
        __syncthreads();
#pragma unroll
        for (int l = 0; l < 16; l++) {
            T av[4], bv[4];
#pragma unroll
            for (int q = 0; q < 4; q++) { av[q] = As[l][tx + 16 * q]; bv[q] = Bs[l][ty + 16 * q]; }
#pragma unroll
            for (int p = 0; p < 4; p++)
#pragma unroll
                for (int q = 0; q < 4; q++) acc[p][q] = fma(av[p], bv[q], acc[p][q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 4; p++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int gi = i0 + tx + 16 * p, gj = j0 + ty + 16 * q;
            if (gi < mr && gj < nc) C[(size_t)gj * ldc + gi] = acc[p][q];
        }
}

template <typename T>
__global__ void k_copy_cols(const T *src, int lds, T *dst, int ldd, int rows, int cols)
{
    const size_t total = (size_t)rows * cols;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t c = t / rows, r = t % rows;
        dst[c * ldd + r] = src[c * lds + r];
    }
}

// ------------------------------------------------------------ host wrappers
// dynamic shared memory for the single-CTA kernels, when it fits
static int smem_for(const void *fn, size_t bytes)
{
    static thread_local int max_optin = -1;
    if (max_optin < 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    if (bytes + 1024 > (size_t)max_optin) return 0;
    if (bytes > 48 * 1024) PGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return 1;
}
void launch_analyse_qr(const AnaArgs &a, cudaStream_t s)
{
    const size_t bytes = sizeof(double) * (7 * (size_t)(a.dim + 1) + 2);
    const int use = smem_for((const void *)k_analyse, bytes);
    PGB_PROF(PK_ANALYSE, s, k_analyse<<<1, 32, use ? bytes : 0, s>>>(a, use));
    PGB_LAUNCHED();
}
static bool bisect_fits(int dim)
{
    return dim <= PAR_DIM_MAX && smem_for((const void *)k_bisect, sizeof(double) * 2 * (size_t)dim) != 0;
}
static void launch_bisect(const double *d, const double *e, int n, double *sig, cudaStream_t s)
{
    // one warp per CTA, so that each singular value's Sturm sequences (an
    // FP64 division per step) have an SM's FP64 pipe to themselves
    const int wpb = 1;
    k_bisect<<<(n + wpb - 1) / wpb, 32 * wpb, sizeof(double) * 2 * (size_t)n, s>>>(d, e, n, sig);
    PGB_LAUNCHED();
}
void launch_analyse(const AnaArgs &a, cudaStream_t s)
{
    // the smallest triplets (which = 'S') keep the QR path: their twisted
    // vectors on the Golub-Kahan form are not reliable near sigma = 0
    if (a.small_side || !a.wz || a.dim > 1024 || !bisect_fits(a.dim)) {
        launch_analyse_qr(a, s);
        return;
    }
    PGB_PROF(PK_ANALYSE, s, {
        k_ana_qr<<<1, 32, 0, s>>>(a);
        PGB_LAUNCHED();
        launch_bisect(a.a1, a.b1, a.dim, a.w, s);
        k_ana_twisted<<<(a.dim + 31) / 32, 32, 0, s>>>(a);
        PGB_LAUNCHED();
        k_ana_finish<<<1, ((a.dim + 31) / 32) * 32, 0, s>>>(a);
        PGB_LAUNCHED();
    });
}
void launch_sweeps(const SweepArgs &a, cudaStream_t s)
{
    const int nsw = a.dim - a.k;
    const size_t chain_bytes = sizeof(double) * 2 * (size_t)(a.dim + 1);
    const size_t apply_bytes = sizeof(double) * APPLY_WARPS * (size_t)(a.dim + 1);
    if (a.small_side || !a.wz || nsw < 1 || nsw > 1024 || a.dim > PAR_DIM_MAX ||
        !smem_for((const void *)k_irl_chain, chain_bytes) || !smem_for((const void *)k_irl_apply, apply_bytes)) {
        const size_t bytes = sizeof(double) * 6 * (size_t)(a.dim + 1);
        const int use = smem_for((const void *)k_irl_sweeps, bytes);
        PGB_PROF(PK_SWEEPS, s, k_irl_sweeps<<<1, 256, use ? bytes : 0, s>>>(a, use));
        PGB_LAUNCHED();
        return;
    }
    const int pblocks = (a.dim + 1 + APPLY_WARPS - 1) / APPLY_WARPS;
    const int qblocks = (a.dim + APPLY_WARPS - 1) / APPLY_WARPS;
    PGB_PROF(PK_SWEEPS, s, {
        k_irl_chain<<<1, ((nsw + 31) / 32) * 32, chain_bytes, s>>>(a);
        PGB_LAUNCHED();
        k_irl_apply<<<pblocks + qblocks, APPLY_WARPS * 32, apply_bytes, s>>>(a, pblocks);
        PGB_LAUNCHED();
    });
}
void launch_ritz_prep_qr(const RitzArgs &a, cudaStream_t s)
{
    const size_t bytes = sizeof(double) * 6 * (size_t)(a.dim + 1);
    const int use = smem_for((const void *)k_ritz_prep, bytes);
    PGB_PROF(PK_RITZ, s, k_ritz_prep<<<1, 256, use ? bytes : 0, s>>>(a, use));
    PGB_LAUNCHED();
}
bool launch_ritz_prep(const RitzArgs &a, cudaStream_t s)
{
    if (a.mstart != 1 || !a.wz || !a.flag || a.k < 1 || !bisect_fits(a.dim)) return false;
    PGB_PROF(PK_RITZ, s, {
        k_ritz_qr<<<1, 256, 0, s>>>(a);
        PGB_LAUNCHED();
        launch_bisect(a.D, a.E, a.dim, a.w + 2 * (a.dim + 1), s);
        k_ritz_vecs<<<(a.k + 31) / 32, 32, 0, s>>>(a);
        PGB_LAUNCHED();
    });
    return true;
}
// C = op(A) op(B) (out of place)
template <typename T>
void gemm(int mr, int nc, int kk, const T *A, int lda, bool ta, const double *B, int ldb, bool tb, T *C, int ldc,
          cudaStream_t s)
{
    if (mr <= 0 || nc <= 0) return;
    if (sizeof(T) == sizeof(double) && !ta &&
        gemm_f64_tc(mr, nc, kk, (const double *)A, lda, B, ldb, tb, (double *)C, ldc, s))
        return;
    dim3 grid((mr + 63) / 64, (nc + 63) / 64);
    PGB_PROF(PK_GEMM, s, k_gemm<T><<<grid, 256, 0, s>>>(mr, nc, kk, A, lda, ta ? 1 : 0, B, ldb, tb ? 1 : 0, C, ldc));
    PGB_LAUNCHED();
}
template <typename T>
void copy_cols(const T *src, int lds, T *dst, int ldd, int rows, int cols, cudaStream_t s)
{
    if (rows <= 0 || cols <= 0) return;
    k_copy_cols<T><<<device_info().nb, 256, 0, s>>>(src, lds, dst, ldd, rows, cols);
    PGB_LAUNCHED();
}
template void gemm<double>(int, int, int, const double *, int, bool, const double *, int, bool, double *, int,
                           cudaStream_t);
template void gemm<float>(int, int, int, const float *, int, bool, const double *, int, bool, float *, int,
                          cudaStream_t);
template void copy_cols<double>(const double *, int, double *, int, int, int, cudaStream_t);
template void copy_cols<float>(const float *, int, float *, int, int, int, cudaStream_t);

}  // namespace pgb
