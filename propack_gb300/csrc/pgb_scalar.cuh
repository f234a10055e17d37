// pgb_scalar.cuh -- scalar FP64 building blocks of the small bidiagonal
// computations (plane rotations, 2x2 singular values, dbdqr, drefinebounds),
// shared by the single-problem kernels and the batched solver.
#pragma once
#include "pgb.cuh"

namespace pgb {

// --------------------------------------------------------- scalar helpers
// plane rotation [c s; -s c][f; g] = [r; 0]; cosine made positive when
// |f| > |g| (the dlartg convention)
__device__ __forceinline__ void lartg(double f, double g, double &c, double &s, double &r)
{
    if (g == 0.0) { c = 1.0; s = 0.0; r = f; return; }
    if (f == 0.0) { c = 0.0; s = 1.0; r = g; return; }
    // one reciprocal hypotenuse (overflow-safe) instead of hypot + 2 divides
    const double rh = rhypot(f, g);
    double cc = f * rh, ss = g * rh;
    double rr = fma(f, cc, g * ss);
    if (fabs(f) > fabs(g) && cc < 0.0) { cc = -cc; ss = -ss; rr = -rr; }
    c = cc; s = ss; r = rr;
}

// singular values of [f g; 0 h]: smax + smin = hypot(|f|+|h|, g),
// smax - smin = hypot(|f|-|h|, g), smin = |f h| / smax
__device__ __forceinline__ void sv2x2(double f, double g, double h, double &smin, double &smax)
{
    const double fa = fabs(f), ga = fabs(g), ha = fabs(h);
    const double mx = 0.5 * (hypot(fa + ha, ga) + hypot(fa - ha, ga));
    smax = mx;
    smin = mx > 0.0 ? (fa / mx) * ha : 0.0;
}

// dbdqr (double/dbsvd.F:87-157); thread 0.  With Qt != nullptr the
// (n+1) x (n+1) matrix Q' is formed (ldq).
__device__ inline void bdqr_dev(int ignorelast, int n, double *D, double *E, double *c1, double *c2, double *Qt, int ldq)
{
    double cs, sn, r;
    if (n < 1) return;
#define QT(a, b) Qt[(size_t)((b)-1) * ldq + ((a)-1)]
    if (Qt) {
        for (int j = 1; j <= n + 1; j++) {
            for (int i = 1; i <= n + 1; i++) QT(i, j) = 0.0;
            QT(j, j) = 1.0;
        }
    }
    int i;
    for (i = 1; i <= n - 1; i++) {
        lartg(D[i - 1], E[i - 1], cs, sn, r);
        D[i - 1] = r;
        E[i - 1] = sn * D[i];
        D[i] = cs * D[i];
        if (Qt) {
            for (int j = 1; j <= i; j++) {
                QT(i + 1, j) = -sn * QT(i, j);
                QT(i, j) = cs * QT(i, j);
            }
            QT(i, i + 1) = sn;
            QT(i + 1, i + 1) = cs;
        }
    }
    if (!ignorelast) {
        lartg(D[n - 1], E[n - 1], cs, sn, r);
        D[n - 1] = r;
        E[n - 1] = 0.0;
        *c1 = sn;
        *c2 = cs;
        if (Qt) {
            for (int j = 1; j <= i; j++) {
                QT(i + 1, j) = -sn * QT(i, j);
                QT(i, j) = cs * QT(i, j);
            }
            QT(i, i + 1) = sn;
            QT(i + 1, i + 1) = cs;
        }
    }
#undef QT
}

// drefinebounds (double/dbsvd.F:162-231); thread 0
__device__ inline void refinebounds_dev(int n, int k, const double *theta, double *bound, double tol, double eps34)
{
    if (k <= 1) return;
    for (int i = 1; i <= k; i++) {
        for (int l = -1; l <= 1; l += 2) {
            if ((l == 1 && i < k) || (l == -1 && i > 1)) {
                if (fabs(theta[i - 1] - theta[i + l - 1]) < eps34 * theta[i - 1]) {
                    if (bound[i - 1] > tol && bound[i + l - 1] > tol) {
                        bound[i + l - 1] = hypot(bound[i - 1], bound[i + l - 1]);
                        bound[i - 1] = 0.0;
                    }
                }
            }
        }
    }
    for (int i = 1; i <= k; i++) {
        if (i < k || k == n) {
            double gap;
            if (i == 1) {
                gap = fabs(theta[i - 1] - theta[i]) - fmax(bound[i - 1], bound[i]);
            } else if (i == n) {
                gap = fabs(theta[i - 2] - theta[i - 1]) - fmax(bound[i - 2], bound[i - 1]);
            } else {
                gap = fabs(theta[i - 1] - theta[i]) - fmax(bound[i - 1], bound[i]);
                const double g2 = fabs(theta[i - 2] - theta[i - 1]) - fmax(bound[i - 2], bound[i - 1]);
                if (g2 < gap) gap = g2;
            }
            if (gap > bound[i - 1]) bound[i - 1] = bound[i - 1] * (bound[i - 1] / gap);
        }
    }
}

}  // namespace pgb
