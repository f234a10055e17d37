// pgb_bidiag.cuh -- lane-parallel numerics for the small upper bidiagonal R
// (diagonal d[0..n-1], superdiagonal e[0..n-2]) that the IRL analysis and
// the Ritz-vector step need.
//
// Why not the QR iteration the reference uses (Lapack_Util/dbdsqr.f):
// its rotation chain is one dependent sequence of FP64 operations, and on
// this GPU an FP64 instruction issued for one thread occupies the FP64 pipe
// as long as one issued for a full warp (2 FP64 lanes per clock per SM), so
// a thread-serial chain runs ~30x slower than on a CPU core.  The methods
// here keep every lane of a warp busy instead:
//
//   singular values   warp multisection on the Golub-Kahan tridiagonal
//                     TGK = tridiag(b; 0; b), b = (d1, e1, d2, e2, ..., dn),
//                     whose eigenvalues are +-sigma_i.  The Sturm count of
//                     TGK - x I (LDL' pivots of a zero-diagonal matrix)
//                     locates sigma_i to high relative accuracy (Demmel &
//                     Kahan 1990, section 7); 32 lanes evaluate 31 points per
//                     round, 5 bits per round.
//   vectors           the twisted factorization of TGK - sigma I (Parlett &
//                     Dhillon 1997; the "getvec" step of MRRR): forward and
//                     backward pivot sequences, twist index r = argmin
//                     |gamma_r|, then z from both ends.  z = (x1, y1, x2,
//                     y2, ...)/sqrt(2) with R x = sigma y; one lane per value.
//
// All functions are plain arithmetic on caller-provided storage, so the same
// code serves any dimension.
#pragma once
#include "pgb.cuh"

namespace pgb {

// b[j], j = 0..2n-2: off-diagonal of TGK; b2 = b*b
__device__ __forceinline__ double tgk_b(const double *d, const double *e, int j)
{
    return (j & 1) ? e[j >> 1] : d[j >> 1];
}

// number of negative pivots of TGK - lam I (size N = 2n)
__device__ __forceinline__ int tgk_negcount(int N, const double *b2, double lam, double pivmin)
{
    double D = -lam;
    if (fabs(D) < pivmin) D = -pivmin;
    int cnt = D < 0.0;
    for (int j = 1; j < N; j++) {
        D = -lam - b2[j - 1] / D;
        if (fabs(D) < pivmin) D = -pivmin;
        cnt += D < 0.0;
    }
    return cnt;
}

// sigma_t (t = 1: largest) of R by warp multisection; all lanes return it.
// hi0: an upper bound of sigma_max (Gershgorin of TGK).
__device__ inline double warp_sigma(int n, const double *b2, int t, double hi0, double pivmin)
{
    const int lane = threadIdx.x & 31, N = 2 * n;
    double lo = 0.0, hi = hi0;
    for (int round = 0; round < 64; round++) {
        if (hi - lo <= 2.0 * EPS * hi) break;
        const double p = lo + (hi - lo) * ((double)(lane + 1) / 33.0);
        // #(sigma > p) = 2n - negcount(p) for p > 0
        const int above = N - tgk_negcount(N, b2, p, pivmin);
        const unsigned bal = __ballot_sync(0xffffffffu, above >= t);
        const int q = __popc(bal);  // counts are monotone: lanes 0..q-1 satisfy
        const double plo = __shfl_sync(0xffffffffu, p, q > 0 ? q - 1 : 0);
        const double phi = __shfl_sync(0xffffffffu, p, q < 32 ? q : 31);
        const double nlo = q > 0 ? plo : lo, nhi = q < 32 ? phi : hi;
        if (nlo == lo && nhi == hi) break;  // no representable progress
        lo = nlo;
        hi = nhi;
    }
    return 0.5 * (lo + hi);
}

// Twisted factorization of TGK - lam I.  Dp/Dm: N scratch each.  When z is
// given it receives the unit eigenvector; returns |z_N| of the unit vector.
__device__ inline double tgk_twisted(const double *d, const double *e, int n, double lam, double pivmin, double *Dp,
                              double *Dm, double *z)
{
    const int N = 2 * n;
    double D = -lam;
    if (fabs(D) < pivmin) D = -pivmin;
    Dp[0] = D;
    for (int j = 1; j < N; j++) {
        const double bj = tgk_b(d, e, j - 1);
        D = -lam - (bj * bj) / D;
        if (fabs(D) < pivmin) D = -pivmin;
        Dp[j] = D;
    }
    D = -lam;
    if (fabs(D) < pivmin) D = -pivmin;
    Dm[N - 1] = D;
    for (int j = N - 2; j >= 0; j--) {
        const double bj = tgk_b(d, e, j);
        D = -lam - (bj * bj) / D;
        if (fabs(D) < pivmin) D = -pivmin;
        Dm[j] = D;
    }
    // gamma_j = Dp_j + Dm_j - (T - lam I)_jj = Dp_j + Dm_j + lam
    int r = 0;
    double gmin = fabs(Dp[0] + Dm[0] + lam);
    for (int j = 1; j < N; j++) {
        const double g = fabs(Dp[j] + Dm[j] + lam);
        if (g < gmin) { gmin = g; r = j; }
    }
    // z_r = 1; z_j = -(b_j / Dp_j) z_{j+1} above r, -(b_{j-1} / Dm_j) z_{j-1} below
    double nrm2 = 1.0, zN = (r == N - 1) ? 1.0 : 0.0;
    if (z) z[r] = 1.0;
    double zz = 1.0;
    for (int j = r - 1; j >= 0; j--) {
        zz = -(tgk_b(d, e, j) / Dp[j]) * zz;
        if (z) z[j] = zz;
        nrm2 += zz * zz;
    }
    zz = 1.0;
    for (int j = r + 1; j < N; j++) {
        zz = -(tgk_b(d, e, j - 1) / Dm[j]) * zz;
        if (z) z[j] = zz;
        nrm2 += zz * zz;
        if (j == N - 1) zN = zz;
    }
    const double inv = 1.0 / sqrt(nrm2);
    if (z)
        for (int j = 0; j < N; j++) z[j] *= inv;
    return fabs(zN) * inv;
}

// Gershgorin bound of TGK and the pivot guard (LAPACK dstebz's pivmin)
__device__ __forceinline__ void tgk_bounds(const double *d, const double *e, int n, double &gersh, double &pivmin)
{
    double g = 0.0, bmax2 = 0.0;
    const int N = 2 * n;
    for (int j = 0; j < N; j++) {
        const double left = j > 0 ? fabs(tgk_b(d, e, j - 1)) : 0.0;
        const double right = j < N - 1 ? fabs(tgk_b(d, e, j)) : 0.0;
        g = fmax(g, left + right);
        if (j < N - 1) bmax2 = fmax(bmax2, right * right);
    }
    gersh = g * (1.0 + 4.0 * EPS) + SFMIN;
    pivmin = SFMIN * fmax(1.0, bmax2);
}

}  // namespace pgb
