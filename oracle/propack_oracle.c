/*
 * propack_oracle.c -- CPU restatement of PROPACK 2.1's double-precision
 * Lanczos bidiagonalisation with partial reorthogonalisation.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle of the tests of the
 * GPU library in propack_gb300/, and the timed multi-core CPU baseline in
 * bench.py.  Nothing in the product links, loads or calls it.
 *
 * Every routine follows the reference's Fortran line by line in control flow
 * (file:line citations are into the PROPACK 2.1 source tree):
 *   lanbpro        double/dlanbpro.F:1-549   (dset_mu :555, dcompute_int :581,
 *                                             dupdate_mu :628, dupdate_nu :684)
 *   reorth/cgs/mgs double/dreorth.F:5-210, double/dmgs.risc.F:11-84
 *   getu0          double/dgetu0.F:11-89     (dlarnv/dlaruv: Lapack_Util)
 *   safescal       double/dsafescal.F:4-55
 *   bsvdstep/bdqr/refinebounds  double/dbsvd.F:5-231
 *   ritzvec        double/dritzvec.F:1-199
 *   ovwr GEMMs     double/dgemm_ovwr.F:5-87
 *   lansvd         double/dlansvd.F:1-291
 *   lansvd_irl     double/dlansvd_irl.F:1-419
 * The LAPACK pieces the reference calls (dbdsqr for the Ritz values and the
 * last row of the left vectors, dbdsdc for the full SVD of the bidiagonal)
 * are served by bdsqr_upper() below: an implicit zero-shift / shifted QR
 * iteration after Demmel & Kahan (SIAM J. Sci. Stat. Comput. 11, 1990), the
 * method dbdsqr implements.  Singular values agree with LAPACK to rounding;
 * singular vectors agree up to the sign of each (u_i, v_i) pair.
 *
 * Random numbers: dlarnv(idist=2) draws from the 48-bit multiplicative
 * congruential generator of LAPACK's dlaruv, x_{i+1} = a*x_i mod 2^48 with
 * a = 33952834046453, returning 2*x/2^48 - 1.  dgetu0 seeds it with
 * (1,3,5,7) in base-4096 digits on every call (dgetu0.F:47-50).
 *
 * Calling convention: gfortran's (all scalars by reference, hidden size_t
 * lengths for CHARACTER arguments appended last), so the same harness
 * drives this file and the GPU library.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef void (*aprod_t)(const char *transa, const int *m, const int *n,
                        const double *x, double *y, double *dparm, int *iparm,
                        size_t transa_len);

#define EPS_D (1.1102230246251565e-16) /* dlamch('e') = 2^-53 */
#define SFMIN_D (2.2250738585072014e-308) /* dlamch('s') */
#define KAPPA_LANBPRO (0.717)              /* dlanbpro.F:118 (double literal) */
#define KAPPA_GETU0 ((double)0.717f)       /* dgetu0.F:30 (REAL literal)      */
#define FUDGE_LANBPRO (1.01)               /* dlanbpro.F:117                  */
#define NTRY_REORTH 5                      /* dreorth.F:64                    */

/* ---------------------------------------------------------------- stats */
/* Counters of double/stat.h:6-15 (timers are never assigned there). */
typedef struct {
    long nopx, nreorth, ndot, nitref, nbsvd, nrestart, nlandim, nsing;
    long nelr; /* passes of the extended local reorthogonalisation (not in stat.h) */
} oracle_stat_t;
static oracle_stat_t st;

void oracle_clearstat(void) { memset(&st, 0, sizeof st); }
long oracle_nelr(void) { return st.nelr; }
void oracle_getstat(long *out8)
{
    out8[0] = st.nopx; out8[1] = st.nreorth; out8[2] = st.ndot;
    out8[3] = st.nitref; out8[4] = st.nbsvd; out8[5] = st.nrestart;
    out8[6] = st.nlandim; out8[7] = st.nsing;
}

static int omp_threads = 0; /* 0: OpenMP default */
void oracle_set_threads(int t) { omp_threads = t; }
static int nthr(void)
{
#ifdef _OPENMP
    return omp_threads > 0 ? omp_threads : omp_get_max_threads();
#else
    return 1;
#endif
}
#define PAR_MIN 8192 /* vectors shorter than this run serially */

/* ------------------------------------------------------ level-1 kernels */
/* OpenMP forms of double/dblasext.F (pdnrm2 :6, pdscal :38, pdaxpy :92,
 * pddot :121).  The 2-norm is a plain sum of squares. */
static double v_dot(int n, const double *x, const double *y)
{
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static) if (n >= PAR_MIN) num_threads(nthr())
    for (int i = 0; i < n; i++) s += x[i] * y[i];
    return s;
}
static double v_nrm2(int n, const double *x) { return sqrt(v_dot(n, x, x)); }
static void v_axpy(int n, double a, const double *x, double *y)
{
#pragma omp parallel for schedule(static) if (n >= PAR_MIN) num_threads(nthr())
    for (int i = 0; i < n; i++) y[i] += a * x[i];
}
static void v_scal(int n, double a, double *x)
{
#pragma omp parallel for schedule(static) if (n >= PAR_MIN) num_threads(nthr())
    for (int i = 0; i < n; i++) x[i] *= a;
}
static void v_zero(int n, double *x) { memset(x, 0, sizeof(double) * (size_t)n); }

/* dsafescal.F:4-55: x <- x/alpha without forming 1/alpha when that would
 * overflow. */
static void safescal(int n, double alpha, double *x)
{
    if (fabs(alpha) >= SFMIN_D) {
        v_scal(n, 1.0 / alpha, x);
    } else {
        for (int i = 0; i < n; i++) x[i] = x[i] / alpha;
    }
}

/* ------------------------------------------------------------- dlarnv */
#define LCG_A 33952834046453ULL
#define LCG_MASK ((1ULL << 48) - 1ULL)
static uint64_t lcg_seed(int s1, int s2, int s3, int s4)
{
    return ((uint64_t)s1 << 36) | ((uint64_t)s2 << 24) | ((uint64_t)s3 << 12) | (uint64_t)s4;
}
/* dlarnv(2, iseed, n, x): uniform(-1,1) from the dlaruv sequence. */
static uint64_t larnv_pm1(uint64_t seed, int n, double *x)
{
    const double r48 = 1.0 / 281474976710656.0; /* 2^-48 */
    for (int i = 0; i < n; i++) {
        seed = (seed * LCG_A) & LCG_MASK;
        x[i] = 2.0 * ((double)seed * r48) - 1.0;
    }
    return seed;
}

/* ------------------------------------------------------------ dlartg */
/* Plane rotation [c s; -s c][f; g] = [r; 0], LAPACK sign convention:
 * when |f| > |g| the cosine is made positive. */
static void lartg(double f, double g, double *c, double *s, double *r)
{
    if (g == 0.0) { *c = 1.0; *s = 0.0; *r = f; return; }
    if (f == 0.0) { *c = 0.0; *s = 1.0; *r = g; return; }
    double rr = hypot(f, g);
    double cc = f / rr, ss = g / rr;
    if (fabs(f) > fabs(g) && cc < 0.0) { cc = -cc; ss = -ss; rr = -rr; }
    *c = cc; *s = ss; *r = rr;
}

/* -------------------------------------------------------------- reorth */
/* dcgs (dreorth.F:106-210): block classical Gram-Schmidt over the column
 * ranges [s_i, e_i] of index[] (1-based, terminated by a value > k or <= 0). */
static void cgs(int n, int k, const double *V, int ldv, double *vnew, const int *index, double *work)
{
    int i = 0;
    while (index[i] <= k && index[i] > 0) {
        int p = index[i], q = index[i + 1], l = q - p + 1;
        st.ndot += l;
        if (l > 0) {
            const double *Vp = V + (size_t)(p - 1) * ldv;
            for (int c = 0; c < l; c++) work[c] = v_dot(n, Vp + (size_t)c * ldv, vnew);
#pragma omp parallel for schedule(static) if (n >= PAR_MIN) num_threads(nthr())
            for (int r = 0; r < n; r++) {
                double acc = 0.0;
                for (int c = 0; c < l; c++) acc += Vp[(size_t)c * ldv + r] * work[c];
                vnew[r] -= acc;
            }
        }
        i += 2;
    }
}

/* dmgs / pdmgs (dmgs.risc.F:11-84, :87-): modified Gram-Schmidt over the
 * same ranges.  As in the reference, the update with column i-1 and the
 * projection onto column i share one pass over vnew (vn0 = vnew - coef V_i-1;
 * newcoef += vn0 V_i), which is the separate dot + axpy of MGS in the same
 * order of operations.  Unlike dcgs, an empty range (p > q) ends the sweep. */
static void mgs(int n, int k, const double *V, int ldv, double *vnew, const int *index)
{
    if (k <= 0 || n <= 0) return;
    int ib = 0, p = index[0], q = index[1];
    while (p <= k && p > 0 && p <= q) {
        st.ndot += q - p + 1;
        double coef = v_dot(n, V + (size_t)(p - 1) * ldv, vnew);
        for (int i = p + 1; i <= q; i++) {
            const double *vprev = V + (size_t)(i - 2) * ldv, *vi = V + (size_t)(i - 1) * ldv;
            double newcoef = 0.0;
#pragma omp parallel for reduction(+ : newcoef) schedule(static) if (n >= PAR_MIN) num_threads(nthr())
            for (int j = 0; j < n; j++) {
                const double vn0 = vnew[j] + (-coef) * vprev[j];
                newcoef += vi[j] * vn0;
                vnew[j] = vn0;
            }
            coef = newcoef;
        }
        v_axpy(n, -coef, V + (size_t)(q - 1) * ldv, vnew);
        ib += 2;
        p = index[ib];
        q = index[ib + 1];
    }
}

/* dreorth (dreorth.F:5-101): iterate until ||v'|| > alpha*||v||, at most
 * NTRY times; a vector that keeps collapsing is set to zero. */
static void reorth(int n, int k, const double *V, int ldv, double *vnew, double *normvnew,
                   const int *index, double alpha, double *work, int iflag)
{
    if (k <= 0 || n <= 0) return;
    for (int itry = 0; itry < NTRY_REORTH; itry++) {
        double normvnew_0 = *normvnew;
        if (iflag == 1) cgs(n, k, V, ldv, vnew, index, work);
        else mgs(n, k, V, ldv, vnew, index);
        st.ndot += k;
        *normvnew = v_nrm2(n, vnew);
        if (*normvnew > alpha * normvnew_0) { st.nreorth++; return; }
    }
    *normvnew = 0.0;
    v_zero(n, vnew);
    st.nreorth++;
}

/* --------------------------------------------------------------- getu0 */
/* dgetu0.F:11-89: a pseudo-random vector in span(op(A)) orthogonal to
 * U(:,1:j); also returns ||op(A) x|| / ||x||. work >= max(m,n) + j. */
static void getu0(char transa, int m, int n, int j, int ntry, double *u0, double *u0norm,
                  const double *U, int ldu, aprod_t aprod, double *dparm, int *iparm, int *ierr,
                  int icgs, double *anormest, double *work)
{
    uint64_t seed = lcg_seed(1, 3, 5, 7);
    int rsize, usize;
    char ta[2] = {transa, 0};
    if (transa == 'n' || transa == 'N') { rsize = n; usize = m; }
    else { rsize = m; usize = n; }
    *ierr = 0;
    double *x = work, *w2 = work + rsize;
    for (int itry = 0; itry < ntry; itry++) {
        seed = larnv_pm1(seed, rsize, x);
        double nrm = v_nrm2(rsize, x);
        aprod(ta, &m, &n, x, u0, dparm, iparm, 1);
        st.nopx++;
        *u0norm = v_nrm2(usize, u0);
        *anormest = *u0norm / nrm;
        if (j >= 1) {
            int index[3] = {1, j, j + 1};
            reorth(usize, j, U, ldu, u0, u0norm, index, KAPPA_GETU0, w2, icgs);
        }
        if (*u0norm > 0) return;
    }
    *ierr = -1;
}

/* ------------------------------------------------ omega recurrences */
/* dset_mu (dlanbpro.F:555-577) */
static void set_mu(int k, double *mu, const int *index, double val)
{
    int i = 0;
    while (index[i] <= k && index[i] > 0) {
        int p = index[i], q = index[i + 1];
        for (int j = p; j <= q; j++) mu[j - 1] = val;
        i += 2;
    }
}

/* dcompute_int (dlanbpro.F:581-624).  Fortran DO-variable exit values
 * are reproduced: after `do s=k,lo,-1` runs out, s = lo-1; after
 * `do i=s+1,j` runs out, i = j+1. */
static void compute_int(const double *mu, int j, double delta, double eta, int *index)
{
    if (delta < eta) return; /* reference warns and leaves index untouched */
    int ip = 0, i = 0, k, s;
    index[0] = 0;
    while (i < j) {
        for (k = i + 1; k <= j; k++)
            if (fabs(mu[k - 1]) > delta) break;
        if (k > j) break;
        int lo = i > 1 ? i : 1;
        for (s = k; s >= lo; s--)
            if (fabs(mu[s - 1]) < eta) break;
        index[ip++] = s + 1;
        for (i = s + 1; i <= j; i++)
            if (fabs(mu[i - 1]) < eta) break;
        index[ip++] = i - 1;
    }
    index[ip] = j + 1;
}

/* dupdate_mu (dlanbpro.F:628-679); alpha, beta are B(:,1), B(:,2). */
static void update_mu(double *mumax, double *mu, const double *nu, int j, const double *alpha,
                      const double *beta, double anorm, double eps1)
{
    double d;
    if (j == 1) {
        d = eps1 * (hypot(alpha[j - 1], beta[j - 1]) + alpha[0]) + eps1 * anorm;
        mu[0] = eps1 / beta[0];
        *mumax = fabs(mu[0]);
    } else {
        mu[0] = alpha[0] * nu[0] - alpha[j - 1] * mu[0];
        d = eps1 * (hypot(alpha[j - 1], beta[j - 1]) + alpha[0]) + eps1 * anorm;
        mu[0] = (mu[0] + copysign(d, mu[0])) / beta[j - 1];
        *mumax = fabs(mu[0]);
        for (int k = 2; k <= j - 1; k++) {
            mu[k - 1] = alpha[k - 1] * nu[k - 1] + beta[k - 2] * nu[k - 2] - alpha[j - 1] * mu[k - 1];
            d = eps1 * (hypot(alpha[j - 1], beta[j - 1]) + hypot(alpha[k - 1], beta[k - 2])) + eps1 * anorm;
            mu[k - 1] = (mu[k - 1] + copysign(d, mu[k - 1])) / beta[j - 1];
            if (fabs(mu[k - 1]) > *mumax) *mumax = fabs(mu[k - 1]);
        }
        mu[j - 1] = beta[j - 2] * nu[j - 2];
        d = eps1 * (hypot(alpha[j - 1], beta[j - 1]) + hypot(alpha[j - 1], beta[j - 2])) + eps1 * anorm;
        mu[j - 1] = (mu[j - 1] + copysign(d, mu[j - 1])) / beta[j - 1];
        if (fabs(mu[j - 1]) > *mumax) *mumax = fabs(mu[j - 1]);
    }
    mu[j] = 1.0;
}

/* dupdate_nu (dlanbpro.F:684-723) */
static void update_nu(double *numax, const double *mu, double *nu, int j, const double *alpha,
                      const double *beta, double anorm, double eps1)
{
    if (j > 1) {
        *numax = 0.0;
        for (int k = 1; k <= j - 1; k++) {
            nu[k - 1] = beta[k - 1] * mu[k] + alpha[k - 1] * mu[k - 1] - beta[j - 2] * nu[k - 1];
            double d = eps1 * (hypot(alpha[k - 1], beta[k - 1]) + hypot(alpha[j - 1], beta[j - 2])) + eps1 * anorm;
            nu[k - 1] = (nu[k - 1] + copysign(d, nu[k - 1])) / alpha[j - 1];
            if (fabs(nu[k - 1]) > *numax) *numax = fabs(nu[k - 1]);
        }
        nu[j - 1] = 1.0;
    }
}

/* ------------------------------------------------------------ lanbpro */
/* dlanbpro.F:1-549.  B is held as balpha[] = B(:,1), bbeta[] = B(:,2).
 * *kp is the target dimension on entry, the dimension reached on exit. */
static void lanbpro(int m, int n, int k0, int *kp, aprod_t aprod, double *U, int ldu, double *V, int ldv,
                    double *balpha, double *bbeta, double *rnorm, double *doption, const int *ioption,
                    double *dparm, int *iparm, int *ierr)
{
    int k = *kp;
    const double eps = EPS_D;
    const double eps34 = pow(eps, 0.75);
    const int mn = m > n ? m : n;
    const double epsn = (double)mn * eps;
    const double epsn2 = sqrt((double)mn) * eps;
    double delta, eta, anorm, anormest = 0, s = 0, alpha, beta, a1, b1, amax, mumax, numax;
    int force_reorth, full_reorth, j0;
    const int icgs = ioption[0], ielr = ioption[1];

    delta = doption[0] < 0 ? sqrt(eps / k) : doption[0];
    eta = doption[1] < 0 ? eps34 / sqrt((double)k) : doption[1];
    full_reorth = (delta <= eta || delta == 0.0);
    if (doption[2] > 0) {
        anorm = doption[2];
    } else if (k0 > 0) {
        anorm = hypot(balpha[0], bbeta[0]);
        if (anorm <= 0) { *ierr = -1; doption[2] = anorm; return; }
    } else {
        anorm = 0.0;
    }
    *ierr = 0;

    double *mu = calloc((size_t)k + 2, sizeof(double));
    double *nu = calloc((size_t)k + 2, sizeof(double));
    int *index = calloc((size_t)2 * k + 4, sizeof(int));
    double *wis = calloc((size_t)2 * mn + 2 * (size_t)k + 8, sizeof(double));
    double *wrk = calloc((size_t)2 * mn + 2 * (size_t)k + 8, sizeof(double));

    if (*rnorm == 0.0) {
        getu0('n', m, n, k0, 3, U + (size_t)k0 * ldu, rnorm, U, ldu, aprod, dparm, iparm, ierr, icgs,
              &anormest, wrk);
        if (anormest > anorm) anorm = anormest;
    }

    if (k0 == 0) {
        amax = 0.0;
        alpha = 0.0;
        beta = *rnorm;
        force_reorth = 0;
        if (n > m)
            getu0('n', m, n, 0, 1, wis, &s, U, ldu, aprod, dparm, iparm, ierr, icgs, &anormest, wrk);
        else
            getu0('t', m, n, 0, 1, wis, &s, V, ldv, aprod, dparm, iparm, ierr, icgs, &anormest, wrk);
        if (FUDGE_LANBPRO * anormest > anorm) anorm = FUDGE_LANBPRO * anormest;
        j0 = 1;
        if (beta != 0.0) safescal(m, beta, U);
        mu[0] = 1.0;
        nu[0] = 1.0;
    } else {
        force_reorth = 1;
        alpha = balpha[k0 - 1];
        beta = *rnorm;
        if (k0 < k && beta * delta < anorm * eps) { full_reorth = 1; *ierr = k0; }
        index[0] = 1; index[1] = k0; index[2] = k0 + 1;
        v_scal(m, *rnorm, U + (size_t)k0 * ldu);
        reorth(m, k0, U, ldu, U + (size_t)k0 * ldu, rnorm, index, KAPPA_LANBPRO, wrk, icgs);
        safescal(m, *rnorm, U + (size_t)k0 * ldu);
        set_mu(k0, mu, index, epsn2);
        set_mu(k0, nu, index, epsn2);
        beta = *rnorm;
        bbeta[k0 - 1] = beta;
        amax = 0.0;
        for (int j = 1; j <= k0; j++) {
            if (balpha[j - 1] > amax) amax = balpha[j - 1];
            if (bbeta[j - 1] > amax) amax = bbeta[j - 1];
            if (j == 1) {
                if (FUDGE_LANBPRO * alpha > anorm) anorm = FUDGE_LANBPRO * alpha;
            } else if (j == 2) {
                a1 = bbeta[0] / amax;
                a1 = FUDGE_LANBPRO * amax *
                     sqrt((balpha[0] / amax) * (balpha[0] / amax) + a1 * a1 + balpha[1] / amax * a1);
                if (a1 > anorm) anorm = a1;
            } else {
                a1 = balpha[j - 2] / amax;
                b1 = bbeta[j - 2] / amax;
                a1 = FUDGE_LANBPRO * amax * sqrt(a1 * a1 + b1 * b1 + a1 * bbeta[j - 3] / amax + balpha[j - 1] / amax * b1);
                if (a1 > anorm) anorm = a1;
            }
        }
        j0 = k0 + 1;
    }
    numax = 0.0;
    mumax = 0.0;

    for (int j = j0; j <= k; j++) {
        double *vj = V + (size_t)(j - 1) * ldv;
        double *uj = U + (size_t)(j - 1) * ldu;
        double *uj1 = U + (size_t)j * ldu;

        /* alpha_j v_j = A' u_j - beta_j v_{j-1}   (dlanbpro.F:288-335) */
        aprod("t", &m, &n, uj, vj, dparm, iparm, 1);
        st.nopx++;
        if (j == 1) {
            alpha = v_nrm2(n, vj);
            if (FUDGE_LANBPRO * alpha > anorm) anorm = FUDGE_LANBPRO * alpha;
        } else {
            v_axpy(n, -beta, vj - ldv, vj);
            alpha = v_nrm2(n, vj);
            if (j > 1 && ielr > 0 && alpha < KAPPA_LANBPRO * beta) {
                for (int i = 1; i <= ielr; i++) {
                    st.nelr++;
                    s = v_dot(n, vj - ldv, vj);
                    v_axpy(n, -s, vj - ldv, vj);
                    if (beta != 0.0) { beta = beta + s; bbeta[j - 2] = beta; }
                    s = v_nrm2(n, vj);
                    if (s >= KAPPA_LANBPRO * alpha) break;
                    alpha = s;
                }
                nu[j - 2] = eps;
                alpha = s;
            }
            balpha[j - 1] = alpha;
            if (alpha > amax) amax = alpha;
            if (j == 2) {
                a1 = bbeta[0] / amax;
                a1 = FUDGE_LANBPRO * amax *
                     sqrt((balpha[0] / amax) * (balpha[0] / amax) + a1 * a1 + balpha[1] / amax * a1);
            } else {
                a1 = balpha[j - 2] / amax;
                b1 = bbeta[j - 2] / amax;
                a1 = FUDGE_LANBPRO * amax * sqrt(a1 * a1 + b1 * b1 + a1 * bbeta[j - 3] / amax + balpha[j - 1] / amax * b1);
            }
            if (a1 > anorm) anorm = a1;
        }

        /* nu recurrence and reorthogonalisation of v_j (:340-367) */
        if (!full_reorth && alpha != 0.0) update_nu(&numax, mu, nu, j, balpha, bbeta, anorm, epsn2);
        if ((full_reorth || numax > delta || force_reorth) && alpha != 0.0) {
            if (full_reorth || eta == 0.0) {
                index[0] = 1; index[1] = j - 1; index[2] = j;
            } else if (!force_reorth) {
                compute_int(nu, j - 1, delta, eta, index);
            }
            reorth(n, j - 1, V, ldv, vj, &alpha, index, KAPPA_LANBPRO, wrk, icgs);
            set_mu(j - 1, nu, index, eps);
            numax = eta;
            force_reorth = !force_reorth;
        }

        /* invariant subspace test (:372-409) */
        if (alpha < anorm * epsn && j < k) {
            *rnorm = alpha;
            alpha = 0.0;
            getu0('t', m, n, j - 1, 3, vj, &alpha, V, ldv, aprod, dparm, iparm, ierr, icgs, &anormest, wrk);
            if (alpha == 0.0) {
                k = j - 1;
                *ierr = -j;
                goto done;
            } else {
                safescal(n, alpha, vj);
                alpha = 0.0;
                force_reorth = 1;
                if (delta > 0) full_reorth = 0;
            }
        } else if (j > 1 && !full_reorth && j < k && (delta * alpha < anorm * eps)) {
            *ierr = j;
        }
        balpha[j - 1] = alpha;
        if (alpha != 0.0) safescal(n, alpha, vj);

        /* beta_{j+1} u_{j+1} = A v_j - alpha_j u_j   (:420-458) */
        aprod("n", &m, &n, vj, uj1, dparm, iparm, 1);
        st.nopx++;
        v_axpy(m, -alpha, uj, uj1);
        beta = v_nrm2(m, uj1);
        if (ielr > 0 && beta < KAPPA_LANBPRO * alpha) {
            for (int i = 1; i <= ielr; i++) {
                st.nelr++;
                s = v_dot(m, uj, uj1);
                v_axpy(m, -s, uj, uj1);
                if (alpha != 0.0) { alpha = alpha + s; balpha[j - 1] = alpha; }
                s = v_nrm2(m, uj1);
                if (s >= KAPPA_LANBPRO * beta) break;
                beta = s;
            }
            mu[j - 1] = eps;
            beta = s;
        }
        bbeta[j - 1] = beta;
        if (beta > amax) amax = beta;
        if (j <= 1) {
            a1 = hypot(balpha[0], bbeta[0]);
        } else {
            a1 = balpha[j - 1] / amax;
            a1 = amax * sqrt(a1 * a1 + (bbeta[j - 1] / amax) * (bbeta[j - 1] / amax) + a1 * bbeta[j - 2] / amax);
        }
        if (a1 > anorm) anorm = a1;

        /* mu recurrence and reorthogonalisation of u_{j+1} (:463-498) */
        if (!full_reorth && beta != 0.0) update_mu(&mumax, mu, nu, j, balpha, bbeta, anorm, epsn2);
        if ((full_reorth || mumax > delta || force_reorth) && beta != 0.0) {
            if (full_reorth || eta == 0.0) {
                index[0] = 1; index[1] = j; index[2] = j + 1;
            } else if (!force_reorth) {
                compute_int(mu, j, delta, eta, index);
            } else {
                for (int i = 0; i < 2 * j + 1; i++) {
                    if (index[i] == j) { index[i] = j + 1; break; }
                }
            }
            reorth(m, j, U, ldu, uj1, &beta, index, KAPPA_LANBPRO, wrk, icgs);
            set_mu(j, mu, index, eps);
            mumax = eta;
            force_reorth = !force_reorth;
        }

        /* invariant subspace test (:503-539) */
        if (beta < anorm * epsn && j < k) {
            *rnorm = beta;
            beta = 0.0;
            getu0('n', m, n, j, 3, uj1, &beta, U, ldu, aprod, dparm, iparm, ierr, icgs, &anormest, wrk);
            if (beta == 0.0) {
                k = j;
                *ierr = -j;
                goto done;
            } else {
                safescal(m, beta, uj1);
                beta = 0.0;
                force_reorth = 1;
                if (delta > 0) full_reorth = 0;
            }
        } else if (!full_reorth && j < k && (delta * beta < anorm * eps)) {
            *ierr = j;
        }
        bbeta[j - 1] = beta;
        if (beta != 0.0 && beta != 1.0) safescal(m, beta, uj1);
        *rnorm = beta;
    }
done:
    doption[2] = anorm;
    *kp = k;
    free(mu); free(nu); free(index); free(wis); free(wrk);
}

/* --------------------------------------------------------- bidiagonal */
/* dbsvdstep (dbsvd.F:5-82): one implicit LQ sweep with shift sigma on the
 * (k+1) x k lower bidiagonal (D, E), accumulating the left rotations into
 * U (m rows) and the right rotations into V (n rows). */
static void rot_cols(int rows, double *x, double *y, double c, double s)
{
    for (int r = 0; r < rows; r++) {
        double t = c * x[r] + s * y[r];
        y[r] = c * y[r] - s * x[r];
        x[r] = t;
    }
}
static void bsvdstep(int dou, int dov, int m, int n, int k, double sigma, double *D, double *E, double *U,
                     int ldu, double *V, int ldv)
{
    double c, s, x, y, r;
    if (k <= 1) return;
    x = D[0] * D[0] - sigma * sigma;
    y = E[0] * D[0];
    for (int i = 1; i <= k - 1; i++) {
        if (i > 1) lartg(x, y, &c, &s, &E[i - 2]);
        else lartg(x, y, &c, &s, &r);
        x = c * D[i - 1] + s * E[i - 1];
        E[i - 1] = -s * D[i - 1] + c * E[i - 1];
        D[i - 1] = x;
        y = s * D[i];
        D[i] = c * D[i];
        if (dou && m > 0) rot_cols(m, U + (size_t)(i - 1) * ldu, U + (size_t)i * ldu, c, s);
        lartg(x, y, &c, &s, &D[i - 1]);
        x = c * E[i - 1] + s * D[i];
        D[i] = -s * E[i - 1] + c * D[i];
        E[i - 1] = x;
        y = s * E[i];
        E[i] = c * E[i];
        if (dov && n > 0) rot_cols(n, V + (size_t)(i - 1) * ldv, V + (size_t)i * ldv, c, s);
    }
    lartg(x, y, &c, &s, &E[k - 2]);
    x = c * D[k - 1] + s * E[k - 1];
    E[k - 1] = -s * D[k - 1] + c * E[k - 1];
    D[k - 1] = x;
    if (dou && m > 0) rot_cols(m, U + (size_t)(k - 1) * ldu, U + (size_t)k * ldu, c, s);
}

/* dbdqr (dbsvd.F:87-157): QR of the (n+1) x n lower bidiagonal; on return
 * [0 .. 0 c1 c2]' = Q'[0 .. 0 1]'.  With jobq, Qt ((n+1)x(n+1), ldq)
 * receives Q'. */
static void bdqr(int ignorelast, int jobq, int n, double *D, double *E, double *c1, double *c2, double *Qt,
                 int ldq)
{
    double cs, sn, r;
    int i;
    if (n < 1) return;
#define QT(a, b) Qt[(size_t)((b)-1) * ldq + ((a)-1)]
    if (jobq) {
        for (int j = 1; j <= n + 1; j++) {
            for (int ii = 1; ii <= n + 1; ii++) QT(ii, j) = 0.0;
            QT(j, j) = 1.0;
        }
    }
    for (i = 1; i <= n - 1; i++) {
        lartg(D[i - 1], E[i - 1], &cs, &sn, &r);
        D[i - 1] = r;
        E[i - 1] = sn * D[i];
        D[i] = cs * D[i];
        if (jobq) {
            for (int j = 1; j <= i; j++) {
                QT(i + 1, j) = -sn * QT(i, j);
                QT(i, j) = cs * QT(i, j);
            }
            QT(i, i + 1) = sn;
            QT(i + 1, i + 1) = cs;
        }
    }
    /* here i == n, the Fortran DO variable's exit value */
    if (!ignorelast) {
        lartg(D[n - 1], E[n - 1], &cs, &sn, &r);
        D[n - 1] = r;
        E[n - 1] = 0.0;
        *c1 = sn;
        *c2 = cs;
        if (jobq) {
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

/* drefinebounds (dbsvd.F:162-231): gap-theorem refinement. */
static void refinebounds(int n, int k, const double *theta, double *bound, double tol, double eps34)
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
                double g2 = fabs(theta[i - 2] - theta[i - 1]) - fmax(bound[i - 2], bound[i - 1]);
                if (g2 < gap) gap = g2;
            }
            if (gap > bound[i - 1]) bound[i - 1] = bound[i - 1] * (bound[i - 1] / gap);
        }
    }
}

/* Singular values of the 2x2 upper triangular [f g; 0 h]:
 * smax + smin = hypot(|f|+|h|, g), smax - smin = hypot(|f|-|h|, g),
 * smin = |f h| / smax. */
static void sv2x2(double f, double g, double h, double *smin, double *smax)
{
    double fa = fabs(f), ga = fabs(g), ha = fabs(h);
    double sp = hypot(fa + ha, ga), sm = hypot(fa - ha, ga);
    double mx = 0.5 * (sp + sm);
    *smax = mx;
    *smin = mx > 0 ? (fa / mx) * ha : 0.0;
}

/* Apply a chain of plane rotations to columns lo..hi of a (rows x *)
 * column-major matrix: pair (c, c+1) gets (cs[i], sn[i]) in the order
 * given by fwd. */
static void chain_cols(int rows, double *A, int lda, int lo, int cnt, const double *cs, const double *sn, int fwd)
{
    if (rows <= 0) return;
    for (int t = 0; t < cnt; t++) {
        int i = fwd ? t : cnt - 1 - t;
        double *x = A + (size_t)(lo + i) * lda, *y = x + lda;
        double c = cs[i], s = sn[i];
        for (int r = 0; r < rows; r++) {
            double tmp = y[r];
            y[r] = c * tmp - s * x[r];
            x[r] = s * tmp + c * x[r];
        }
    }
}
/* Same, on rows lo..hi of an (* x cols) column-major matrix. */
static void chain_rows(int cols, double *A, int lda, int lo, int cnt, const double *cs, const double *sn, int fwd)
{
    if (cols <= 0) return;
    for (int t = 0; t < cnt; t++) {
        int i = fwd ? t : cnt - 1 - t;
        double c = cs[i], s = sn[i];
        for (int col = 0; col < cols; col++) {
            double *x = A + (size_t)col * lda + lo + i, *y = x + 1;
            double tmp = *y;
            *y = c * tmp - s * (*x);
            *x = s * tmp + c * (*x);
        }
    }
}

/* Upper bidiagonal SVD (d[n], e[n-1]) by implicit QR; the role of LAPACK
 * dbdsqr / dbdsdc in the reference.  VT (n x ncvt, ldvt) is premultiplied
 * by the transposed right rotations, U (nru x n, ldu) postmultiplied by
 * the left rotations.  Returns 0, or >0 if it did not converge. */
static int bdsqr_upper(int n, double *d, double *e, int ncvt, double *vt, int ldvt, int nru, double *u, int ldu)
{
    const double eps = EPS_D, unfl = SFMIN_D;
    const int maxitr = 6;
    if (n <= 0) return 0;
    double *w = malloc(sizeof(double) * 4 * (size_t)(n + 1));
    double *c1 = w, *s1 = w + n, *c2 = w + 2 * n, *s2 = w + 3 * n;
    int info = 0;
    if (n > 1) {
        double tolmul = fmax(10.0, fmin(100.0, pow(eps, -0.125)));
        double tol = tolmul * eps;
        double smax = 0.0;
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
        double thresh = fmax(tol * sminoa, maxitr * (double)n * (double)n * unfl);
        long maxit = (long)maxitr * n * n, iter = 0;
        int oldll = -1, oldm = -1, idir = 0, m = n - 1; /* 0-based bottom of the active block */
        double sminl = 0.0;
        while (m > 0) {
            if (iter > maxit) { info = 1; break; }
            /* find the bottom unreduced block [ll, m] */
            int ll;
            double smin;
            smax = fabs(d[m]);
            smin = smax;
            int split = -1;
            for (ll = m - 1; ll >= 0; ll--) {
                double abss = fabs(d[ll]), abse = fabs(e[ll]);
                if (abse <= thresh) { split = ll; break; }
                smin = fmin(smin, abss);
                smax = fmax(smax, fmax(abss, abse));
            }
            (void)smin;
            if (split >= 0) {
                e[split] = 0.0;
                if (split == m - 1) { m -= 1; continue; }
                ll = split + 1;
            } else {
                ll = 0;
            }
            /* block [ll, m], m - ll >= 1 */
            if (ll > oldm || m < oldll) idir = (fabs(d[ll]) >= fabs(d[m])) ? 1 : 2;
            int deflated = 0;
            if (idir == 1) {
                if (fabs(e[m - 1]) <= tol * fabs(d[m])) { e[m - 1] = 0.0; continue; }
                double mu = fabs(d[ll]);
                sminl = mu;
                for (int l3 = ll; l3 <= m - 1; l3++) {
                    if (fabs(e[l3]) <= tol * mu) { e[l3] = 0.0; deflated = 1; break; }
                    mu = fabs(d[l3 + 1]) * (mu / (mu + fabs(e[l3])));
                    sminl = fmin(sminl, mu);
                }
            } else {
                if (fabs(e[ll]) <= tol * fabs(d[ll])) { e[ll] = 0.0; continue; }
                double mu = fabs(d[m]);
                sminl = mu;
                for (int l3 = m - 1; l3 >= ll; l3--) {
                    if (fabs(e[l3]) <= tol * mu) { e[l3] = 0.0; deflated = 1; break; }
                    mu = fabs(d[l3]) * (mu / (mu + fabs(e[l3])));
                    sminl = fmin(sminl, mu);
                }
            }
            if (deflated) continue;
            oldll = ll;
            oldm = m;
            /* shift */
            double shift, sll, rdum;
            if ((double)n * tol * (sminl / smax) <= fmax(eps, 0.01 * tol)) {
                shift = 0.0;
            } else {
                if (idir == 1) { sll = fabs(d[ll]); sv2x2(d[m - 1], e[m - 1], d[m], &shift, &rdum); }
                else { sll = fabs(d[m]); sv2x2(d[ll], e[ll], d[ll + 1], &shift, &rdum); }
                if (sll > 0.0 && (shift / sll) * (shift / sll) < eps) shift = 0.0;
            }
            iter += m - ll;
            int cnt = m - ll;
            double cs, sn, r, oldcs, oldsn, f, g, h;
            if (shift == 0.0) {
                if (idir == 1) {
                    cs = 1.0; oldcs = 1.0; oldsn = 0.0;
                    for (int i = ll; i <= m - 1; i++) {
                        lartg(d[i] * cs, e[i], &cs, &sn, &r);
                        if (i > ll) e[i - 1] = oldsn * r;
                        lartg(oldcs * r, d[i + 1] * sn, &oldcs, &oldsn, &d[i]);
                        c1[i - ll] = cs; s1[i - ll] = sn; c2[i - ll] = oldcs; s2[i - ll] = oldsn;
                    }
                    h = d[m] * cs;
                    d[m] = h * oldcs;
                    e[m - 1] = h * oldsn;
                    chain_rows(ncvt, vt, ldvt, ll, cnt, c1, s1, 1);
                    chain_cols(nru, u, ldu, ll, cnt, c2, s2, 1);
                    if (fabs(e[m - 1]) <= thresh) e[m - 1] = 0.0;
                } else {
                    cs = 1.0; oldcs = 1.0; oldsn = 0.0;
                    for (int i = m; i >= ll + 1; i--) {
                        lartg(d[i] * cs, e[i - 1], &cs, &sn, &r);
                        if (i < m) e[i] = oldsn * r;
                        lartg(oldcs * r, d[i - 1] * sn, &oldcs, &oldsn, &d[i]);
                        c1[i - ll - 1] = cs; s1[i - ll - 1] = -sn;
                        c2[i - ll - 1] = oldcs; s2[i - ll - 1] = -oldsn;
                    }
                    h = d[ll] * cs;
                    d[ll] = h * oldcs;
                    e[ll] = h * oldsn;
                    chain_rows(ncvt, vt, ldvt, ll, cnt, c2, s2, 0);
                    chain_cols(nru, u, ldu, ll, cnt, c1, s1, 0);
                    if (fabs(e[ll]) <= thresh) e[ll] = 0.0;
                }
            } else {
                double cosr, sinr, cosl, sinl;
                if (idir == 1) {
                    f = (fabs(d[ll]) - shift) * (copysign(1.0, d[ll]) + shift / d[ll]);
                    g = e[ll];
                    for (int i = ll; i <= m - 1; i++) {
                        lartg(f, g, &cosr, &sinr, &r);
                        if (i > ll) e[i - 1] = r;
                        f = cosr * d[i] + sinr * e[i];
                        e[i] = cosr * e[i] - sinr * d[i];
                        g = sinr * d[i + 1];
                        d[i + 1] = cosr * d[i + 1];
                        lartg(f, g, &cosl, &sinl, &r);
                        d[i] = r;
                        f = cosl * e[i] + sinl * d[i + 1];
                        d[i + 1] = cosl * d[i + 1] - sinl * e[i];
                        if (i < m - 1) { g = sinl * e[i + 1]; e[i + 1] = cosl * e[i + 1]; }
                        c1[i - ll] = cosr; s1[i - ll] = sinr; c2[i - ll] = cosl; s2[i - ll] = sinl;
                    }
                    e[m - 1] = f;
                    chain_rows(ncvt, vt, ldvt, ll, cnt, c1, s1, 1);
                    chain_cols(nru, u, ldu, ll, cnt, c2, s2, 1);
                    if (fabs(e[m - 1]) <= thresh) e[m - 1] = 0.0;
                } else {
                    f = (fabs(d[m]) - shift) * (copysign(1.0, d[m]) + shift / d[m]);
                    g = e[m - 1];
                    for (int i = m; i >= ll + 1; i--) {
                        lartg(f, g, &cosr, &sinr, &r);
                        if (i < m) e[i] = r;
                        f = cosr * d[i] + sinr * e[i - 1];
                        e[i - 1] = cosr * e[i - 1] - sinr * d[i];
                        g = sinr * d[i - 1];
                        d[i - 1] = cosr * d[i - 1];
                        lartg(f, g, &cosl, &sinl, &r);
                        d[i] = r;
                        f = cosl * e[i - 1] + sinl * d[i - 1];
                        d[i - 1] = cosl * d[i - 1] - sinl * e[i - 1];
                        if (i > ll + 1) { g = sinl * e[i - 2]; e[i - 2] = cosl * e[i - 2]; }
                        c1[i - ll - 1] = cosr; s1[i - ll - 1] = -sinr;
                        c2[i - ll - 1] = cosl; s2[i - ll - 1] = -sinl;
                    }
                    e[ll] = f;
                    if (fabs(e[ll]) <= thresh) e[ll] = 0.0;
                    chain_rows(ncvt, vt, ldvt, ll, cnt, c2, s2, 0);
                    chain_cols(nru, u, ldu, ll, cnt, c1, s1, 0);
                }
            }
        }
    }
    /* make the singular values non-negative */
    for (int i = 0; i < n; i++) {
        if (d[i] < 0.0) {
            d[i] = -d[i];
            for (int c = 0; c < ncvt; c++) vt[(size_t)c * ldvt + i] = -vt[(size_t)c * ldvt + i];
        }
    }
    /* sort decreasingly (selection sort, swapping vectors along) */
    for (int i = 0; i < n - 1; i++) {
        int isub = i;
        double smx = d[i];
        for (int j = i + 1; j < n; j++)
            if (d[j] > smx) { smx = d[j]; isub = j; }
        if (isub != i) {
            d[isub] = d[i];
            d[i] = smx;
            for (int c = 0; c < ncvt; c++) {
                double t = vt[(size_t)c * ldvt + i];
                vt[(size_t)c * ldvt + i] = vt[(size_t)c * ldvt + isub];
                vt[(size_t)c * ldvt + isub] = t;
            }
            for (int r = 0; r < nru; r++) {
                double t = u[(size_t)i * ldu + r];
                u[(size_t)i * ldu + r] = u[(size_t)isub * ldu + r];
                u[(size_t)isub * ldu + r] = t;
            }
        }
    }
    free(w);
    return info;
}

/* Exported for the oracle's own unit tests (bidiagonal SVD vs numpy). */
int oracle_bdsqr(int n, double *d, double *e, int ncvt, double *vt, int ldvt, int nru, double *u, int ldu)
{
    return bdsqr_upper(n, d, e, ncvt, vt, ldvt, nru, u, ldu);
}

/* ---------------------------------------------------------- ovwr GEMM */
/* dgemm_ovwr_left (dgemm_ovwr.F:56-87): A(:,1:nc) <- A(:,1:kk) * op(B),
 * op(B) = B(1:kk,1:nc) ('n') or B(1:nc,1:kk)' ('t'), in place, by row
 * blocks. */
static void gemm_ovwr_left(char transb, int m, int nc, int kk, double *A, int lda, const double *B, int ldb)
{
    if (m <= 0 || nc <= 0 || kk <= 0) return;
    const int RB = 64;
    int nblk = (m + RB - 1) / RB;
#pragma omp parallel for schedule(static) if (m >= 2 * RB) num_threads(nthr())
    for (int b = 0; b < nblk; b++) {
        int r0 = b * RB, rn = (m - r0 < RB) ? m - r0 : RB;
        double *tmp = malloc(sizeof(double) * (size_t)RB * nc);
        for (int c = 0; c < nc; c++) {
            double *t = tmp + (size_t)c * RB;
            for (int r = 0; r < rn; r++) t[r] = 0.0;
            for (int l = 0; l < kk; l++) {
                double bl = (transb == 'n') ? B[(size_t)c * ldb + l] : B[(size_t)l * ldb + c];
                const double *a = A + (size_t)l * lda + r0;
                for (int r = 0; r < rn; r++) t[r] += a[r] * bl;
            }
        }
        for (int c = 0; c < nc; c++)
            memcpy(A + (size_t)c * lda + r0, tmp + (size_t)c * RB, sizeof(double) * rn);
        free(tmp);
    }
}

/* ------------------------------------------------------------ ritzvec */
/* dritzvec.F:1-199.  D, E: copies of B(:,1), B(:,2) (overwritten). */
static void ritzvec(char which, int jobu, int jobv, int m, int n, int k, int dim, double *D, double *E,
                    double *U, int ldu, double *V, int ldv)
{
    int dp1 = dim + 1;
    double *Mt = calloc((size_t)dp1 * dp1, sizeof(double));
    double *P = calloc((size_t)dim * dim, sizeof(double));
    double *Qt = calloc((size_t)dim * dim, sizeof(double));
    double *X = calloc((size_t)dp1 * dp1, sizeof(double));
    double c1 = 0, c2 = 0;
    int ignorelast = (dim == (m < n ? m : n));
    bdqr(ignorelast, jobu, dim, D, E, &c1, &c2, Mt, dp1);
    for (int i = 0; i < dim; i++) { P[(size_t)i * dim + i] = 1.0; Qt[(size_t)i * dim + i] = 1.0; }
    bdsqr_upper(dim, D, E, dim, Qt, dim, dim, P, dim);
    /* X = P' * Mt(1:dim, 1:dim+1), stored in rows 1..dim of a (dim+1) ld */
    for (int c = 0; c < dp1; c++)
        for (int r = 0; r < dim; r++) {
            double acc = 0.0;
            for (int l = 0; l < dim; l++) acc += P[(size_t)r * dim + l] * Mt[(size_t)c * dp1 + l];
            X[(size_t)c * dp1 + r] = acc;
        }
    int mstart = (which == 's' || which == 'S') ? dim - k + 1 : 1;
    if (jobu) gemm_ovwr_left('t', m, k, dp1, U, ldu, X + (mstart - 1), dp1);
    if (jobv) gemm_ovwr_left('t', n, k, dim, V, ldv, Qt + (mstart - 1), dim);
    free(Mt); free(P); free(Qt); free(X);
}

static int is_yes(const char *c) { return c[0] == 'y' || c[0] == 'Y'; }

/* ------------------------------------------------------------- lansvd */
/* dlansvd.F:1-291. */
void oracle_dlansvd(const char *jobu, const char *jobv, int *m_, int *n_, int *k_, int *kmax_, aprod_t aprod,
                    double *U, int *ldu_, double *Sigma, double *bnd, double *V, int *ldv_, double *tolin,
                    double *work, int *lwork, int *iwork, int *liwork, double *doption, int *ioption, int *info,
                    double *dparm, int *iparm, size_t ljobu, size_t ljobv)
{
    (void)work; (void)lwork; (void)iwork; (void)liwork; (void)ljobu; (void)ljobv;
    int m = *m_, n = *n_, k = *k_, kmax = *kmax_, ldu = *ldu_, ldv = *ldv_;
    const double eps = EPS_D, eps34 = pow(eps, 0.75);
    const int mn = m > n ? m : n;
    const double epsn = (double)mn * eps / 2.0;
    int lanmax = kmax;
    if (n + 1 < lanmax) lanmax = n + 1;
    if (m + 1 < lanmax) lanmax = m + 1;
    double tol = fmin(1.0, fmax(16.0 * eps, *tolin));
    double anorm = 0.0, rnorm;
    int ierr = 0, j, jold, neig, dj;
    double *B = calloc((size_t)2 * lanmax + 2, sizeof(double));  /* alpha | beta */
    double *B1 = calloc((size_t)2 * lanmax + 2, sizeof(double));
    double *wb = calloc((size_t)lanmax + 2, sizeof(double));
    double *wrk = calloc((size_t)2 * mn + 8, sizeof(double));
    double *balpha = B, *bbeta = B + lanmax;

    rnorm = v_nrm2(m, U);
    if (rnorm == 0.0)
        getu0('n', m, n, 0, 1, U, &rnorm, U, ldu, aprod, dparm, iparm, &ierr, ioption[0], &anorm, wrk);

    st.nsing = k;
    *info = 0;
    neig = 0;
    jold = 0;
    j = k + (8 > k ? 8 : k) + 1;
    if (j > lanmax) j = lanmax;
    while (neig < k) {
        lanbpro(m, n, jold, &j, aprod, U, ldu, V, ldv, balpha, bbeta, &rnorm, doption, ioption, dparm, iparm,
                &ierr);
        jold = j;
        memcpy(B1, B, sizeof(double) * 2 * lanmax);
        for (int i = 0; i <= j; i++) wb[i] = 0.0;
        bdqr(j == (m < n ? m : n), 0, j, B1, B1 + lanmax, &wb[j - 1], &wb[j], NULL, lanmax + 1);
        bdsqr_upper(j, B1, B1 + lanmax, 0, NULL, 1, 1, wb, 1);
        st.nbsvd++;
        if (j > 5) anorm = B1[0];
        else anorm = fmax(anorm, B1[0]);
        for (int i = 0; i < j; i++) wb[i] = fabs(rnorm * wb[i]);
        refinebounds(m < n ? m : n, j, B1, wb, epsn * anorm, eps34);
        int lim = j < k ? j : k;
        for (int i = 0; i < lim; i++) bnd[i] = wb[i];
        int i = 0;
        neig = 0;
        while (i < lim) {
            if (wb[i] <= tol * B1[i]) { Sigma[neig] = B1[i]; neig++; i++; }
            else i = k;
        }
        if (ierr < 0) {
            if (j < k) *info = j;
            break;
        }
        if (j >= lanmax) {
            if (neig < k) *info = -1;
            break;
        }
        if (neig > 1) {
            dj = j / 2;
            int d2 = ((k - neig) * (j - 6)) / (2 * neig + 1);
            if (d2 < dj) dj = d2;
            dj = dj < 2 ? 2 : dj;
            dj = dj > 100 ? 100 : dj;
        } else {
            dj = j / 2;
            dj = dj < 10 ? 10 : dj;
            dj = dj > 100 ? 100 : dj;
        }
        j = j + dj < lanmax ? j + dj : lanmax;
    }
    if ((neig >= k || *info > 0) && (is_yes(jobu) || is_yes(jobv))) {
        memcpy(B1, B, sizeof(double) * 2 * lanmax);
        ritzvec('L', is_yes(jobu), is_yes(jobv), m, n, neig, jold, B1, B1 + lanmax, U, ldu, V, ldv);
    }
    *k_ = neig;
    st.nlandim = j;
    free(B); free(B1); free(wb); free(wrk);
}

/* --------------------------------------------------------- lansvd_irl */
/* dlansvd_irl.F:1-419. */
void oracle_dlansvd_irl(const char *which, const char *jobu, const char *jobv, int *m_, int *n_, int *dim_,
                        int *p_, int *neig_, int *maxiter_, aprod_t aprod, double *U, int *ldu_, double *Sigma,
                        double *bnd, double *V, int *ldv_, double *tolin, double *work, int *lwork, int *iwork,
                        int *liwork, double *doption, int *ioption, int *info, double *dparm, int *iparm,
                        size_t lwhich, size_t ljobu, size_t ljobv)
{
    (void)work; (void)lwork; (void)iwork; (void)liwork; (void)lwhich; (void)ljobu; (void)ljobv;
    int m = *m_, n = *n_, dim = *dim_, p = *p_, neig = *neig_, maxiter = *maxiter_, ldu = *ldu_, ldv = *ldv_;
    const double eps = EPS_D, eps34 = pow(eps, 0.75);
    const int mn = m > n ? m : n;
    const double epsn = (double)mn * eps / 2.0;
    const int small_side = which[0] == 's' || which[0] == 'S';
    if (n + 1 < dim) dim = n + 1;
    if (m + 1 < dim) dim = m + 1;
    int k = dim - p;
    double tol = fmin(1.0, fmax(16.0 * eps, *tolin));
    double anorm = 0.0, rnorm;
    int ierr = 0, iter = 0, nconv = 0, kold = 0, dim0 = dim;
    double *balpha = calloc((size_t)dim0 + 2, sizeof(double));
    double *bbeta = calloc((size_t)dim0 + 2, sizeof(double));
    double *a1 = calloc((size_t)dim0 + 2, sizeof(double));
    double *b1 = calloc((size_t)dim0 + 2, sizeof(double));
    double *wb = calloc((size_t)dim0 + 2, sizeof(double));
    double *shifts = calloc((size_t)dim0 + 2, sizeof(double));
    double *P = calloc((size_t)(dim0 + 1) * (dim0 + 1), sizeof(double));
    double *Q = calloc((size_t)dim0 * dim0, sizeof(double));
    double *wrk = calloc((size_t)2 * mn + 8, sizeof(double));

    rnorm = v_nrm2(m, U);
    if (rnorm == 0.0)
        getu0('n', m, n, 0, 1, U, &rnorm, U, ldu, aprod, dparm, iparm, &ierr, ioption[0], &anorm, wrk);

    *info = 0;
    while (nconv < neig && iter < maxiter) {
        lanbpro(m, n, kold, &dim, aprod, U, ldu, V, ldv, balpha, bbeta, &rnorm, doption, ioption, dparm, iparm,
                &ierr);
        kold = k;
        memcpy(a1, balpha, sizeof(double) * dim);
        memcpy(b1, bbeta, sizeof(double) * dim);
        for (int i = 0; i <= dim; i++) wb[i] = 0.0;
        bdqr(dim == (m < n ? m : n), 0, dim, a1, b1, &wb[dim - 1], &wb[dim], NULL, dim + 1);
        bdsqr_upper(dim, a1, b1, 0, NULL, 1, 1, wb, 1);
        st.nbsvd++;
        if (dim > 5) anorm = a1[0];
        else anorm = fmax(anorm, a1[0]);
        for (int i = 0; i < dim; i++) wb[i] = fabs(rnorm * wb[i]);
        if (small_side)
            refinebounds(m < n ? m : n, dim, a1, wb, epsn * anorm, eps34);
        else
            refinebounds(m < n ? m : n, dim < neig ? dim : neig, a1, wb, epsn * anorm, eps34);

        if (small_side) {
            nconv = 0;
            for (int i = dim - neig + 1; i <= dim; i++) {
                if (wb[i - 1] <= tol * a1[0]) {
                    Sigma[nconv] = a1[i - 1];
                    bnd[nconv] = wb[i - 1];
                    nconv++;
                }
            }
        } else {
            int i = 1, lim = dim < neig ? dim : neig;
            nconv = 0;
            while (i <= lim) {
                if (wb[i - 1] <= tol * a1[i - 1]) {
                    Sigma[nconv] = a1[i - 1];
                    bnd[nconv] = wb[i - 1];
                    nconv++;
                    i++;
                } else {
                    i = k + 1;
                }
            }
        }

        if (ierr < 0) {
            if (dim < k) *info = dim;
            break;
        }
        if (nconv < neig) {
            /* exact shifts gated by the relative gap (:304-344) */
            int nshft = 0;
            for (int i = 0; i < dim - k; i++) shifts[i] = 0.0;
            if (small_side) {
                for (int i = 1; i <= k; i++) {
                    double relgap = a1[i - 1] - wb[i - 1] - a1[dim - neig - 1];
                    shifts[nshft] = (relgap > doption[3] * a1[dim - neig - 1]) ? a1[i - 1] : a1[0];
                    nshft++;
                }
            } else {
                for (int i = dim; i >= k + 1; i--) {
                    double relgap = a1[k - 1] - (a1[i - 1] + wb[i - 1]);
                    shifts[nshft] = (relgap > doption[3] * a1[k - 1]) ? a1[i - 1] : 0.0;
                    nshft++;
                }
            }
            /* sweeps accumulating P ((dim+1)^2) and Q (dim^2) (:350-363) */
            memset(P, 0, sizeof(double) * (size_t)(dim + 1) * (dim + 1));
            memset(Q, 0, sizeof(double) * (size_t)dim * dim);
            for (int i = 0; i < dim + 1; i++) P[(size_t)i * (dim + 2)] = 1.0;
            for (int i = 0; i < dim; i++) Q[(size_t)i * (dim + 1)] = 1.0;
            for (int i = dim; i >= k + 1; i--) {
                double shift = shifts[dim - i];
                bsvdstep(1, 1, dim + 1, dim, i, shift, balpha, bbeta, P, dim + 1, Q, dim);
            }
            /* U(:,1:k+1) <- U P(:,1:k+1); V(:,1:k) <- V Q(:,1:k) (:371-398) */
            gemm_ovwr_left('n', m, k + 1, dim + 1, U, ldu, P, dim + 1);
            gemm_ovwr_left('n', n, k, dim, V, ldv, Q, dim);
            rnorm = bbeta[k - 1];
            st.nrestart++;
        }
        iter++;
    }

    if ((nconv >= neig || *info > 0) && (is_yes(jobu) || is_yes(jobv))) {
        memcpy(a1, balpha, sizeof(double) * dim);
        memcpy(b1, bbeta, sizeof(double) * dim);
        ritzvec(which[0], is_yes(jobu), is_yes(jobv), m, n, nconv, dim, a1, b1, U, ldu, V, ldv);
    }
    *neig_ = nconv;
    st.nlandim = dim;
    free(balpha); free(bbeta); free(a1); free(b1); free(wb); free(shifts); free(P); free(Q); free(wrk);
}

/* ---------------------------------------------------- CSR operator */
/* A = S + L diag(w) R' with S (m x n), L (m x r), R (n x r) in CSR; the
 * transposes are built once.  This is the oracle's APROD for the
 * synthetic workloads (the factored low-rank term keeps dense outer
 * products out of the CSR). iparm[0..1] carry the handle pointer. */
typedef struct {
    int rows, cols;
    int64_t *ptr;
    int *idx;
    double *val;
} csr_t;
typedef struct {
    int m, n, r;
    csr_t S, St, L, Lt, R, Rt;
    double *w, *tmp;
} oracle_op_t;

static void csr_transpose(const csr_t *A, csr_t *T)
{
    T->rows = A->cols;
    T->cols = A->rows;
    int64_t nnz = A->ptr[A->rows];
    T->ptr = calloc((size_t)T->rows + 1, sizeof(int64_t));
    T->idx = malloc(sizeof(int) * (size_t)(nnz ? nnz : 1));
    T->val = malloc(sizeof(double) * (size_t)(nnz ? nnz : 1));
    for (int64_t e = 0; e < nnz; e++) T->ptr[A->idx[e] + 1]++;
    for (int i = 0; i < T->rows; i++) T->ptr[i + 1] += T->ptr[i];
    int64_t *pos = malloc(sizeof(int64_t) * (size_t)(T->rows + 1));
    memcpy(pos, T->ptr, sizeof(int64_t) * (size_t)(T->rows + 1));
    for (int i = 0; i < A->rows; i++)
        for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++) {
            int64_t q = pos[A->idx[e]]++;
            T->idx[q] = i;
            T->val[q] = A->val[e];
        }
    free(pos);
}
static void csr_copy(csr_t *D, int rows, int cols, const int64_t *ptr, const int *idx, const double *val)
{
    D->rows = rows;
    D->cols = cols;
    int64_t nnz = ptr[rows];
    D->ptr = malloc(sizeof(int64_t) * (size_t)(rows + 1));
    memcpy(D->ptr, ptr, sizeof(int64_t) * (size_t)(rows + 1));
    D->idx = malloc(sizeof(int) * (size_t)(nnz ? nnz : 1));
    D->val = malloc(sizeof(double) * (size_t)(nnz ? nnz : 1));
    if (nnz) {
        memcpy(D->idx, idx, sizeof(int) * (size_t)nnz);
        memcpy(D->val, val, sizeof(double) * (size_t)nnz);
    }
}
static void csr_free(csr_t *A)
{
    free(A->ptr); free(A->idx); free(A->val);
}
/* y = A x (+ y if accumulate) */
static void csr_mv(const csr_t *A, const double *x, double *y, int accumulate)
{
#pragma omp parallel for schedule(dynamic, 1024) if (A->rows >= PAR_MIN) num_threads(nthr())
    for (int i = 0; i < A->rows; i++) {
        double acc = 0.0;
        for (int64_t e = A->ptr[i]; e < A->ptr[i + 1]; e++) acc += A->val[e] * x[A->idx[e]];
        y[i] = accumulate ? y[i] + acc : acc;
    }
}

void *oracle_op_create(int m, int n, const int64_t *sptr, const int *sidx, const double *sval, int r,
                       const int64_t *lptr, const int *lidx, const double *lval, const int64_t *rptr,
                       const int *ridx, const double *rval, const double *w)
{
    oracle_op_t *op = calloc(1, sizeof(oracle_op_t));
    op->m = m; op->n = n; op->r = r;
    csr_copy(&op->S, m, n, sptr, sidx, sval);
    csr_transpose(&op->S, &op->St);
    if (r > 0) {
        csr_copy(&op->L, m, r, lptr, lidx, lval);
        csr_copy(&op->R, n, r, rptr, ridx, rval);
        csr_transpose(&op->L, &op->Lt);
        csr_transpose(&op->R, &op->Rt);
        op->w = malloc(sizeof(double) * r);
        memcpy(op->w, w, sizeof(double) * r);
        op->tmp = malloc(sizeof(double) * r);
    }
    return op;
}
void oracle_op_destroy(void *h)
{
    oracle_op_t *op = h;
    if (!op) return;
    csr_free(&op->S); csr_free(&op->St);
    if (op->r > 0) {
        csr_free(&op->L); csr_free(&op->Lt); csr_free(&op->R); csr_free(&op->Rt);
        free(op->w); free(op->tmp);
    }
    free(op);
}
/* The APROD of this operator: handle pointer in iparm[0] (low) / [1]. */
void oracle_op_aprod(const char *transa, const int *m, const int *n, const double *x, double *y, double *dparm,
                     int *iparm, size_t len)
{
    (void)m; (void)n; (void)dparm; (void)len;
    uint64_t h = (uint64_t)(uint32_t)iparm[0] | ((uint64_t)(uint32_t)iparm[1] << 32);
    oracle_op_t *op = (oracle_op_t *)(uintptr_t)h;
    int t = (transa[0] == 't' || transa[0] == 'T');
    if (!t) {
        csr_mv(&op->S, x, y, 0);
        if (op->r > 0) {
            csr_mv(&op->Rt, x, op->tmp, 0);
            for (int i = 0; i < op->r; i++) op->tmp[i] *= op->w[i];
            csr_mv(&op->L, op->tmp, y, 1);
        }
    } else {
        csr_mv(&op->St, x, y, 0);
        if (op->r > 0) {
            csr_mv(&op->Lt, x, op->tmp, 0);
            for (int i = 0; i < op->r; i++) op->tmp[i] *= op->w[i];
            csr_mv(&op->R, op->tmp, y, 1);
        }
    }
}

/* One Lanczos step count of work for timing samples: run lanbpro for
 * nsteps from a given start, exposed for the CPU baseline. */
int oracle_lanbpro_sample(int m, int n, int nsteps, aprod_t aprod, double *U, int ldu, double *V, int ldv,
                          double *doption, int *ioption, double *dparm, int *iparm)
{
    double *ba = calloc((size_t)nsteps + 2, sizeof(double));
    double *bb = calloc((size_t)nsteps + 2, sizeof(double));
    double rnorm = v_nrm2(m, U);
    int ierr = 0, k = nsteps;
    lanbpro(m, n, 0, &k, aprod, U, ldu, V, ldv, ba, bb, &rnorm, doption, ioption, dparm, iparm, &ierr);
    free(ba); free(bb);
    return k;
}

/* The complex*16 drivers share the real routines above. */
#include "propack_oracle_z.inc"
