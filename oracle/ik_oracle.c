/*
 * ik_oracle.c -- FP64 CPU restatement of the pyglasstools Irving-Kirkwood path.
 *
 * TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py; never by the product.
 * Field parity is unpinned by the reference itself (its IK loop needs Aboria,
 * Eigen, GSL and MPI, all absent); force and kernel formulas are pinned against
 * the reference headers compiled by oracle/build_ref.sh (see ik_oracle.h).
 *
 * Compiled with -ffp-contract=off so that x86-64 and aarch64 hosts produce the
 * same bits (no fused multiply-add contraction).
 *
 * Every function cites the reference code it restates (paths relative to the
 * pyglasstools repository).
 */
#include "ik_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------- */
/* Gauss-Legendre rule on [-1,1]: Newton iteration on P_n from the three-term
 * recurrence (Golub & Welsch 1969 give the same nodes; this is the classical
 * Newton form).  Replaces gsl_integration_glfixed_table_alloc
 * (irvingkirkwood/cgfunc/FixedPointQuadrature.h:35). */
void ikor_gl_rule(int n, double* x, double* w)
{
    for (int k = 0; k < n; ++k) {
        /* k-th root, descending from +1 */
        long double z = cosl(3.14159265358979323846264338327950288L * (k + 0.75L) / (n + 0.5L));
        long double pp = 0.0L;
        for (int it = 0; it < 100; ++it) {
            long double p0 = 1.0L, p1 = z;
            for (int j = 2; j <= n; ++j) {
                long double p2 = ((2.0L * j - 1.0L) * z * p1 - (j - 1.0L) * p0) / j;
                p0 = p1; p1 = p2;
            }
            if (n == 1) { p1 = z; p0 = 1.0L; }
            pp = n * (z * p1 - p0) / (z * z - 1.0L);
            long double dz = p1 / pp;
            z -= dz;
            if (fabsl(dz) < 1e-19L) break;
        }
        /* recompute derivative at the converged root */
        {
            long double p0 = 1.0L, p1 = z;
            for (int j = 2; j <= n; ++j) {
                long double p2 = ((2.0L * j - 1.0L) * z * p1 - (j - 1.0L) * p0) / j;
                p0 = p1; p1 = p2;
            }
            if (n == 1) { p1 = z; p0 = 1.0L; }
            pp = n * (z * p1 - p0) / (z * z - 1.0L);
        }
        /* store ascending: index n-1-k */
        x[n - 1 - k] = (double)z;
        w[n - 1 - k] = (double)(2.0L / ((1.0L - z * z) * pp * pp));
    }
    if (n % 2 == 1) x[n / 2] = 0.0; /* exact centre node */
}

/* Each rule is built once per process and reused (the reference takes its table from
 * GSL on every call, FixedPointQuadrature.h:35; rebuilding it by Newton iteration in
 * long double on every bond would dominate the loop, most of all where long double is
 * software quad precision, as on aarch64).  The first caller builds under a lock; later
 * callers see the finished table through an acquire load. */
static double gl_tab_x[65][64], gl_tab_w[65][64];
static int gl_tab_ready[65];

static void gl_rule_cached(int n, const double** x, const double** w)
{
    if (!__atomic_load_n(&gl_tab_ready[n], __ATOMIC_ACQUIRE)) {
#pragma omp critical(ikor_rules)
        {
            if (!__atomic_load_n(&gl_tab_ready[n], __ATOMIC_RELAXED)) {
                ikor_gl_rule(n, gl_tab_x[n], gl_tab_w[n]);
                __atomic_store_n(&gl_tab_ready[n], 1, __ATOMIC_RELEASE);
            }
        }
    }
    *x = gl_tab_x[n];
    *w = gl_tab_w[n];
}

/* ------------------------------------------------------------------------- */
/* The pair models, each in the evaluation order of its reference expression (C and
 * C++ both evaluate a*b*c as (a*b)*c; the library is built with -ffp-contract=off):
 *   Polydisperse12     potential/Polydisperse12.h:19-55
 *   LennardJones       potential/LennardJones.h:19-57
 *   ForceShiftedLJ     potential/LennardJones.h:105-124; energy: LennardJones's
 *   Polydisperse10     potential/Polydisperse10.h:19-53
 *   Polydisperse106    potential/Polydisperse106.h:19-53
 *   Polydisperse18     potential/Polydisperse18.h:19-50
 *   PolydisperseLJ     potential/PolydisperseLJ.h:19-50
 *   PolydisperseYukawa potential/PolydisperseYukawa.h:19-55
 * with rsq_cut = scaled_rcut^2 (potential/PairPotential.h:98-113). */
static double poly12_sigma(const ikor_pot* p, double di, double dj)
{
    return 0.5 * (di + dj) * (1 - p->eps * fabs(di - dj));
}

double ikor_force_divr(const ikor_pot* p, double rsq, double di, double dj)
{
    double rcutsq = p->scaled_rcut * p->scaled_rcut;
    double v0 = p->v0, c1 = p->c1, c2 = p->c2, c3 = p->c3, kappa = p->kappa;
    double sigma = p->kind == IKOR_POT_FSLJ ? 0.5 * (di + dj) : poly12_sigma(p, di, dj);
    double actualrcutsq = rcutsq * sigma * sigma;
    if (!(rsq < actualrcutsq)) return 0.0;
    if ((p->kind == IKOR_POT_LJ || p->kind == IKOR_POT_FSLJ) && v0 == 0) return 0.0;
    double r2inv = 1.0 / rsq;
    r2inv *= sigma * sigma;
    double _rsq = rsq / (sigma * sigma);
    double r6inv = r2inv * r2inv * r2inv;
    double r10inv = r2inv * r2inv * r2inv * r2inv * r2inv;
    switch (p->kind) {
    case IKOR_POT_LJ:
        return (4 * v0 * r2inv * r6inv * (12.0 * r6inv - 6.0)) / (sigma * sigma);
    case IKOR_POT_FSLJ: {
        double f = 4 * v0 * r2inv * r6inv * (12.0 * r6inv - 6.0);
        double c2inv = 1.0 / rcutsq;
        double c6inv = c2inv * c2inv * c2inv;
        f -= 4 * v0 * c2inv * c6inv * (12.0 * c6inv - 6.0);
        return f / (sigma * sigma);
    }
    case IKOR_POT_POLY10:
        return (10.0 * v0 * r2inv * r10inv - 2.0 * c1 - 4.0 * c2 * _rsq - 6.0 * c3 * _rsq * _rsq) / (sigma * sigma);
    case IKOR_POT_POLY106:
        return (v0 * (10.0 * r10inv * r2inv - 6.0 * r2inv * r2inv * r2inv * r2inv) - 2.0 * c1 - 4.0 * c2 * _rsq) /
               (sigma * sigma);
    case IKOR_POT_POLY18:
        return (18.0 * v0 * r2inv * r6inv * r6inv * r6inv - 2.0 * c1 - 4.0 * c2 * _rsq) / (sigma * sigma);
    case IKOR_POT_POLYLJ:
        return (12.0 * v0 * r2inv * r6inv * r6inv - 6.0 * v0 * r2inv * r6inv - 2.0 * c1 - 4.0 * c2 * _rsq) /
               (sigma * sigma);
    case IKOR_POT_POLYYUKAWA: {
        double rinv = sqrt(r2inv), rroot = sqrt(_rsq);
        return ((exp(-kappa * rroot) * (rinv + kappa) * v0) * r2inv - 2 * c1 - 4 * c2 * _rsq) / (sigma * sigma);
    }
    default:
        return (12.0 * v0 * r2inv * r6inv * r6inv - 2.0 * c1 - 4.0 * c2 * _rsq) / (sigma * sigma);
    }
}

double ikor_pair_energy(const ikor_pot* p, double rsq, double di, double dj)
{
    double rcutsq = p->scaled_rcut * p->scaled_rcut;
    double v0 = p->v0, c0 = p->c0, c1 = p->c1, c2 = p->c2, c3 = p->c3, kappa = p->kappa;
    double sigma = poly12_sigma(p, di, dj);
    double actualrcutsq = rcutsq * sigma * sigma;
    if (!(rsq < actualrcutsq)) return 0.0;
    double r2inv = 1.0 / rsq;
    r2inv *= sigma * sigma;
    double _rsq = rsq / (sigma * sigma);
    double r6inv = r2inv * r2inv * r2inv;
    double r10inv = r2inv * r2inv * r2inv * r2inv * r2inv;
    switch (p->kind) {
    case IKOR_POT_LJ:
    case IKOR_POT_FSLJ: {
        double r2invcut = 1.0 / actualrcutsq;
        r2invcut *= sigma * sigma;
        double r6invcut = r2invcut * r2invcut * r2invcut;
        return 4 * v0 * r6inv * (r6inv - 1.0) - 4 * v0 * r6invcut * (r6invcut - 1.0);
    }
    case IKOR_POT_POLY10:
        return v0 * r10inv + c0 + c1 * _rsq + c2 * _rsq * _rsq + c3 * _rsq * _rsq * _rsq;
    case IKOR_POT_POLY106:
        return v0 * (r10inv - r2inv * r2inv * r2inv) + c0 + c1 * _rsq + c2 * _rsq * _rsq;
    case IKOR_POT_POLY18:
        return v0 * r6inv * r6inv * r6inv + c0 + c1 * _rsq + c2 * _rsq * _rsq;
    case IKOR_POT_POLYLJ:
        return v0 * r6inv * r6inv - v0 * r6inv + c0 + c1 * _rsq + c2 * _rsq * _rsq;
    case IKOR_POT_POLYYUKAWA: {
        double rinv = sqrt(r2inv), rroot = sqrt(_rsq);
        return v0 * exp(-rroot * kappa) * rinv + c0 + c1 * _rsq + c2 * _rsq * _rsq;
    }
    default:
        return v0 * r6inv * r6inv + c0 + c1 * _rsq + c2 * _rsq * _rsq;
    }
}

/* computeStiffness of each model (Polydisperse12.h:57-73, LennardJones.h:60-75 -- the
 * force-shifted model inherits it --, Polydisperse10.h:56-72, Polydisperse106.h:56-72,
 * Polydisperse18.h:56-72, PolydisperseLJ.h:56-72, PolydisperseYukawa.h:59-76). */
double ikor_bond_stiffness(const ikor_pot* p, double rsq, double di, double dj)
{
    double rcutsq = p->scaled_rcut * p->scaled_rcut;
    double v0 = p->v0, c1 = p->c1, c2 = p->c2, c3 = p->c3, kappa = p->kappa;
    double sigma = poly12_sigma(p, di, dj);
    double actualrcutsq = rcutsq * sigma * sigma;
    if (!(rsq < actualrcutsq)) return 0.0;
    if ((p->kind == IKOR_POT_LJ || p->kind == IKOR_POT_FSLJ) && v0 == 0) return 0.0;
    double r2inv = 1.0 / rsq;
    r2inv *= sigma * sigma;
    double _rsq = rsq / (sigma * sigma);
    double r6inv = r2inv * r2inv * r2inv;
    switch (p->kind) {
    case IKOR_POT_LJ:
    case IKOR_POT_FSLJ:
        return (4 * v0 * r2inv * r6inv * (13.0 * 12.0 * r6inv - 6.0 * 7.0)) / (sigma * sigma);
    case IKOR_POT_POLY10:
        return (110.0 * v0 * r6inv * r6inv + 2.0 * c1 + 12.0 * c2 * _rsq + 30.0 * c3 * _rsq * _rsq) / (sigma * sigma);
    case IKOR_POT_POLY106:
        return (v0 * (110.0 * r6inv * r6inv - 42.0 * r2inv * r2inv * r2inv * r2inv) + 2.0 * c1 + 12.0 * c2 * _rsq) /
               (sigma * sigma);
    case IKOR_POT_POLY18:
        return (342.0 * v0 * r2inv * r6inv * r6inv * r6inv + 2.0 * c1 + 12.0 * c2 * _rsq) / (sigma * sigma);
    case IKOR_POT_POLYLJ:
        return (156.0 * v0 * r2inv * r6inv * r6inv - 42.0 * v0 * r2inv * r6inv + 2.0 * c1 + 4.0 * c2 * _rsq) /
               (sigma * sigma);
    case IKOR_POT_POLYYUKAWA: {
        double rinv = sqrt(r2inv), rroot = sqrt(_rsq);
        return (v0 * exp(-kappa * rroot) * (2 * r2inv + 2 * kappa * rinv + kappa * kappa) * rinv + 2 * c1 +
                12 * c2 * _rsq) / (sigma * sigma);
    }
    default:
        return (156.0 * v0 * r2inv * r6inv * r6inv + 2.0 * c1 + 12.0 * c2 * _rsq) / (sigma * sigma);
    }
}

/* ------------------------------------------------------------------------- */
/* Coarse-graining kernels.
 *   Octic      irvingkirkwood/cgfunc/CGFuncOctic.h:16-29
 *   Rect       irvingkirkwood/cgfunc/CGFuncRect.h  (1/(pi R^2) inside)
 *   Mollifier  irvingkirkwood/cgfunc/CGFuncMollifier.h (C1/(2 pi R^2) exp(-1/(1-r^2/R^2)))
 *   Gaussian   not in the reference: (2 pi w^2)^(-dim/2) exp(-r^2/(2 w^2)) for r < R,
 *              not renormalised for the truncation. */
#define MOLLIFIER_C1 13.46842098743079272180855772032086697297031125109170011102

double ikor_delta(const ikor_cg* cg, int dim, double dr_sq)
{
    double rcutsq = cg->rcut * cg->rcut;
    if (!(dr_sq < rcutsq)) return 0.0;
    switch (cg->kind) {
    case IKOR_CG_OCTIC: {
        double r4 = dr_sq * dr_sq / (rcutsq * rcutsq);
        double r8 = r4 * r4;
        return 15.0 / (8 * M_PI * rcutsq) * (1 - 2 * r4 + r8);
    }
    case IKOR_CG_RECT:
        return 1 / (M_PI * rcutsq);
    case IKOR_CG_MOLLIFIER: {
        double norm = MOLLIFIER_C1 / (2.0 * M_PI * cg->rcut * cg->rcut);
        double r2 = dr_sq / rcutsq;
        return norm * exp(-1.0 / (1 - r2));
    }
    case IKOR_CG_GAUSSIAN: {
        double w2 = cg->width * cg->width;
        double norm = (dim == 3) ? 1.0 / ((2.0 * M_PI * w2) * sqrt(2.0 * M_PI * w2)) : 1.0 / (2.0 * M_PI * w2);
        return norm * exp(-dr_sq / (2.0 * w2));
    }
    }
    return 0.0;
}

/* getObjFunc(s) = getDeltaFunc(x, ri + s*rij)  (CoarseGrainFunction.h:42-45, 78-83) */
static double obj(const ikor_cg* cg, int dim, const double x[3], const double ri[3],
                  const double rij[3], double s)
{
    double p0 = ri[0] + s * rij[0], p1 = ri[1] + s * rij[1], p2 = ri[2] + s * rij[2];
    double d0 = x[0] - p0, d1 = x[1] - p1, d2 = x[2] - p2;
    return ikor_delta(cg, dim, d0 * d0 + d1 * d1 + d2 * d2);
}

/* ---- Gauss-Kronrod 7/15 pair, computed from first principles --------------
 * The 8 Kronrod nodes are the zeros of the Stieltjes polynomial E_8 (even),
 * defined by orthogonality of E_8 to x^k (k < 8) under the weight P_7(x) on
 * [-1,1]; the 15 weights make the rule exact for degree <= 22 (Kronrod 1965;
 * the rule used by QUADPACK's QAG key=1, Piessens et al. 1983). */
static double gk_x[8], gk_wk[8], gk_wg[4]; /* x ascending from 0: gk_x[0]=0 */
static int gk_ready = 0;

static long double legendre_coef7(int m)
{
    /* P_7(x) = (429x^7 - 693x^5 + 315x^3 - 35x)/16 */
    switch (m) { case 7: return 429.0L / 16; case 5: return -693.0L / 16;
                 case 3: return 315.0L / 16; case 1: return -35.0L / 16; }
    return 0.0L;
}

static long double mom7(int m) /* int_{-1}^{1} P_7(x) x^m dx */
{
    long double s = 0.0L;
    for (int l = 1; l <= 7; l += 2) {
        int e = l + m;
        if (e % 2 == 0) s += legendre_coef7(l) * 2.0L / (e + 1);
    }
    return s;
}

static void gk15_build(void)
{
    /* E_8 = x^8 + a6 x^6 + a4 x^4 + a2 x^2 + a0; conditions k = 1,3,5,7 */
    long double M7 = mom7(7), M9 = mom7(9), M11 = mom7(11), M13 = mom7(13), M15 = mom7(15);
    long double a6 = -M9 / M7;
    long double a4 = (-M11 - a6 * M9) / M7;
    long double a2 = (-M13 - a4 * M9 - a6 * M11) / M7;
    long double a0 = (-M15 - a2 * M9 - a4 * M11 - a6 * M13) / M7;
    /* Gauss-7 nodes */
    double gx[7], gw[7];
    ikor_gl_rule(7, gx, gw);
    /* positive Gauss nodes: gx[4], gx[5], gx[6]; Kronrod nodes interlace:
     * 0 < k1 < g1 < k2 < g2 < k3 < g3 < k4 < 1 */
    long double brk[5] = {0.0L, gx[4], gx[5], gx[6], 1.0L};
    long double kn[4];
    for (int r = 0; r < 4; ++r) {
        long double lo = brk[r], hi = brk[r + 1];
        /* bisection then Newton on E_8 */
        for (int it = 0; it < 200; ++it) {
            long double mid = 0.5L * (lo + hi);
            long double x2 = lo * lo, fl = (((x2 + a6) * x2 + a4) * x2 + a2) * x2 + a0;
            long double m2 = mid * mid, fm = (((m2 + a6) * m2 + a4) * m2 + a2) * m2 + a0;
            if ((fl < 0) == (fm < 0)) lo = mid; else hi = mid;
        }
        kn[r] = 0.5L * (lo + hi);
    }
    long double nodes[8] = {0.0L, kn[0], gx[4], kn[1], gx[5], kn[2], gx[6], kn[3]};
    /* weights: exactness on x^(2m), m = 0..7:  w0*[m==0] + 2*sum_i w_i x_i^(2m) = 2/(2m+1) */
    long double A[8][9];
    for (int m = 0; m < 8; ++m) {
        for (int i = 0; i < 8; ++i) {
            long double v = (i == 0) ? (m == 0 ? 1.0L : 0.0L) : 2.0L * powl(nodes[i], 2 * m);
            A[m][i] = v;
        }
        A[m][8] = 2.0L / (2 * m + 1);
    }
    for (int c = 0; c < 8; ++c) { /* Gaussian elimination with partial pivoting */
        int piv = c;
        for (int r = c + 1; r < 8; ++r) if (fabsl(A[r][c]) > fabsl(A[piv][c])) piv = r;
        for (int k = 0; k < 9; ++k) { long double t = A[c][k]; A[c][k] = A[piv][k]; A[piv][k] = t; }
        for (int r = 0; r < 8; ++r) {
            if (r == c) continue;
            long double f = A[r][c] / A[c][c];
            for (int k = c; k < 9; ++k) A[r][k] -= f * A[c][k];
        }
    }
    for (int i = 0; i < 8; ++i) { gk_x[i] = (double)nodes[i]; gk_wk[i] = (double)(A[i][8] / A[i][i]); }
    gk_wg[0] = gw[3]; gk_wg[1] = gw[4]; gk_wg[2] = gw[5]; gk_wg[3] = gw[6];
}

/* built once, as the GL tables: the first caller under a lock, the rest after an acquire load */
static void gk15_init(void)
{
    if (__atomic_load_n(&gk_ready, __ATOMIC_ACQUIRE)) return;
#pragma omp critical(ikor_rules)
    {
        if (!__atomic_load_n(&gk_ready, __ATOMIC_RELAXED)) {
            gk15_build();
            __atomic_store_n(&gk_ready, 1, __ATOMIC_RELEASE);
        }
    }
}

/* exported for the pin tests */
void ikor_gk15_rule(double* x8, double* wk8, double* wg4)
{
    gk15_init();
    memcpy(x8, gk_x, sizeof gk_x); memcpy(wk8, gk_wk, sizeof gk_wk); memcpy(wg4, gk_wg, sizeof gk_wg);
}

/* one GK15 application on [a,b]; QUADPACK-style error estimate */
static double gk15_apply(const ikor_cg* cg, int dim, const double x[3], const double ri[3],
                         const double rij[3], double a, double b, double* err)
{
    double c = 0.5 * (a + b), h = 0.5 * (b - a);
    double fc = obj(cg, dim, x, ri, rij, c);
    double rk = fc * gk_wk[0], rg = 0.0, rabs = fabs(rk);
    double fv1[8], fv2[8];
    for (int i = 1; i < 8; ++i) {
        double f1 = obj(cg, dim, x, ri, rij, c - h * gk_x[i]);
        double f2 = obj(cg, dim, x, ri, rij, c + h * gk_x[i]);
        fv1[i] = f1; fv2[i] = f2;
        rk += gk_wk[i] * (f1 + f2);
        rabs += gk_wk[i] * (fabs(f1) + fabs(f2));
        if (i % 2 == 0) rg += gk_wg[i / 2] * (f1 + f2); /* Gauss nodes at even slots */
    }
    /* centre is a Gauss node for n = 7 (weight gk_wg[0]) */
    rg += gk_wg[0] * fc;
    double mean = 0.5 * rk, rasc = gk_wk[0] * fabs(fc - mean);
    for (int i = 1; i < 8; ++i) rasc += gk_wk[i] * (fabs(fv1[i] - mean) + fabs(fv2[i] - mean));
    double result = rk * h, e = fabs((rk - rg) * h);
    rasc *= fabs(h); rabs *= fabs(h);
    if (rasc != 0.0 && e != 0.0) { double t = pow(200.0 * e / rasc, 1.5); e = rasc * (t < 1.0 ? t : 1.0); }
    if (rabs > 2.2250738585072014e-308 / (50.0 * 2.220446049250313e-16)) {
        double m = 50.0 * 2.220446049250313e-16 * rabs; if (m > e) e = m;
    }
    *err = e;
    return result;
}

/* QAG strategy: repeatedly bisect the subinterval with the largest error
 * estimate until the total estimate meets max(epsabs, epsrel*|I|) or `limit`
 * subintervals exist (Piessens et al. 1983, QUADPACK).  Replaces
 * gsl_integration_qag(..., key=1, ...)  (irvingkirkwood/cgfunc/Quadrature.h:47-49). */
static double qag15(const ikor_cg* cg, int dim, const double x[3], const double ri[3],
                    const double rij[3], double a, double b)
{
    gk15_init();
    int limit = cg->limit > 0 ? cg->limit : 1000;
    if (limit > 4096) limit = 4096;
    double* ia = (double*)malloc(sizeof(double) * 4 * limit);
    double *ib = ia + limit, *ir = ib + limit, *ie = ir + limit;
    int n = 1;
    ia[0] = a; ib[0] = b; ir[0] = gk15_apply(cg, dim, x, ri, rij, a, b, &ie[0]);
    double res = ir[0], err = ie[0];
    while (n < limit) {
        double tol = fmax(cg->epsabs, cg->epsrel * fabs(res));
        if (err <= tol) break;
        int worst = 0;
        for (int k = 1; k < n; ++k) if (ie[k] > ie[worst]) worst = k;
        double a1 = ia[worst], b2 = ib[worst], m = 0.5 * (a1 + b2);
        double e1, e2;
        double r1 = gk15_apply(cg, dim, x, ri, rij, a1, m, &e1);
        double r2 = gk15_apply(cg, dim, x, ri, rij, m, b2, &e2);
        ib[worst] = m; ir[worst] = r1; ie[worst] = e1;
        ia[n] = m; ib[n] = b2; ir[n] = r2; ie[n] = e2; ++n;
        res = 0.0; err = 0.0;
        for (int k = 0; k < n; ++k) { res += ir[k]; err += ie[k]; }
        if (m <= a1 || m >= b2) break; /* interval exhausted */
    }
    free(ia);
    return res;
}

/* Clip the parameter range [0,1] of the segment ri + s*rij to the open ball
 * |x - ri - s*rij| < R.  Returns 0 if empty. */
static int clip_segment(const double u[3], const double b[3], double R, double* s0, double* s1)
{
    double bb = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
    double ub = u[0] * b[0] + u[1] * b[1] + u[2] * b[2];
    double uu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    if (bb == 0.0) { if (uu < R * R) { *s0 = 0; *s1 = 1; return 1; } return 0; }
    double disc = ub * ub - bb * (uu - R * R);
    if (disc <= 0.0) return 0;
    double sq = sqrt(disc);
    /* stable roots */
    double q = ub + (ub >= 0 ? sq : -sq);
    double ra = q / bb, rb = (q != 0.0) ? (uu - R * R) / q : ra;
    double lo = ra < rb ? ra : rb, hi = ra < rb ? rb : ra;
    if (lo < 0.0) lo = 0.0;
    if (hi > 1.0) hi = 1.0;
    if (!(hi > lo)) return 0;
    *s0 = lo; *s1 = hi;
    return 1;
}

/* Exact bond integral (new mode, used as the reference for the learned
 * surrogate and the closed-form GPU mode):
 *   Gaussian: clip to the ball, then the erf closed form along the line;
 *   Octic:    clip to the ball, then GL-5 on the clipped interval (the integrand
 *             is a degree-8 polynomial in s there, integrated exactly);
 *   Rect:     clipped length / (pi R^2);
 *   Mollifier: no closed form -> adaptive GK15 at 1e-12. */
static double bond_exact(const ikor_cg* cg, int dim, const double x[3], const double ri[3], const double rij[3])
{
    double u[3] = {x[0] - ri[0], x[1] - ri[1], x[2] - ri[2]};
    double s0, s1;
    if (cg->kind == IKOR_CG_MOLLIFIER) {
        ikor_cg c2 = *cg; c2.epsabs = 1e-14; c2.epsrel = 1e-12; c2.limit = 2000;
        if (!clip_segment(u, rij, cg->rcut, &s0, &s1)) return 0.0;
        return qag15(&c2, dim, x, ri, rij, s0, s1);
    }
    if (!clip_segment(u, rij, cg->rcut, &s0, &s1)) return 0.0;
    double bb = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
    if (cg->kind == IKOR_CG_RECT) return ikor_delta(cg, dim, 0.0) * (s1 - s0);
    if (cg->kind == IKOR_CG_OCTIC || bb == 0.0) {
        const double *gx, *gw;
        gl_rule_cached(5, &gx, &gw);
        double c = 0.5 * (s0 + s1), h = 0.5 * (s1 - s0), acc = 0.0;
        if (bb == 0.0) return ikor_delta(cg, dim, u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        for (int k = 0; k < 5; ++k) {
            double s = c + h * gx[k];
            double d0 = u[0] - s * rij[0], d1 = u[1] - s * rij[1], d2 = u[2] - s * rij[2];
            double r2 = d0 * d0 + d1 * d1 + d2 * d2;
            double rc2 = cg->rcut * cg->rcut;
            /* inside the clipped interval the untruncated polynomial applies */
            double r4 = r2 * r2 / (rc2 * rc2);
            acc += gw[k] * (15.0 / (8 * M_PI * rc2) * (1 - 2 * r4 + r4 * r4));
        }
        return acc * h;
    }
    /* Gaussian */
    double w = cg->width;
    double ub = u[0] * rij[0] + u[1] * rij[1] + u[2] * rij[2];
    double sstar = ub / bb;
    double p0 = u[0] - sstar * rij[0], p1 = u[1] - sstar * rij[1], p2 = u[2] - sstar * rij[2];
    double dperp2 = p0 * p0 + p1 * p1 + p2 * p2;
    double blen = sqrt(bb);
    double k = blen / (sqrt(2.0) * w);
    double ta = (s0 - sstar) * k, tb = (s1 - sstar) * k;
    double diff;
    if (ta >= 0.0) diff = erfc(ta) - erfc(tb);
    else if (tb <= 0.0) diff = erfc(-tb) - erfc(-ta);
    else diff = erf(tb) - erf(ta);
    double norm = ikor_delta(cg, dim, 0.0);
    return norm * exp(-dperp2 / (2.0 * w * w)) * sqrt(M_PI / 2.0) * (w / blen) * diff;
}

double ikor_bond(const ikor_cg* cg, int dim, const double x[3], const double ri[3], const double rij[3])
{
    if (cg->mode == IKOR_QUAD_EXACT) return bond_exact(cg, dim, x, ri, rij);
    if (cg->mode == IKOR_QUAD_ADAPTIVE) return qag15(cg, dim, x, ri, rij, 0.0, 1.0);
    /* fixed point: GL-n on [0,1]  (CoarseGrainFunction.h:85-88, FixedPointQuadrature.h:39-46) */
    int n = cg->order > 0 ? cg->order : 1;
    if (n > 64) n = 64;
    const double *gx, *gw;
    gl_rule_cached(n, &gx, &gw);
    double acc = 0.0;
    for (int k = 0; k < n; ++k) acc += gw[k] * obj(cg, dim, x, ri, rij, 0.5 + 0.5 * gx[k]);
    return 0.5 * acc;
}

/* ------------------------------------------------------------------------- */
double ikor_max_rcut(double scaled_rcut, int64_t n, const double* diam)
{
    double dmax = diam[0];
    for (int64_t i = 1; i < n; ++i) if (diam[i] > dmax) dmax = diam[i];
    double m = scaled_rcut * dmax;
    return m > dmax ? m : dmax;
}

/* Minimum image along periodic axes: d - L*rint(d/L) (round half to even). */
void ikor_min_image(const ikor_box* box, const double a[3], const double b[3], double out[3])
{
    for (int c = 0; c < 3; ++c) {
        double d = b[c] - a[c];
        if (box->periodic[c]) {
            double k = nearbyint(d / box->L[c]);
            double s = box->L[c] * k;
            d = d - s;
        }
        out[c] = d;
    }
}

/* ---- uniform cell list (the role Aboria's init_neighbour_search plays,
 *      ParticleSystem.cc:13) ------------------------------------------------ */
typedef struct {
    int nc[3];
    double cw[3];
    int64_t* start; /* ncells + 1 */
    int64_t* items; /* particle ids, ascending within a cell */
} cell_list;

static int cell_coord(const ikor_box* box, const cell_list* cl, int c, double x)
{
    if (cl->nc[c] == 1) return 0;
    double t = (x - box->lo[c]) / box->L[c];
    t -= floor(t);
    int k = (int)(t * cl->nc[c]);
    if (k < 0) k = 0;
    if (k >= cl->nc[c]) k = cl->nc[c] - 1;
    return k;
}

static void cell_build(const ikor_box* box, int64_t n, const double* pos, double cs, cell_list* cl)
{
    for (int c = 0; c < 3; ++c) {
        int nc = 1;
        if (box->periodic[c] && c < box->dim) {
            nc = (int)floor(box->L[c] / cs);
            if (nc < 1) nc = 1;
        }
        cl->nc[c] = nc;
        cl->cw[c] = box->L[c] / nc;
    }
    int64_t ncell = (int64_t)cl->nc[0] * cl->nc[1] * cl->nc[2];
    cl->start = (int64_t*)calloc((size_t)ncell + 1, sizeof(int64_t));
    cl->items = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    int64_t* cid = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) {
        int cx = cell_coord(box, cl, 0, pos[3 * i]);
        int cy = cell_coord(box, cl, 1, pos[3 * i + 1]);
        int cz = cell_coord(box, cl, 2, pos[3 * i + 2]);
        cid[i] = ((int64_t)cz * cl->nc[1] + cy) * cl->nc[0] + cx;
        cl->start[cid[i] + 1]++;
    }
    for (int64_t k = 0; k < ncell; ++k) cl->start[k + 1] += cl->start[k];
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)(ncell + 1));
    memcpy(fill, cl->start, sizeof(int64_t) * (size_t)(ncell + 1));
    for (int64_t i = 0; i < n; ++i) cl->items[fill[cid[i]]++] = i; /* ascending i */
    free(fill);
    free(cid);
}

static void cell_free(cell_list* cl) { free(cl->start); free(cl->items); }

/* visit each cell whose particles may lie within `radius` of q, each once */
typedef void (*visit_fn)(void* ctx, int64_t j);
static void cell_query(const ikor_box* box, const cell_list* cl, const double q[3], double radius,
                       visit_fn fn, void* ctx)
{
    int lo[3], hi[3], all[3];
    for (int c = 0; c < 3; ++c) {
        int nc = cl->nc[c];
        if (nc == 1) { lo[c] = 0; hi[c] = 0; all[c] = 1; continue; }
        int reach = (int)ceil(radius / cl->cw[c]);
        if (2 * reach + 1 >= nc) { lo[c] = 0; hi[c] = nc - 1; all[c] = 1; continue; }
        int k = cell_coord(box, cl, c, q[c]);
        lo[c] = k - reach; hi[c] = k + reach; all[c] = 0;
    }
    for (int z = lo[2]; z <= hi[2]; ++z) {
        int cz = all[2] ? z : ((z % cl->nc[2]) + cl->nc[2]) % cl->nc[2];
        for (int y = lo[1]; y <= hi[1]; ++y) {
            int cy = all[1] ? y : ((y % cl->nc[1]) + cl->nc[1]) % cl->nc[1];
            for (int x = lo[0]; x <= hi[0]; ++x) {
                int cx = all[0] ? x : ((x % cl->nc[0]) + cl->nc[0]) % cl->nc[0];
                int64_t cell = ((int64_t)cz * cl->nc[1] + cy) * cl->nc[0] + cx;
                for (int64_t k = cl->start[cell]; k < cl->start[cell + 1]; ++k) fn(ctx, cl->items[k]);
            }
        }
    }
}

static double dot3(const double a[3]) { return a[0] * a[0] + a[1] * a[1] + a[2] * a[2]; }

typedef struct {
    const ikor_box* box; const double* pos; int64_t i; double r2;
    int32_t* out; int64_t cnt; int64_t cap;
} nb_ctx;

static void nb_visit(void* vctx, int64_t j)
{
    nb_ctx* c = (nb_ctx*)vctx;
    if (j == c->i) return;
    double d[3];
    ikor_min_image(c->box, &c->pos[3 * c->i], &c->pos[3 * j], d);
    if (dot3(d) < c->r2) {
        if (c->out && c->cnt < c->cap) c->out[c->cnt] = (int32_t)j;
        c->cnt++;
    }
}

static int cmp_i32(const void* a, const void* b)
{
    int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
    return (x > y) - (x < y);
}

int64_t ikor_neighbors(const ikor_box* box, int64_t n, const double* pos, double radius,
                       int64_t* offs, int32_t* idx)
{
    cell_list cl;
    cell_build(box, n, pos, radius, &cl);
    int64_t total = 0;
    offs[0] = 0;
    for (int64_t i = 0; i < n; ++i) {
        nb_ctx c = {box, pos, i, radius * radius, idx ? idx + total : NULL, 0,
                    idx ? (int64_t)1 << 62 : 0};
        cell_query(box, &cl, &pos[3 * i], radius, nb_visit, &c);
        if (idx) qsort(idx + total, (size_t)c.cnt, sizeof(int32_t), cmp_i32);
        total += c.cnt;
        offs[i + 1] = total;
    }
    cell_free(&cl);
    return total;
}

/* ------------------------------------------------------------------------- */
/* The IK gather: IrvingKirkwood::compute (irvingkirkwood/IrvingKirkwood.h:74-110)
 * with VirialStress::compute_cg (ListofCommonObservables.h:49-82) and the
 * intended KineticStress (ListofCommonObservables.h:131-142, m v(x)v * Delta). */
typedef struct {
    const ikor_box* box; const double* pos; const double* vel; const double* mass;
    const double* diam; const ikor_pot* pot; const ikor_cg* cg;
    const int64_t* noff; const int32_t* nidx;
    const double* x; double* vir; double* kin; int dim;
    const double* disp; double* ela; /* elastic virial (ElasticVirialStress), or NULL */
} g_ctx;

static void g_visit(void* vctx, int64_t i)
{
    g_ctx* c = (g_ctx*)vctx;
    const ikor_box* box = c->box;
    const double* x = c->x;
    double dr[3];
    /* p_i.dx(): x - r_i, minimum image */
    ikor_min_image(box, &c->pos[3 * i], x, dr);
    double R = c->cg->rcut;
    if (!(dot3(dr) < R * R)) return;
    double ri[3] = {x[0] - dr[0], x[1] - dr[1], x[2] - dr[2]};
    double e[3] = {x[0] - ri[0], x[1] - ri[1], x[2] - ri[2]};
    double cgval = ikor_delta(c->cg, c->dim, dot3(e));
    int D = c->dim;
    if (c->vel && c->mass) {
        const double* v = &c->vel[3 * i];
        for (int b = 0; b < D; ++b)
            for (int a = 0; a < D; ++a)
                c->kin[a + D * b] += (c->mass[i] * v[a] * v[b]) * cgval;
    }
    for (int64_t k = c->noff[i]; k < c->noff[i + 1]; ++k) {
        int64_t j = c->nidx[k];
        double rij[3];
        ikor_min_image(box, &c->pos[3 * i], &c->pos[3 * j], rij); /* r_j - r_i */
        double bondval = ikor_bond(c->cg, D, x, ri, rij);
        double fdr = ikor_force_divr(c->pot, dot3(rij), c->diam[i], c->diam[j]);
        double hb = 0.5 * bondval;
        for (int b = 0; b < D; ++b)
            for (int a = 0; a < D; ++a)
                c->vir[a + D * b] += hb * ((fdr * rij[a]) * rij[b]);
        if (c->ela) {
            /* ElasticVirialStress::compute (ListofCommonObservables.h:86-122) through
             * VirialStress::compute_cg (:72-82): the pair force at the displaced
             * separation r + u_ij (u_ij = u_j - u_i) minus the force at r, times
             * 0.5 * bond */
            const double* ui = &c->disp[3 * i];
            const double* uj = &c->disp[3 * j];
            double uij[3] = {uj[0] - ui[0], uj[1] - ui[1], uj[2] - ui[2]};
            double ur[3] = {uij[0] + rij[0], uij[1] + rij[1], uij[2] + rij[2]};
            double f1 = ikor_force_divr(c->pot, dot3(ur), c->diam[i], c->diam[j]);
            for (int b = 0; b < D; ++b)
                for (int a = 0; a < D; ++a) {
                    double t = (f1 * ur[a]) * ur[b] - (fdr * rij[a]) * rij[b];
                    c->ela[a + D * b] += hb * t;
                }
        }
    }
}

static int compute_impl(const ikor_box* box, int64_t n, const double* pos, const double* vel,
                        const double* mass, const double* diam, const double* disp,
                        const ikor_pot* pot, const ikor_cg* cg, double max_rcut, int64_t g0,
                        int64_t g1, const double* grid, double* virial, double* kinetic,
                        double* elastic, int nthreads);

int ikor_compute_range(const ikor_box* box, int64_t n, const double* pos, const double* vel,
                       const double* mass, const double* diam, const ikor_pot* pot,
                       const ikor_cg* cg, double max_rcut, int64_t g0, int64_t g1,
                       const double* grid, double* virial, double* kinetic, int nthreads)
{
    return compute_impl(box, n, pos, vel, mass, diam, NULL, pot, cg, max_rcut, g0, g1, grid, virial,
                        kinetic, NULL, nthreads);
}

int ikor_compute_elastic(const ikor_box* box, int64_t n, const double* pos, const double* disp,
                         const double* diam, const ikor_pot* pot, const ikor_cg* cg,
                         double max_rcut, int64_t g0, int64_t g1, const double* grid,
                         double* virial, double* elastic, int nthreads)
{
    return compute_impl(box, n, pos, NULL, NULL, diam, disp, pot, cg, max_rcut, g0, g1, grid, virial,
                        NULL, elastic, nthreads);
}

static int compute_impl(const ikor_box* box, int64_t n, const double* pos, const double* vel,
                        const double* mass, const double* diam, const double* disp,
                        const ikor_pot* pot, const ikor_cg* cg, double max_rcut, int64_t g0,
                        int64_t g1, const double* grid, double* virial, double* kinetic,
                        double* elastic, int nthreads)
{
    int D = box->dim;
    if (D != 2 && D != 3) return -1;
    if (n < 0 || g1 < g0) return -1;
    for (int c = 0; c < D; ++c)
        if (box->periodic[c] && (2.0 * max_rcut >= box->L[c] || 2.0 * cg->rcut >= box->L[c])) return -2;
    int64_t* noff = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 1));
    int64_t nnz = ikor_neighbors(box, n, pos, max_rcut, noff, NULL);
    int32_t* nidx = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1));
    ikor_neighbors(box, n, pos, max_rcut, noff, nidx);
    cell_list cl;
    cell_build(box, n, pos, cg->rcut, &cl);
    int64_t DD = (int64_t)D * D;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t g = g0; g < g1; ++g) {
        double* vir = &virial[(g - g0) * DD];
        double* kin = kinetic ? &kinetic[(g - g0) * DD] : NULL;
        double* ela = elastic ? &elastic[(g - g0) * DD] : NULL;
        double kdummy[9];
        for (int k = 0; k < DD; ++k) { vir[k] = 0.0; if (kin) kin[k] = 0.0; if (ela) ela[k] = 0.0; }
        g_ctx c = {box, pos, vel, mass, diam, pot, cg, noff, nidx, &grid[3 * g], vir,
                   kin ? kin : kdummy, D, disp, ela};
        if (!kin) { c.vel = NULL; }
        cell_query(box, &cl, &grid[3 * g], cg->rcut, g_visit, &c);
    }
    cell_free(&cl);
    free(noff);
    free(nidx);
    return 0;
}

int ikor_compute(const ikor_box* box, int64_t n, const double* pos, const double* vel,
                 const double* mass, const double* diam, const ikor_pot* pot,
                 const ikor_cg* cg, double max_rcut, int64_t g, const double* grid,
                 double* virial, double* kinetic, int nthreads)
{
    return ikor_compute_range(box, n, pos, vel, mass, diam, pot, cg, max_rcut, 0, g, grid,
                              virial, kinetic, nthreads);
}

/* ThermoCalculator::compute pair part (thermo/ThermoCalculator.h:68-90):
 * sum over i < j of F (x) r_ij with F = forceDivR * r_ij. */
void ikor_global_virial(const ikor_box* box, int64_t n, const double* pos, const double* diam,
                        const ikor_pot* pot, double max_rcut, double* out)
{
    int D = box->dim;
    for (int k = 0; k < D * D; ++k) out[k] = 0.0;
    int64_t* noff = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 1));
    int64_t nnz = ikor_neighbors(box, n, pos, max_rcut, noff, NULL);
    int32_t* nidx = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1));
    ikor_neighbors(box, n, pos, max_rcut, noff, nidx);
    for (int64_t i = 0; i < n; ++i)
        for (int64_t k = noff[i]; k < noff[i + 1]; ++k) {
            int64_t j = nidx[k];
            if (!(i < j)) continue;
            double rij[3];
            ikor_min_image(box, &pos[3 * j], &pos[3 * i], rij); /* p_j.dx() = r_i - r_j */
            double f = ikor_force_divr(pot, dot3(rij), diam[i], diam[j]);
            for (int b = 0; b < D; ++b)
                for (int a = 0; a < D; ++a) out[a + D * b] += (f * rij[a]) * rij[b];
        }
    free(noff);
    free(nidx);
}

/* ThermoCalculator::compute (thermo/ThermoCalculator.h:68-90) with every global observable
 * of thermo/module-thermo.cpp:7-20: particles i in id order, neighbours j within max_rcut
 * with i < j, r_ij = p_j.dx() = r_i - r_j (min image), then everything times 1/vol
 * (ThermoProperty.h divideByVolume; vol = SimBox::vol, SimBox.cc:15-22).
 *   PotentialEnergy      sum getPairEnergy                      (ListofCommonObservables.h:10-28)
 *   VirialStress         (f r_a) r_b                            (:43-70)
 *   ElasticVirialStress  F1_a (u+r)_b - F_a r_b, u = u_j - u_i  (:86-122)
 *   KineticStress        (m v_a) v_b per particle               (:125-140)
 *   BornStiffnessTensor  (s r_i + F_i) r_j n_k n_l, n = r/|r|   (:150-183)
 * out: [0] energy, [1..] virial, elastic virial, kinetic (D x D each, index a + D b), Born
 * (D^4, index i + D (j + D (k + D l))).  disp / vel / mass may be NULL (zero / zero / one). */
void ikor_global_thermo(const ikor_box* box, int64_t n, const double* pos, const double* vel, const double* mass,
                        const double* diam, const double* disp, const ikor_pot* pot, double max_rcut, double* out)
{
    int D = box->dim, D2 = D * D, D4 = D2 * D2;
    double* pe = out;
    double* vir = out + 1;
    double* ela = vir + D2;
    double* kin = ela + D2;
    double* born = kin + D2;
    for (int k = 0; k < 1 + 3 * D2 + D4; ++k) out[k] = 0.0;
    int64_t* noff = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 1));
    int64_t nnz = ikor_neighbors(box, n, pos, max_rcut, noff, NULL);
    int32_t* nidx = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1));
    ikor_neighbors(box, n, pos, max_rcut, noff, nidx);
    double vol = D == 2 ? box->L[0] * box->L[1] : box->L[0] * box->L[1] * box->L[2];
    for (int64_t i = 0; i < n; ++i) {
        double m = mass ? mass[i] : 1.0;
        if (vel)
            for (int b = 0; b < D; ++b)
                for (int a = 0; a < D; ++a) kin[a + D * b] += m * vel[3 * i + a] * vel[3 * i + b];
        for (int64_t k = noff[i]; k < noff[i + 1]; ++k) {
            int64_t j = nidx[k];
            if (!(i < j)) continue;
            double rij[3];
            ikor_min_image(box, &pos[3 * j], &pos[3 * i], rij);
            double rsq = dot3(rij);
            pe[0] += ikor_pair_energy(pot, rsq, diam[i], diam[j]);
            double f = ikor_force_divr(pot, rsq, diam[i], diam[j]);
            double F[3] = {f * rij[0], f * rij[1], f * rij[2]};
            for (int b = 0; b < D; ++b)
                for (int a = 0; a < D; ++a) vir[a + D * b] += F[a] * rij[b];
            if (disp) {
                double w[3];
                for (int c = 0; c < 3; ++c) w[c] = (disp[3 * j + c] - disp[3 * i + c]) + rij[c];
                double f1 = ikor_force_divr(pot, dot3(w), diam[i], diam[j]);
                double F1[3] = {f1 * w[0], f1 * w[1], f1 * w[2]};
                for (int b = 0; b < D; ++b)
                    for (int a = 0; a < D; ++a) ela[a + D * b] += F1[a] * w[b] - F[a] * rij[b];
            }
            double st = ikor_bond_stiffness(pot, rsq, diam[i], diam[j]);
            double nr = sqrt(rsq);
            double nv[3] = {rij[0] / nr, rij[1] / nr, rij[2] / nr};
            for (int l = 0; l < D; ++l)
                for (int kk = 0; kk < D; ++kk)
                    for (int jj = 0; jj < D; ++jj)
                        for (int ii = 0; ii < D; ++ii)
                            born[ii + D * (jj + D * (kk + D * l))] += (st * rij[ii] + F[ii]) * rij[jj] * nv[kk] * nv[l];
        }
    }
    double iv = 1 / vol;
    for (int k = 0; k < 1 + 3 * D2 + D4; ++k) out[k] = out[k] * iv;
    free(noff);
    free(nidx);
}

/* Threads an OpenMP region of the oracle runs on after asking for `requested` (0: the
 * default); 1 when the library was built without OpenMP. */
int ikor_threads(int requested)
{
#ifdef _OPENMP
    if (requested > 0) omp_set_num_threads(requested);
    int n = 1;
#pragma omp parallel
    {
#pragma omp single
        n = omp_get_num_threads();
    }
    return n;
#else
    (void)requested;
    return 1;
#endif
}
