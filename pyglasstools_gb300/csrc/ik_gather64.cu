// ik_gather64.cu -- the plain FP64 Irving-Kirkwood gather (one thread per grid
// point) and scalar bond-integral evaluation.
//
// Straight FP64 restatement of IrvingKirkwood::compute
// (irvingkirkwood/IrvingKirkwood.h:74-110): per grid point, particles i with
// |x - r_i| < R (minimum image, ri = x - dx), kinetic term m v(x)v Delta(x - ri),
// and for each force-active bond (i, j) the Gauss-Legendre bond integral of
// FixedPointCGFunc::getBondFunc (cgfunc/CoarseGrainFunction.h:85-88) times
// 0.5 * forceDivR * r_ij (x) r_ij (ListofCommonObservables.h:57-81).
#include "ik_kernels.h"

// Exact bond integral (no reference counterpart; the answer the fixed-point rule and
// the learned surrogate approximate): clip the segment r_i + s r_ij, s in [0, 1], to
// the open ball |x - r| < R, then
//   Gaussian: the error-function closed form along the line,
//   others:   Gauss-Legendre on the clipped interval (exact for the octic's degree-8
//             polynomial at n >= 5).
__device__ double ik_bond64_exact(const IkCG& cg, const double* xs, const double* ws, int nq, const double x[3],
                                  const double ri[3], const double rij[3])
{
    const double u0 = x[0] - ri[0], u1 = x[1] - ri[1], u2 = x[2] - ri[2];
    const double bb = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
    const double ub = u0 * rij[0] + u1 * rij[1] + u2 * rij[2];
    const double uu = u0 * u0 + u1 * u1 + u2 * u2;
    if (bb == 0.0) return ik_delta64(cg, uu);
    const double disc = ub * ub - bb * (uu - cg.rcutsq);
    if (!(disc > 0.0)) return 0.0;
    const double sq = sqrt(disc);
    const double qq = ub + (ub >= 0.0 ? sq : -sq); // roots without cancellation
    const double ra = qq / bb, rb = qq != 0.0 ? (uu - cg.rcutsq) / qq : ra;
    const double s0 = fmax(fmin(ra, rb), 0.0), s1 = fmin(fmax(ra, rb), 1.0);
    if (!(s1 > s0)) return 0.0;
    if (cg.kind == 1) {
        const double w = cg.width, sstar = ub / bb;
        const double p0 = u0 - sstar * rij[0], p1 = u1 - sstar * rij[1], p2 = u2 - sstar * rij[2];
        const double dperp2 = p0 * p0 + p1 * p1 + p2 * p2;
        const double blen = sqrt(bb), k = blen / (1.4142135623730951 * w);
        const double ta = (s0 - sstar) * k, tb = (s1 - sstar) * k;
        double diff;
        if (ta >= 0.0) diff = erfc(ta) - erfc(tb);
        else if (tb <= 0.0) diff = erfc(-tb) - erfc(-ta);
        else diff = erf(tb) - erf(ta);
        return cg.norm * exp(-dperp2 / (2.0 * w * w)) * 1.2533141373155003 * (w / blen) * diff;
    }
    double acc = 0.0;
    for (int k = 0; k < nq; ++k) {
        const double s = s0 + (s1 - s0) * xs[k];
        const double d0 = u0 - s * rij[0], d1 = u1 - s * rij[1], d2 = u2 - s * rij[2];
        const double r2 = fmin(d0 * d0 + d1 * d1 + d2 * d2, cg.rcutsq * (1.0 - 1e-15)); // inside by construction
        acc += ws[k] * ik_delta64(cg, r2);
    }
    return 0.5 * acc * (s1 - s0);
}

// Integrand of the bond integral: Delta(|x - (r_i + s r_ij)|^2)
// (CoarseGrainFunction::getObjFunc, cgfunc/CoarseGrainFunction.h:42-48).
__device__ __forceinline__ double ik_obj64(const IkCG& cg, const double x[3], const double ri[3],
                                           const double rij[3], double s)
{
    const double p0 = ri[0] + s * rij[0], p1 = ri[1] + s * rij[1], p2 = ri[2] + s * rij[2];
    const double d0 = x[0] - p0, d1 = x[1] - p1, d2 = x[2] - p2;
    return ik_delta64(cg, d0 * d0 + d1 * d1 + d2 * d2);
}

// One Gauss-Kronrod 7/15 application on [a, b] with the QUADPACK error estimate
// (Piessens et al. 1983): |K15 - G7| scaled by (200 |K15 - G7| / asc)^1.5, bounded below
// by 50 eps times the integral of |f|.
__device__ double ik_gk15(const IkCG& cg, const IkGK& gk, const double x[3], const double ri[3],
                          const double rij[3], double a, double b, double* err)
{
    const double c = 0.5 * (a + b), h = 0.5 * (b - a);
    const double fc = ik_obj64(cg, x, ri, rij, c);
    double rk = fc * gk.wk[0], rg = 0.0, rabs = fabs(rk);
    double f1[8], f2[8];
#pragma unroll
    for (int i = 1; i < 8; ++i) {
        f1[i] = ik_obj64(cg, x, ri, rij, c - h * gk.x[i]);
        f2[i] = ik_obj64(cg, x, ri, rij, c + h * gk.x[i]);
        rk += gk.wk[i] * (f1[i] + f2[i]);
        rabs += gk.wk[i] * (fabs(f1[i]) + fabs(f2[i]));
        if (i % 2 == 0) rg += gk.wg[i / 2] * (f1[i] + f2[i]);
    }
    rg += gk.wg[0] * fc;
    const double mean = 0.5 * rk;
    double rasc = gk.wk[0] * fabs(fc - mean);
#pragma unroll
    for (int i = 1; i < 8; ++i) rasc += gk.wk[i] * (fabs(f1[i] - mean) + fabs(f2[i] - mean));
    double e = fabs((rk - rg) * h);
    rasc *= fabs(h);
    rabs *= fabs(h);
    if (rasc != 0.0 && e != 0.0) e = rasc * fmin(pow(200.0 * e / rasc, 1.5), 1.0);
    const double eps = 2.220446049250313e-16;
    if (rabs > 2.2250738585072014e-308 / (50.0 * eps)) e = fmax(e, 50.0 * eps * rabs);
    *err = e;
    return rk * h;
}

// AdaptiveCGFunc::getBondFunc (cgfunc/CoarseGrainFunction.h:124-127): gsl_integration_qag
// with key 1 (GK15) on [0, 1] to max(abserr, relerr |B|), at most neval subintervals
// (cgfunc/Quadrature.h:47-49).  Strategy of QUADPACK's QAG: bisect the subinterval with
// the largest error estimate, sums recomputed in subinterval order.  Subintervals live in
// the thread's local memory (at most IK_QAG_MAXSUB); a tolerance missed when they run out
// sets IK_ST_QUAD_FAIL (the reference's GSL error handler would abort there).
__device__ double ik_bond64_qag(const IkCG& cg, const IkGK& gk, const double x[3], const double ri[3],
                                const double rij[3], int* status)
{
    double ia[IK_QAG_MAXSUB], ib[IK_QAG_MAXSUB], ir[IK_QAG_MAXSUB], ie[IK_QAG_MAXSUB];
    const int limit = cg.neval < 1 ? 1 : (cg.neval > IK_QAG_MAXSUB ? IK_QAG_MAXSUB : cg.neval);
    int n = 1;
    ia[0] = 0.0;
    ib[0] = 1.0;
    ir[0] = ik_gk15(cg, gk, x, ri, rij, 0.0, 1.0, &ie[0]);
    double res = ir[0], err = ie[0];
    bool done = false;
    while (n < limit) {
        if (err <= fmax(cg.abserr, cg.relerr * fabs(res))) { done = true; break; }
        int worst = 0;
        for (int k = 1; k < n; ++k)
            if (ie[k] > ie[worst]) worst = k;
        const double a1 = ia[worst], b2 = ib[worst], m = 0.5 * (a1 + b2);
        double e1, e2;
        const double r1 = ik_gk15(cg, gk, x, ri, rij, a1, m, &e1);
        const double r2 = ik_gk15(cg, gk, x, ri, rij, m, b2, &e2);
        ib[worst] = m; ir[worst] = r1; ie[worst] = e1;
        ia[n] = m; ib[n] = b2; ir[n] = r2; ie[n] = e2;
        ++n;
        res = 0.0;
        err = 0.0;
        for (int k = 0; k < n; ++k) { res += ir[k]; err += ie[k]; }
        if (m <= a1 || m >= b2) { done = true; break; } // interval exhausted
    }
    if (!done && !(err <= fmax(cg.abserr, cg.relerr * fabs(res)))) atomicOr(status, IK_ST_QUAD_FAIL);
    return res;
}

// ADAPT: the instantiation that carries the adaptive mode (its subinterval arrays cost
// local memory and registers the other modes do not pay).
template <bool ADAPT>
__device__ __forceinline__ double ik_bond64(const IkCG& cg, const double* xs, const double* ws, int nq,
                                            const IkGK& gk, int* status, const double x[3], const double ri[3],
                                            const double rij[3])
{
    if (cg.mode == IK_QUAD_EXACT_DEV) return ik_bond64_exact(cg, xs, ws, nq, x, ri, rij);
    if (ADAPT && cg.mode == IK_QUAD_ADAPTIVE_DEV) return ik_bond64_qag(cg, gk, x, ri, rij, status);
    double acc = 0.0;
    for (int k = 0; k < nq; ++k) {
        double s = xs[k];
        double p0 = ri[0] + s * rij[0], p1 = ri[1] + s * rij[1], p2 = ri[2] + s * rij[2];
        double d0 = x[0] - p0, d1 = x[1] - p1, d2 = x[2] - p2;
        acc += ws[k] * ik_delta64(cg, d0 * d0 + d1 * d1 + d2 * d2);
    }
    return 0.5 * acc;
}

template <int DIM, bool ADAPT>
__global__ void __launch_bounds__(128) k_gather64(const GatherArgs64 a)
{
    constexpr int NC = DIM == 2 ? 3 : 6;
    int64_t gidx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gidx >= a.ngrid) return;
    const IkGeom& g = a.g;
    double x[3] = {a.grid[3 * gidx], a.grid[3 * gidx + 1], a.grid[3 * gidx + 2]};
    double vir[NC], kin[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) { vir[c] = 0.0; kin[c] = 0.0; }
    const double R2 = a.cg.rcutsq;
    int home[3], lo[3], hi[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (c >= DIM || g.nc[c] == 1) { lo[c] = hi[c] = 0; home[c] = 0; continue; }
        home[c] = ik_cell_coord(g, c, x[c]);
        if (a.all[c]) { lo[c] = 0; hi[c] = g.nc[c] - 1; }
        else { lo[c] = home[c] - a.reach[c]; hi[c] = home[c] + a.reach[c]; }
    }
    const bool want_kin = (a.fields & 2) && a.vel;
    for (int zz = lo[2]; zz <= hi[2]; ++zz) {
        int wz = DIM == 3 ? ik_wrap(zz, g.nc[2]) : 0;
        for (int yy = lo[1]; yy <= hi[1]; ++yy) {
            int wy = ik_wrap(yy, g.nc[1]);
            for (int xx = lo[0]; xx <= hi[0]; ++xx) {
                int wx = ik_wrap(xx, g.nc[0]);
                int cell = (wz * g.nc[1] + wy) * g.nc[0] + wx;
                int e = a.cell_start[cell + 1];
                for (int q = a.cell_start[cell]; q < e; ++q) {
                    int i = a.sorted[q];
                    const double* pi = a.pos + 3 * (size_t)i;
                    double d0 = ik_minimg(__dsub_rn(x[0], pi[0]), g.L[0], g.periodic[0]);
                    double d1 = ik_minimg(__dsub_rn(x[1], pi[1]), g.L[1], g.periodic[1]);
                    double d2 = ik_minimg(__dsub_rn(x[2], pi[2]), g.L[2], g.periodic[2]);
                    if (!(ik_dot3(d0, d1, d2) < R2)) continue;
                    double ri[3] = {x[0] - d0, x[1] - d1, x[2] - d2};
                    if (want_kin) {
                        double e0 = x[0] - ri[0], e1 = x[1] - ri[1], e2 = x[2] - ri[2];
                        double cgval = ik_delta64(a.cg, e0 * e0 + e1 * e1 + e2 * e2);
                        double m = a.mass ? a.mass[i] : 1.0;
                        const double* v = a.vel + 3 * (size_t)i;
                        kin[0] += (m * v[0] * v[0]) * cgval;
                        kin[1] += (m * v[1] * v[1]) * cgval;
                        if (DIM == 2) {
                            kin[2] += (m * v[0] * v[1]) * cgval;
                        } else {
                            kin[2] += (m * v[2] * v[2]) * cgval;
                            kin[3] += (m * v[0] * v[1]) * cgval;
                            kin[4 % NC] += (m * v[0] * v[2]) * cgval;
                            kin[5 % NC] += (m * v[1] * v[2]) * cgval;
                        }
                    }
                    int nbq = a.nb[q];
                    const IkB64* bq = a.bonds + (size_t)q * a.maxb;
                    for (int k = 0; k < nbq; ++k) {
                        IkB64 b = bq[k];
                        double rij[3] = {b.x, b.y, b.z};
                        double bond = ik_bond64<ADAPT>(a.cg, a.xs, a.ws, a.nq, a.gk, a.status, x, ri, rij);
                        if (a.ecoef) { // elastic field: precomputed coefficients (0.5 included)
                            const double* cc = a.ecoef + ((size_t)q * a.maxb + k) * NC;
#pragma unroll
                            for (int cc_i = 0; cc_i < NC; ++cc_i) vir[cc_i] += bond * cc[cc_i];
                            continue;
                        }
                        double hb = 0.5 * bond, f = b.w;
                        vir[0] += hb * ((f * rij[0]) * rij[0]);
                        vir[1] += hb * ((f * rij[1]) * rij[1]);
                        if (DIM == 2) {
                            vir[2] += hb * ((f * rij[0]) * rij[1]);
                        } else {
                            vir[2] += hb * ((f * rij[2]) * rij[2]);
                            vir[3] += hb * ((f * rij[0]) * rij[1]);
                            vir[4 % NC] += hb * ((f * rij[0]) * rij[2]);
                            vir[5 % NC] += hb * ((f * rij[1]) * rij[2]);
                        }
                    }
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        if (a.fields & 1) a.out_vir[gidx * NC + c] = vir[c];
        if (a.fields & 2) a.out_kin[gidx * NC + c] = kin[c];
    }
}

cudaError_t launch_gather64(const GatherArgs64& a, cudaStream_t st)
{
    int threads = 128;
    int blocks = (int)((a.ngrid + threads - 1) / threads);
    if (blocks == 0) return cudaSuccess;
    const bool adapt = a.cg.mode == IK_QUAD_ADAPTIVE_DEV;
    if (a.g.dim == 2) adapt ? k_gather64<2, true><<<blocks, threads, 0, st>>>(a) : k_gather64<2, false><<<blocks, threads, 0, st>>>(a);
    else adapt ? k_gather64<3, true><<<blocks, threads, 0, st>>>(a) : k_gather64<3, false><<<blocks, threads, 0, st>>>(a);
    return cudaGetLastError();
}

struct EvalBondArgs {
    IkCG cg;
    int nq;
    double xs[64], ws[64];
    IkGK gk;
    int* status;
};

__global__ void k_eval_bond(const EvalBondArgs a, int m, const double* __restrict__ x,
                            const double* __restrict__ ri, const double* __restrict__ rij,
                            double* __restrict__ bond, double* __restrict__ delta)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    double xx[3] = {x[3 * k], x[3 * k + 1], x[3 * k + 2]};
    double rr[3] = {ri[3 * k], ri[3 * k + 1], ri[3 * k + 2]};
    double bb[3] = {rij[3 * k], rij[3 * k + 1], rij[3 * k + 2]};
    bond[k] = ik_bond64<true>(a.cg, a.xs, a.ws, a.nq, a.gk, a.status, xx, rr, bb);
    double e0 = xx[0] - rr[0], e1 = xx[1] - rr[1], e2 = xx[2] - rr[2];
    delta[k] = ik_delta64(a.cg, e0 * e0 + e1 * e1 + e2 * e2);
}

cudaError_t launch_eval_bond(const IkCG& cg, int dim, const double* xs, const double* ws, int nq,
                             const IkGK& gk, int* status, int m, const double* x, const double* ri,
                             const double* rij, double* bond, double* delta, cudaStream_t st)
{
    (void)dim;
    EvalBondArgs a;
    a.cg = cg;
    a.nq = nq;
    a.gk = gk;
    a.status = status;
    for (int k = 0; k < nq && k < 64; ++k) { a.xs[k] = xs[k]; a.ws[k] = ws[k]; }
    int threads = 128, blocks = (m + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    k_eval_bond<<<blocks, threads, 0, st>>>(a, m, x, ri, rij, bond, delta);
    return cudaGetLastError();
}
