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

__device__ __forceinline__ double ik_bond64(const IkCG& cg, const double* xs, const double* ws, int nq,
                                            const double x[3], const double ri[3], const double rij[3])
{
    if (cg.mode == IK_QUAD_EXACT_DEV) return ik_bond64_exact(cg, xs, ws, nq, x, ri, rij);
    double acc = 0.0;
    for (int k = 0; k < nq; ++k) {
        double s = xs[k];
        double p0 = ri[0] + s * rij[0], p1 = ri[1] + s * rij[1], p2 = ri[2] + s * rij[2];
        double d0 = x[0] - p0, d1 = x[1] - p1, d2 = x[2] - p2;
        acc += ws[k] * ik_delta64(cg, d0 * d0 + d1 * d1 + d2 * d2);
    }
    return 0.5 * acc;
}

template <int DIM>
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
                        double bond = ik_bond64(a.cg, a.xs, a.ws, a.nq, x, ri, rij);
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
    if (a.g.dim == 2) k_gather64<2><<<blocks, threads, 0, st>>>(a);
    else k_gather64<3><<<blocks, threads, 0, st>>>(a);
    return cudaGetLastError();
}

struct EvalBondArgs {
    IkCG cg;
    int nq;
    double xs[64], ws[64];
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
    bond[k] = ik_bond64(a.cg, a.xs, a.ws, a.nq, xx, rr, bb);
    double e0 = xx[0] - rr[0], e1 = xx[1] - rr[1], e2 = xx[2] - rr[2];
    delta[k] = ik_delta64(a.cg, e0 * e0 + e1 * e1 + e2 * e2);
}

cudaError_t launch_eval_bond(const IkCG& cg, int dim, const double* xs, const double* ws, int nq, int m,
                             const double* x, const double* ri, const double* rij, double* bond,
                             double* delta, cudaStream_t st)
{
    (void)dim;
    EvalBondArgs a;
    a.cg = cg;
    a.nq = nq;
    for (int k = 0; k < nq && k < 64; ++k) { a.xs[k] = xs[k]; a.ws[k] = ws[k]; }
    int threads = 128, blocks = (m + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    k_eval_bond<<<blocks, threads, 0, st>>>(a, m, x, ri, rij, bond, delta);
    return cudaGetLastError();
}
