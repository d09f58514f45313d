// ik_common.cuh -- shared device/host definitions of the GB300 Irving-Kirkwood engine.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define IK_MAXB_2D 16   // default force-active bonds per particle (grows on overflow)
#define IK_MAXB_3D 32
#define IK_WARPS_GATHER 8
#define IK_P 4          // grid points per warp group in the FP32 gather
#define IK_SQ_CONT (1 << 30) // staged-entry flag: further bonds of a particle already staged
#define IK_MAXB_LIMIT 1023   // force-active bonds (and elastic neighbours) per particle

// device status word bits (ctx->d_status)
#define IK_ST_BOND_OVERFLOW 1
#define IK_ST_HALO_OVERFLOW 2
#define IK_ST_BAD_INPUT     4
#define IK_ST_NEIGH_OVERFLOW 8
#define IK_QUAD_EXACT_DEV 2 /* IK_QUAD_EXACT of the C ABI */
#define IK_QUAD_ADAPTIVE_DEV 1 /* IK_QUAD_ADAPTIVE of the C ABI */
#define IK_ST_QUAD_FAIL     64  /* an adaptive bond integral missed its tolerance within its subintervals */
#define IK_QAG_MAXSUB       64  /* subintervals one adaptive bond integral may hold on the device */
#define IK_ST_MMA_TIMEOUT   16  /* a tensor-core completion wait gave up */
#define IK_ST_MLP_OVERFLOW  32  /* the surrogate record buffer overflowed */
#define IK_ST_BOND_RANGE    128 /* FP32 path: 2^25 or more bond records (staged-entry word) */

// Box + cell grid.  Cells tile [lo, lo+L) per axis; nc[c] = 1 on non-periodic axes.
struct IkGeom {
    int dim;
    int nc[3];
    int ncell;
    int reach_bond[3];   // stencil half-width for the bond search (cells)
    int all_bond[3];     // 1: stencil covers the whole axis once
    double L[3], lo[3], cw[3];
    double invL[3];      // 1 / L (used for minimum-image rounding only)
    float cwhi[3], cwlo[3]; // cell width as a double-float pair (FP32 hi + lo)
    int periodic[3];
};

// Pair potential (potential/*.h), one struct for the eight models of the reference.
// kind = IKP_* (the values of ik_pot_kind of the C ABI).  Parameters in a common layout:
//   v0    energy scale (LennardJones / ForceShiftedLennardJones: eps)
//   eps   non-additivity of sigma_ij (LennardJones: vareps; ForceShifted: unused)
//   c0-c3 smoothing polynomial (c3: Polydisperse10 only); kappa (PolydisperseYukawa)
#define IKP_POLY12 0
#define IKP_LJ 1
#define IKP_FSLJ 2
#define IKP_POLY10 3
#define IKP_POLY106 4
#define IKP_POLY18 5
#define IKP_POLYLJ 6
#define IKP_POLYYUKAWA 7
struct IkPot {
    int kind;
    double rcutsq;       // scaled_rcut^2
    double v0, eps, c0, c1, c2, c3, kappa;
    double max_rcut_sq;
};

// Coarse-graining function, in the two forms the kernels use.
struct IkCG {
    int kind;            // IK_CG_*
    int mode;            // IK_QUAD_*
    int order;           // GL points
    double rcut, rcutsq, width;
    double norm;         // prefactor of Delta (Gaussian: (2 pi w^2)^(-d/2), octic 15/(8 pi R^2), ...)
    // FP32 tuned path works in scaled coordinates u = kappa * x:
    //   Gaussian: kappa = sqrt(log2(e) / (2 w^2)), Delta = norm * 2^(-|u|^2), cut |u|^2 < R2s
    //   others:   kappa = 1/R, q = |u|^2 in [0,1)
    float kappa;
    float R2s;           // scaled squared support radius
    double mollifier_norm;
    // adaptive
    int neval;
    double relerr, abserr;
};

// Gauss-Kronrod 7/15 rule on [-1, 1]: x[0] = 0, x[1..7] the positive nodes ascending
// (Kronrod nodes at odd slots, the 7-point Gauss nodes at even slots), Kronrod weights
// wk[8], Gauss weights wg[4] of the nodes 0, x[2], x[4], x[6].
struct IkGK {
    double x[8], wk[8], wg[4];
};

// GL nodes on [-1,1] (ascending) and weights, FP64 + FP32 copies (max 64 points).
struct IkGL {
    int n;
    double x[64], w[64];
    float t[32], wt[32];   // symmetric form: t_k = x_k/2 for the positive half, weights
    float w0;              // centre weight (odd n), else 0
    int npairs;
};

// ---------------------------------------------------------------------------
// FP64 helpers with explicit rounding (no contraction) so the neighbour and
// selection tests are bit-identical to the CPU oracle (compiled with
// -ffp-contract=off).
__device__ __forceinline__ double ik_minimg(double d, double L, int periodic)
{
    if (periodic) {
        double k = rint(__ddiv_rn(d, L));
        d = __dsub_rn(d, __dmul_rn(L, k));
    }
    return d;
}

__device__ __forceinline__ double ik_dot2(double a, double b)
{
    return __dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b));
}
__device__ __forceinline__ double ik_dot3(double a, double b, double c)
{
    return __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c));
}

// computeForceDivR / computeEnergy of the eight models in FP64, each in the evaluation
// order of its reference expression (C++ left-to-right), every operation rounded
// explicitly so that no FMA contraction changes a bit against the CPU oracle.
//   Polydisperse12   potential/Polydisperse12.h:19-55
//   LennardJones     potential/LennardJones.h:19-57 (force needs eps != 0)
//   ForceShiftedLJ   potential/LennardJones.h:105-124 (sigma without vareps; energy of LJ)
//   Polydisperse10   potential/Polydisperse10.h:19-53
//   Polydisperse106  potential/Polydisperse106.h:19-53
//   Polydisperse18   potential/Polydisperse18.h:19-50
//   PolydisperseLJ   potential/PolydisperseLJ.h:19-50
//   PolydisperseYukawa potential/PolydisperseYukawa.h:19-55 (exp: CUDA's, <= 2 ulp from libm)
// sigma_ij: 0.5 (d_i + d_j) (1 - eps |d_i - d_j|); the force-shifted LJ force uses
// 0.5 (d_i + d_j).  `force` selects the force's sigma (the energy of the force-shifted
// model is the truncated LJ one, with the non-additive sigma).
__device__ __forceinline__ double ik_sigma_eps(double eps, double di, double dj)
{
    return __dmul_rn(__dmul_rn(0.5, __dadd_rn(di, dj)), __dsub_rn(1.0, __dmul_rn(eps, fabs(__dsub_rn(di, dj)))));
}
__device__ __forceinline__ double ik_sigma64(const IkPot& p, double di, double dj, bool force = true)
{
    if (force && p.kind == IKP_FSLJ) return __dmul_rn(0.5, __dadd_rn(di, dj));
    return ik_sigma_eps(p.eps, di, dj);
}
// the force is non-zero only inside the cut-off (and, for the LJ models, for eps != 0)
__device__ __forceinline__ bool ik_active64(const IkPot& p, double rsq, double sigma)
{
    double actual = __dmul_rn(__dmul_rn(p.rcutsq, sigma), sigma);
    if ((p.kind == IKP_LJ || p.kind == IKP_FSLJ) && p.v0 == 0.0) return false;
    return rsq < actual;
}
// 4 v0 r2inv r6inv (12 r6inv - 6), left to right
__device__ __forceinline__ double ik_lj_fterm(double v0, double r2inv, double r6inv)
{
    return __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(4.0, v0), r2inv), r6inv),
                     __dsub_rn(__dmul_rn(12.0, r6inv), 6.0));
}
__device__ __forceinline__ double ik_force64(const IkPot& p, double rsq, double sigma)
{
    const double s2 = __dmul_rn(sigma, sigma);
    const double r2inv = __dmul_rn(__ddiv_rn(1.0, rsq), s2);
    const double rs = __ddiv_rn(rsq, s2);
    const double r6inv = __dmul_rn(__dmul_rn(r2inv, r2inv), r2inv);
    double t;
    switch (p.kind) {
    case IKP_LJ:
        return __ddiv_rn(ik_lj_fterm(p.v0, r2inv, r6inv), s2);
    case IKP_FSLJ: {
        t = ik_lj_fterm(p.v0, r2inv, r6inv);
        const double c2inv = __ddiv_rn(1.0, p.rcutsq);
        const double c6inv = __dmul_rn(__dmul_rn(c2inv, c2inv), c2inv);
        return __ddiv_rn(__dsub_rn(t, ik_lj_fterm(p.v0, c2inv, c6inv)), s2);
    }
    case IKP_POLY10: {
        const double r10 = __dmul_rn(__dmul_rn(r6inv, r2inv), r2inv);
        t = __dmul_rn(__dmul_rn(__dmul_rn(10.0, p.v0), r2inv), r10);
        t = __dsub_rn(t, __dmul_rn(2.0, p.c1));
        t = __dsub_rn(t, __dmul_rn(__dmul_rn(4.0, p.c2), rs));
        t = __dsub_rn(t, __dmul_rn(__dmul_rn(__dmul_rn(6.0, p.c3), rs), rs));
        return __ddiv_rn(t, s2);
    }
    case IKP_POLY106: {
        const double r10 = __dmul_rn(__dmul_rn(r6inv, r2inv), r2inv);
        const double a = __dmul_rn(__dmul_rn(10.0, r10), r2inv);
        const double b = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(6.0, r2inv), r2inv), r2inv), r2inv);
        t = __dmul_rn(p.v0, __dsub_rn(a, b));
        t = __dsub_rn(t, __dmul_rn(2.0, p.c1));
        t = __dsub_rn(t, __dmul_rn(__dmul_rn(4.0, p.c2), rs));
        return __ddiv_rn(t, s2);
    }
    case IKP_POLY18:
        t = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(18.0, p.v0), r2inv), r6inv), r6inv), r6inv);
        t = __dsub_rn(t, __dmul_rn(2.0, p.c1));
        t = __dsub_rn(t, __dmul_rn(__dmul_rn(4.0, p.c2), rs));
        return __ddiv_rn(t, s2);
    case IKP_POLYLJ:
        t = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(12.0, p.v0), r2inv), r6inv), r6inv);
        t = __dsub_rn(t, __dmul_rn(__dmul_rn(__dmul_rn(6.0, p.v0), r2inv), r6inv));
        t = __dsub_rn(t, __dmul_rn(2.0, p.c1));
        t = __dsub_rn(t, __dmul_rn(__dmul_rn(4.0, p.c2), rs));
        return __ddiv_rn(t, s2);
    case IKP_POLYYUKAWA: {
        const double rinv = __dsqrt_rn(r2inv), rroot = __dsqrt_rn(rs);
        const double e = exp(__dmul_rn(-p.kappa, rroot));
        t = __dmul_rn(__dmul_rn(__dmul_rn(e, __dadd_rn(rinv, p.kappa)), p.v0), r2inv);
        t = __dsub_rn(t, __dmul_rn(2.0, p.c1));
        t = __dsub_rn(t, __dmul_rn(__dmul_rn(4.0, p.c2), rs));
        return __ddiv_rn(t, s2);
    }
    default: // IKP_POLY12
        t = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(12.0, p.v0), r2inv), r6inv), r6inv);
        t = __dsub_rn(t, __dmul_rn(2.0, p.c1));
        t = __dsub_rn(t, __dmul_rn(__dmul_rn(4.0, p.c2), rs));
        return __ddiv_rn(t, s2);
    }
}
// computeEnergy; call with sigma = ik_sigma64(p, di, dj, false) and the cut-off test
// rsq < rcutsq sigma^2 (no eps != 0 condition for the LJ energies).
__device__ __forceinline__ double ik_energy64(const IkPot& p, double rsq, double sigma)
{
    const double s2 = __dmul_rn(sigma, sigma);
    const double r2inv = __dmul_rn(__ddiv_rn(1.0, rsq), s2);
    const double rs = __ddiv_rn(rsq, s2);
    const double r6inv = __dmul_rn(__dmul_rn(r2inv, r2inv), r2inv);
    double t;
    switch (p.kind) {
    case IKP_LJ:
    case IKP_FSLJ: {
        const double actual = __dmul_rn(__dmul_rn(p.rcutsq, sigma), sigma);
        const double c2inv = __dmul_rn(__ddiv_rn(1.0, actual), s2);
        const double c6inv = __dmul_rn(__dmul_rn(c2inv, c2inv), c2inv);
        const double a = __dmul_rn(__dmul_rn(__dmul_rn(4.0, p.v0), r6inv), __dsub_rn(r6inv, 1.0));
        const double b = __dmul_rn(__dmul_rn(__dmul_rn(4.0, p.v0), c6inv), __dsub_rn(c6inv, 1.0));
        return __dsub_rn(a, b);
    }
    case IKP_POLY10: {
        const double r10 = __dmul_rn(__dmul_rn(r6inv, r2inv), r2inv);
        t = __dadd_rn(__dmul_rn(p.v0, r10), p.c0);
        t = __dadd_rn(t, __dmul_rn(p.c1, rs));
        t = __dadd_rn(t, __dmul_rn(__dmul_rn(p.c2, rs), rs));
        return __dadd_rn(t, __dmul_rn(__dmul_rn(__dmul_rn(p.c3, rs), rs), rs));
    }
    case IKP_POLY106: {
        const double r10 = __dmul_rn(__dmul_rn(r6inv, r2inv), r2inv);
        t = __dadd_rn(__dmul_rn(p.v0, __dsub_rn(r10, r6inv)), p.c0);
        break;
    }
    case IKP_POLY18:
        t = __dadd_rn(__dmul_rn(__dmul_rn(__dmul_rn(p.v0, r6inv), r6inv), r6inv), p.c0);
        break;
    case IKP_POLYLJ:
        t = __dsub_rn(__dmul_rn(__dmul_rn(p.v0, r6inv), r6inv), __dmul_rn(p.v0, r6inv));
        t = __dadd_rn(t, p.c0);
        break;
    case IKP_POLYYUKAWA: {
        const double rinv = __dsqrt_rn(r2inv), rroot = __dsqrt_rn(rs);
        t = __dadd_rn(__dmul_rn(__dmul_rn(p.v0, exp(__dmul_rn(-rroot, p.kappa))), rinv), p.c0);
        break;
    }
    default: // IKP_POLY12
        t = __dadd_rn(__dmul_rn(__dmul_rn(p.v0, r6inv), r6inv), p.c0);
        break;
    }
    t = __dadd_rn(t, __dmul_rn(p.c1, rs));
    return __dadd_rn(t, __dmul_rn(__dmul_rn(p.c2, rs), rs));
}

// computeStiffness (the bond stiffness, second derivative of the pair energy) of the eight
// models in FP64, reference expression order: Polydisperse12.h:57-73, LennardJones.h:60-75
// (also the force-shifted model's: it does not override it), Polydisperse10.h:56-72,
// Polydisperse106.h:56-72, Polydisperse18.h:56-72, PolydisperseLJ.h:56-72 (its c2 term is
// 4 c2 r^2 as written there), PolydisperseYukawa.h:59-76.  Call with
// sigma = ik_sigma64(p, di, dj, false) and ik_active64's test on that sigma.
__device__ __forceinline__ double ik_stiffness64(const IkPot& p, double rsq, double sigma)
{
    const double s2 = __dmul_rn(sigma, sigma);
    const double r2inv = __dmul_rn(__ddiv_rn(1.0, rsq), s2);
    const double rs = __ddiv_rn(rsq, s2);
    const double r6inv = __dmul_rn(__dmul_rn(r2inv, r2inv), r2inv);
    double t;
    switch (p.kind) {
    case IKP_LJ:
    case IKP_FSLJ:
        t = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(4.0, p.v0), r2inv), r6inv),
                      __dsub_rn(__dmul_rn(156.0, r6inv), 42.0));
        return __ddiv_rn(t, s2);
    case IKP_POLY10:
        t = __dmul_rn(__dmul_rn(__dmul_rn(110.0, p.v0), r6inv), r6inv);
        t = __dadd_rn(t, __dmul_rn(2.0, p.c1));
        t = __dadd_rn(t, __dmul_rn(__dmul_rn(12.0, p.c2), rs));
        t = __dadd_rn(t, __dmul_rn(__dmul_rn(__dmul_rn(30.0, p.c3), rs), rs));
        return __ddiv_rn(t, s2);
    case IKP_POLY106: {
        const double a = __dmul_rn(__dmul_rn(110.0, r6inv), r6inv);
        const double b = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(42.0, r2inv), r2inv), r2inv), r2inv);
        t = __dmul_rn(p.v0, __dsub_rn(a, b));
        t = __dadd_rn(t, __dmul_rn(2.0, p.c1));
        t = __dadd_rn(t, __dmul_rn(__dmul_rn(12.0, p.c2), rs));
        return __ddiv_rn(t, s2);
    }
    case IKP_POLY18:
        t = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(342.0, p.v0), r2inv), r6inv), r6inv), r6inv);
        t = __dadd_rn(t, __dmul_rn(2.0, p.c1));
        t = __dadd_rn(t, __dmul_rn(__dmul_rn(12.0, p.c2), rs));
        return __ddiv_rn(t, s2);
    case IKP_POLYLJ:
        t = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(156.0, p.v0), r2inv), r6inv), r6inv);
        t = __dsub_rn(t, __dmul_rn(__dmul_rn(__dmul_rn(42.0, p.v0), r2inv), r6inv));
        t = __dadd_rn(t, __dmul_rn(2.0, p.c1));
        t = __dadd_rn(t, __dmul_rn(__dmul_rn(4.0, p.c2), rs));
        return __ddiv_rn(t, s2);
    case IKP_POLYYUKAWA: {
        const double rinv = __dsqrt_rn(r2inv), rroot = __dsqrt_rn(rs);
        const double e = exp(__dmul_rn(-p.kappa, rroot));
        const double q = __dadd_rn(__dadd_rn(__dmul_rn(2.0, r2inv), __dmul_rn(__dmul_rn(2.0, p.kappa), rinv)),
                                   __dmul_rn(p.kappa, p.kappa));
        t = __dmul_rn(__dmul_rn(__dmul_rn(p.v0, e), q), rinv);
        t = __dadd_rn(t, __dmul_rn(2.0, p.c1));
        t = __dadd_rn(t, __dmul_rn(__dmul_rn(12.0, p.c2), rs));
        return __ddiv_rn(t, s2);
    }
    default: // IKP_POLY12
        t = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(156.0, p.v0), r2inv), r6inv), r6inv);
        t = __dadd_rn(t, __dmul_rn(2.0, p.c1));
        t = __dadd_rn(t, __dmul_rn(__dmul_rn(12.0, p.c2), rs));
        return __ddiv_rn(t, s2);
    }
}

// Coarse-graining kernels in FP64 (CGFuncOctic.h:16-29, CGFuncRect.h,
// CGFuncMollifier.h; Gaussian added).  Returns Delta(dr_sq).
__device__ __forceinline__ double ik_delta64(const IkCG& cg, double dr_sq)
{
    if (!(dr_sq < cg.rcutsq)) return 0.0;
    switch (cg.kind) {
    case 0: { // octic
        double r4 = dr_sq * dr_sq / (cg.rcutsq * cg.rcutsq);
        double r8 = r4 * r4;
        return cg.norm * (1 - 2 * r4 + r8);
    }
    case 1: // gaussian
        return cg.norm * exp(-dr_sq / (2.0 * cg.width * cg.width));
    case 2: // rect
        return cg.norm;
    default: { // mollifier
        double r2 = dr_sq / cg.rcutsq;
        return cg.mollifier_norm * exp(-1.0 / (1 - r2));
    }
    }
}

// ---------------------------------------------------------------------------
// cell coordinate of a position along axis c (wrapped into [0, nc))
__device__ __forceinline__ int ik_cell_coord(const IkGeom& g, int c, double x)
{
    if (g.nc[c] == 1) return 0;
    double t = (x - g.lo[c]) / g.L[c];
    t -= floor(t);
    int k = (int)(t * g.nc[c]);
    return k < 0 ? 0 : (k >= g.nc[c] ? g.nc[c] - 1 : k);
}

__device__ __forceinline__ int ik_wrap(int k, int n)
{
    k %= n;
    return k < 0 ? k + n : k;
}

// Particle record of the FP32 path, in cell-sorted order (16 bytes): position
// relative to the lower corner of its cell (unscaled), and the linear cell index.
struct __align__(16) IkPRec {
    float x, y, z;
    int cell;
};

// FP64 bond record of the plain path: r_ij and forceDivR.
struct __align__(16) IkB64 { double x, y, z, w; };
__host__ __device__ __forceinline__ IkB64 make_ikb64(double x, double y, double z, double w)
{
    IkB64 b; b.x = x; b.y = y; b.z = z; b.w = w; return b;
}
