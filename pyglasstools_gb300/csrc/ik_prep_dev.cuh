// ik_prep_dev.cuh -- device functions of the FP32 path's per-frame preparation, shared
// by the per-frame kernels (ik_bonds.cu) and the batch-wide ones (ik_batch.cu): the
// double-float cell-relative position of a particle, the per-cell sort and pack, the
// FP32 pair forces and the force-active bonds of one particle.
#pragma once
#include "ik_kernels.h"

// Cell (linear index) of a particle at pos[0..2] and its position relative to the
// lower corner of the cell as a double-float pair (hi = FP32 rounding, lo = FP32
// rounding of the remainder; hi + lo carries ~48 bits).
__device__ __forceinline__ int ik_bin32_one(const IkGeom& g, const double* __restrict__ pos, float4& relhi,
                                            float4& rello)
{
    double r[3] = {0.0, 0.0, 0.0};
    int cc[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (a >= g.dim || g.nc[a] == 1) continue;
        double t = (pos[a] - g.lo[a]) * g.invL[a];
        t -= floor(t);
        int k = (int)(t * g.nc[a]);
        k = k < 0 ? 0 : (k >= g.nc[a] ? g.nc[a] - 1 : k);
        cc[a] = k;
        r[a] = t * g.L[a] - k * g.cw[a];
    }
    float hx = (float)r[0], hy = (float)r[1], hz = (float)r[2];
    relhi = make_float4(hx, hy, hz, 0.f);
    rello = make_float4((float)(r[0] - hx), (float)(r[1] - hy), (float)(r[2] - hz), 0.f);
    return (cc[2] * g.nc[1] + cc[1]) * g.nc[0] + cc[0];
}

// The tests of k_validate on the IEEE-754 bits: finite, and for a 2D position z == 0
// (positions), finite and > 0 (diameters).
__device__ __forceinline__ bool ik_pos_ok(const double* p, int dim)
{
    const long long EXP = 0x7ff0000000000000LL, ABS = 0x7fffffffffffffffLL;
    const long long x = __double_as_longlong(p[0]), y = __double_as_longlong(p[1]), z = __double_as_longlong(p[2]);
    return (x & EXP) != EXP && (y & EXP) != EXP && (z & EXP) != EXP && (dim == 3 || (z & ABS) == 0);
}
__device__ __forceinline__ bool ik_diam_ok(double d)
{
    const long long v = __double_as_longlong(d);
    return (v & 0x7ff0000000000000LL) != 0x7ff0000000000000LL && v > 0;
}

// Sort the ids of one cell (insertion sort: cells hold a handful of particles; fixes the
// order the atomic ranks left).
__device__ __forceinline__ void ik_sort_cell(int s, int e, int* __restrict__ sorted)
{
    for (int a = s + 1; a < e; ++a) {
        const int v = sorted[a];
        int b = a - 1;
        while (b >= s && sorted[b] > v) { sorted[b + 1] = sorted[b]; --b; }
        sorted[b + 1] = v;
    }
}

// Pack the particle at cell-list position p (id ig = sorted[p]): its records in
// prec / plo / pos64 / kin / diam32, indexed by p.  relhi / rello are indexed by ig (the
// cell list's ids; a batch's: id0 = the frame's first); pos / vel / mass / diam are the
// frame's own arrays, indexed by ig - id0.  cell = the cell's index in the frame
// (IkPRec::cell).
__device__ __forceinline__ void ik_pack_one(int dim, int cell, int p, int ig, int id0,
                                            const float4* __restrict__ relhi, const float4* __restrict__ rello,
                                            const double* __restrict__ pos, const double* __restrict__ vel,
                                            const double* __restrict__ mass, const double* __restrict__ diam,
                                            IkPRec* __restrict__ prec, float4* __restrict__ plo,
                                            IkB64* __restrict__ pos64, float4* __restrict__ kin,
                                            float* __restrict__ diam32)
{
    const int i = ig - id0;
    const float4 h = relhi[ig];
    IkPRec r;
    r.x = h.x;
    r.y = h.y;
    r.z = h.z;
    r.cell = cell;
    prec[p] = r;
    plo[p] = rello[ig];
    pos64[p] = make_ikb64(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], diam[i]);
    const double m = mass ? mass[i] : 1.0;
    const double vx = vel ? vel[3 * i] : 0.0, vy = vel ? vel[3 * i + 1] : 0.0, vz = vel ? vel[3 * i + 2] : 0.0;
    if (dim == 2) {
        kin[p] = make_float4((float)(m * vx * vx), (float)(m * vy * vy), (float)(m * vx * vy), 0.f);
    } else {
        kin[2 * p] = make_float4((float)(m * vx * vx), (float)(m * vy * vy), (float)(m * vz * vz),
                                 (float)(m * vx * vy));
        kin[2 * p + 1] = make_float4((float)(m * vx * vz), (float)(m * vy * vz), 0.f, 0.f);
    }
    diam32[p] = (float)diam[i];
}

// b = o + (pj - pi) for double-float operands (o = ohi + olo, p = hi + lo), rounded
// once to FP32 at the end: TwoSum for the two leading additions, the small terms
// added after.  Accurate to ~1 ulp of the FP32 result.
__device__ __forceinline__ float ik_df_diff(float ohi, float olo, float hj, float lj, float hi_, float li)
{
    float s = hj - hi_;
    float bb = s - hj;
    float e = (hj - (s - bb)) + (-hi_ - bb);
    float t = ohi + s;
    float b2 = t - ohi;
    float e2 = (ohi - (t - b2)) + (s - b2);
    return t + ((e + e2) + (olo + (lj - li)));
}

// ---------------------------------------------------------------------------
// FP32 force of the eight pair models (the expressions of potential/*.h with FP32
// constants; r2inv = sigma^2 / r^2, rs = r^2 / sigma^2, s2 = sigma^2).
// Built on the host once per launch (its FP64 set-up, a division among it, would cost
// every thread of a bond build ~40 operations on GB300's narrow FP64 pipe).
struct IkPotF {
    int kind;
    float rc2, eps_s, v0, v0x4, c1x2, c2x4, c3x6, kappa, shift;
    float mr2; // max_rcut^2
};
__host__ __device__ inline IkPotF ik_potf(const IkPot& p)
{
    IkPotF q;
    q.kind = p.kind;
    q.mr2 = (float)p.max_rcut_sq;
    const bool lj = p.kind == IKP_LJ || p.kind == IKP_FSLJ;
    q.rc2 = lj && p.v0 == 0.0 ? 0.f : (float)p.rcutsq; // eps = 0: no force (LennardJones.h:48)
    q.eps_s = p.kind == IKP_FSLJ ? 0.f : (float)p.eps;
    q.v0 = (float)p.v0;
    q.v0x4 = (float)(4.0 * p.v0);
    q.c1x2 = (float)(2.0 * p.c1);
    q.c2x4 = (float)(4.0 * p.c2);
    q.c3x6 = (float)(6.0 * p.c3);
    q.kappa = (float)p.kappa;
    const double c2inv = 1.0 / p.rcutsq, c6inv = c2inv * c2inv * c2inv;
    q.shift = (float)(4.0 * p.v0 * c2inv * c6inv * (12.0 * c6inv - 6.0)); // LennardJones.h:117-119
    return q;
}
template <int KIND>
__device__ __forceinline__ float ik_force32(const IkPotF& q, float r2, float s2)
{
    const float r2inv = s2 / r2, rs = r2 / s2;
    const float r6 = r2inv * r2inv * r2inv;
    float t;
    switch (KIND) {
    case IKP_LJ: t = q.v0x4 * r2inv * r6 * (12.f * r6 - 6.f); break;
    case IKP_FSLJ: t = q.v0x4 * r2inv * r6 * (12.f * r6 - 6.f) - q.shift; break;
    case IKP_POLY10: {
        const float r10 = r6 * r2inv * r2inv;
        t = 10.f * q.v0 * r2inv * r10 - q.c1x2 - q.c2x4 * rs - q.c3x6 * rs * rs;
        break;
    }
    case IKP_POLY106: {
        const float r10 = r6 * r2inv * r2inv;
        t = q.v0 * (10.f * r10 * r2inv - 6.f * r6 * r2inv) - q.c1x2 - q.c2x4 * rs;
        break;
    }
    case IKP_POLY18: t = 18.f * q.v0 * r2inv * r6 * r6 * r6 - q.c1x2 - q.c2x4 * rs; break;
    case IKP_POLYLJ: t = q.v0 * r2inv * r6 * (12.f * r6 - 6.f) - q.c1x2 - q.c2x4 * rs; break;
    case IKP_POLYYUKAWA: {
        const float rinv = sqrtf(r2inv), rroot = sqrtf(rs);
        t = expf(-q.kappa * rroot) * (rinv + q.kappa) * q.v0 * r2inv - q.c1x2 - q.c2x4 * rs;
        break;
    }
    default: t = 12.f * q.v0 * r2inv * r6 * r6 - q.c1x2 - q.c2x4 * rs; break;
    }
    return t / s2;
}

// The FP64 selection of a bond (k_bonds64's test, bit for bit): within max_rcut and
// force-active.  The FP32 kernels call it for pairs whose FP32 distance lies within
// 2e-5 (relative) of a cut-off, so that both paths keep exactly the same bonds.
__device__ __forceinline__ bool ik_select64_r(const IkPot& pot, double dx, double dy, double dz, double di,
                                              double dj)
{
    const double rsq = ik_dot3(dx, dy, dz);
    if (!(rsq < pot.max_rcut_sq)) return false;
    return ik_active64(pot, rsq, ik_sigma64(pot, di, dj));
}
// Minimum image by division, as the oracle (boxes with fewer than three cells on an axis).
__device__ __forceinline__ bool ik_select64(const IkGeom& g, const IkPot& pot, const IkB64& a, const IkB64& b)
{
    return ik_select64_r(pot, ik_minimg(__dsub_rn(b.x, a.x), g.L[0], g.periodic[0]),
                         ik_minimg(__dsub_rn(b.y, a.y), g.L[1], g.periodic[1]),
                         ik_minimg(__dsub_rn(b.z, a.z), g.L[2], g.periodic[2]), a.w, b.w);
}
// With three or more cells per axis a stencil candidate near a cut-off lies within
// max_rcut <= L/3 of the particle, so the oracle's image count rint(d / L) is exactly
// minus the stencil's wrap shift s (the image of b used is b + s L): the same
// d - L k without the divisions.
__device__ __forceinline__ bool ik_select64_shift(const IkGeom& g, const IkPot& pot, const IkB64& a,
                                                  const IkB64& b, int sx, int sy, int sz)
{
    return ik_select64_r(pot, __dsub_rn(__dsub_rn(b.x, a.x), __dmul_rn(g.L[0], (double)(-sx))),
                         __dsub_rn(__dsub_rn(b.y, a.y), __dmul_rn(g.L[1], (double)(-sy))),
                         __dsub_rn(__dsub_rn(b.z, a.z), __dmul_rn(g.L[2], (double)(-sz))), a.w, b.w);
}

// ---------------------------------------------------------------------------
// Force-active bonds, one thread per particle (particles in cell order, so that
// neighbouring threads walk the same candidate cells and their loads hit in L1).
// Each candidate of the 3^d stencil is screened in FP32 from the cell-relative
// positions; survivors are re-measured from the double-float positions, so that r_ij
// carries only its final FP32 rounding -- the r^-14 force amplifies position rounding
// for strongly overlapping pairs.  (On axes with fewer than three cells the stencil is
// not the minimum image; those pairs are re-measured in FP64.)
// Output record (16 B): {hb_x, hb_y, hb_z, f'} with hb = kappa * r_ij / 2 (scaled half
// bond, r_ij = r_j - r_i) and f' = 2 forceDivR / kappa^2, so that
// f' * hb (x) hb = 0.5 * forceDivR * r_ij (x) r_ij.  Written at a fixed stride of
// `maxb` records per particle in candidate order (stencil cell with x fastest, then
// ascending sorted index): deterministic.  ALLAX: some axis has fewer than three cells.
// Without ALLAX a stencil row's three cells (x = hx - 1, hx, hx + 1) are distinct and,
// unless the row wraps in x, consecutive in the cell list: the row's candidates are one
// contiguous index range (two at the box's x edges), walked in the same order as cell
// by cell, with the x offset of a candidate's cell read from the range's inner cell
// boundaries.  One loop per row instead of one per cell: fewer loop set-ups, no integer
// division for the wrap, and less divergence between the lanes' ragged cell counts.
// The bonds of particle p (cell order); cell_start is the frame's cell list (indices
// into prec / plo / pos64 / tmp / nb, which may be a batch's); pf = ik_potf(pot); returns
// the number of force-active bonds (those beyond maxb are counted, not stored).  qidx /
// qcode: this thread's survivor queue in shared memory, IK_BOND_QUEUE entries at stride
// qstride (unused with ALLAX).
#define IK_BOND_QUEUE 16
template <int DIM, int KIND, bool ALLAX>
__device__ __forceinline__ int ik_bonds32_particle(const IkGeom& g, const IkPot& pot, const IkPotF& pf, float kappa,
                                                   int p,
                                                   const IkPRec* __restrict__ prec,
                                                   const float* __restrict__ diam32,
                                                   const int* __restrict__ cell_start,
                                                   const float4* __restrict__ plo,
                                                   const IkB64* __restrict__ pos64, float4* __restrict__ tmp,
                                                   int maxb, int* __restrict__ nb, int* __restrict__ status,
                                                   int* __restrict__ maxnb, int* __restrict__ qidx,
                                                   unsigned char* __restrict__ qcode, int qstride)
{
    const IkPRec me = prec[p];
    const int c = me.cell;
    const int home[3] = {c % g.nc[0], (c / g.nc[0]) % g.nc[1], c / (g.nc[0] * g.nc[1])};
    int lo[3], len[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (a >= DIM || g.nc[a] == 1) { lo[a] = 0; len[a] = 1; }
        else if (g.all_bond[a]) { lo[a] = 0; len[a] = g.nc[a]; }
        else { lo[a] = home[a] - 1; len[a] = 3; }
    }
    const bool allx = ALLAX && (len[0] > 3 || (g.all_bond[0] && g.nc[0] > 1));
    const bool ally = ALLAX && (len[1] > 3 || (g.all_bond[1] && g.nc[1] > 1));
    const bool allz = ALLAX && DIM == 3 && (len[2] > 3 || (g.all_bond[2] && g.nc[2] > 1));
    const float L0 = (float)g.L[0], L1 = (float)g.L[1], L2 = (float)g.L[2];
    const float rc2 = pf.rc2, mr2 = pf.mr2, eps = pf.eps_s;
    const float screen_f = 1.0f + 1e-4f;
    const float di = diam32[p];
    const float4 mlo = plo[p];
    const float hk = 0.5f * kappa, fk = 2.0f / (kappa * kappa);
    float4* out = tmp + (size_t)p * maxb;
    int cnt = 0;
    // one candidate q, cell offset (ox, oy, oz) + (olx, oly, olz) as double-float pairs:
    // screen = the two FP32 tests (within max_rcut, within the pair's cut-off, both with a
    // 1e-4 margin); measure = the rest for a candidate that passed (re-measure, the exact
    // decision, the force, the record).  (sx, sy, sz): the stencil's wrap shifts, used by
    // the FP64 re-decision.
    auto screen_rec = [&](const IkPRec& o, float dj, float ox, float oy, float oz) { // o = prec[q], dj = diam32[q]
        float bx = ox + (o.x - me.x), by = oy + (o.y - me.y), bz = DIM == 3 ? oz + (o.z - me.z) : 0.f;
        if (allx) bx -= L0 * rintf(bx / L0);
        if (ally) by -= L1 * rintf(by / L1);
        if (allz) bz -= L2 * rintf(bz / L2);
        const float r2 = bx * bx + by * by + bz * bz;
        if (!(r2 < mr2 * screen_f)) return false;
        const float sig = 0.5f * (di + dj) * (1.f - eps * fabsf(di - dj));
        const float s2 = sig * sig;
        return r2 < rc2 * s2 * screen_f;
    };
    auto screen = [&](int q, float ox, float oy, float oz) { return screen_rec(prec[q], diam32[q], ox, oy, oz); };
    auto measure = [&](int q, float ox, float olx, float oy, float oly, float oz, float olz, int sx, int sy, int sz) {
        const IkPRec o = prec[q];
        const float dj = diam32[q];
        const float sig = 0.5f * (di + dj) * (1.f - eps * fabsf(di - dj));
        const float s2 = sig * sig;
        float bx, by, bz = 0.f;
        if (!(allx || ally || allz)) {
            const float4 lq = plo[q];
            bx = ik_df_diff(ox, olx, o.x, lq.x, me.x, mlo.x);
            by = ik_df_diff(oy, oly, o.y, lq.y, me.y, mlo.y);
            if (DIM == 3) bz = ik_df_diff(oz, olz, o.z, lq.z, me.z, mlo.z);
        } else {
            const IkB64 pi = pos64[p], pj = pos64[q];
            double dx = pj.x - pi.x, dy = pj.y - pi.y;
            dx = fma(-g.L[0], rint(dx * g.invL[0]), dx);
            dy = fma(-g.L[1], rint(dy * g.invL[1]), dy);
            bx = (float)dx;
            by = (float)dy;
            if (DIM == 3) {
                double dz = pj.z - pi.z;
                dz = fma(-g.L[2], rint(dz * g.invL[2]), dz);
                bz = (float)dz;
            }
        }
        const float r2 = bx * bx + by * by + bz * bz;
        const float rt = rc2 * s2;
        bool act = r2 < mr2 && r2 < rt;
        if (fabsf(r2 - rt) <= 2e-5f * rt || fabsf(r2 - mr2) <= 2e-5f * mr2) { // at a cut-off: FP64
            if (ALLAX) act = ik_select64(g, pot, pos64[p], pos64[q]);
            else act = ik_select64_shift(g, pot, pos64[p], pos64[q], sx, sy, sz);
        }
        if (act) {
            const float f = ik_force32<KIND>(pf, r2, s2);
            if (cnt < maxb) out[cnt] = make_float4(hk * bx, hk * by, hk * bz, fk * f);
            ++cnt;
        }
    };
    if constexpr (ALLAX) {
        for (int iz = 0; iz < len[2]; ++iz) {
            const int uz = lo[2] + iz;
            const int wz = DIM == 3 ? ik_wrap(uz, g.nc[2]) : 0;
            const float kz = (float)(uz - home[2]);
            const float oz = DIM == 3 ? kz * g.cwhi[2] : 0.f, olz = DIM == 3 ? kz * g.cwlo[2] : 0.f;
            for (int iy = 0; iy < len[1]; ++iy) {
                const int uy = lo[1] + iy;
                const int wy = ik_wrap(uy, g.nc[1]);
                const float ky = (float)(uy - home[1]);
                const float oy = ky * g.cwhi[1], oly = ky * g.cwlo[1];
                for (int ix = 0; ix < len[0]; ++ix) {
                    const int ux = lo[0] + ix;
                    const int wx = ik_wrap(ux, g.nc[0]);
                    const float kx = (float)(ux - home[0]);
                    const float ox = kx * g.cwhi[0], olx = kx * g.cwlo[0];
                    const int cell = (wz * g.nc[1] + wy) * g.nc[0] + wx;
                    const int qe = cell_start[cell + 1];
                    for (int q = cell_start[cell]; q < qe; ++q)
                        if (q != p && screen(q, ox, oy, oz)) measure(q, ox, olx, oy, oly, oz, olz, 0, 0, 0);
                }
            }
        }
    } else {
        // every axis has one cell (len 1) or at least three (len 3, distinct cells).
        // Two passes so that the costly part runs with the lanes busy: the screen of every
        // candidate first, its survivors (≈ 6 of ≈ 37 in the headline workload) queued in
        // this thread's column of shared memory as (index, cell offset code), then the
        // measurement of the queued ones in candidate order (the records' order is the
        // same as measuring each one where it is found).
        const int nx = g.nc[0], hx = home[0];
        const int ny = g.nc[1], hy = home[1], nz = g.nc[2], hz = home[2];
        int ns = 0;
        auto drain = [&]() {
            for (int t = 0; t < ns; ++t) {
                const int q = qidx[t * qstride];
                const int code = qcode[t * qstride];
                const int kx = code % 3 - 1, ky = code / 3 % 3 - 1, kz = code / 9 - 1;
                const float kxf = (float)kx, kyf = (float)ky, kzf = (float)kz;
                const int ux = hx + kx, uy = hy + ky, uz = hz + kz;
                measure(q, kxf * g.cwhi[0], kxf * g.cwlo[0], kyf * g.cwhi[1], kyf * g.cwlo[1],
                        DIM == 3 ? kzf * g.cwhi[2] : 0.f, DIM == 3 ? kzf * g.cwlo[2] : 0.f, (ux >= nx) - (ux < 0),
                        (uy >= ny) - (uy < 0), DIM == 3 ? (uz >= nz) - (uz < 0) : 0);
            }
            ns = 0;
        };
        // the row's cells in stencil order as one or two runs of consecutive x:
        // run 0 = [xa0, xb0] starting at x offset ka0, run 1 = [xa1, xb1] (empty: xb1 < xa1)
        int xa0, xb0, ka0, xa1, xb1, ka1;
        if (len[0] == 1) { xa0 = 0; xb0 = 0; ka0 = 0; xa1 = 1; xb1 = 0; ka1 = 0; }
        else if (hx == 0) { xa0 = nx - 1; xb0 = nx - 1; ka0 = -1; xa1 = 0; xb1 = 1; ka1 = 0; }
        else if (hx == nx - 1) { xa0 = nx - 2; xb0 = nx - 1; ka0 = -1; xa1 = 0; xb1 = 0; ka1 = 1; }
        else { xa0 = hx - 1; xb0 = hx + 1; ka0 = -1; xa1 = 1; xb1 = 0; ka1 = 0; }
        for (int iz = 0; iz < len[2]; ++iz) {
            const int uz = lo[2] + iz;
            const int wz = DIM == 3 ? (uz < 0 ? uz + nz : (uz >= nz ? uz - nz : uz)) : 0;
            const float kz = (float)(uz - hz);
            const float oz = DIM == 3 ? kz * g.cwhi[2] : 0.f;
            for (int iy = 0; iy < len[1]; ++iy) {
                const int uy = lo[1] + iy;
                const int wy = uy < 0 ? uy + ny : (uy >= ny ? uy - ny : uy);
                const float ky = (float)(uy - hy);
                const float oy = ky * g.cwhi[1];
                const int row_code = 3 * (uy - hy + 1) + 9 * (uz - hz + 1) + 1; // + kx
                const int* rs = cell_start + (wz * ny + wy) * nx;
#pragma unroll
                for (int run = 0; run < 2; ++run) {
                    const int xa = run ? xa1 : xa0, xb = run ? xb1 : xb0, ka = run ? ka1 : ka0;
                    if (xb < xa) continue;
                    const int qa = rs[xa], qe = rs[xb + 1];
                    // inner cell boundaries of the run (past its end where it has fewer cells)
                    const int b1 = xb >= xa + 1 ? rs[xa + 1] : qe, b2 = xb >= xa + 2 ? rs[xa + 2] : qe;
                    const float kaf = (float)ka;
                    // the next candidate's record and diameter are loaded before the
                    // current one is screened, so that their latency overlaps the test
                    // (fused preparation 19.6 -> 18.4 us per frame)
                    IkPRec nxt = qa < qe ? prec[qa] : me;
                    float ndj = qa < qe ? diam32[qa] : di;
                    for (int q = qa; q < qe; ++q) {
                        const IkPRec cur = nxt;
                        const float cdj = ndj;
                        if (q + 1 < qe) { nxt = prec[q + 1]; ndj = diam32[q + 1]; }
                        if (q == p) continue;
                        // the candidate cell's x offset (-1, 0 or 1: exactly the float the
                        // cell-by-cell walk converts)
                        const float kxf = kaf + (q >= b1 ? 1.f : 0.f) + (q >= b2 ? 1.f : 0.f);
                        if (screen_rec(cur, cdj, kxf * g.cwhi[0], oy, oz)) {
                            qidx[ns * qstride] = q;
                            qcode[ns * qstride] = (unsigned char)(row_code + (int)kxf);
                            if (++ns == IK_BOND_QUEUE) drain();
                        }
                    }
                }
            }
        }
        drain();
    }
    nb[p] = cnt < maxb ? cnt : maxb;
    if (cnt > maxb) { // rare: grow the capacity and recompute (host side)
        atomicOr(status, IK_ST_BOND_OVERFLOW);
        atomicMax(maxnb, cnt);
    }
    return cnt;
}

