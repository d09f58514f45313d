// ik_bonds.cu -- per-frame preparation of the tuned FP32 path: particle packing in
// cell order, the force-active bond list (one warp per particle) and its compaction
// into a CSR layout, and a multi-block exclusive scan.
//
// Replaces, for the tuned path, the Aboria neighbour search around each particle and
// the per-(grid point, pair) force evaluation of IrvingKirkwood::compute
// (irvingkirkwood/IrvingKirkwood.h:93-105 with potential/Polydisperse12.h:38-55): here
// the force of every directed bond is evaluated once per frame.
#include "ik_kernels.h"

#define FULL 0xffffffffu

// ---------------------------------------------------------------------------
// Cell index of every particle (atomic rank inside the cell; the order is fixed by
// the per-cell sort) and its position relative to the lower corner of its cell, as a
// double-float pair (hi = FP32 rounding, lo = FP32 rounding of the remainder; hi + lo
// carries ~48 bits).  One thread per particle, original order.
__global__ void k_bin32(const double* __restrict__ pos, int n, IkGeom g, int* __restrict__ cell_of,
                        int* __restrict__ rank, int* __restrict__ cell_count, float4* __restrict__ relhi,
                        float4* __restrict__ rello)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double r[3] = {0.0, 0.0, 0.0};
    int cc[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (a >= g.dim || g.nc[a] == 1) continue;
        double t = (pos[3 * i + a] - g.lo[a]) * g.invL[a];
        t -= floor(t);
        int k = (int)(t * g.nc[a]);
        k = k < 0 ? 0 : (k >= g.nc[a] ? g.nc[a] - 1 : k);
        cc[a] = k;
        r[a] = t * g.L[a] - k * g.cw[a];
    }
    int c = (cc[2] * g.nc[1] + cc[1]) * g.nc[0] + cc[0];
    cell_of[i] = c;
    rank[i] = atomicAdd(&cell_count[c], 1);
    float hx = (float)r[0], hy = (float)r[1], hz = (float)r[2];
    relhi[i] = make_float4(hx, hy, hz, 0.f);
    rello[i] = make_float4((float)(r[0] - hx), (float)(r[1] - hy), (float)(r[2] - hz), 0.f);
}

// Pack the particles in cell order: the double-float cell-relative position, the raw
// FP64 position, kinetic coefficients m v(x)v, FP32 diameter.  One thread per sorted
// particle.
__global__ void k_pack32(IkGeom g, int n, const int* __restrict__ sorted, const int* __restrict__ cell_of,
                         const float4* __restrict__ relhi, const float4* __restrict__ rello,
                         const double* __restrict__ pos, const double* __restrict__ vel,
                         const double* __restrict__ mass, const double* __restrict__ diam,
                         IkPRec* __restrict__ prec, float4* __restrict__ plo, IkB64* __restrict__ pos64,
                         float4* __restrict__ kin, float* __restrict__ diam32)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int i = sorted[p];
    float4 h = relhi[i];
    IkPRec r;
    r.x = h.x;
    r.y = h.y;
    r.z = h.z;
    r.cell = cell_of[i];
    prec[p] = r;
    plo[p] = rello[i];
    pos64[p] = make_ikb64(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], diam[i]);
    double m = mass ? mass[i] : 1.0;
    double vx = vel ? vel[3 * i] : 0.0, vy = vel ? vel[3 * i + 1] : 0.0, vz = vel ? vel[3 * i + 2] : 0.0;
    if (g.dim == 2) {
        kin[p] = make_float4((float)(m * vx * vx), (float)(m * vy * vy), (float)(m * vx * vy), 0.f);
    } else {
        kin[2 * p] = make_float4((float)(m * vx * vx), (float)(m * vy * vy), (float)(m * vz * vz), (float)(m * vx * vy));
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
struct IkPotF {
    int kind;
    float rc2, eps_s, v0, v0x4, c1x2, c2x4, c3x6, kappa, shift;
};
__device__ __forceinline__ IkPotF ik_potf(const IkPot& p)
{
    IkPotF q;
    q.kind = p.kind;
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
template <int DIM, int KIND, bool ALLAX>
__global__ void __launch_bounds__(128) k_bonds32t(IkGeom g, IkPot pot, float kappa, int n,
                                                  const IkPRec* __restrict__ prec,
                                                  const float* __restrict__ diam32,
                                                  const int* __restrict__ cell_start,
                                                  const float4* __restrict__ plo,
                                                  const IkB64* __restrict__ pos64, float4* __restrict__ tmp,
                                                  int maxb, int* __restrict__ nb, int* __restrict__ status,
                                                  int* __restrict__ maxnb, unsigned long long* nbond_total)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
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
    const IkPotF pf = ik_potf(pot);
    const float rc2 = pf.rc2, mr2 = (float)pot.max_rcut_sq, eps = pf.eps_s;
    const float screen = 1.0f + 1e-4f;
    const float di = diam32[p];
    const float4 mlo = plo[p];
    const float hk = 0.5f * kappa, fk = 2.0f / (kappa * kappa);
    float4* out = tmp + (size_t)p * maxb;
    int cnt = 0;
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
                for (int q = cell_start[cell]; q < qe; ++q) {
                    if (q == p) continue;
                    const IkPRec o = prec[q];
                    float bx = ox + (o.x - me.x), by = oy + (o.y - me.y), bz = DIM == 3 ? oz + (o.z - me.z) : 0.f;
                    if (allx) bx -= L0 * rintf(bx / L0);
                    if (ally) by -= L1 * rintf(by / L1);
                    if (allz) bz -= L2 * rintf(bz / L2);
                    float r2 = bx * bx + by * by + bz * bz;
                    if (!(r2 < mr2 * screen)) continue;
                    const float dj = diam32[q];
                    const float sig = 0.5f * (di + dj) * (1.f - eps * fabsf(di - dj));
                    const float s2 = sig * sig;
                    if (!(r2 < rc2 * s2 * screen)) continue;
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
                    r2 = bx * bx + by * by + bz * bz;
                    const float rt = rc2 * s2;
                    bool act = r2 < mr2 && r2 < rt;
                    if (fabsf(r2 - rt) <= 2e-5f * rt || fabsf(r2 - mr2) <= 2e-5f * mr2) { // at a cut-off: FP64
                        if (ALLAX) act = ik_select64(g, pot, pos64[p], pos64[q]);
                        else act = ik_select64_shift(g, pot, pos64[p], pos64[q], (ux > wx) - (ux < wx),
                                                     (uy > wy) - (uy < wy), DIM == 3 ? (uz > wz) - (uz < wz) : 0);
                    }
                    if (act) {
                        const float f = ik_force32<KIND>(pf, r2, s2);
                        if (cnt < maxb) out[cnt] = make_float4(hk * bx, hk * by, hk * bz, fk * f);
                        ++cnt;
                    }
                }
            }
        }
    }
    nb[p] = cnt < maxb ? cnt : maxb;
    if (cnt > maxb) { // rare: grow the capacity and recompute (host side)
        atomicOr(status, IK_ST_BOND_OVERFLOW);
        atomicMax(maxnb, cnt);
    }
    if (nbond_total) { // force-active directed bonds of the frame (one atomic per warp)
        const unsigned act = __activemask();
        const int tot = __reduce_add_sync(act, cnt);
        if ((threadIdx.x & 31) == __ffs(act) - 1) atomicAdd(nbond_total, (unsigned long long)tot);
    }
}

// Compact the fixed-stride records into CSR order (boff = exclusive scan of nb); the
// first thread also stores the number of bonds, boff[n], in the frame's counters.
__global__ void k_bond_compact(int n, int maxb, const int* __restrict__ nb, const int* __restrict__ boff,
                               const float4* __restrict__ tmp, float4* __restrict__ bonds,
                               unsigned long long* __restrict__ nbond_total)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) *nbond_total = (unsigned long long)boff[n];
    int p = t / maxb, k = t - p * maxb;
    if (p >= n) return;
    if (k < nb[p]) bonds[boff[p] + k] = tmp[(size_t)p * maxb + k];
}

// ---------------------------------------------------------------------------
// Exclusive scan of n ints (any n < 2^31): per-block sums, then each block adds the
// sum of the blocks before it and scans its own tile.  Tiles of 4096 (1024 x 4).
__device__ __forceinline__ int ik_block_excl_scan(int v, int* wsum)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int w = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
        int wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(FULL, wi, o);
            if (lane >= o) wi += t;
        }
        wsum[lane] = wi - w;
    }
    __syncthreads();
    int r = wsum[wid] + incl - v;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(1024) k_scan_sums(const int* __restrict__ in, int n, int* __restrict__ bsum)
{
    __shared__ int red[32];
    int base = blockIdx.x * 4096 + threadIdx.x * 4, s = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) s += (base + k < n) ? in[base + k] : 0;
    s = __reduce_add_sync(FULL, s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        int t = red[threadIdx.x];
        t = __reduce_add_sync(FULL, t);
        if (threadIdx.x == 0) bsum[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(1024) k_scan_apply(const int* __restrict__ in, int n, const int* __restrict__ bsum,
                                                     int* __restrict__ out)
{
    __shared__ int wsum[32];
    __shared__ int prefix_s;
    // sum of the blocks before this one
    int pre = 0;
    for (int b = threadIdx.x; b < (int)blockIdx.x; b += blockDim.x) pre += bsum[b];
    pre = __reduce_add_sync(FULL, pre);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = pre;
    __syncthreads();
    if (threadIdx.x < 32) {
        int t = wsum[threadIdx.x];
        t = __reduce_add_sync(FULL, t);
        if (threadIdx.x == 0) prefix_s = t;
    }
    __syncthreads();
    const int prefix = prefix_s;
    int base = blockIdx.x * 4096 + threadIdx.x * 4;
    int v[4], s = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) { v[k] = (base + k < n) ? in[base + k] : 0; s += v[k]; }
    int run = prefix + ik_block_excl_scan(s, wsum);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = run;
}

cudaError_t launch_scan(const int* in, int n, int* out, int* bsum, cudaStream_t st)
{
    if (n <= 65536) { // one CTA walks the tiles with a carry: one launch
        k_scan<<<1, 1024, 0, st>>>(in, n, out);
        return cudaGetLastError();
    }
    int blocks = (n + 4095) / 4096;
    if (blocks < 1) blocks = 1;
    k_scan_sums<<<blocks, 1024, 0, st>>>(in, n, bsum);
    k_scan_apply<<<blocks, 1024, 0, st>>>(in, n, bsum, out);
    return cudaGetLastError();
}

cudaError_t launch_bin32(const double* pos, int n, IkGeom g, int* cell_of, int* rank, int* cell_count, float4* relhi,
                         float4* rello, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_bin32<<<(n + 255) / 256, 256, 0, st>>>(pos, n, g, cell_of, rank, cell_count, relhi, rello);
    return cudaGetLastError();
}

// Sort the ids of each cell (insertion sort: cells hold a handful of particles; fixes
// the order the atomic ranks left) and pack the cell's particles in that order: the
// two steps of k_cell_sort_pack + k_pack32 in one launch, one thread per cell.
__global__ void k_cell_sort_pack32(IkGeom g, const int* __restrict__ cell_start, int* __restrict__ sorted,
                                   const float4* __restrict__ relhi, const float4* __restrict__ rello,
                                   const double* __restrict__ pos, const double* __restrict__ vel,
                                   const double* __restrict__ mass, const double* __restrict__ diam,
                                   IkPRec* __restrict__ prec, float4* __restrict__ plo, IkB64* __restrict__ pos64,
                                   float4* __restrict__ kin, float* __restrict__ diam32)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncell) return;
    const int s = cell_start[c], e = cell_start[c + 1];
    for (int a = s + 1; a < e; ++a) {
        const int v = sorted[a];
        int b = a - 1;
        while (b >= s && sorted[b] > v) { sorted[b + 1] = sorted[b]; --b; }
        sorted[b + 1] = v;
    }
    for (int p = s; p < e; ++p) {
        const int i = sorted[p];
        const float4 h = relhi[i];
        IkPRec r;
        r.x = h.x;
        r.y = h.y;
        r.z = h.z;
        r.cell = c;
        prec[p] = r;
        plo[p] = rello[i];
        pos64[p] = make_ikb64(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], diam[i]);
        const double m = mass ? mass[i] : 1.0;
        const double vx = vel ? vel[3 * i] : 0.0, vy = vel ? vel[3 * i + 1] : 0.0, vz = vel ? vel[3 * i + 2] : 0.0;
        if (g.dim == 2) {
            kin[p] = make_float4((float)(m * vx * vx), (float)(m * vy * vy), (float)(m * vx * vy), 0.f);
        } else {
            kin[2 * p] = make_float4((float)(m * vx * vx), (float)(m * vy * vy), (float)(m * vz * vz),
                                     (float)(m * vx * vy));
            kin[2 * p + 1] = make_float4((float)(m * vx * vz), (float)(m * vy * vz), 0.f, 0.f);
        }
        diam32[p] = (float)diam[i];
    }
}

cudaError_t launch_sort_pack32(IkGeom g, const int* cell_start, int* sorted, const float4* relhi, const float4* rello,
                               const double* pos, const double* vel, const double* mass, const double* diam,
                               IkPRec* prec, float4* plo, IkB64* pos64, float4* kin, float* diam32, cudaStream_t st)
{
    if (g.ncell <= 0) return cudaSuccess;
    k_cell_sort_pack32<<<(g.ncell + 127) / 128, 128, 0, st>>>(g, cell_start, sorted, relhi, rello, pos, vel, mass,
                                                              diam, prec, plo, pos64, kin, diam32);
    return cudaGetLastError();
}

cudaError_t launch_pack32(IkGeom g, int n, const int* sorted, const int* cell_of, const float4* relhi,
                          const float4* rello, const double* pos, const double* vel, const double* mass,
                          const double* diam, IkPRec* prec, float4* plo, IkB64* pos64, float4* kin, float* diam32,
                          cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_pack32<<<(n + 255) / 256, 256, 0, st>>>(g, n, sorted, cell_of, relhi, rello, pos, vel, mass, diam, prec, plo,
                                              pos64, kin, diam32);
    return cudaGetLastError();
}

cudaError_t launch_bonds32(int dim, IkGeom g, IkPot pot, float kappa, int n, const IkPRec* prec,
                            const float* diam32, const int* cell_start, const float4* plo, const IkB64* pos64,
                            float4* tmp, int maxb, int* nb, int* status, int* maxnb,
                            unsigned long long* nbond_total, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const int threads = 128;
    const int blocks = (n + threads - 1) / threads;
    auto go = [&](auto kernel) {
        kernel<<<blocks, threads, 0, st>>>(g, pot, kappa, n, prec, diam32, cell_start, plo, pos64, tmp, maxb, nb,
                                           status, maxnb, nbond_total);
    };
    bool allax = false;
    for (int a = 0; a < dim; ++a) allax = allax || (g.all_bond[a] && g.nc[a] > 1);
#define IK_BONDS32_KIND(K)                                                        \
    case K:                                                                       \
        if (dim == 2) allax ? go(k_bonds32t<2, K, true>) : go(k_bonds32t<2, K, false>); \
        else allax ? go(k_bonds32t<3, K, true>) : go(k_bonds32t<3, K, false>);   \
        break;
    switch (pot.kind) {
        IK_BONDS32_KIND(IKP_LJ)
        IK_BONDS32_KIND(IKP_FSLJ)
        IK_BONDS32_KIND(IKP_POLY10)
        IK_BONDS32_KIND(IKP_POLY106)
        IK_BONDS32_KIND(IKP_POLY18)
        IK_BONDS32_KIND(IKP_POLYLJ)
        IK_BONDS32_KIND(IKP_POLYYUKAWA)
    default: IK_BONDS32_KIND(IKP_POLY12)
    }
#undef IK_BONDS32_KIND
    return cudaGetLastError();
}

cudaError_t launch_bond_compact(int n, int maxb, const int* nb, const int* boff, const float4* tmp, float4* bonds,
                                unsigned long long* nbond_total, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    long long t = (long long)n * maxb;
    k_bond_compact<<<(int)((t + 255) / 256), 256, 0, st>>>(n, maxb, nb, boff, tmp, bonds, nbond_total);
    return cudaGetLastError();
}
