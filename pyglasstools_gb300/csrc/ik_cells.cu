// ik_cells.cu -- cell list (counting sort), FP32/FP64 force-active bond lists and the
// bit-exact FP64 candidate neighbour list.
//
// Replaces the Aboria cell list and its two radius searches in
// IrvingKirkwood::compute (irvingkirkwood/IrvingKirkwood.h:80-95) and
// ParticleSystem::init_neighbour_search (ParticleSystem.cc:13).
#include "ik_common.cuh"
#include "ik_kernels.h"
#include <algorithm>

// ---------------------------------------------------------------------------
// 1. cell id + rank within the cell (atomic, order fixed later by k_cell_sort)
__global__ void k_bin(const double* __restrict__ pos, int n, IkGeom g, int* __restrict__ cell_of,
                      int* __restrict__ rank, int* __restrict__ cell_count, int* __restrict__ status)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) atomicOr(status, IK_ST_BAD_INPUT);
    int cx = ik_cell_coord(g, 0, x);
    int cy = ik_cell_coord(g, 1, y);
    int cz = g.dim == 3 ? ik_cell_coord(g, 2, z) : 0;
    int c = (cz * g.nc[1] + cy) * g.nc[0] + cx;
    cell_of[i] = c;
    rank[i] = atomicAdd(&cell_count[c], 1);
}

// 1b. FP32 frame staging (pos 3n | vel 3n | mass n | diam n) widened to the slot's FP64
//     arrays (exact: every float is a double); vel/mass may be null (not uploaded).
__global__ void k_widen_frame(const float* __restrict__ st, int n, double* __restrict__ pos,
                              double* __restrict__ vel, double* __restrict__ mass, double* __restrict__ diam)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = 0; k < 3; ++k) {
        pos[3 * i + k] = (double)st[3 * i + k];
        if (vel) vel[3 * i + k] = (double)st[3 * (size_t)n + 3 * i + k];
    }
    if (mass) mass[i] = (double)st[6 * (size_t)n + i];
    diam[i] = (double)st[7 * (size_t)n + i];
}

// 2. exclusive scan of n ints into out[0..n] (single CTA of 1024 threads; tiles of
//    4096 with a running carry).  Used for cell starts and neighbour offsets.
__global__ void __launch_bounds__(1024) k_scan(const int* __restrict__ in, int n, int* __restrict__ out)
{
    __shared__ int wsum[32];
    __shared__ int carry_s;
    int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) carry_s = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 4096) {
        int v[4], s = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            int idx = base + tid * 4 + k;
            v[k] = idx < n ? in[idx] : 0;
            s += v[k];
        }
        int incl = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) wsum[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            int w = wsum[lane];
            int wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += t;
            }
            wsum[lane] = wi - w; // exclusive warp offsets
        }
        __syncthreads();
        int run = carry_s + wsum[wid] + incl - s;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            int idx = base + tid * 4 + k;
            if (idx < n) out[idx] = run;
            run += v[k];
        }
        __syncthreads();
        if (tid == 1023) carry_s = run;
        __syncthreads();
    }
    if (tid == 0) out[n] = carry_s;
}

// 3. scatter particle ids into cell order
__global__ void k_scatter(const int* __restrict__ cell_of, const int* __restrict__ rank,
                          const int* __restrict__ cell_start, int n, int* __restrict__ sorted)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    sorted[cell_start[cell_of[i]] + rank[i]] = i;
}

// 4. per cell: sort ids ascending (deterministic order), then write the FP32
//    particle records, kinetic coefficients and FP32 diameters in sorted order.
__global__ void k_cell_sort_pack(IkGeom g, const int* __restrict__ cell_start, int* __restrict__ sorted,
                                 const double* __restrict__ pos, const double* __restrict__ vel,
                                 const double* __restrict__ mass, const double* __restrict__ diam,
                                 IkPRec* __restrict__ prec, float4* __restrict__ kin,
                                 float* __restrict__ diam32, int want_pack)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncell) return;
    int s = cell_start[c], e = cell_start[c + 1];
    for (int a = s + 1; a < e; ++a) { // insertion sort (cells hold a handful of particles)
        int v = sorted[a], b = a - 1;
        while (b >= s && sorted[b] > v) { sorted[b + 1] = sorted[b]; --b; }
        sorted[b + 1] = v;
    }
    if (!want_pack) return;
    int cx = c % g.nc[0], cy = (c / g.nc[0]) % g.nc[1], cz = c / (g.nc[0] * g.nc[1]);
    double ox = g.lo[0] + cx * g.cw[0], oy = g.lo[1] + cy * g.cw[1], oz = g.lo[2] + cz * g.cw[2];
    for (int p = s; p < e; ++p) {
        int i = sorted[p];
        double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
        x -= g.L[0] * floor((x - g.lo[0]) / g.L[0]);
        y -= g.L[1] * floor((y - g.lo[1]) / g.L[1]);
        if (g.dim == 3) z -= g.L[2] * floor((z - g.lo[2]) / g.L[2]);
        IkPRec r;
        r.x = (float)(x - ox);
        r.y = (float)(y - oy);
        r.z = g.dim == 3 ? (float)(z - oz) : 0.0f;
        r.cell = c;
        prec[p] = r;
        double m = mass ? mass[i] : 1.0;
        double vx = vel ? vel[3 * i] : 0.0, vy = vel ? vel[3 * i + 1] : 0.0, vz = vel ? vel[3 * i + 2] : 0.0;
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

// ---------------------------------------------------------------------------
// Stencil enumeration shared by the bond builders.  For axis c: if all_bond[c]
// the axis is scanned once over all its cells (offset computed per pair by the
// minimum image), else offsets -reach..+reach around the home cell.
struct StencilAxis { int lo, hi, all; };
__device__ __forceinline__ StencilAxis ik_axis(const IkGeom& g, int c, int home)
{
    StencilAxis a;
    if (g.nc[c] == 1) { a.lo = 0; a.hi = 0; a.all = 1; return a; }
    if (g.all_bond[c]) { a.lo = 0; a.hi = g.nc[c] - 1; a.all = 1; return a; }
    a.lo = home - g.reach_bond[c]; a.hi = home + g.reach_bond[c]; a.all = 0;
    return a;
}

// 5b. FP64 force-active bond records (plain path): {rij.x, rij.y, rij.z, forceDivR}
//     in sorted-particle order, bit-identical selection to the oracle.
__global__ void k_bonds64(IkGeom g, IkPot pot, int n, const int* __restrict__ sorted,
                          const int* __restrict__ cell_of, const double* __restrict__ pos,
                          const double* __restrict__ diam, const int* __restrict__ cell_start,
                          IkB64* __restrict__ bonds, int maxb, int* __restrict__ nb,
                          int* __restrict__ status, int* __restrict__ maxnb)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int i = sorted[p];
    int c = cell_of[i];
    int cx = c % g.nc[0], cy = (c / g.nc[0]) % g.nc[1], cz = c / (g.nc[0] * g.nc[1]);
    double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2], di = diam[i];
    int cnt = 0;
    StencilAxis az = ik_axis(g, 2, cz), ay = ik_axis(g, 1, cy), ax = ik_axis(g, 0, cx);
    for (int zz = az.lo; zz <= az.hi; ++zz) {
        int wz = g.dim == 3 ? ik_wrap(zz, g.nc[2]) : 0;
        for (int yy = ay.lo; yy <= ay.hi; ++yy) {
            int wy = ik_wrap(yy, g.nc[1]);
            for (int xx = ax.lo; xx <= ax.hi; ++xx) {
                int wx = ik_wrap(xx, g.nc[0]);
                int cell = (wz * g.nc[1] + wy) * g.nc[0] + wx;
                int e = cell_start[cell + 1];
                for (int q = cell_start[cell]; q < e; ++q) {
                    int j = sorted[q];
                    if (j == i) continue;
                    double dx = ik_minimg(__dsub_rn(pos[3 * j], xi), g.L[0], g.periodic[0]);
                    double dy = ik_minimg(__dsub_rn(pos[3 * j + 1], yi), g.L[1], g.periodic[1]);
                    double dz = ik_minimg(__dsub_rn(pos[3 * j + 2], zi), g.L[2], g.periodic[2]);
                    double rsq = ik_dot3(dx, dy, dz);
                    if (!(rsq < pot.max_rcut_sq)) continue;
                    double sig = ik_sigma64(pot, di, diam[j]);
                    if (!ik_active64(pot, rsq, sig)) continue;
                    double f = ik_force64(pot, rsq, sig);
                    if (cnt < maxb) bonds[(size_t)p * maxb + cnt] = make_ikb64(dx, dy, dz, f);
                    ++cnt;
                }
            }
        }
    }
    nb[p] = cnt < maxb ? cnt : maxb;
    if (cnt > maxb) { // rare: grow the capacity and recompute (host side)
        atomicOr(status, IK_ST_BOND_OVERFLOW);
        atomicMax(maxnb, cnt);
    }
}

// ---------------------------------------------------------------------------
// 5b. Bonds of the elastic virial field (ElasticVirialStress::compute,
//     ListofCommonObservables.h:86-122, through VirialStress::compute_cg, :72-82):
//     every neighbour within max_rcut of the undisplaced frame, u_ij = u_j - u_i,
//     coefficient C = 0.5 (f(|r+u|) (r+u)(x)(r+u) - f(|r|) r(x)r), all in FP64; a
//     record is kept when either force is non-zero.  Written for both gathers at a
//     fixed stride of maxb per particle (cell order): FP64 {r_ij} + C (NC doubles),
//     FP32 {kappa r_ij / 2} + C (float4 x CW).
__global__ void k_bonds64e(IkGeom g, IkPot pot, float kappa, int n, const int* __restrict__ sorted,
                           const int* __restrict__ cell_of, const double* __restrict__ pos,
                           const double* __restrict__ disp, const double* __restrict__ diam,
                           const int* __restrict__ cell_start, IkB64* __restrict__ b64,
                           double* __restrict__ c64, float4* __restrict__ b32, float4* __restrict__ c32,
                           int maxb, int* __restrict__ nb, int* __restrict__ status, int* __restrict__ maxnb)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int NC = g.dim == 2 ? 3 : 6, CW = g.dim == 2 ? 1 : 2;
    const int i = sorted[p];
    const int c = cell_of[i];
    const int cx = c % g.nc[0], cy = (c / g.nc[0]) % g.nc[1], cz = c / (g.nc[0] * g.nc[1]);
    const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2], di = diam[i];
    const double uxi = disp[3 * i], uyi = disp[3 * i + 1], uzi = disp[3 * i + 2];
    const float hk = 0.5f * kappa;
    int cnt = 0;
    StencilAxis az = ik_axis(g, 2, cz), ay = ik_axis(g, 1, cy), ax = ik_axis(g, 0, cx);
    for (int zz = az.lo; zz <= az.hi; ++zz) {
        const int wz = g.dim == 3 ? ik_wrap(zz, g.nc[2]) : 0;
        for (int yy = ay.lo; yy <= ay.hi; ++yy) {
            const int wy = ik_wrap(yy, g.nc[1]);
            for (int xx = ax.lo; xx <= ax.hi; ++xx) {
                const int wx = ik_wrap(xx, g.nc[0]);
                const int cell = (wz * g.nc[1] + wy) * g.nc[0] + wx;
                const int e = cell_start[cell + 1];
                for (int q = cell_start[cell]; q < e; ++q) {
                    const int j = sorted[q];
                    if (j == i) continue;
                    const double dx = ik_minimg(__dsub_rn(pos[3 * j], xi), g.L[0], g.periodic[0]);
                    const double dy = ik_minimg(__dsub_rn(pos[3 * j + 1], yi), g.L[1], g.periodic[1]);
                    const double dz = ik_minimg(__dsub_rn(pos[3 * j + 2], zi), g.L[2], g.periodic[2]);
                    const double rsq = ik_dot3(dx, dy, dz);
                    if (!(rsq < pot.max_rcut_sq)) continue;
                    const double sig = ik_sigma64(pot, di, diam[j]);
                    const double f = ik_active64(pot, rsq, sig) ? ik_force64(pot, rsq, sig) : 0.0;
                    const double ux = __dadd_rn(__dsub_rn(disp[3 * j], uxi), dx);
                    const double uy = __dadd_rn(__dsub_rn(disp[3 * j + 1], uyi), dy);
                    const double uz = __dadd_rn(__dsub_rn(disp[3 * j + 2], uzi), dz);
                    const double usq = ik_dot3(ux, uy, uz);
                    const double f1 = ik_active64(pot, usq, sig) ? ik_force64(pot, usq, sig) : 0.0;
                    if (f == 0.0 && f1 == 0.0) continue;
                    if (cnt < maxb) {
                        const double r[3] = {dx, dy, dz}, u[3] = {ux, uy, uz};
                        const int ia[6] = {0, 1, 2, 0, 0, 1}, ib[6] = {0, 1, 2, 1, 2, 2};
                        const int ia2[3] = {0, 1, 0}, ib2[3] = {0, 1, 1};
                        double cc[6];
                        for (int k = 0; k < NC; ++k) {
                            const int a_ = g.dim == 2 ? ia2[k] : ia[k], b_ = g.dim == 2 ? ib2[k] : ib[k];
                            cc[k] = 0.5 * __dsub_rn(__dmul_rn(__dmul_rn(f1, u[a_]), u[b_]),
                                                    __dmul_rn(__dmul_rn(f, r[a_]), r[b_]));
                        }
                        const size_t rec = (size_t)p * maxb + cnt;
                        b64[rec] = make_ikb64(dx, dy, dz, 0.0);
                        for (int k = 0; k < NC; ++k) c64[rec * NC + k] = cc[k];
                        b32[rec] = make_float4(hk * (float)dx, hk * (float)dy, hk * (float)dz, 0.f);
                        c32[rec * CW] = make_float4((float)cc[0], (float)cc[1], (float)cc[2], NC > 3 ? (float)cc[3] : 0.f);
                        if (CW == 2) c32[rec * CW + 1] = make_float4((float)cc[4], (float)cc[5], 0.f, 0.f);
                    }
                    ++cnt;
                }
            }
        }
    }
    nb[p] = cnt < maxb ? cnt : maxb;
    if (cnt > maxb) {
        atomicOr(status, IK_ST_BOND_OVERFLOW);
        atomicMax(maxnb, cnt);
    }
}

// ---------------------------------------------------------------------------
// 6. Candidate neighbour list (FP64, |r_ij|^2 < radius^2, j != i), CSR by
//    original particle id; count pass, scan, fill pass, per-row sort.
template <bool FILL>
__global__ void k_neigh(IkGeom g, int n, double r2cut, const int* __restrict__ sorted,
                        const int* __restrict__ cell_of, const double* __restrict__ pos,
                        const int* __restrict__ cell_start, int* __restrict__ count,
                        const int* __restrict__ offs, int* __restrict__ idx)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = cell_of[i];
    int cx = c % g.nc[0], cy = (c / g.nc[0]) % g.nc[1], cz = c / (g.nc[0] * g.nc[1]);
    double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
    int cnt = 0, base = FILL ? offs[i] : 0;
    StencilAxis az = ik_axis(g, 2, cz), ay = ik_axis(g, 1, cy), ax = ik_axis(g, 0, cx);
    for (int zz = az.lo; zz <= az.hi; ++zz) {
        int wz = g.dim == 3 ? ik_wrap(zz, g.nc[2]) : 0;
        for (int yy = ay.lo; yy <= ay.hi; ++yy) {
            int wy = ik_wrap(yy, g.nc[1]);
            for (int xx = ax.lo; xx <= ax.hi; ++xx) {
                int wx = ik_wrap(xx, g.nc[0]);
                int cell = (wz * g.nc[1] + wy) * g.nc[0] + wx;
                int e = cell_start[cell + 1];
                for (int q = cell_start[cell]; q < e; ++q) {
                    int j = sorted[q];
                    if (j == i) continue;
                    double dx = ik_minimg(__dsub_rn(pos[3 * j], xi), g.L[0], g.periodic[0]);
                    double dy = ik_minimg(__dsub_rn(pos[3 * j + 1], yi), g.L[1], g.periodic[1]);
                    double dz = ik_minimg(__dsub_rn(pos[3 * j + 2], zi), g.L[2], g.periodic[2]);
                    if (ik_dot3(dx, dy, dz) < r2cut) {
                        if (FILL) idx[base + cnt] = j;
                        ++cnt;
                    }
                }
            }
        }
    }
    if (!FILL) { count[i] = cnt; return; }
    int* row = idx + base;
    for (int a = 1; a < cnt; ++a) {
        int v = row[a], b = a - 1;
        while (b >= 0 && row[b] > v) { row[b + 1] = row[b]; --b; }
        row[b + 1] = v;
    }
}
cudaError_t launch_neigh(bool fill, IkGeom g, int n, double r2cut, const int* sorted, const int* cell_of,
                         const double* pos, const int* cell_start, int* count, const int* offs, int* idx,
                         cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    int blocks = (n + 127) / 128;
    if (fill) k_neigh<true><<<blocks, 128, 0, st>>>(g, n, r2cut, sorted, cell_of, pos, cell_start, count, offs, idx);
    else k_neigh<false><<<blocks, 128, 0, st>>>(g, n, r2cut, sorted, cell_of, pos, cell_start, count, offs, idx);
    return cudaGetLastError();
}

// 7. particles within radius of a point (flag per particle, FP64 min-image)
__global__ void k_point_query(IkGeom g, int n, const double* __restrict__ pos, double px, double py,
                              double pz, double r2cut, unsigned char* __restrict__ flag)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double dx = ik_minimg(__dsub_rn(px, pos[3 * i]), g.L[0], g.periodic[0]);
    double dy = ik_minimg(__dsub_rn(py, pos[3 * i + 1]), g.L[1], g.periodic[1]);
    double dz = ik_minimg(__dsub_rn(pz, pos[3 * i + 2]), g.L[2], g.periodic[2]);
    flag[i] = ik_dot3(dx, dy, dz) < r2cut ? 1 : 0;
}

// 8. scalar evaluations for the Python-facing getPairForceDivR / getBondFunc
__global__ void k_eval_pair(IkPot pot, int m, const double* __restrict__ rij, const double* __restrict__ di,
                            const double* __restrict__ dj, double* __restrict__ f, double* __restrict__ en)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    double rsq = ik_dot3(rij[3 * k], rij[3 * k + 1], rij[3 * k + 2]);
    const double sig = ik_sigma64(pot, di[k], dj[k]);
    f[k] = ik_active64(pot, rsq, sig) ? ik_force64(pot, rsq, sig) : 0.0;
    // computeEnergy: its own sigma (force-shifted LJ: the non-additive one) and cut-off
    const double sie = ik_sigma64(pot, di[k], dj[k], false);
    en[k] = rsq < __dmul_rn(__dmul_rn(pot.rcutsq, sie), sie) ? ik_energy64(pot, rsq, sie) : 0.0;
}

// 9. FP32 FMA throughput probe: IK_FMA_PROBE_CHAINS independent FFMA chains per thread.
__global__ void __launch_bounds__(256) k_fma_probe(int iters, float* out)
{
    float a[IK_FMA_PROBE_CHAINS];
    float m = 1.0f + 1e-7f * threadIdx.x, c = 1e-7f;
#pragma unroll
    for (int k = 0; k < IK_FMA_PROBE_CHAINS; ++k) a[k] = (float)k * 1e-3f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < IK_FMA_PROBE_CHAINS; ++k) a[k] = fmaf(a[k], m, c);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < IK_FMA_PROBE_CHAINS; ++k) s += a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

cudaError_t launch_fma_probe(int blocks, int threads, int iters, float* out)
{
    k_fma_probe<<<blocks, threads>>>(iters, out);
    return cudaGetLastError();
}

// 10. frame validation at upload: finite positions, diameters > 0, z == 0 in 2D
__global__ void k_validate(const double* __restrict__ pos, const double* __restrict__ diam, int n, int dim,
                           int* __restrict__ status)
{
    // integer tests on the IEEE-754 bits (no FP64 instructions): finite = exponent
    // field not all ones; d > 0 = sign clear and not +0; z == 0 = all bits but the sign clear
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long* p = reinterpret_cast<const long long*>(pos) + 3 * (size_t)i;
    long long x = p[0], y = p[1], z = p[2], d = reinterpret_cast<const long long*>(diam)[i];
    const long long EXP = 0x7ff0000000000000LL, ABS = 0x7fffffffffffffffLL;
    bool ok = (x & EXP) != EXP && (y & EXP) != EXP && (z & EXP) != EXP && (d & EXP) != EXP && d > 0 &&
              (dim == 3 || (z & ABS) == 0);
    if (!ok) atomicOr(status, IK_ST_BAD_INPUT);
}

// Host copies of a batch as one kernel (the copies of many small frames without a copy
// node each): thread w copies word w of the concatenation, its copy found by a binary
// search of the offsets, and applies the copy's checks (the tests of k_validate on the
// IEEE-754 bits).
__global__ void k_io_copy(const IkIoCopy* __restrict__ d, int n, long long total, int* __restrict__ status)
{
    const long long EXP = 0x7ff0000000000000LL, ABS = 0x7fffffffffffffffLL;
    bool ok = true;
    for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < total;
         w += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(&d[mid].off) <= w) lo = mid;
            else hi = mid - 1;
        }
        const long long k = w - __ldg(&d[lo].off);
        const long long v = d[lo].src[k];
        d[lo].dst[k] = v;
        const int check = __ldg(&d[lo].check);
        if (check == 1) ok = ok && (v & EXP) != EXP && (__ldg(&d[lo].dim) == 3 || k % 3 != 2 || (v & ABS) == 0);
        else if (check == 2) ok = ok && (v & EXP) != EXP && v > 0;
    }
    if (!ok) atomicOr(status, IK_ST_BAD_INPUT);
}

cudaError_t launch_io_copy(const IkIoCopy* d, int n, long long total, int* status, int sm_count, cudaStream_t st)
{
    if (n <= 0 || total <= 0) return cudaSuccess;
    const int T = 256;
    const long long want = (total + T - 1) / T;
    const int blocks = (int)std::min<long long>(want, (long long)sm_count * 8);
    k_io_copy<<<blocks, T, 0, st>>>(d, n, total, status);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// 10. Global thermodynamic observables (ThermoCalculator::compute,
//     thermo/ThermoCalculator.h:68-90): one thread per particle in cell order; its kinetic
//     term m v (x) v and, over the stencil, every neighbour j within max_rcut with a
//     larger id (unique pairs i < j as there), r_ij = r_i - r_j (Aboria's p_j.dx()):
//       energy, virial F (x) r, elastic virial F1 (x) (u + r) - F (x) r with u = u_j - u_i,
//       and the Born tensor (s r_i + F_i) r_j n_k n_l = (s + f) r_i r_j r_k r_l / r^2,
//       kept as its fully symmetric components (i <= j <= k <= l).
//     FP64 per thread, then a fixed-order block reduction into per-block partials; the
//     final sums run over the blocks in order (k_thermo_final): deterministic.
template <int DIM>
struct ThermoLayout {
    static constexpr int D2 = DIM * DIM;
    static constexpr int NB = DIM == 2 ? 5 : 15; // symmetric 4-tensor components
    static constexpr int NQ = 1 + 3 * D2 + NB;
};

template <int DIM>
__global__ void __launch_bounds__(128) k_thermo64(IkGeom g, IkPot pot, int n, const int* __restrict__ sorted,
                                                  const int* __restrict__ cell_of, const double* __restrict__ pos,
                                                  const double* __restrict__ vel, const double* __restrict__ mass,
                                                  const double* __restrict__ diam, const double* __restrict__ disp,
                                                  const int* __restrict__ cell_start, double* __restrict__ partial)
{
    using TL = ThermoLayout<DIM>;
    constexpr int D2 = TL::D2, NQ = TL::NQ;
    double acc[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k) acc[k] = 0.0;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) {
        const int i = sorted[p];
        const double m = mass ? mass[i] : 1.0;
        if (vel) {
#pragma unroll
            for (int b = 0; b < DIM; ++b)
#pragma unroll
                for (int a = 0; a < DIM; ++a)
                    acc[1 + 2 * D2 + a + DIM * b] = __dmul_rn(__dmul_rn(m, vel[3 * i + a]), vel[3 * i + b]);
        }
        const int c = cell_of[i];
        const int cx = c % g.nc[0], cy = (c / g.nc[0]) % g.nc[1], cz = c / (g.nc[0] * g.nc[1]);
        const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2], di = diam[i];
        StencilAxis az = ik_axis(g, 2, cz), ay = ik_axis(g, 1, cy), ax = ik_axis(g, 0, cx);
        for (int zz = az.lo; zz <= az.hi; ++zz) {
            const int wz = DIM == 3 ? ik_wrap(zz, g.nc[2]) : 0;
            for (int yy = ay.lo; yy <= ay.hi; ++yy) {
                const int wy = ik_wrap(yy, g.nc[1]);
                for (int xx = ax.lo; xx <= ax.hi; ++xx) {
                    const int wx = ik_wrap(xx, g.nc[0]);
                    const int cell = (wz * g.nc[1] + wy) * g.nc[0] + wx;
                    const int e = cell_start[cell + 1];
                    for (int q = cell_start[cell]; q < e; ++q) {
                        const int j = sorted[q];
                        if (j <= i) continue;
                        double r[3];
                        r[0] = ik_minimg(__dsub_rn(xi, pos[3 * j]), g.L[0], g.periodic[0]);
                        r[1] = ik_minimg(__dsub_rn(yi, pos[3 * j + 1]), g.L[1], g.periodic[1]);
                        r[2] = ik_minimg(__dsub_rn(zi, pos[3 * j + 2]), g.L[2], g.periodic[2]);
                        const double rsq = ik_dot3(r[0], r[1], r[2]);
                        if (!(rsq < pot.max_rcut_sq)) continue;
                        const double dj = diam[j];
                        const double sie = ik_sigma64(pot, di, dj, false); // energy / stiffness sigma
                        if (rsq < __dmul_rn(__dmul_rn(pot.rcutsq, sie), sie)) acc[0] += ik_energy64(pot, rsq, sie);
                        const double sig = ik_sigma64(pot, di, dj);
                        const double f = ik_active64(pot, rsq, sig) ? ik_force64(pot, rsq, sig) : 0.0;
#pragma unroll
                        for (int b = 0; b < DIM; ++b)
#pragma unroll
                            for (int a = 0; a < DIM; ++a) acc[1 + a + DIM * b] += __dmul_rn(__dmul_rn(f, r[a]), r[b]);
                        if (disp) {
                            double w[3];
#pragma unroll
                            for (int k = 0; k < 3; ++k) w[k] = __dadd_rn(__dsub_rn(disp[3 * j + k], disp[3 * i + k]), r[k]);
                            const double wsq = ik_dot3(w[0], w[1], w[2]);
                            const double f1 = ik_active64(pot, wsq, sig) ? ik_force64(pot, wsq, sig) : 0.0;
#pragma unroll
                            for (int b = 0; b < DIM; ++b)
#pragma unroll
                                for (int a = 0; a < DIM; ++a)
                                    acc[1 + D2 + a + DIM * b] += __dsub_rn(__dmul_rn(__dmul_rn(f1, w[a]), w[b]),
                                                                           __dmul_rn(__dmul_rn(f, r[a]), r[b]));
                        }
                        const double st = ik_active64(pot, rsq, sie) ? ik_stiffness64(pot, rsq, sie) : 0.0;
                        const double cb = (st + f) / rsq;
                        int u = 1 + 3 * D2;
#pragma unroll
                        for (int a = 0; a < DIM; ++a)
#pragma unroll
                            for (int b = a; b < DIM; ++b)
#pragma unroll
                                for (int k = b; k < DIM; ++k)
#pragma unroll
                                    for (int l = k; l < DIM; ++l) acc[u++] += cb * r[a] * r[b] * r[k] * r[l];
                    }
                }
            }
        }
    }
    // block reduction: warps by shuffles (fixed tree), then the warps in order
    __shared__ double red[4][NQ];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
        double v = acc[k];
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < NQ) {
        double v = red[0][threadIdx.x];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v += red[w][threadIdx.x];
        partial[(size_t)blockIdx.x * NQ + threadIdx.x] = v;
    }
}

__global__ void k_thermo_final(const double* __restrict__ partial, int nblocks, int nq, double inv_vol,
                               double* __restrict__ out)
{
    const int k = threadIdx.x;
    if (k >= nq) return;
    double v = 0.0;
    for (int b = 0; b < nblocks; ++b) v += partial[(size_t)b * nq + k];
    out[k] = v * inv_vol;
}

int ik_thermo_nq(int dim) { return dim == 2 ? ThermoLayout<2>::NQ : ThermoLayout<3>::NQ; }

cudaError_t launch_thermo64(const IkGeom& g, const IkPot& pot, int n, const int* sorted, const int* cell_of,
                            const double* pos, const double* vel, const double* mass, const double* diam,
                            const double* disp, const int* cell_start, double* partial, int nblocks,
                            double inv_vol, double* out, cudaStream_t st)
{
    if (nblocks > 0) {
        if (g.dim == 2)
            k_thermo64<2><<<nblocks, 128, 0, st>>>(g, pot, n, sorted, cell_of, pos, vel, mass, diam, disp,
                                                   cell_start, partial);
        else
            k_thermo64<3><<<nblocks, 128, 0, st>>>(g, pot, n, sorted, cell_of, pos, vel, mass, diam, disp,
                                                   cell_start, partial);
    }
    k_thermo_final<<<1, 64, 0, st>>>(partial, nblocks, ik_thermo_nq(g.dim), inv_vol, out);
    return cudaGetLastError();
}
