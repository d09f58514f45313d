// ik_bonds.cu -- per-frame preparation of the tuned FP32 path: particle packing in
// cell order, the force-active bond list (one warp per particle) and its compaction
// into a CSR layout, and a multi-block exclusive scan.
//
// Replaces, for the tuned path, the Aboria neighbour search around each particle and
// the per-(grid point, pair) force evaluation of IrvingKirkwood::compute
// (irvingkirkwood/IrvingKirkwood.h:93-105 with potential/Polydisperse12.h:38-55): here
// the force of every directed bond is evaluated once per frame.
#include "ik_prep_dev.cuh"

#define FULL 0xffffffffu

// ---------------------------------------------------------------------------
// Cell index of every particle (atomic rank inside the cell; the order is fixed by
// the per-cell sort) and its position relative to the lower corner of its cell, as a
// double-float pair (hi = FP32 rounding, lo = FP32 rounding of the remainder; hi + lo
// carries ~48 bits).  One thread per particle, original order.
__global__ void k_bin32(const double* __restrict__ pos, int n, IkGeom g, int* __restrict__ cell_of,
                        int* __restrict__ rank, int* __restrict__ cell_count, float4* __restrict__ relhi,
                        float4* __restrict__ rello, int* __restrict__ status)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 rh, rl;
    if (!ik_pos_ok(pos + 3 * (size_t)i, g.dim)) atomicOr(status, IK_ST_BAD_INPUT); // k_validate's test
    const int c = ik_bin32_one(g, pos + 3 * (size_t)i, rh, rl);
    cell_of[i] = c;
    rank[i] = atomicAdd(&cell_count[c], 1);
    relhi[i] = rh;
    rello[i] = rl;
}

// ---------------------------------------------------------------------------
// Force-active bonds of a frame, one thread per particle (ik_bonds32_particle).
template <int DIM, int KIND, bool ALLAX>
__global__ void __launch_bounds__(128) k_bonds32t(IkGeom g, IkPot pot, IkPotF pf, float kappa, int n,
                                                  const IkPRec* __restrict__ prec,
                                                  const float* __restrict__ diam32,
                                                  const int* __restrict__ cell_start,
                                                  const float4* __restrict__ plo,
                                                  const IkB64* __restrict__ pos64, float4* __restrict__ tmp,
                                                  int maxb, int* __restrict__ nb, int* __restrict__ status,
                                                  int* __restrict__ maxnb, unsigned long long* nbond_total)
{
    __shared__ int s_qidx[IK_BOND_QUEUE * 128];
    __shared__ unsigned char s_qcode[IK_BOND_QUEUE * 128];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int cnt = ik_bonds32_particle<DIM, KIND, ALLAX>(g, pot, pf, kappa, p, prec, diam32, cell_start, plo,
                                                          pos64, tmp, maxb, nb, status, maxnb, s_qidx + threadIdx.x,
                                                          s_qcode + threadIdx.x, 128);
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
                         float4* rello, int* status, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_bin32<<<(n + 255) / 256, 256, 0, st>>>(pos, n, g, cell_of, rank, cell_count, relhi, rello, status);
    return cudaGetLastError();
}

// Sort the ids of each cell (insertion sort: cells hold a handful of particles; fixes
// the order the atomic ranks left) and pack the cell's particles in that order, one
// thread per cell.  (A frame alone has too few cells for the batch kernel's split into
// a sort per cell and a pack per particle to pay: its barrier lengthens the chain of
// dependent loads.)
__global__ void __launch_bounds__(128) k_cell_sort_pack32(IkGeom g, const int* __restrict__ cell_start,
                                                          int* __restrict__ sorted, const float4* __restrict__ relhi,
                                                          const float4* __restrict__ rello,
                                                          const double* __restrict__ pos,
                                                          const double* __restrict__ vel,
                                                          const double* __restrict__ mass,
                                                          const double* __restrict__ diam, IkPRec* __restrict__ prec,
                                                          float4* __restrict__ plo, IkB64* __restrict__ pos64,
                                                          float4* __restrict__ kin, float* __restrict__ diam32,
                                                          int* __restrict__ status)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncell) return;
    const int s = cell_start[c], e = cell_start[c + 1];
    ik_sort_cell(s, e, sorted);
    for (int p = s; p < e; ++p) {
        const int ig = sorted[p];
        if (!ik_diam_ok(diam[ig])) atomicOr(status, IK_ST_BAD_INPUT); // k_validate's test
        ik_pack_one(g.dim, c, p, ig, 0, relhi, rello, pos, vel, mass, diam, prec, plo, pos64, kin, diam32);
    }
}

cudaError_t launch_sort_pack32(IkGeom g, const int* cell_start, int* sorted, const float4* relhi, const float4* rello,
                               const double* pos, const double* vel, const double* mass, const double* diam,
                               IkPRec* prec, float4* plo, IkB64* pos64, float4* kin, float* diam32, int* status,
                               cudaStream_t st)
{
    if (g.ncell <= 0) return cudaSuccess;
    k_cell_sort_pack32<<<(g.ncell + 127) / 128, 128, 0, st>>>(g, cell_start, sorted, relhi, rello, pos, vel, mass,
                                                              diam, prec, plo, pos64, kin, diam32, status);
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
    const IkPotF pf = ik_potf(pot);
    auto go = [&](auto kernel) {
        kernel<<<blocks, threads, 0, st>>>(g, pot, pf, kappa, n, prec, diam32, cell_start, plo, pos64, tmp, maxb, nb,
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
