// ik_batch.cu -- batch-wide preparation kernels of a fused batch: every stage of the
// FP32 path runs once over all frames of a batch (ik_compute_batch), instead of once per
// frame.  Frames keep their own boxes, grids and cell lists; their particles, cells,
// grid points and work items are concatenated in batch order, and every kernel finds
// the frame ("slot") of its particle, cell or value by a binary search over the batch's
// offsets.  Each stage computes exactly what the per-frame kernels compute (the same
// device functions, ik_prep_dev.cuh), so that a fused batch gives bit-identical fields.
//
// Launch sequence of a fused batch (all on one stream, recorded once as a CUDA graph):
//   k_bin32_batch       cell of every particle, its rank in the cell, double-float
//                       cell-relative position; zeroes the slots' counters; checks the
//                       positions (finite, z == 0 in 2D)
//   launch_scan         cell starts over the batch's concatenated cell counts
//   k_scatter           particle ids to cell order
//   k_sort_pack32_batch per cell: sorted ids, packed records; checks the diameters
//   k_bonds32t_batch    per particle: force-active bonds (records at a fixed stride)
//   k_gather32 (BATCH)  per work item of every frame: the stress field
//   k_pairs_to_f64_batch double-float sums -> each slot's FP64 fields
// Replaces, for a list of frames, the per-frame loop of IrvingKirkwood::compute over
// grid points (irvingkirkwood/IrvingKirkwood.h:76) run once per frame by analyze
// (pyglasstools/__init__.py:119-122).
#include "ik_prep_dev.cuh"
#include "../../include/ik_gb300.h"

#include <algorithm>

#define FULL 0xffffffffu

namespace {

// The slot of x: the last s with offs[s] <= x (offs ascending, nslots + 1 entries; an
// empty slot shares its offset with the next and is skipped).
__device__ __forceinline__ int ik_batch_slot(const int* __restrict__ offs, int nslots, int x)
{
    int lo = 0, hi = nslots - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(offs + mid) <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int ik_batch_slot64(const long long* __restrict__ offs, int nslots, long long x)
{
    int lo = 0, hi = nslots - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(offs + mid) <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Also checks every position (as k_validate does at an upload): a batch whose frames were
// copied in by its own graph is validated here, without a launch per frame.
__global__ void k_bin32_batch(const IkBatchSlot* __restrict__ S, const int* __restrict__ p_offs, int nslots,
                              int ptot, int* __restrict__ cell_of, int* __restrict__ rank,
                              int* __restrict__ cell_count, float4* __restrict__ relhi, float4* __restrict__ rello,
                              int* __restrict__ status)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    // the slots' counters (bonds, pairs, triples, surrogate records and fallbacks) start at
    // zero; the later stages add
    for (int k = i; k < 5 * nslots; k += gridDim.x * blockDim.x) S[k / 5].geo.cnt[k % 5] = 0ull;
    if (i >= ptot) return;
    const int s = ik_batch_slot(p_offs, nslots, i);
    const IkBatchSlot& sl = S[s];
    float4 rh, rl;
    const double* pi = sl.pos + 3 * (size_t)(i - sl.geo.p_off);
    if (!ik_pos_ok(pi, sl.geo.g.dim)) atomicOr(status, IK_ST_BAD_INPUT);
    const int c = sl.geo.c_off + ik_bin32_one(sl.geo.g, pi, rh, rl);
    cell_of[i] = c;
    rank[i] = atomicAdd(&cell_count[c], 1);
    relhi[i] = rh;
    rello[i] = rl;
}

// As k_cell_sort_pack32 over the batch's cells: a CTA sorts its 128 cells, then packs
// their particles (cell_of holds batch cell indices; a particle's frame is found by a
// search of the particle offsets), checking every diameter as k_validate does.
__global__ void __launch_bounds__(128) k_sort_pack32_batch(const IkBatchSlot* __restrict__ S,
                                                           const int* __restrict__ p_offs, int nslots, int ctot,
                                                           const int* __restrict__ cell_start,
                                                           int* __restrict__ sorted, const int* __restrict__ cell_of,
                                                           const float4* __restrict__ relhi,
                                                           const float4* __restrict__ rello,
                                                           IkPRec* __restrict__ prec, float4* __restrict__ plo,
                                                           IkB64* __restrict__ pos64, float4* __restrict__ kin,
                                                           float* __restrict__ diam32, int* __restrict__ status)
{
    const int c0 = blockIdx.x * blockDim.x, c = c0 + threadIdx.x;
    if (c < ctot) ik_sort_cell(cell_start[c], cell_start[c + 1], sorted);
    __syncthreads();
    const int pe = cell_start[min(c0 + (int)blockDim.x, ctot)];
    for (int p = cell_start[c0] + threadIdx.x; p < pe; p += blockDim.x) {
        const int ig = sorted[p];
        const IkBatchSlot& sl = S[ik_batch_slot(p_offs, nslots, ig)];
        if (!ik_diam_ok(sl.diam[ig - sl.geo.p_off])) atomicOr(status, IK_ST_BAD_INPUT);
        ik_pack_one(sl.geo.g.dim, cell_of[ig] - sl.geo.c_off, p, ig, sl.geo.p_off, relhi, rello, sl.pos, sl.vel,
                    sl.mass, sl.diam, prec, plo, pos64, kin, diam32);
    }
}

// Eight CTAs per SM (64 registers, a few bytes of spill): the bond build waits on its loads,
// and more resident warps hide that better (fused preparation 21.2 -> 19.4 us per frame).
template <int DIM, int KIND>
__global__ void __launch_bounds__(128, 8) k_bonds32t_batch(const IkBatchSlot* __restrict__ S,
                                                        const int* __restrict__ p_offs, int nslots, int ptot,
                                                        IkPot pot, IkPotF pf, float kappa,
                                                        const IkPRec* __restrict__ prec,
                                                        const float* __restrict__ diam32,
                                                        const int* __restrict__ cell_start,
                                                        const float4* __restrict__ plo,
                                                        const IkB64* __restrict__ pos64, float4* __restrict__ tmp,
                                                        int maxb, int* __restrict__ nb, int* __restrict__ status,
                                                        int* __restrict__ maxnb)
{
    __shared__ int s_qidx[IK_BOND_QUEUE * 128];
    __shared__ unsigned char s_qcode[IK_BOND_QUEUE * 128];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= ptot) return;
    const int s = ik_batch_slot(p_offs, nslots, p);
    const IkBatchSlot& sl = S[s];
    const int* cs = cell_start + sl.geo.c_off;
    int* qi = s_qidx + threadIdx.x;
    unsigned char* qc = s_qcode + threadIdx.x;
    const int cnt = sl.allax ? ik_bonds32_particle<DIM, KIND, true>(sl.geo.g, pot, pf, kappa, p, prec, diam32, cs,
                                                                    plo, pos64, tmp, maxb, nb, status, maxnb, qi, qc,
                                                                    128)
                             : ik_bonds32_particle<DIM, KIND, false>(sl.geo.g, pot, pf, kappa, p, prec, diam32, cs,
                                                                     plo, pos64, tmp, maxb, nb, status, maxnb, qi, qc,
                                                                     128);
    // force-active directed bonds per slot: one atomic per slot present in the warp
    const unsigned act = __activemask();
    const unsigned grp = __match_any_sync(act, s);
    const int tot = __reduce_add_sync(grp, cnt);
    if ((int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(&sl.geo.cnt[0], (unsigned long long)tot);
}

// out = ((double)hi + (double)lo) * scale into the slot's field, as k_pairs_to_f64;
// a field the batch does not compute is written as zeros.
__global__ void k_pairs_to_f64_batch(const IkBatchSlot* __restrict__ S, const long long* __restrict__ v_offs,
                                     int nslots, long long vtot, const float2* __restrict__ vin,
                                     const float2* __restrict__ kin, double svir, double skin, int fields)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= vtot) return;
    const int s = ik_batch_slot64(v_offs, nslots, k);
    const IkBatchSlot& sl = S[s];
    const long long o = k - __ldg(v_offs + s);
    if (sl.out_vir) {
        const float2 v = vin[k];
        sl.out_vir[o] = (fields & IK_FIELD_VIRIAL) ? ((double)v.x + (double)v.y) * svir : 0.0;
    }
    if (sl.out_kin) {
        const float2 v = kin[k];
        sl.out_kin[o] = (fields & IK_FIELD_KINETIC) ? ((double)v.x + (double)v.y) * skin : 0.0;
    }
}

} // namespace

cudaError_t launch_batch_prepare(const IkBatchLaunch& b, int dim, const IkPot& pot, float kappa, cudaStream_t st)
{
    const int T = 256;
    const int bin_threads = std::max(b.ptot, 5 * b.nslots);
    k_bin32_batch<<<(bin_threads + T - 1) / T, T, 0, st>>>(b.slots, b.p_offs, b.nslots, b.ptot, b.cell_of, b.rank,
                                                           b.cell_count, b.relhi, b.rello, b.status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if ((e = launch_scan(b.cell_count, b.ctot, b.cell_start, b.bsum, st)) != cudaSuccess) return e;
    if (b.ptot > 0) {
        k_scatter<<<(b.ptot + T - 1) / T, T, 0, st>>>(b.cell_of, b.rank, b.cell_start, b.ptot, b.sorted);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (b.ctot > 0) {
        k_sort_pack32_batch<<<(b.ctot + 127) / 128, 128, 0, st>>>(b.slots, b.p_offs, b.nslots, b.ctot, b.cell_start,
                                                                  b.sorted, b.cell_of, b.relhi, b.rello, b.prec, b.plo,
                                                                  b.pos64, b.kin, b.diam32, b.status);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (b.ptot > 0) {
        const int blocks = (b.ptot + 127) / 128;
        const IkPotF pf = ik_potf(pot);
        auto go = [&](auto kernel) {
            kernel<<<blocks, 128, 0, st>>>(b.slots, b.p_offs, b.nslots, b.ptot, pot, pf, kappa, b.prec, b.diam32,
                                           b.cell_start, b.plo, b.pos64, b.tmp, b.maxb, b.nb, b.status, b.maxnb);
        };
#define IK_BONDS32B_KIND(K)                                                   \
    case K:                                                                   \
        if (dim == 2) go(k_bonds32t_batch<2, K>);                            \
        else go(k_bonds32t_batch<3, K>);                                     \
        break;
        switch (pot.kind) {
            IK_BONDS32B_KIND(IKP_LJ)
            IK_BONDS32B_KIND(IKP_FSLJ)
            IK_BONDS32B_KIND(IKP_POLY10)
            IK_BONDS32B_KIND(IKP_POLY106)
            IK_BONDS32B_KIND(IKP_POLY18)
            IK_BONDS32B_KIND(IKP_POLYLJ)
            IK_BONDS32B_KIND(IKP_POLYYUKAWA)
        default: IK_BONDS32B_KIND(IKP_POLY12)
        }
#undef IK_BONDS32B_KIND
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_batch_finish(const IkBatchLaunch& b, const float2* vir2, const float2* kin2, double svir,
                                double skin, int fields, cudaStream_t st)
{
    if (b.vtot <= 0) return cudaSuccess;
    k_pairs_to_f64_batch<<<(int)((b.vtot + 255) / 256), 256, 0, st>>>(b.slots, b.v_offs, b.nslots, b.vtot, vir2, kin2,
                                                                      svir, skin, fields);
    return cudaGetLastError();
}
