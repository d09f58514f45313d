// ik_gather32_batch.cu -- the FP32 gather of a fused batch (k_gather32 with BATCH set,
// a fourth translation unit, compiled in parallel): the work items of every frame of
// the batch in one persistent launch, each item's slot giving its geometry.  The
// fixed-point rule with two symmetric node pairs (Gauss-Legendre order 4 or 5), the four
// coarse-graining kernels, plain or Kahan-compensated per-lane sums.
#include "ik_gather32_kernel.cuh"

template <int DIM, bool KAHAN>
static cudaError_t launch_batch_kind(const GatherArgs32& a, int kind, int blocks, int threads, size_t smem,
                                     cudaStream_t st)
{
    switch (kind) {
    case 0: return ik_launch_gather32_kernel<DIM, 0, KAHAN, 2, 0, false, false, true>(a, blocks, threads, smem, st);
    case 1: return ik_launch_gather32_kernel<DIM, 1, KAHAN, 2, 0, false, false, true>(a, blocks, threads, smem, st);
    case 2: return ik_launch_gather32_kernel<DIM, 2, KAHAN, 2, 0, false, false, true>(a, blocks, threads, smem, st);
    default: return ik_launch_gather32_kernel<DIM, 3, KAHAN, 2, 0, false, false, true>(a, blocks, threads, smem, st);
    }
}

cudaError_t launch_gather32_batch(const GatherArgs32& a, int kind, bool kahan, int blocks, int threads, size_t smem,
                                  cudaStream_t st)
{
    if (a.npairs != 2 || !a.slots || !a.item_slot || a.bcoef || a.boff || a.maxb > 63) return cudaErrorInvalidValue;
    if (a.geo.g.dim == 2) return kahan ? launch_batch_kind<2, true>(a, kind, blocks, threads, smem, st)
                                       : launch_batch_kind<2, false>(a, kind, blocks, threads, smem, st);
    return kahan ? launch_batch_kind<3, true>(a, kind, blocks, threads, smem, st)
                 : launch_batch_kind<3, false>(a, kind, blocks, threads, smem, st);
}
