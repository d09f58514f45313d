// ik_gather32_exact.cu -- the FP32 gather with closed-form bond integrals of the
// truncated Gaussian (a third translation unit, compiled in parallel): quadrature mode 2
// (the closed form on bonds whose far end lies outside the support, the fixed-point
// rule elsewhere: the same bonds the learned surrogate stands in for) and mode 3 (the
// closed form on every bond).  Gaussian kernel only, plain per-lane sums (merged across
// lanes and chunks with TwoSum), as in surrogate mode.
#include "ik_gather32_kernel.cuh"

template <int DIM>
static cudaError_t launch_qm(const GatherArgs32& a, int qm, int blocks, int threads, size_t smem, cudaStream_t st)
{
    const bool split = a.maxb > 63; // more than 63 bonds per particle: several staged entries
    if (qm == 3)
        return split ? ik_launch_gather32_kernel<DIM, 1, false, 0, 3, false, true>(a, blocks, threads, smem, st)
                     : ik_launch_gather32_kernel<DIM, 1, false, 0, 3, false, false>(a, blocks, threads, smem, st);
    if (a.npairs == 2 && !split)
        return ik_launch_gather32_kernel<DIM, 1, false, 2, 2, false, false>(a, blocks, threads, smem, st);
    return ik_launch_gather32_kernel<DIM, 1, false, 0, 2, false, true>(a, blocks, threads, smem, st);
}

cudaError_t launch_gather32_exact(const GatherArgs32& a, int kind, bool kahan, int qm, int blocks, int threads,
                                  size_t smem, cudaStream_t st)
{
    (void)kahan; // plain per-lane sums in these modes
    if (kind != 1 || (qm != 2 && qm != 3) || a.bcoef) return cudaErrorInvalidValue;
    return a.geo.g.dim == 2 ? launch_qm<2>(a, qm, blocks, threads, smem, st) : launch_qm<3>(a, qm, blocks, threads, smem, st);
}
