// ik_gather32_aux.cu -- the FP32 gather variants instantiated apart from the headline
// ones (a second translation unit, compiled in parallel): the elastic field, and the
// frames with more than 63 bonds per particle (SPLIT staging, runtime node count).
#include "ik_gather32_kernel.cuh"

template <int DIM, int NP, int QM, bool ELA, bool KAHAN>
static cudaError_t launch_kinds(const GatherArgs32& a, int kind, int blocks, int threads, size_t smem,
                                cudaStream_t st)
{
    switch (kind) {
    case 0: return ik_launch_gather32_kernel<DIM, 0, KAHAN, NP, QM, ELA, true>(a, blocks, threads, smem, st);
    case 1: return ik_launch_gather32_kernel<DIM, 1, KAHAN, NP, QM, ELA, true>(a, blocks, threads, smem, st);
    case 2: return ik_launch_gather32_kernel<DIM, 2, KAHAN, NP, QM, ELA, true>(a, blocks, threads, smem, st);
    default: return ik_launch_gather32_kernel<DIM, 3, KAHAN, NP, QM, ELA, true>(a, blocks, threads, smem, st);
    }
}

cudaError_t launch_gather32_aux(const GatherArgs32& a, int kind, bool kahan, int qm, int blocks, int threads,
                                size_t smem, cudaStream_t st)
{
    const bool d2 = a.geo.g.dim == 2;
    if (a.bcoef) { // elastic field: plain per-lane sums, fixed-point rule
        if (qm) return cudaErrorInvalidValue;
        if (a.npairs == 2) return d2 ? launch_kinds<2, 2, 0, true, false>(a, kind, blocks, threads, smem, st)
                                     : launch_kinds<3, 2, 0, true, false>(a, kind, blocks, threads, smem, st);
        return d2 ? launch_kinds<2, 0, 0, true, false>(a, kind, blocks, threads, smem, st)
                  : launch_kinds<3, 0, 0, true, false>(a, kind, blocks, threads, smem, st);
    }
    if (qm >= 2) return launch_gather32_exact(a, kind, kahan, qm, blocks, threads, smem, st);
    if (qm == 1) { // Gaussian kernel only, plain per-lane sums
        if (kind != 1 || kahan) return cudaErrorInvalidValue;
        return d2 ? ik_launch_gather32_kernel<2, 1, false, 0, 1, false, true>(a, blocks, threads, smem, st)
                  : ik_launch_gather32_kernel<3, 1, false, 0, 1, false, true>(a, blocks, threads, smem, st);
    }
    if (kahan) return d2 ? launch_kinds<2, 0, 0, false, true>(a, kind, blocks, threads, smem, st)
                         : launch_kinds<3, 0, 0, false, true>(a, kind, blocks, threads, smem, st);
    return d2 ? launch_kinds<2, 0, 0, false, false>(a, kind, blocks, threads, smem, st)
              : launch_kinds<3, 0, 0, false, false>(a, kind, blocks, threads, smem, st);
}
