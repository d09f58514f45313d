// ik_gather32.cu -- launchers of the tuned FP32 gather (k_gather32, in
// ik_gather32_kernel.cuh) for frames with at most 63 bonds per particle, and the FP64
// conversion of its double-float results.  The elastic-field variants and the
// variants for more bonds per particle are instantiated in ik_gather32_aux.cu (a
// second translation unit, compiled in parallel).
#include "ik_gather32_kernel.cuh"
template <int DIM, int KIND, bool KAHAN, int NP, int QM = 0>
static cudaError_t launch_one(const GatherArgs32& a, int blocks, int threads, size_t smem, cudaStream_t st)
{
    return ik_launch_gather32_kernel<DIM, KIND, KAHAN, NP, QM, false, false>(a, blocks, threads, smem, st);
}

template <int DIM, bool KAHAN, int NP>
static cudaError_t launch_kind(const GatherArgs32& a, int kind, int blocks, int threads, size_t smem,
                               cudaStream_t st)
{
    switch (kind) {
    case 0: return launch_one<DIM, 0, KAHAN, NP>(a, blocks, threads, smem, st);
    case 1: return launch_one<DIM, 1, KAHAN, NP>(a, blocks, threads, smem, st);
    case 2: return launch_one<DIM, 2, KAHAN, NP>(a, blocks, threads, smem, st);
    default: return launch_one<DIM, 3, KAHAN, NP>(a, blocks, threads, smem, st);
    }
}

template <int DIM, bool KAHAN>
static cudaError_t launch_np(const GatherArgs32& a, int kind, int blocks, int threads, size_t smem, cudaStream_t st)
{
    if (a.npairs == 2) return launch_kind<DIM, KAHAN, 2>(a, kind, blocks, threads, smem, st);
    return launch_kind<DIM, KAHAN, 0>(a, kind, blocks, threads, smem, st);
}

cudaError_t launch_gather32(const GatherArgs32& a, int kind, bool kahan, int qm, int blocks, int threads,
                            size_t smem, cudaStream_t st)
{
    if (a.bcoef || a.maxb > 63) return launch_gather32_aux(a, kind, kahan, qm, blocks, threads, smem, st);
    if (qm >= 2) return launch_gather32_exact(a, kind, kahan, qm, blocks, threads, smem, st);
    if (qm == 1) { // Gaussian kernel only, plain per-lane sums
        if (kind != 1 || kahan) return cudaErrorInvalidValue;
        if (a.geo.g.dim == 2) return a.npairs == 2 ? launch_one<2, 1, false, 2, 1>(a, blocks, threads, smem, st)
                                               : launch_one<2, 1, false, 0, 1>(a, blocks, threads, smem, st);
        return a.npairs == 2 ? launch_one<3, 1, false, 2, 1>(a, blocks, threads, smem, st)
                             : launch_one<3, 1, false, 0, 1>(a, blocks, threads, smem, st);
    }
    if (a.geo.g.dim == 2) return kahan ? launch_np<2, true>(a, kind, blocks, threads, smem, st)
                                   : launch_np<2, false>(a, kind, blocks, threads, smem, st);
    return kahan ? launch_np<3, true>(a, kind, blocks, threads, smem, st)
                 : launch_np<3, false>(a, kind, blocks, threads, smem, st);
}

// Double-float pairs -> FP64, scaled: out = ((double)hi + (double)lo) * scale.  One
// thread per value (fully populated warps: the FP64 pipe is narrow on this GPU).
// With surrogate corrections (fixed point, 2^-32 units) added to the virial before scaling.
__global__ void k_pairs_to_f64(const float2* __restrict__ vin, const unsigned long long* __restrict__ corr,
                               double* __restrict__ vout, double svir, const float2* __restrict__ kin,
                               double* __restrict__ kout, double skin, int count)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    if (vout) {
        const float2 v = vin[k];
        double s = (double)v.x + (double)v.y;
        if (corr) s += (double)(long long)corr[k] * 2.3283064365386963e-10;
        vout[k] = s * svir;
    }
    if (kout) {
        const float2 v = kin[k];
        kout[k] = ((double)v.x + (double)v.y) * skin;
    }
}

cudaError_t launch_pairs_to_f64(const float2* vin, const unsigned long long* corr, double* vout, double svir,
                                const float2* kin, double* kout, double skin, long long count, cudaStream_t st)
{
    if (count <= 0 || (!vout && !kout)) return cudaSuccess;
    k_pairs_to_f64<<<(int)((count + 255) / 256), 256, 0, st>>>(vin, corr, vout, svir, kin, kout, skin, (int)count);
    return cudaGetLastError();
}
