// ik_gather32.cu -- the tuned FP32 Irving-Kirkwood gather for sm_103a.
//
// Computes, for every grid point x_g,
//   T(x_g) = sum_{i: |x_g - r_i| < R} sum_{j in bonds(i)} c_ij * int_0^1 Delta(x_g - r_i - s r_ij) ds
//          + sum_{i: |x_g - r_i| < R} m_i v_i (x) v_i Delta(x_g - r_i)
// the loop of IrvingKirkwood::compute (irvingkirkwood/IrvingKirkwood.h:74-110) with
// VirialStress::compute_cg (ListofCommonObservables.h:72-82) and the intended
// KineticStress (ListofCommonObservables.h:131-148), c_ij = 0.5 * forceDivR * r_ij (x) r_ij.
//
// Organisation (one warp = one worker, persistent, dynamic work queue):
//   * a work item is a range of grid-point groups inside one spatial bin of
//     bw^dim cells; the warp stages the bin's halo (particles of the cells within
//     R) into its private shared memory as scaled, bin-relative FP32 positions;
//   * a group is IK_P grid points; lanes test 32 staged particles at a time
//     against the group (FP32, with an FP64 re-check inside a thin band around R
//     so the selection equals the FP64 rule), accumulate the kinetic term, and
//     push (particle, bond, grid mask) slots of accepted particles into a
//     per-warp queue; every full batch of 32 slots is processed with all lanes
//     busy: per slot, the bond integral by symmetric Gauss-Legendre for each grid
//     point of the group, accumulated in FP32 (optionally Kahan-compensated);
//   * the group's partial sums are combined across lanes with a transposing
//     butterfly (each shuffle level halves the values per lane) and written in FP64.
#include "ik_kernels.h"

#define FULL 0xffffffffu

__device__ __forceinline__ float ik_ex2(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float ik_rcp(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Kernel value K(q) in scaled coordinates (normalisation applied on output).
template <int KIND>
__device__ __forceinline__ float ik_kern(float q, float R2s)
{
    if (KIND == 0) {            // octic: q = r^2/R^2, (1 - q^2)^2 inside
        float u = fmaxf(fmaf(-q, q, 1.0f), 0.0f);
        return u * u;
    } else if (KIND == 1) {     // gaussian: q = r^2 * log2(e)/(2 w^2)
        return q < R2s ? ik_ex2(-q) : 0.0f;
    } else if (KIND == 2) {     // rect
        return q < 1.0f ? 1.0f : 0.0f;
    } else {                    // mollifier: exp(-1/(1-q))
        return q < 1.0f ? ik_ex2(-1.4426950408889634f * ik_rcp(1.0f - q)) : 0.0f;
    }
}

template <int DIM>
struct Vec { float v[3]; };

// Transposing butterfly: each lane holds V values (V power of two >= 32 is not
// required); after the call lane l holds the warp total of value indices
// idx(l, k), k < max(V/32, 1), where idx is given by ik_red_index.
template <int V>
__device__ __forceinline__ void ik_warp_transpose_reduce(float (&val)[V], int lane)
{
    int cur = V;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        if (cur > 1) {
            int half = cur >> 1;
            bool up = (lane & o) != 0;
#pragma unroll
            for (int k = 0; k < V / 2; ++k) {
                if (k < half) {
                    float send = up ? val[k] : val[k + half];
                    float keep = up ? val[k + half] : val[k];
                    float recv = __shfl_xor_sync(FULL, send, o);
                    val[k] = keep + recv;
                }
            }
            cur = half;
        } else {
            val[0] += __shfl_xor_sync(FULL, val[0], o);
        }
    }
}
// value index held in slot k of lane `lane` after ik_warp_transpose_reduce<V>
template <int V>
__device__ __forceinline__ int ik_red_index(int lane, int k)
{
    int idx = 0, cur = V;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        if (cur > 1) {
            int half = cur >> 1;
            if (lane & o) idx += half;
            cur = half;
        }
    }
    return idx + k;
}

__host__ __device__ constexpr int ik_pow2_ceil(int x) { int p = 1; while (p < x) p <<= 1; return p; }

template <int DIM, int KIND, bool KAHAN>
__global__ void __launch_bounds__(256, 2) k_gather32(const GatherArgs32 a)
{
    constexpr int NC = DIM == 2 ? 3 : 6;       // unique tensor components
    constexpr int NV = DIM == 2 ? 2 : 3;       // float4 per bond record
    constexpr int P = IK_P;
    constexpr int VR = ik_pow2_ceil(2 * P * NC); // reduction width (virial + kinetic)

    extern __shared__ float4 smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    float4* stage = smem + (size_t)warp * (a.halo_cap + a.qcap / 4);
    int* queue = reinterpret_cast<int*>(stage + a.halo_cap);

    const float R2s = a.R2s, margin = a.margin, kappa = a.kappa;
    const bool want_kin = (a.fields & 2) != 0;
    unsigned long long my_pairs = 0, my_triples = 0;

    for (;;) {
        int w = 0;
        if (lane == 0) w = atomicAdd(a.work_counter, 1);
        w = __shfl_sync(FULL, w, 0);
        if (w >= a.nitems) break;
        const int4 it = a.items[w];
        const int gend = a.items[w + 1].w;

        // halo cell box (unwrapped cell coordinates)
        int h0[3], hn[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            int cc = c == 0 ? it.x : (c == 1 ? it.y : it.z);
            if (c >= DIM || a.g.nc[c] == 1) { h0[c] = 0; hn[c] = 1; }
            else { h0[c] = cc - a.reach[c]; hn[c] = a.bw[c] + 2 * a.reach[c]; }
        }
        const int nh = hn[0] * hn[1] * hn[2];

        int hc = 0;
        bool first = true;
        while (hc < nh) {
            // ---- stage cells [hc, ...) until the warp's halo buffer is full
            int nst = 0;
            for (;;) {
                int cid = hc + lane;
                int cstart = 0, ccnt = 0;
                float ox = 0.f, oy = 0.f, oz = 0.f;
                if (cid < nh) {
                    int ix = cid % hn[0], iy = (cid / hn[0]) % hn[1], iz = cid / (hn[0] * hn[1]);
                    int ux = h0[0] + ix, uy = h0[1] + iy, uz = h0[2] + iz;
                    int wx = ik_wrap(ux, a.g.nc[0]), wy = ik_wrap(uy, a.g.nc[1]);
                    int wz = DIM == 3 ? ik_wrap(uz, a.g.nc[2]) : 0;
                    int cell = (wz * a.g.nc[1] + wy) * a.g.nc[0] + wx;
                    cstart = a.cell_start[cell];
                    ccnt = a.cell_start[cell + 1] - cstart;
                    ox = (ux - it.x) * a.cws[0];
                    oy = (uy - it.y) * a.cws[1];
                    oz = DIM == 3 ? (uz - it.z) * a.cws[2] : 0.f;
                }
                int incl = ccnt;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    int t = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o) incl += t;
                }
                unsigned fit = __ballot_sync(FULL, cid < nh && nst + incl <= a.halo_cap);
                // cells fit as a prefix; count leading ones
                int k = __popc(fit & ~(fit + 1u)) ; // length of the run of ones from bit 0
                if ((fit & 1u) == 0) k = 0;
                if (k == 0) {
                    if (nst == 0 && hc < nh) {
                        // a single cell exceeds the halo buffer: report and skip it
                        if (lane == 0) atomicOr(a.status, IK_ST_HALO_OVERFLOW);
                        ++hc;
                        continue;
                    }
                    break;
                }
                if (lane < k) {
                    int dst = nst + incl - ccnt;
                    for (int t = 0; t < ccnt; ++t) {
                        int q = cstart + t;
                        IkPRec r = a.prec[q];
                        int nbq = a.nb[q];
                        float4 s;
                        s.x = fmaf(kappa, r.x, ox);
                        s.y = fmaf(kappa, r.y, oy);
                        s.z = DIM == 3 ? fmaf(kappa, r.z, oz) : 0.f;
                        s.w = __int_as_float((q << 6) | nbq);
                        stage[dst + t] = s;
                    }
                }
                nst += __shfl_sync(FULL, incl, k - 1);
                hc += k;
                if (k < 32 || hc >= nh) break;
            }
            __syncwarp();

            // ---- process the item's groups against the staged particles
            for (int gs = it.w; gs < gend; gs += P) {
                float gu[P][3];
                int gi[P];
#pragma unroll
                for (int p = 0; p < P; ++p) {
                    if (gs + p < gend) {
                        float4 v = a.gpts[gs + p];
                        gu[p][0] = v.x; gu[p][1] = v.y; gu[p][2] = v.z;
                        gi[p] = __float_as_int(v.w);
                    } else {
                        gu[p][0] = gu[p][1] = gu[p][2] = 1e18f;
                        gi[p] = -1;
                    }
                }
                float acc[P][NC], cmp[P][NC], kac[P][NC];
#pragma unroll
                for (int p = 0; p < P; ++p)
#pragma unroll
                    for (int c = 0; c < NC; ++c) { acc[p][c] = 0.f; cmp[p][c] = 0.f; kac[p][c] = 0.f; }

                // one 32-slot batch of (staged particle, bond, mask)
                auto process_slot = [&](int e) {
                    int s = e >> 10, k = (e >> 4) & 63, m = e & 15;
                    float4 sp = stage[s];
                    int q = __float_as_int(sp.w) >> 6;
                    const float4* rec = a.bonds + ((size_t)q * a.maxb + k) * NV;
                    float4 r0 = __ldg(rec), r1 = __ldg(rec + 1);
                    float4 r2v = NV == 3 ? __ldg(rec + 2) : make_float4(0.f, 0.f, 0.f, 0.f);
                    float hbx, hby, hbz, hh, cf[NC];
                    if (DIM == 2) {
                        hbx = r0.x; hby = r0.y; hbz = 0.f; hh = r0.z;
                        cf[0] = r0.w; cf[1] = r1.x; cf[2] = r1.y;
                    } else {
                        hbx = r0.x; hby = r0.y; hbz = r0.z; hh = r0.w;
                        cf[0] = r1.x; cf[1] = r1.y; cf[2] = r1.z; cf[3] = r1.w;
                        cf[4] = r2v.x; cf[5] = r2v.y;
                    }
                    float mx0 = sp.x + hbx, my0 = sp.y + hby, mz0 = sp.z + hbz; // bond midpoint
#pragma unroll
                    for (int p = 0; p < P; ++p) {
                        float mx = gu[p][0] - mx0, my = gu[p][1] - my0;
                        float M = mx * mx, mb = mx * hbx;
                        M = fmaf(my, my, M);
                        mb = fmaf(my, hby, mb);
                        if (DIM == 3) {
                            float mz = gu[p][2] - mz0;
                            M = fmaf(mz, mz, M);
                            mb = fmaf(mz, hbz, mb);
                        }
                        // r^2(xi) = M - 2 xi mb + xi^2 hh  at the GL nodes
                        float B = a.w0 != 0.f ? a.w0 * ik_kern<KIND>(M, R2s) : 0.f;
#pragma unroll 4
                        for (int t = 0; t < a.npairs; ++t) {
                            float xi = a.xi[t];
                            float base = fmaf(xi * xi, hh, M);
                            float d = 2.f * xi * mb;
                            float kp = ik_kern<KIND>(base - d, R2s);
                            float km = ik_kern<KIND>(base + d, R2s);
                            B = fmaf(a.w[t], kp + km, B);
                        }
                        B = ((m >> p) & 1) ? B : 0.f;
#pragma unroll
                        for (int c = 0; c < NC; ++c) {
                            if (KAHAN) {
                                float y = fmaf(B, cf[c], -cmp[p][c]);
                                float t2 = acc[p][c] + y;
                                cmp[p][c] = (t2 - acc[p][c]) - y;
                                acc[p][c] = t2;
                            } else {
                                acc[p][c] = fmaf(B, cf[c], acc[p][c]);
                            }
                        }
                    }
                    my_triples += __popc(m);
                };

                int qn = 0;
                for (int base = 0; base < nst; base += 32) {
                    int s = base + lane;
                    int mask = 0, cnt = 0;
                    if (s < nst) {
                        float4 sp = stage[s];
                        int wq = __float_as_int(sp.w);
                        int q = wq >> 6;
#pragma unroll
                        for (int p = 0; p < P; ++p) {
                            float dx = gu[p][0] - sp.x, dy = gu[p][1] - sp.y;
                            float r2 = fmaf(dy, dy, dx * dx);
                            if (DIM == 3) { float dz = gu[p][2] - sp.z; r2 = fmaf(dz, dz, r2); }
                            bool in = r2 < R2s;
                            if (fabsf(r2 - R2s) < margin && gi[p] >= 0) {
                                // boundary band: decide with the FP64 rule of the reference
                                int i = a.sorted[q];
                                const double* xg = a.grid + 3 * (size_t)gi[p];
                                double ddx = ik_minimg(__dsub_rn(xg[0], a.pos[3 * i]), a.g.L[0], a.g.periodic[0]);
                                double ddy = ik_minimg(__dsub_rn(xg[1], a.pos[3 * i + 1]), a.g.L[1], a.g.periodic[1]);
                                double ddz = ik_minimg(__dsub_rn(xg[2], a.pos[3 * i + 2]), a.g.L[2], a.g.periodic[2]);
                                in = ik_dot3(ddx, ddy, ddz) < a.R2;
                            }
                            if (in) {
                                mask |= 1 << p;
                                if (want_kin) {
                                    float kv = ik_kern<KIND>(KIND == 1 ? r2 : r2, R2s);
                                    if (DIM == 2) {
                                        float4 kc = __ldg(a.kin + q);
                                        kac[p][0] = fmaf(kv, kc.x, kac[p][0]);
                                        kac[p][1] = fmaf(kv, kc.y, kac[p][1]);
                                        kac[p][2] = fmaf(kv, kc.z, kac[p][2]);
                                    } else {
                                        float4 k0 = __ldg(a.kin + 2 * q), k1 = __ldg(a.kin + 2 * q + 1);
                                        kac[p][0] = fmaf(kv, k0.x, kac[p][0]);
                                        kac[p][1] = fmaf(kv, k0.y, kac[p][1]);
                                        kac[p][2] = fmaf(kv, k0.z, kac[p][2]);
                                        kac[p][NC > 3 ? 3 : 0] = fmaf(kv, k0.w, kac[p][NC > 3 ? 3 : 0]);
                                        kac[p][NC > 4 ? 4 : 0] = fmaf(kv, k1.x, kac[p][NC > 4 ? 4 : 0]);
                                        kac[p][NC > 5 ? 5 : 0] = fmaf(kv, k1.y, kac[p][NC > 5 ? 5 : 0]);
                                    }
                                }
                            }
                        }
                        cnt = mask ? (wq & 63) : 0;
                        my_pairs += __popc(mask);
                    }
                    int incl = cnt;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        int t = __shfl_up_sync(FULL, incl, o);
                        if (lane >= o) incl += t;
                    }
                    int tot = __shfl_sync(FULL, incl, 31);
                    int off = qn + incl - cnt;
                    int entry = (s << 10) | mask;
                    for (int k = 0; k < cnt; ++k) queue[off + k] = entry | (k << 4);
                    qn += tot;
                    __syncwarp();
                    while (qn >= 32) {
                        qn -= 32;
                        process_slot(queue[qn + lane]);
                    }
                    __syncwarp();
                }
                if (lane < qn) process_slot(queue[lane]);
                __syncwarp();

                // ---- combine lanes and write the group's results (FP64)
                float red[VR];
#pragma unroll
                for (int p = 0; p < P; ++p)
#pragma unroll
                    for (int c = 0; c < NC; ++c) {
                        red[p * NC + c] = KAHAN ? acc[p][c] - cmp[p][c] : acc[p][c];
                        red[P * NC + p * NC + c] = kac[p][c];
                    }
#pragma unroll
                for (int k = 2 * P * NC; k < VR; ++k) red[k] = 0.f;
                ik_warp_transpose_reduce<VR>(red, lane);
                constexpr int PER = VR >= 32 ? VR / 32 : 1;
#pragma unroll
                for (int k = 0; k < PER; ++k) {
                    int idx = ik_red_index<VR>(lane, k);
                    bool dup = VR < 32 && (lane & ((32 / VR) - 1)) != 0; // duplicated copies
                    if (idx < 2 * P * NC && !dup) {
                        int kinf = idx >= P * NC;
                        int r = kinf ? idx - P * NC : idx;
                        int p = r / NC, c = r - p * NC;
                        int g = -1;
#pragma unroll
                        for (int pp = 0; pp < P; ++pp) if (pp == p) g = gi[pp];
                        if (g >= 0 && (kinf ? want_kin : (a.fields & 1))) {
                            double* out = kinf ? a.out_kin : a.out_vir;
                            double v = (double)red[k] * (kinf ? a.kin_scale : a.vir_scale);
                            size_t o = (size_t)g * NC + c;
                            out[o] = first ? v : out[o] + v;
                        }
                    }
                }
            }
            first = false;
            __syncwarp();
        }
    }
    // counters
    for (int o = 16; o; o >>= 1) {
        my_pairs += __shfl_xor_sync(FULL, my_pairs, o);
        my_triples += __shfl_xor_sync(FULL, my_triples, o);
    }
    if (lane == 0) {
        atomicAdd(a.cnt_pairs, my_pairs);
        atomicAdd(a.cnt_triples, my_triples);
    }
}

template <int DIM, int KIND, bool KAHAN>
static cudaError_t launch_one(const GatherArgs32& a, int blocks, int threads, size_t smem, cudaStream_t st)
{
    auto kfn = k_gather32<DIM, KIND, KAHAN>;
    cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kfn<<<blocks, threads, smem, st>>>(a);
    return cudaGetLastError();
}

template <int DIM, bool KAHAN>
static cudaError_t launch_kind(const GatherArgs32& a, int kind, int blocks, int threads, size_t smem,
                               cudaStream_t st)
{
    switch (kind) {
    case 0: return launch_one<DIM, 0, KAHAN>(a, blocks, threads, smem, st);
    case 1: return launch_one<DIM, 1, KAHAN>(a, blocks, threads, smem, st);
    case 2: return launch_one<DIM, 2, KAHAN>(a, blocks, threads, smem, st);
    default: return launch_one<DIM, 3, KAHAN>(a, blocks, threads, smem, st);
    }
}

cudaError_t launch_gather32(const GatherArgs32& a, int kind, bool kahan, int blocks, int threads,
                            size_t smem, cudaStream_t st)
{
    if (a.g.dim == 2) return kahan ? launch_kind<2, true>(a, kind, blocks, threads, smem, st)
                                   : launch_kind<2, false>(a, kind, blocks, threads, smem, st);
    return kahan ? launch_kind<3, true>(a, kind, blocks, threads, smem, st)
                 : launch_kind<3, false>(a, kind, blocks, threads, smem, st);
}

int gather32_regs(int dim, int kind, bool kahan)
{
    cudaFuncAttributes fa;
    cudaError_t e;
    if (dim == 2) e = kahan ? cudaFuncGetAttributes(&fa, k_gather32<2, 1, true>)
                            : cudaFuncGetAttributes(&fa, k_gather32<2, 1, false>);
    else e = kahan ? cudaFuncGetAttributes(&fa, k_gather32<3, 1, true>)
                   : cudaFuncGetAttributes(&fa, k_gather32<3, 1, false>);
    (void)kind;
    return e == cudaSuccess ? fa.numRegs : -1;
}
