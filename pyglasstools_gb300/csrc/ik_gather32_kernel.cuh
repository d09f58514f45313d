// ik_gather32_kernel.cuh -- the tuned FP32 Irving-Kirkwood gather for sm_103a (kernel
// template; instantiated by ik_gather32.cu and ik_gather32_aux.cu).
//
// Computes, for every grid point x_g,
//   T(x_g) = sum_{i: |x_g - r_i| < R} sum_{j in bonds(i)} c_ij * int_0^1 Delta(x_g - r_i - s r_ij) ds
//          + sum_{i: |x_g - r_i| < R} m_i v_i (x) v_i Delta(x_g - r_i)
// i.e. the loop of IrvingKirkwood::compute (irvingkirkwood/IrvingKirkwood.h:74-110) with
// VirialStress::compute_cg (ListofCommonObservables.h:72-82) and the intended
// KineticStress (ListofCommonObservables.h:131-148), c_ij = 0.5 * forceDivR * r_ij (x) r_ij.
//
// Organisation (one warp = one worker, persistent, dynamic work queue):
//   * a work item is a range of grid-point groups inside one spatial bin of bw^dim
//     cells; the warp stages the bin's halo (particles of the cells within R) into its
//     private shared memory as scaled, bin-relative FP32 positions;
//   * a group is IK_P grid points (2 in the 3D Kahan variants); lanes test 32 staged particles at a time against
//     the group (FP32, with an FP64 re-check inside a thin band around R so that the
//     selection equals the FP64 rule), accumulate the kinetic term, and push
//     (particle, bond, grid mask) slots of accepted particles into a per-warp queue;
//     every full batch of 32 slots is processed with all lanes busy: per slot, the
//     bond integral by symmetric Gauss-Legendre for each grid point of the group;
//   * accumulation: every lane sums its slots of a group in FP32 (optionally with
//     Kahan compensation, one update per pair of slots in flight: their two products
//     summed first); the 32 lane partials of the virial are combined with
//     error-free transformations (TwoSum) in a transposing butterfly -- each shuffle
//     level halves the values a lane holds -- those of the kinetic term (a few kernel
//     values per lane) with plain adds, and the result is kept as a double-float pair
//     (hi, lo) between the chunks of an item and written as FP64 on its last chunk;
//   * quadrature modes (QM): 0 the fixed-point rule; 1 surrogate mode: a bond whose far
//     end r_j lies outside the support becomes a record {M, m.h, |h|^2, B_fixed} +
//     {grid point, bond} for the learned surrogate (ik_mlp.cu) instead of a term of the
//     sum; 2 the same bonds by the closed form of the truncated Gaussian (the segment
//     clipped to the support, error functions along it), the rule elsewhere; 3 the
//     closed form for every bond.
// Bond records (CSR, 16 B): {hb = kappa r_ij / 2, f' = 2 forceDivR / kappa^2}; the
// stress coefficient is f' hb (x) hb.
#pragma once
#include "ik_kernels.h"

#define FULL 0xffffffffu
#define IK_BATCH_ROUND 16 // fused batch: consecutive work items a CTA takes per round

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
    if (KIND == 0) {            // octic: q = r^2/R^2, (1 - q^2)^2 inside (1 - q^2 <= 1: the
                                // saturation only clips at 0)
        float u = __saturatef(fmaf(-q, q, 1.0f));
        return u * u;
    } else if (KIND == 1) {     // gaussian: q = r^2 * log2(e)/(2 w^2), cut at q = R2s.  The
                                // cut as a saturated FMA: (R2s - q) * 2^100 is >= 1 for every
                                // float q < R2s (they differ by >= 1 ulp of R2s) and <= 0 else
        const float inside = __saturatef(fmaf(-q, 0x1p100f, R2s * 0x1p100f));
        return ik_ex2(-q) * inside;
    } else if (KIND == 2) {     // rect
        return q < 1.0f ? 1.0f : 0.0f;
    } else {                    // mollifier: exp(-1/(1-q))
        return q < 1.0f ? ik_ex2(-1.4426950408889634f * ik_rcp(1.0f - q)) : 0.0f;
    }
}
// Two kernel values, packed.  Gaussian: the two cuts (saturated FMAs) and exponentials
// are scalar, their product one packed multiply.
template <int KIND>
__device__ __forceinline__ unsigned long long ik_kern2(unsigned long long q2, float R2s);

// erfc(x) for x >= 0 by Hastings' rational approximation (Abramowitz & Stegun,
// Handbook of Mathematical Functions, 7.1.26): erfc(x) = t (a1 + t (a2 + t (a3 +
// t (a4 + t a5)))) exp(-x^2), t = 1 / (1 + p x), with |error| <= 1.5e-7.
__device__ __forceinline__ float ik_erfc_hastings(float x)
{
    const float t = ik_rcp(fmaf(0.3275911f, x, 1.0f));
    float q = fmaf(1.061405429f, t, -1.453152027f);
    q = fmaf(q, t, 1.421413741f);
    q = fmaf(q, t, -0.284496736f);
    q = fmaf(q, t, 0.254829592f);
    return q * t * ik_ex2(-1.4426950408889634f * x * x);
}
// erf(zb) - erf(za) from erfc of |za| and |zb|: with s = sign,
// (s_b - s_a) + s_a erfc|za| - s_b erfc|zb| -- the difference of the two small tails
// when both lie on one side (no cancellation), branch-free.
__device__ __forceinline__ float ik_erf_diff(float za, float zb)
{
    const float sa = za < 0.f ? -1.f : 1.f, sb = zb < 0.f ? -1.f : 1.f;
    return fmaf(sa, ik_erfc_hastings(fabsf(za)), fmaf(-sb, ik_erfc_hastings(fabsf(zb)), sb - sa));
}

// The bond integral of the truncated Gaussian in closed form, in the gather's scaled
// units (kernel 2^-q, q = |scaled r|^2, support q < R2s):
//   int_{-1}^{1} 2^{-r^2(xi)} [r^2(xi) < R2s] dxi,  r^2(xi) = hh (xi - xi0)^2 + d2,
// with xi0 = mb / hh the foot of the grid point on the bond's line and d2 its squared
// distance from the line (from a cross product: no cancellation near the line).  The
// segment is clipped to the support, |xi - xi0| < sqrt((R2s - d2) / hh), and
//   = 2^{-d2} sqrt(pi) / (2 sqrt(a)) (erf(sqrt(a) (hi - xi0)) - erf(sqrt(a) (lo - xi0))),
// a = ln 2 hh, with the error functions of ik_erf_diff.
__device__ __forceinline__ float ik_bond_gauss_exact(float d2, float mb, float hh, float R2s)
{
    const float ihh = ik_rcp(hh);
    const float t2 = (R2s - d2) * ihh;
    if (!(t2 > 0.f)) return 0.f;
    const float xi0 = mb * ihh, tc = sqrtf(t2);
    const float sa = sqrtf(0.69314718055994531f * hh);
    // z = sqrt(a) (end - xi0) at the clipped ends, from tc directly where the clip holds
    const float za = xi0 - tc > -1.f ? -sa * tc : sa * (-1.f - xi0);
    const float zb = xi0 + tc < 1.f ? sa * tc : sa * (1.f - xi0);
    if (!(zb > za)) return 0.f;
    return ik_ex2(-d2) * (0.88622692545275801f * ik_rcp(sa)) * ik_erf_diff(za, zb);
}

// Kernel value of a particle already selected by the (FP64) support rule.
template <int KIND>
__device__ __forceinline__ float ik_kern_in(float q)
{
    if (KIND == 1) return ik_ex2(-q);
    if (KIND == 0) { float u = fmaxf(fmaf(-q, q, 1.0f), 0.0f); return u * u; }
    if (KIND == 2) return 1.0f;
    return q < 1.0f ? ik_ex2(-1.4426950408889634f * ik_rcp(1.0f - q)) : 0.0f;
}

// TwoSum (Knuth): s + e == a + b exactly.
__device__ __forceinline__ void ik_two_sum(float a, float b, float& s, float& e)
{
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__host__ __device__ constexpr int ik_pow2_ceil(int x) { int p = 1; while (p < x) p <<= 1; return p; }

// Packed FP32 pairs (sm_100+ f32x2 arithmetic): two grid points evaluated per instruction.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float a, float b)
{
    f32x2 r;
    asm("mov.b64 %0, {%1,%2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void up2(f32x2 r, float& a, float& b)
{
    asm("mov.b64 {%0,%1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b)
{
    f32x2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b)
{
    f32x2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b)
{
    f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c)
{
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

template <int KIND>
__device__ __forceinline__ f32x2 ik_kern2(f32x2 q2, float R2s)
{
    float qa, qb;
    up2(q2, qa, qb);
    if (KIND == 1) {
        const float ia = __saturatef(fmaf(-qa, 0x1p100f, R2s * 0x1p100f));
        const float ib = __saturatef(fmaf(-qb, 0x1p100f, R2s * 0x1p100f));
        return mul2(pk2(ik_ex2(-qa), ik_ex2(-qb)), pk2(ia, ib));
    }
    return pk2(ik_kern<KIND>(qa, R2s), ik_kern<KIND>(qb, R2s));
}

// Compensated transposing butterfly over a warp: on entry each lane holds V values
// (hi[k], lo[k] = 0); after the call lane l holds, for k < max(V/32, 1), the warp sum
// of value ik_red_index<V>(l, k) as hi[k] + lo[k] (hi + lo exact to ~2 ulp of the
// sum, i.e. the accumulation of the 32 partials is compensated).
template <int V>
__device__ __forceinline__ void ik_warp_reduce_cmp(float (&hi)[V], float (&lo)[V], int lane)
{
#pragma unroll
    for (int lev = 0; lev < 5; ++lev) {
        const int o = 16 >> lev;
        const int cur = (V >> lev) > 1 ? (V >> lev) : 1;
        if (cur > 1) {
            const int half = cur >> 1;
            const bool up = (lane & o) != 0;
#pragma unroll
            for (int k = 0; k < V / 2; ++k) {
                if (k < half) {
                    float sh = up ? hi[k] : hi[k + half];
                    float sl = up ? lo[k] : lo[k + half];
                    float kh = up ? hi[k + half] : hi[k];
                    float kl = up ? lo[k + half] : lo[k];
                    float rh = __shfl_xor_sync(FULL, sh, o);
                    float rl = __shfl_xor_sync(FULL, sl, o);
                    float s, e;
                    ik_two_sum(kh, rh, s, e);
                    hi[k] = s;
                    lo[k] = e + (kl + rl);
                }
            }
        } else {
            float rh = __shfl_xor_sync(FULL, hi[0], o);
            float rl = __shfl_xor_sync(FULL, lo[0], o);
            float s, e;
            ik_two_sum(hi[0], rh, s, e);
            hi[0] = s;
            lo[0] = e + (lo[0] + rl);
        }
    }
}
// The same transposing butterfly with plain FP32 adds (index mapping as above).  The
// per-lane partial sums already carry the rounding of their own accumulation, which a
// compensated combination of 32 partials does not remove; the plain tree adds the
// rounding of 5 adds per value to the ~(terms per lane) adds each lane made.
template <int V>
__device__ __forceinline__ void ik_warp_reduce_plain(float (&hi)[V], int lane)
{
#pragma unroll
    for (int lev = 0; lev < 5; ++lev) {
        const int o = 16 >> lev;
        const int cur = (V >> lev) > 1 ? (V >> lev) : 1;
        if (cur > 1) {
            const int half = cur >> 1;
            const bool up = (lane & o) != 0;
#pragma unroll
            for (int k = 0; k < V / 2; ++k) {
                if (k < half) {
                    const float sh = up ? hi[k] : hi[k + half];
                    const float kh = up ? hi[k + half] : hi[k];
                    hi[k] = kh + __shfl_xor_sync(FULL, sh, o);
                }
            }
        } else {
            hi[0] += __shfl_xor_sync(FULL, hi[0], o);
        }
    }
}

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

// NP: number of symmetric Gauss-Legendre node pairs (compile-time when > 0; 0 = runtime).
// QM: quadrature mode -- 0 fixed-point rule; 1 surrogate (bonds crossing the edge of the
// support become records); 2 closed form on those bonds; 3 closed form on every bond
// (2 and 3: the Gaussian kernel only).
// SPLIT: particles with more than 63 bonds are staged as several entries (one per 63
// bonds; the entry word holds 6 count bits); the other variants need maxb <= 63.
// BATCH: a fused batch -- work items of every slot in one launch; each item's slot
// (a.item_slot) gives the geometry (copied to the warp's shared memory when the slot
// changes) and the counters; particle, bond, grid and output indices are the batch's.
template <int DIM, int KIND, bool KAHAN, int NP, int QM, bool ELA, bool SPLIT, bool BATCH>
__global__ void __launch_bounds__(256, 2) k_gather32(const GatherArgs32 a)
{
    constexpr int NC = DIM == 2 ? 3 : 6;       // unique tensor components
    // grid points per group: IK_P, but 2 for the 3D Kahan variants, whose per-lane sums and
    // compensations of 4 points x 6 components spill (the fused 3D Kahan gather ran 516 ->
    // 445 us per frame with 2; the plain 3D variants stay at IK_P, where 2 is slower)
    constexpr int P = (DIM == 3 && KAHAN) ? 2 : IK_P;
    constexpr bool MLPM = QM == 1;
    static_assert(QM < 2 || KIND == 1, "closed-form bond integrals: Gaussian kernel only");
    static_assert(!BATCH || (QM == 0 && !ELA && !SPLIT), "fused batches: fixed-point rule, virial and kinetic");

    // CSR bond records are addressed by (offset << 6 | count) words: 2^25 records at most
    if (a.boff && a.boff[a.nprec] >= (1 << 25)) {
        if (threadIdx.x == 0 && blockIdx.x == 0) atomicOr(a.status, IK_ST_BOND_RANGE);
        return;
    }
    extern __shared__ float4 smem[];
    __shared__ int s_next; // next item of this CTA's share
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_next = 0;
    // the geometry of the current item: the frame's (kernel parameter) or, in a fused
    // batch, the item's slot's (a copy in this warp's shared memory)
    __shared__ GatherGeo s_geo[BATCH ? IK_WARPS_GATHER : 1];
    const GatherGeo& G = BATCH ? s_geo[warp] : a.geo;
    int cur_slot = -1;
    const float4* bonds_w = a.bonds; // the item's slot's bond records (fused batch: offset)
    __syncthreads();
    // per warp: staged particles (float4 x,y,z, bits(bond offset << 6 | bond count)),
    // their cell-order indices (3D; 2D keeps them in the unused z word), and the slot
    // queue.  halo_cap is a multiple of 32.
    constexpr int SQW = DIM == 3 ? 1 : 0;
    float4* stage = smem + (size_t)warp * (a.halo_cap + SQW * a.halo_cap / 4 + a.qcap / 4);
    int* sq = reinterpret_cast<int*>(stage + a.halo_cap);
    int* queue = sq + SQW * a.halo_cap;

    const float R2s = a.R2s, margin = a.margin, kappa = a.kappa;
    const float cull_r2 = 1.001f * R2s + margin; // staging: within R of the bin's box, FP32 slack
    // culling the staged halo pays in 3D (a one-cell bin keeps ~3/4 of its 27-cell halo);
    // 2D bins of several cells keep ~7/8, less than the second pass over them costs
    bool cull = DIM == 3 && G.cull;
    const bool want_kin = (a.fields & 2) != 0;
    const int npairs = NP > 0 ? NP : a.npairs;
    unsigned my_pairs = 0, my_triples = 0; // per lane, flushed to the 64-bit counters
    // surrogate records: this warp's current chunk [wfill, wend) of the record buffer
    long long wfill = 0, wend = 0;
    unsigned long long my_records = 0;
    auto emit = [&](int cmask, const float4 (&crec)[P], const int (&gidx)[P], int bidx) {
        const int cnt = __popc(cmask);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += t;
        }
        const int tot = __shfl_sync(FULL, incl, 31);
        if (tot == 0) return;
        if (wfill + tot > wend) {
            for (long long k = wfill + lane; k < wend; k += 32) a.mlp_rid[k] = make_int2(-1, 0);
            unsigned long long nb = 0;
            if (lane == 0) nb = atomicAdd(a.mlp_count, (unsigned long long)IK_MLP_CHUNK);
            nb = __shfl_sync(FULL, nb, 0);
            if ((long long)nb + IK_MLP_CHUNK > a.mlp_cap) { // overflow: reported, replayed larger
                if (lane == 0) atomicOr(a.status, IK_ST_MLP_OVERFLOW);
                wfill = wend = 0;
                return;
            }
            wfill = (long long)nb;
            wend = wfill + IK_MLP_CHUNK;
        }
        long long o = wfill + incl - cnt;
#pragma unroll
        for (int p = 0; p < P; ++p)
            if (cmask & (1 << p)) {
                a.mlp_rec[o] = crec[p];
                a.mlp_rid[o] = make_int2(gidx[p], bidx);
                ++o;
            }
        wfill += tot;
        my_records += (unsigned long long)cnt;
    };

    // pair and triple counts to the frame's counters (fused batch: the current slot's)
    auto flush_counters = [&]() {
        if (!BATCH || cur_slot >= 0) {
            unsigned long long p2 = my_pairs, t2 = my_triples;
            for (int o = 16; o; o >>= 1) {
                p2 += __shfl_xor_sync(FULL, p2, o);
                t2 += __shfl_xor_sync(FULL, t2, o);
            }
            if (lane == 0 && (p2 | t2)) {
                atomicAdd(BATCH ? G.cnt + 1 : a.cnt_pairs, p2);
                atomicAdd(BATCH ? G.cnt + 2 : a.cnt_triples, t2);
            }
        }
        my_pairs = my_triples = 0;
    };

    for (;;) {
        // work items: first this CTA's contiguous share (spatial neighbours, L1 reuse
        // across its warps), then a global counter over the remaining tail
        // (fused batch: rounds of IK_BATCH_ROUND consecutive items per CTA, CTA after CTA,
        // so that the whole GPU works through the frames in order -- a frame's particles
        // and bonds are fetched into L2 once -- while a CTA's warps share their items'
        // halos in L1; the last eighth from the global counter)
        int w = 0;
        if (lane == 0) {
            if (BATCH) {
                const long long span = (long long)gridDim.x * IK_BATCH_ROUND;
                const long long nstatic = ((long long)a.nitems * 7 / 8) / span * span;
                const int k = atomicAdd(&s_next, 1);
                const long long ws = (long long)(k / IK_BATCH_ROUND) * span +
                                     (long long)blockIdx.x * IK_BATCH_ROUND + k % IK_BATCH_ROUND;
                w = ws < nstatic ? (int)ws : (int)nstatic + atomicAdd(a.work_counter, 1);
            } else {
                const int per = (int)(((long long)a.nitems * 7 / 8) / gridDim.x);
                const int k = atomicAdd(&s_next, 1);
                w = k < per ? (int)blockIdx.x * per + k : per * (int)gridDim.x + atomicAdd(a.work_counter, 1);
            }
        }
        w = __shfl_sync(FULL, w, 0);
        if (w >= a.nitems) break;
        if constexpr (BATCH) { // the item's slot: its geometry into this warp's copy
            const int sl = __ldg(a.item_slot + w);
            if (sl != cur_slot) {
                flush_counters();
                const int* src = reinterpret_cast<const int*>(&a.slots[sl].geo);
                int* dst = reinterpret_cast<int*>(&s_geo[warp]);
                for (int k = lane; k < (int)(sizeof(GatherGeo) / 4); k += 32) dst[k] = __ldg(src + k);
                __syncwarp();
                cur_slot = sl;
                cull = DIM == 3 && G.cull;
                bonds_w = a.bonds + (size_t)G.p_off * a.maxb;
            }
        }
        const int4 it = a.items[w];
        const int gend = a.items[w + 1].w;

        // halo cell box (unwrapped cell coordinates)
        int h0[3], hn[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            int cc = c == 0 ? it.x : (c == 1 ? it.y : it.z);
            if (c >= DIM || G.g.nc[c] == 1) { h0[c] = 0; hn[c] = 1; }
            else { h0[c] = cc - G.reach[c]; hn[c] = G.bw[c] + 2 * G.reach[c]; }
        }
        const int nh = hn[0] * hn[1] * hn[2];
        // the bin's box in scaled bin-relative coordinates, [0, bw cws) per axis (cells past
        // the box edge only shrink it: conservative)
        const float bxs = G.bw[0] * G.cws[0], bys = G.bw[1] * G.cws[1], bzs = DIM == 3 ? G.bw[2] * G.cws[2] : 0.f;
        auto near_bin = [&](const IkPRec& r, float ox, float oy, float oz) {
            const float sx = fmaf(kappa, r.x, ox), sy = fmaf(kappa, r.y, oy);
            const float dx = fmaxf(fmaxf(-sx, sx - bxs), 0.f), dy = fmaxf(fmaxf(-sy, sy - bys), 0.f);
            float d2 = fmaf(dy, dy, dx * dx);
            if (DIM == 3) {
                const float sz = fmaf(kappa, r.z, oz);
                const float dz = fmaxf(fmaxf(-sz, sz - bzs), 0.f);
                d2 = fmaf(dz, dz, d2);
            }
            return d2 < cull_r2;
        };

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
                    int wx = ik_wrap(ux, G.g.nc[0]), wy = ik_wrap(uy, G.g.nc[1]);
                    int wz = DIM == 3 ? ik_wrap(uz, G.g.nc[2]) : 0;
                    int cell = (wz * G.g.nc[1] + wy) * G.g.nc[0] + wx + G.c_off;
                    cstart = a.cell_start[cell];
                    ccnt = a.cell_start[cell + 1] - cstart;
                    ox = (ux - it.x) * G.cws[0];
                    oy = (uy - it.y) * G.cws[1];
                    oz = DIM == 3 ? (uz - it.z) * G.cws[2] : 0.f;
                }
                // staged entries of the cell: one per particle (with cull: only those
                // within R of the bin's box -- the others cannot reach any of its grid
                // points), and one more per further 63 bonds where a particle has more
                // (the entry word holds 6 count bits)
                int cent = ccnt;
                if ((SPLIT || cull) && cid < nh) {
                    cent = 0;
                    for (int t = 0; t < ccnt; ++t) {
                        const int q = cstart + t;
                        if (cull && !near_bin(a.prec[q], ox, oy, oz)) continue;
                        if (SPLIT) {
                            const int nbq = a.boff ? a.boff[q + 1] - a.boff[q] : a.nb[q];
                            cent += nbq > 63 ? (nbq + 62) / 63 : 1;
                        } else {
                            ++cent;
                        }
                    }
                }
                int incl = cent;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    int t = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o) incl += t;
                }
                unsigned fit = __ballot_sync(FULL, cid < nh && nst + incl <= a.halo_cap);
                int k = __popc(fit & ~(fit + 1u)); // length of the run of ones from bit 0
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
                    int dst = nst + incl - cent;
                    for (int t = 0; t < ccnt; ++t) {
                        int q = cstart + t;
                        IkPRec r = a.prec[q];
                        if (cull && !near_bin(r, ox, oy, oz)) continue;
                        int b0, nbq;
                        if (a.boff) { b0 = a.boff[q]; nbq = a.boff[q + 1] - b0; }
                        else { b0 = (q - G.p_off) * a.maxb; nbq = a.nb[q]; }
                        float4 s;
                        s.x = fmaf(kappa, r.x, ox);
                        s.y = fmaf(kappa, r.y, oy);
                        s.z = DIM == 3 ? fmaf(kappa, r.z, oz) : 0.f;
                        if (!SPLIT || nbq <= 63) {
                            s.w = __int_as_float((b0 << 6) | nbq);
                            if (DIM == 2) s.z = __int_as_float(q);
                            stage[dst] = s;
                            if (DIM == 3) sq[dst] = q;
                            ++dst;
                        } else { // continuation entries carry IK_SQ_CONT
                            for (int j = 0; j < nbq; j += 63) {
                                s.w = __int_as_float(((b0 + j) << 6) | min(nbq - j, 63));
                                if (DIM == 2) s.z = __int_as_float(j ? (q | IK_SQ_CONT) : q);
                                stage[dst] = s;
                                if (DIM == 3) sq[dst] = j ? (q | IK_SQ_CONT) : q;
                                ++dst;
                            }
                        }
                    }
                }
                nst += __shfl_sync(FULL, incl, k - 1);
                hc += k;
                if (k < 32 || hc >= nh) break;
            }
            __syncwarp();
            const bool last = hc >= nh; // this chunk holds the item's last halo cells

            // ---- process the item's groups against the staged particles
            for (int gs = it.w; gs < gend; gs += P) {
                // the group's grid points, packed in pairs (0,1), (2,3) for f32x2 arithmetic
                f32x2 g2[P / 2][3];
                int gi[P];
#pragma unroll
                for (int j = 0; j < P / 2; ++j) {
                    float4 v0 = make_float4(1e18f, 1e18f, 1e18f, __int_as_float(-1)), v1 = v0;
                    if (gs + 2 * j < gend) v0 = a.gpts[gs + 2 * j];
                    if (gs + 2 * j + 1 < gend) v1 = a.gpts[gs + 2 * j + 1];
                    g2[j][0] = pk2(v0.x, v1.x);
                    g2[j][1] = pk2(v0.y, v1.y);
                    g2[j][2] = pk2(v0.z, v1.z);
                    gi[2 * j] = __float_as_int(v0.w);
                    gi[2 * j + 1] = __float_as_int(v1.w);
                }
                float acc[P][NC], cmp[P][NC], kac[P][NC];
#pragma unroll
                for (int p = 0; p < P; ++p)
#pragma unroll
                    for (int c = 0; c < NC; ++c) { acc[p][c] = 0.f; cmp[p][c] = 0.f; kac[p][c] = 0.f; }

                // packed sums of the grid-point pairs; in the Kahan variant also their running
                // compensations, kept negated (cn = -c: y = B cf + cn, t = acc + y,
                // cn = y - (t - acc), acc = t -- Kahan's summation, two points per instruction)
                f32x2 acc2[P / 2][NC], cn2[P / 2][KAHAN ? NC : 1];
#pragma unroll
                for (int j = 0; j < P / 2; ++j) {
#pragma unroll
                    for (int c = 0; c < NC; ++c) acc2[j][c] = 0ull;
#pragma unroll
                    for (int c = 0; c < (KAHAN ? NC : 1); ++c) cn2[j][c] = 0ull;
                }

                // one slot: staged particle s, its bond k, grid mask m.  The loads are
                // separate so that two batches can be in flight before either computes.
                auto load_slot = [&](int e, float4& sp, float4& b) {
                    sp = stage[e >> 10];
                    b = __ldg(bonds_w + (__float_as_int(sp.w) >> 6) + ((e >> 4) & 63));
                };
                // Kahan lane sums: the two slots in flight are added to the compensated sums
                // as one term (their products summed first: one Kahan update per pair)
                constexpr bool PAIRK = KAHAN && NP > 0 && QM == 0 && !ELA;
                f32x2 pB[PAIRK ? P / 2 : 1], pcf[PAIRK ? NC : 1];
                // mode 0: accumulate; 1: keep B and the coefficients for the next call;
                // 2: accumulate together with the kept ones
                auto process_slot = [&](int e, const float4& sp, const float4& b, int mode = 0) {
                    const int m = e & 15;
                    const float hbx = b.x, hby = b.y, hbz = b.z;
                    const float hh = DIM == 3 ? fmaf(hbz, hbz, fmaf(hby, hby, hbx * hbx)) : fmaf(hby, hby, hbx * hbx);
                    float cf[NC];
                    if constexpr (ELA) { // elastic field: the bond's own coefficient
                        const int bi = (__float_as_int(sp.w) >> 6) + ((e >> 4) & 63);
                        const float4 c0 = __ldg(a.bcoef + (size_t)bi * (DIM == 2 ? 1 : 2));
                        cf[0] = c0.x;
                        cf[1] = c0.y;
                        cf[2] = c0.z;
                        if (DIM == 3) {
                            const float4 c1 = __ldg(a.bcoef + (size_t)bi * 2 + 1);
                            cf[3 % NC] = c0.w;
                            cf[4 % NC] = c1.x;
                            cf[5 % NC] = c1.y;
                        }
                    } else {
                        const float fx = b.w * hbx, fy = b.w * hby;
                        cf[0] = fx * hbx;
                        cf[1] = fy * hby;
                        if (DIM == 2) {
                            cf[2] = fx * hby;
                        } else {
                            const float fz = b.w * hbz;
                            cf[2] = fz * hbz;
                            cf[3 % NC] = fx * hby;
                            cf[4 % NC] = fx * hbz;
                            cf[5 % NC] = fy * hbz;
                        }
                    }
                    const float mx0 = sp.x + hbx, my0 = sp.y + hby, mz0 = sp.z + hbz; // bond midpoint
                    float4 crec[P];
                    int cmask = 0;
                    if constexpr (NP > 0 && QM != 3) {
                        // packed path: two grid points per f32x2 instruction
                        const f32x2 mid2x = pk2(mx0, mx0), mid2y = pk2(my0, my0), mid2z = pk2(mz0, mz0);
                        const f32x2 hb2x = pk2(hbx, hbx), hb2y = pk2(hby, hby), hb2z = pk2(hbz, hbz);
                        f32x2 cq2[NP], cf2[NC];
#pragma unroll
                        for (int t = 0; t < NP; ++t) { const float v = a.xi2[t] * hh; cq2[t] = pk2(v, v); }
#pragma unroll
                        for (int c = 0; c < NC; ++c) cf2[c] = pk2(cf[c], cf[c]);
                        if (PAIRK && mode == 1) {
#pragma unroll
                            for (int c = 0; c < NC; ++c) pcf[c % (PAIRK ? NC : 1)] = cf2[c];
                        }
#pragma unroll
                        for (int j = 0; j < P / 2; ++j) {
                            const f32x2 mx = sub2(g2[j][0], mid2x), my = sub2(g2[j][1], mid2y);
                            f32x2 M = fma2(my, my, mul2(mx, mx));
                            f32x2 mb = fma2(my, hb2y, mul2(mx, hb2x));
                            if (DIM == 3) {
                                const f32x2 mz = sub2(g2[j][2], mid2z);
                                M = fma2(mz, mz, M);
                                mb = fma2(mz, hb2z, mb);
                            }
                            float Ma, Mb;
                            up2(M, Ma, Mb);
                            // node sums of the two grid points packed (the same roundings as
                            // per point: w0 K(M) + sum_t w_t (K(r+) + K(r-)))
                            f32x2 B2 = mul2(pk2(a.w0, a.w0), ik_kern2<KIND>(M, R2s));
#pragma unroll
                            for (int t = 0; t < NP; ++t) {
                                const f32x2 base = add2(M, cq2[t]);
                                const f32x2 rp = fma2(pk2(a.m2xi[t], a.m2xi[t]), mb, base);
                                const f32x2 rm = fma2(pk2(-a.m2xi[t], -a.m2xi[t]), mb, base);
                                B2 = fma2(pk2(a.w[t], a.w[t]), add2(ik_kern2<KIND>(rp, R2s), ik_kern2<KIND>(rm, R2s)), B2);
                            }
                            float Ba, Bb;
                            up2(B2, Ba, Bb);
                            f32x2 B;
                            if constexpr (MLPM) { // r_j outside the support: a record, not a term
                                const f32x2 rj2 = fma2(pk2(-2.f, -2.f), mb, add2(M, pk2(hh, hh)));
                                float ra, rb, mba, mbb;
                                up2(rj2, ra, rb);
                                up2(mb, mba, mbb);
                                if ((m & (1 << (2 * j))) && ra >= R2s) {
                                    crec[2 * j] = make_float4(Ma, mba, hh, Ba);
                                    cmask |= 1 << (2 * j);
                                    Ba = 0.f;
                                }
                                if ((m & (2 << (2 * j))) && rb >= R2s) {
                                    crec[2 * j + 1] = make_float4(Mb, mbb, hh, Bb);
                                    cmask |= 2 << (2 * j);
                                    Bb = 0.f;
                                }
                            }
                            if constexpr (QM == 2) { // r_j outside the support: the closed form
                                const f32x2 rj2 = fma2(pk2(-2.f, -2.f), mb, add2(M, pk2(hh, hh)));
                                float ra, rb;
                                up2(rj2, ra, rb);
                                const bool ca = (m & (1 << (2 * j))) && ra >= R2s, cb = (m & (2 << (2 * j))) && rb >= R2s;
                                if (ca || cb) {
                                    // squared distance from the bond's line: |m x h|^2 / hh
                                    f32x2 cr = fma2(mx, hb2y, mul2(pk2(-1.f, -1.f), mul2(my, hb2x)));
                                    f32x2 c2 = mul2(cr, cr);
                                    if (DIM == 3) {
                                        const f32x2 mz = sub2(g2[j][2], mid2z);
                                        const f32x2 cy = fma2(mz, hb2x, mul2(pk2(-1.f, -1.f), mul2(mx, hb2z)));
                                        const f32x2 cx = fma2(my, hb2z, mul2(pk2(-1.f, -1.f), mul2(mz, hb2y)));
                                        c2 = fma2(cy, cy, fma2(cx, cx, c2));
                                    }
                                    float c2a, c2b, mba, mbb;
                                    up2(c2, c2a, c2b);
                                    up2(mb, mba, mbb);
                                    const float ihh = ik_rcp(hh);
                                    if (ca) Ba = ik_bond_gauss_exact(c2a * ihh, mba, hh, R2s);
                                    if (cb) Bb = ik_bond_gauss_exact(c2b * ihh, mbb, hh, R2s);
                                }
                            }
                            B = pk2((m & (1 << (2 * j))) ? Ba : 0.f, (m & (2 << (2 * j))) ? Bb : 0.f);
                            if (PAIRK && mode == 1) { pB[j % (PAIRK ? P / 2 : 1)] = B; continue; }
#pragma unroll
                            for (int c = 0; c < NC; ++c) {
                                if constexpr (KAHAN) {
                                    const f32x2 y = (PAIRK && mode == 2)
                                                        ? fma2(B, cf2[c], fma2(pB[j % (PAIRK ? P / 2 : 1)], pcf[c % (PAIRK ? NC : 1)], cn2[j][c]))
                                                        : fma2(B, cf2[c], cn2[j][c]);
                                    const f32x2 t2 = add2(acc2[j][c], y);
                                    cn2[j][c] = sub2(y, sub2(t2, acc2[j][c]));
                                    acc2[j][c] = t2;
                                } else {
                                    acc2[j][c] = fma2(B, cf2[c], acc2[j][c]);
                                }
                            }
                        }
                    } else {
                        float cq[NP > 0 ? NP : 1];
                        if constexpr (NP > 0) {
#pragma unroll
                            for (int t = 0; t < NP; ++t) cq[t] = a.xi2[t] * hh;
                        }
#pragma unroll
                        for (int p = 0; p < P; ++p) {
                            float gx, gy, gz, t0, t1, t2;
                            up2(g2[p >> 1][0], t0, t1);
                            gx = (p & 1) ? t1 : t0;
                            up2(g2[p >> 1][1], t0, t1);
                            gy = (p & 1) ? t1 : t0;
                            up2(g2[p >> 1][2], t0, t2);
                            gz = (p & 1) ? t2 : t0;
                            const float mx = gx - mx0, my = gy - my0;
                            float M = mx * mx, mb = mx * hbx;
                            M = fmaf(my, my, M);
                            mb = fmaf(my, hby, mb);
                            if (DIM == 3) {
                                const float mz = gz - mz0;
                                M = fmaf(mz, mz, M);
                                mb = fmaf(mz, hbz, mb);
                            }
                            // r^2(xi) = M - 2 xi mb + xi^2 hh at the symmetric nodes +-xi
                            float B = QM == 3 ? 0.f : a.w0 * ik_kern<KIND>(M, R2s);
                            if constexpr (QM == 3) {
                                // the closed form; d2 = |m x h|^2 / hh
                                float c2;
                                if (DIM == 2) {
                                    const float cr = fmaf(mx, hby, -my * hbx);
                                    c2 = cr * cr;
                                } else {
                                    const float mz = gz - mz0;
                                    const float cx = fmaf(my, hbz, -mz * hby), cy = fmaf(mz, hbx, -mx * hbz),
                                                cz = fmaf(mx, hby, -my * hbx);
                                    c2 = fmaf(cz, cz, fmaf(cy, cy, cx * cx));
                                }
                                B = ik_bond_gauss_exact(c2 * ik_rcp(hh), mb, hh, R2s);
                            } else if constexpr (NP > 0) {
#pragma unroll
                                for (int t = 0; t < NP; ++t) {
                                    const float base = M + cq[t];
                                    const float kp = ik_kern<KIND>(fmaf(a.m2xi[t], mb, base), R2s);
                                    const float km = ik_kern<KIND>(fmaf(-a.m2xi[t], mb, base), R2s);
                                    B = fmaf(a.w[t], kp + km, B);
                                }
                            } else {
#pragma unroll 1
                                for (int t = 0; t < npairs; ++t) {
                                    const float base = fmaf(a.xi2[t], hh, M);
                                    const float kp = ik_kern<KIND>(fmaf(a.m2xi[t], mb, base), R2s);
                                    const float km = ik_kern<KIND>(fmaf(-a.m2xi[t], mb, base), R2s);
                                    B = fmaf(a.w[t], kp + km, B);
                                }
                            }
                            if constexpr (QM == 2) {
                                if ((m & (1 << p)) && fmaf(-2.f, mb, M + hh) >= R2s) {
                                    float c2;
                                    if (DIM == 2) {
                                        const float cr = fmaf(mx, hby, -my * hbx);
                                        c2 = cr * cr;
                                    } else {
                                        const float mz = gz - mz0;
                                        const float cx = fmaf(my, hbz, -mz * hby), cy = fmaf(mz, hbx, -mx * hbz),
                                                    cz = fmaf(mx, hby, -my * hbx);
                                        c2 = fmaf(cz, cz, fmaf(cy, cy, cx * cx));
                                    }
                                    B = ik_bond_gauss_exact(c2 * ik_rcp(hh), mb, hh, R2s);
                                }
                            }
                            B = (m & (1 << p)) ? B : 0.f;
                            if constexpr (MLPM) {
                                if ((m & (1 << p)) && fmaf(-2.f, mb, M + hh) >= R2s) {
                                    crec[p] = make_float4(M, mb, hh, B);
                                    cmask |= 1 << p;
                                    B = 0.f;
                                }
                            }
#pragma unroll
                            for (int c = 0; c < NC; ++c) {
                                if (KAHAN) {
                                    const float y = fmaf(B, cf[c], -cmp[p][c]);
                                    const float t2 = acc[p][c] + y;
                                    cmp[p][c] = (t2 - acc[p][c]) - y;
                                    acc[p][c] = t2;
                                } else {
                                    acc[p][c] = fmaf(B, cf[c], acc[p][c]);
                                }
                            }
                        }
                    }
                    my_triples += __popc(m);
                    if constexpr (MLPM) emit(cmask, crec, gi, (__float_as_int(sp.w) >> 6) + ((e >> 4) & 63));
                };

                int qn = 0;
                for (int base = 0; base < nst; base += 32) {
                    const int s = base + lane;
                    int mask = 0, cnt = 0;
                    if (s < nst) {
                        const float4 sp = stage[s];
                        const int sqv = DIM == 2 ? __float_as_int(sp.z) : sq[s];
                        const int q = SPLIT ? sqv & (IK_SQ_CONT - 1) : sqv;
                        const bool own = !SPLIT || sqv == q; // not a continuation: the kinetic term
                        float4 k0 = make_float4(0.f, 0.f, 0.f, 0.f), k1 = k0;
                        if (want_kin && own) { // issued before the tests so the latency overlaps them
                            k0 = __ldg(a.kin + (DIM == 2 ? q : 2 * q));
                            if (DIM == 3) k1 = __ldg(a.kin + 2 * q + 1);
                        }
                        // inside: r2 - R2s < 0 (the sign of an exact-zero-free difference);
                        // band: |r2 - R2s| < margin, looked at only when the closest of the
                        // group's differences is that small.  Padding points sit at 1e18:
                        // never inside, never in the band.
                        float r2v[P], dv[P];
                        int band = 0;
                        {
                            const f32x2 sx = pk2(sp.x, sp.x), sy = pk2(sp.y, sp.y), sz = pk2(sp.z, sp.z);
                            const f32x2 R2p = pk2(R2s, R2s);
#pragma unroll
                            for (int j = 0; j < P / 2; ++j) {
                                const f32x2 dx = sub2(g2[j][0], sx), dy = sub2(g2[j][1], sy);
                                f32x2 r2 = fma2(dy, dy, mul2(dx, dx));
                                if (DIM == 3) { const f32x2 dz = sub2(g2[j][2], sz); r2 = fma2(dz, dz, r2); }
                                up2(r2, r2v[2 * j], r2v[2 * j + 1]);
                                up2(sub2(r2, R2p), dv[2 * j], dv[2 * j + 1]);
                                mask |= (int)((__float_as_uint(dv[2 * j]) >> 31) | ((__float_as_uint(dv[2 * j + 1]) >> 31) << 1))
                                        << (2 * j);
                            }
                        }
                        float dmin = fabsf(dv[0]);
#pragma unroll
                        for (int p = 1; p < P; ++p) dmin = fminf(dmin, fabsf(dv[p]));
                        if (dmin < margin) {
#pragma unroll
                            for (int p = 0; p < P; ++p) band |= fabsf(dv[p]) < margin ? (1 << p) : 0;
                        }
                        if (band) { // rare: inside the thin band around R decide with the FP64 rule
                            const IkB64 pq = a.pos64[q];
#pragma unroll
                            for (int p = 0; p < P; ++p) {
                                if (!(band & (1 << p))) continue;
                                const double* xg = a.grid + 3 * (size_t)(MLPM ? gi[p] : __float_as_int(__ldg(&a.gpts[gs + p].w)));
                                const double ddx = ik_minimg(__dsub_rn(xg[0], pq.x), G.g.L[0], G.g.periodic[0]);
                                const double ddy = ik_minimg(__dsub_rn(xg[1], pq.y), G.g.L[1], G.g.periodic[1]);
                                const double ddz = ik_minimg(__dsub_rn(xg[2], pq.z), G.g.L[2], G.g.periodic[2]);
                                mask = ik_dot3(ddx, ddy, ddz) < a.R2 ? (mask | (1 << p)) : (mask & ~(1 << p));
                            }
                        }
                        if (mask) {
                            cnt = __float_as_int(sp.w) & 63;
                            if (want_kin && own) {
#pragma unroll
                                for (int p = 0; p < P; ++p) {
                                    const float kv = (mask & (1 << p)) ? ik_kern_in<KIND>(r2v[p]) : 0.f;
                                    kac[p][0] = fmaf(kv, k0.x, kac[p][0]);
                                    kac[p][1] = fmaf(kv, k0.y, kac[p][1]);
                                    kac[p][2] = fmaf(kv, k0.z, kac[p][2]);
                                    if (DIM == 3) {
                                        kac[p][3 % NC] = fmaf(kv, k0.w, kac[p][3 % NC]);
                                        kac[p][4 % NC] = fmaf(kv, k1.x, kac[p][4 % NC]);
                                        kac[p][5 % NC] = fmaf(kv, k1.y, kac[p][5 % NC]);
                                    }
                                }
                            }
                            my_pairs += own ? __popc(mask) : 0;
                        }
                    }
                    int incl = cnt;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        int t = __shfl_up_sync(FULL, incl, o);
                        if (lane >= o) incl += t;
                    }
                    const int tot = __reduce_add_sync(FULL, cnt); // beside the scan, not after it
                    const int off = qn + incl - cnt;
                    const int entry = (s << 10) | mask;
                    for (int k = 0; k < cnt; ++k) queue[off + k] = entry | (k << 4);
                    qn += tot;
                    __syncwarp();
                    // two batches in flight; in surrogate mode one at a time: the records of a
                    // second slot in flight spilled 68 bytes (its gather 192.8 -> 165.8 us per frame)
                    while (!MLPM && qn >= 64) {
                        const int e1 = queue[qn - 32 + lane], e2 = queue[qn - 64 + lane];
                        qn -= 64;
                        float4 sp1, b1, sp2, b2;
                        load_slot(e1, sp1, b1);
                        load_slot(e2, sp2, b2);
                        process_slot(e1, sp1, b1, PAIRK ? 1 : 0);
                        process_slot(e2, sp2, b2, PAIRK ? 2 : 0);
                    }
                    while (qn >= 32) { // at most one pass outside surrogate mode (qn < 64 here)
                        qn -= 32;
                        const int e1 = queue[qn + lane];
                        float4 sp1, b1;
                        load_slot(e1, sp1, b1);
                        process_slot(e1, sp1, b1);
                    }
                    __syncwarp();
                }
                if (MLPM ? qn > 0 : lane < qn) { // surrogate mode: all lanes (emission is warp-wide)
                    const int e1 = lane < qn ? queue[lane] : (queue[0] & ~15); // mask 0 on idle lanes
                    float4 sp1, b1;
                    load_slot(e1, sp1, b1);
                    process_slot(e1, sp1, b1);
                }
                __syncwarp();

                // ---- combine lanes: virial, then kinetic, each a transposing butterfly
                //      of VH values (compensated in the Kahan variant); results are
                //      written as unscaled double-float pairs (hi, lo), merged across
                //      chunks of an item with TwoSum, converted to FP64 later
                if constexpr (NP > 0 && QM != 3) {
#pragma unroll
                    for (int j = 0; j < P / 2; ++j)
#pragma unroll
                        for (int c = 0; c < NC; ++c) {
                            up2(acc2[j][c], acc[2 * j][c], acc[2 * j + 1][c]);
                            if constexpr (KAHAN) {
                                float n0, n1;
                                up2(cn2[j][c % (KAHAN ? NC : 1)], n0, n1);
                                cmp[2 * j][c] = -n0;
                                cmp[2 * j + 1][c] = -n1;
                            }
                        }
                }
                constexpr int VH = ik_pow2_ceil(P * NC);
                static_assert(VH == 16 || VH == 32, "butterfly width");
                float vh[VH], vl[VH], kh[VH], kl[VH];
#pragma unroll
                for (int p = 0; p < P; ++p)
#pragma unroll
                    for (int c = 0; c < NC; ++c) {
                        vh[p * NC + c] = acc[p][c];
                        vl[p * NC + c] = KAHAN ? -cmp[p][c] : 0.f;
                        kh[p * NC + c] = kac[p][c];
                        kl[p * NC + c] = 0.f;
                    }
#pragma unroll
                for (int k = P * NC; k < VH; ++k) { vh[k] = vl[k] = kh[k] = kl[k] = 0.f; }
                if constexpr (KAHAN) { // compensated lanes: compensated combination of the virial
                    ik_warp_reduce_cmp<VH>(vh, vl, lane);
                    // the kinetic partials are plain per-lane sums of ~4 terms (one
                    // kernel value per particle): their combination stays plain
                    ik_warp_reduce_plain<VH>(kh, lane);
                } else {
                    ik_warp_reduce_plain<VH>(vh, lane);
                    ik_warp_reduce_plain<VH>(kh, lane);
                }
                // VH == 16: lanes 2k and 2k+1 both hold value k -> the even lane writes
                // the virial, the odd lane the kinetic value; VH == 32: one value per lane
#pragma unroll
                for (int f = 0; f < (VH == 16 ? 1 : 2); ++f) {
                    const bool kin_here = VH == 16 ? (lane & 1) != 0 : f == 1;
                    const int idx = ik_red_index<VH>(lane, 0);
                    const float h = kin_here ? kh[0] : vh[0], l = kin_here ? kl[0] : vl[0];
                    const bool want = kin_here ? want_kin : (a.fields & 1);
                    if (idx < P * NC && want) {
                        const int p = idx / NC, c = idx - p * NC;
                        int g = -1;
#pragma unroll
                        if constexpr (MLPM) {
                            for (int pp = 0; pp < P; ++pp) if (pp == p) g = gi[pp];
                        } else { // reloaded: fewer live registers through the group
                            g = gs + p < gend ? __float_as_int(__ldg(&a.gpts[gs + p].w)) : -1;
                        }
                        if (g >= 0) {
                            float2* out = kin_here ? a.out_kin : a.out_vir;
                            const size_t o = (size_t)g * NC + c;
                            float fh = h, fl = l;
                            if (!first) { // another chunk of the same item: compensated add
                                const float2 old = out[o];
                                float s2, e2;
                                ik_two_sum(old.x, h, s2, e2);
                                fh = s2;
                                fl = e2 + (old.y + l);
                            }
                            if (a.direct64 && last) { // the value is final: FP64 into the field
                                double* o64;
                                size_t oo = o;
                                if constexpr (BATCH) {
                                    const IkBatchSlot& sl = a.slots[cur_slot];
                                    o64 = kin_here ? sl.out_kin : sl.out_vir;
                                    oo = (size_t)(g - sl.g_off) * NC + c;
                                } else {
                                    o64 = kin_here ? a.out64_kin : a.out64_vir;
                                }
                                o64[oo] = ((double)fh + (double)fl) * (kin_here ? a.s64_kin : a.s64_vir);
                            } else {
                                out[o] = make_float2(fh, fl);
                            }
                        }
                    }
                }
            }
            first = false;
            __syncwarp();
        }
    }
    if constexpr (MLPM)
        for (long long k = wfill + lane; k < wend; k += 32) a.mlp_rid[k] = make_int2(-1, 0);
    flush_counters();
    if constexpr (MLPM) {
        for (int o = 16; o; o >>= 1) my_records += __shfl_xor_sync(FULL, my_records, o);
        if (lane == 0) atomicAdd(a.cnt_records, my_records);
    }
}

template <int DIM, int KIND, bool KAHAN, int NP, int QM, bool ELA, bool SPLIT, bool BATCH = false>
static cudaError_t ik_launch_gather32_kernel(const GatherArgs32& a, int blocks, int threads, size_t smem,
                                             cudaStream_t st)
{
    auto kfn = k_gather32<DIM, KIND, KAHAN, NP, QM, ELA, SPLIT, BATCH>;
    cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kfn<<<blocks, threads, smem, st>>>(a);
    return cudaGetLastError();
}
