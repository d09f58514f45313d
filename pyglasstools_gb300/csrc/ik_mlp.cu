// ik_mlp.cu -- learned surrogate of the bond integral of a truncated Gaussian
// coarse-graining kernel (sm_103a).
//
// The bond integral B = int_0^1 Delta(x - r_i - s r_ij) ds (fixed point:
// irvingkirkwood/cgfunc/CoarseGrainFunction.h:85-88; adaptive GSL quadrature:
// CoarseGrainFunction.h:124-127 with cgfunc/Quadrature.h:47-49) is least accurate under a
// fixed-point rule on bonds that cross the edge of the kernel's support, where the
// integrand jumps to zero.  A 4 -> 64 -> 64 -> 64 -> 1 SiLU network stands in for the
// quadrature on exactly those bonds.  Everything here is in units of the width w:
//   K(r^2) = exp(-r^2 / 2) for r < 3, else 0           (un-normalised)
//   B(d, a, b) = int_0^1 K(d^2 + (a + s (b - a))^2) ds
// with d the distance from the grid point to the bond's line, a and b the signed
// positions of r_i (inside the support) and r_j (outside) along it, reflected so
// that b > 0.  The clipped part of the segment is known in closed form: it ends where
// the line leaves the ball, at t_c = sqrt(9 - d^2), a fraction s1 = (t_c - a)/(b - a)
// of the bond.  Four-point Gauss-Legendre on it is the first approximation (base; its
// relative error is below 1e-4 on this domain); the network predicts the scaled
// relative correction y = (B / base - 1) * MLP_YSCALE from x = (t_c / 3, a/4, b/4,
// 2 (w - 1.5)), so that B = base (1 + y / MLP_YSCALE).  The network's own error is
// scaled down by the same factor in B, which is what lets BF16 operands meet a 1e-6
// bound on B.
//
// Kernels:
//   k_mlp_samples   seeded samples of the crossing-bond domain and their labels by
//                   global adaptive quadrature (bisection of the worst interval, error
//                   from a 10/20-point Gauss-Legendre pair) on the clipped interval, FP64;
//   k_mlp_train     forward + backward of one mini-batch in FP32 (one sample per
//                   thread, activations in shared memory), per-CTA gradient partials;
//   k_mlp_adam      fixed-order reduction of the partials + Adam (deterministic);
//   k_mlp_deploy    FP32 parameters -> BF16 operand tiles in the tensor-core layout;
//   k_mlp_infer_tc  inference on the 5th-generation tensor cores: per 128-row tile,
//                   tcgen05.mma (kind::f16, BF16 in, FP32 accumulators in TMEM) for the
//                   three hidden layers with their biases, tcgen05.ld epilogues (SiLU)
//                   that write the next layer's operand (BF16) back to shared memory; the
//                   first layer is split three ways (x_hi W_hi + x_lo W_hi + x_hi W_lo);
//                   four warpgroups per CTA, each through its own tiles, share the weights;
//   k_mlp_infer_simt the same BF16 arithmetic on the CUDA cores (cross-check), or FP32.
#include "ik_kernels.h"
#include "../../include/ik_gb300.h"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

constexpr int H = 64, NIN = 4, TILE = 128;
constexpr int O_W1 = 0, O_B1 = O_W1 + H * NIN, O_W2 = O_B1 + H, O_B2 = O_W2 + H * H, O_W3 = O_B2 + H,
              O_B3 = O_W3 + H * H, O_W4 = O_B3 + H, O_B4 = O_W4 + H, NPAR = O_B4 + 1;
constexpr int NPART = NPAR + 1; // + loss
constexpr double LMAX = 2.5;    // longest bond sampled (units of w)
constexpr float MLP_YSCALE = 1.0e4f;        // network output = (B / base - 1) * MLP_YSCALE
constexpr float MLP_YINV = 1.0f / MLP_YSCALE;
constexpr double MLP_BASE_MIN = 1e-6;       // targets are 0 below this baseline
// four-point Gauss-Legendre on [-1, 1]: nodes +-GL4X0, +-GL4X1, weights GL4W0, GL4W1
constexpr double GL4X0 = 0.33998104358485626480, GL4X1 = 0.86113631159405257522;
constexpr double GL4W0 = 0.65214515486254614263, GL4W1 = 0.34785484513745385737;

// deployed blob (bytes): BF16 operand tiles in the no-swizzle K-major layout, then FP32.
// The hidden layers' biases ride on the tensor cores: the input operand carries 1.0 in
// its columns 12 and 13, and each bias enters as a BF16 pair (hi, lo) in columns 12 and 13
// of a B operand -- of W1 itself for the first layer, of a 64 x 16 bias tile (zero
// elsewhere) multiplied by the same input operand for the other two.
constexpr int DB_W1 = 0;                   // 64 x 16 bf16 (K padded from 4)  2048 B
constexpr int DB_W2 = DB_W1 + 64 * 16 * 2; // 64 x 64 bf16                     8192 B
constexpr int DB_W3 = DB_W2 + 64 * 64 * 2; // 64 x 64 bf16                     8192 B
constexpr int DB_B2 = DB_W3 + 64 * 64 * 2; // 64 x 16 bf16 bias tile of layer 2  2048 B
constexpr int DB_B3 = DB_B2 + 64 * 16 * 2; // 64 x 16 bf16 bias tile of layer 3  2048 B
constexpr int DB_F = DB_B3 + 64 * 16 * 2;  // floats: b1, b2, b3 (64 each), w4 (64, bf16-rounded), b4
constexpr int DB_NF = 4 * 64 + 1;
constexpr int DB_BYTES = (DB_F + DB_NF * 4 + 15) / 16 * 16;

} // namespace

// ---------------------------------------------------------------------------- shared math
__host__ __device__ inline void mlp_inputs(float d, float a, float b, float w, float x[4])
{
    const float dd = d * (1.0f / 3.0f);
    const float t = 1.0f - dd * dd;
    x[0] = t > 0.0f ? sqrtf(t) : 0.0f; // t_c / 3
    x[1] = 0.25f * a;
    x[2] = 0.25f * b;
    x[3] = 2.0f * (w - 1.5f);
}

// Gauss-Legendre-4 baseline on the clipped segment (see the header comment):
// base = s1 / 2 * sum_k w_k exp(-(d^2 + t_k^2) / 2), t_k = a + s1 l (1 + x_k) / 2
__host__ __device__ inline float mlp_base(float d, float a, float b)
{
    const float tc = sqrtf(fmaxf(9.0f - d * d, 0.0f));
    const float l = b - a;
    const float s1 = l > 0.0f ? fminf(fmaxf((tc - a) / l, 0.0f), 1.0f) : 0.0f;
    const float h = 0.5f * s1 * l, m = a + h, d2 = d * d;
    const float t0 = m - h * (float)GL4X1, t1 = m - h * (float)GL4X0, t2 = m + h * (float)GL4X0,
                t3 = m + h * (float)GL4X1;
    const float sum = (float)GL4W1 * (expf(-0.5f * (d2 + t0 * t0)) + expf(-0.5f * (d2 + t3 * t3))) +
                      (float)GL4W0 * (expf(-0.5f * (d2 + t1 * t1)) + expf(-0.5f * (d2 + t2 * t2)));
    return 0.5f * s1 * sum;
}

__device__ __forceinline__ float silu_exact(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu_grad(float z)
{
    const float s = 1.0f / (1.0f + expf(-z));
    return s * (1.0f + z * (1.0f - s));
}
__device__ __forceinline__ float tanh_approx(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// SiLU for the deployed network: z * sigmoid(z), sigmoid(z) = 1/2 + tanh(z/2)/2
__device__ __forceinline__ float silu_fast(float z) { return z * fmaf(0.5f, tanh_approx(0.5f * z), 0.5f); }
__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// SplitMix64 (Steele, Lea and Flood 2014) as a counter-based generator
__device__ __forceinline__ unsigned long long mix64(unsigned long long z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double u01(unsigned long long seed, long long i, int k)
{
    unsigned long long h = mix64(seed ^ mix64((unsigned long long)i * 4 + (unsigned long long)k));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

// ---------------------------------------------------------------------------- samples + labels
struct MlpGL {
    double x10[10], w10[10], x20[20], w20[20];
};

__device__ double mlp_seg(const MlpGL& q, double d2, double a, double l, double lo, double hi, bool fine)
{
    // int_lo^hi exp(-(d^2 + (a + s l)^2) / 2) ds by Gauss-Legendre (10 or 20 points)
    const double c = 0.5 * (lo + hi), h = 0.5 * (hi - lo);
    const int n = fine ? 20 : 10;
    const double* x = fine ? q.x20 : q.x10;
    const double* w = fine ? q.w20 : q.w10;
    double acc = 0.0;
    for (int k = 0; k < n; ++k) {
        const double s = c + h * x[k];
        const double t = a + s * l;
        acc += w[k] * exp(-0.5 * (d2 + t * t));
    }
    return acc * h;
}

// Global adaptive quadrature of B on the clipped interval [0, s1]: every interval
// carries the 20-point value and |G20 - G10| as its error; the worst is bisected
// until the total error is below max(1e-14, 1e-12 |B|) (QUADPACK's QAG strategy with
// a Gauss-Legendre pair for the estimate).
__device__ double mlp_label(const MlpGL& q, double d, double a, double b)
{
    const double tc = sqrt(fmax(9.0 - d * d, 0.0));
    const double l = b - a;
    double s1 = l > 0.0 ? (tc - a) / l : 1.0;
    s1 = fmin(fmax(s1, 0.0), 1.0);
    if (!(s1 > 0.0)) return 0.0;
    constexpr int LIM = 24;
    double ia[LIM], ib[LIM], ir[LIM], ie[LIM];
    const double d2 = d * d;
    ia[0] = 0.0; ib[0] = s1;
    ir[0] = mlp_seg(q, d2, a, l, 0.0, s1, true);
    ie[0] = fabs(ir[0] - mlp_seg(q, d2, a, l, 0.0, s1, false));
    int n = 1;
    double res = ir[0], err = ie[0];
    while (n < LIM && err > fmax(1e-14, 1e-12 * fabs(res))) {
        int worst = 0;
        for (int k = 1; k < n; ++k) if (ie[k] > ie[worst]) worst = k;
        const double lo = ia[worst], hi = ib[worst], m = 0.5 * (lo + hi);
        const double r1 = mlp_seg(q, d2, a, l, lo, m, true), r2 = mlp_seg(q, d2, a, l, m, hi, true);
        ie[worst] = fabs(r1 - mlp_seg(q, d2, a, l, lo, m, false));
        ib[worst] = m; ir[worst] = r1;
        ia[n] = m; ib[n] = hi; ir[n] = r2;
        ie[n] = fabs(r2 - mlp_seg(q, d2, a, l, m, hi, false));
        ++n;
        res = 0.0; err = 0.0;
        for (int k = 0; k < n; ++k) { res += ir[k]; err += ie[k]; }
    }
    return res;
}

// Sample i of the crossing-bond domain: d ~ U[0,3); the inside end a ~ U over the part
// of (-tc, tc) from which a bond of length <= LMAX can leave the support; the length
// so that the outside end b lies in [tc, min(a + LMAX, 4)]; w = 1 or 2.
__global__ void k_mlp_samples(long long n, unsigned long long seed, MlpGL q, float4* feats, double* labels,
                              float* targets)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double d = 3.0 * u01(seed, i, 0);
    const double tc = sqrt(fmax(9.0 - d * d, 0.0));
    const double alo = fmax(-tc, tc - LMAX);
    const double a = alo + (tc - alo) * u01(seed, i, 1);
    const double llo = tc - a, lhi = fmin(LMAX, 4.0 - a);
    const double b = a + llo + (lhi - llo) * u01(seed, i, 2);
    const double w = u01(seed, i, 3) < 0.5 ? 1.0 : 2.0;
    const double B = mlp_label(q, d, a, b);
    feats[i] = make_float4((float)d, (float)a, (float)b, (float)w);
    labels[i] = B;
    // target y = (B / base - 1) * MLP_YSCALE, the baseline from the FP32 features (what
    // the network sees), in FP64
    const double df = (float)d, af = (float)a, bf = (float)b;
    const double tcf = sqrt(fmax(9.0 - df * df, 0.0));
    const double l = bf - af;
    const double s1 = l > 0.0 ? fmin(fmax((tcf - af) / l, 0.0), 1.0) : 0.0;
    const double h = 0.5 * s1 * l, m = af + h, d2 = df * df;
    auto e = [&](double t) { return exp(-0.5 * (d2 + t * t)); };
    const double base = 0.5 * s1 * (GL4W1 * (e(m - h * GL4X1) + e(m + h * GL4X1)) +
                                    GL4W0 * (e(m - h * GL4X0) + e(m + h * GL4X0)));
    // where the baseline is below 1e-6 the label's own tolerance (1e-14 absolute) is no
    // longer small against the network's share of B (below 1e-9 of B there): target 0; the
    // target is clipped to [-8, 8] (the baseline's relative error is below 1e-4 here)
    targets[i] = base > MLP_BASE_MIN ? (float)fmin(fmax((B / base - 1.0) * (double)MLP_YSCALE, -8.0), 8.0) : 0.0f;
}

// ---------------------------------------------------------------------------- training
// One mini-batch tile of 128 samples per CTA iteration; one sample per thread.
// Shared memory: X[128][4], Z1..Z3[128][65] (pre-activations, then their gradients),
// Hs[128][65] (activations of the layer being differentiated), W1, W2, W3, W4, biases.
constexpr int TS = 65; // padded row stride
constexpr size_t TRAIN_SMEM =
    sizeof(float) * (128 * 4 + 4 * 128 * TS + 2 * 64 * 64 + 64 * 4 + 4 * 64 + 1 + 128 + 128);

struct TrainArgs {
    const float* params;   // NPAR master parameters
    const float4* feats;
    const float* targets;
    long long nsamples;    // a power of two
    long long pos0;        // first position of this step in the epoch's permutation
    unsigned long long perm_a, perm_b;  // position -> sample: (p * a + b) mod nsamples
    int tiles_per_cta;
    long long valid;       // samples of the batch that are real (ragged batches)
    float inv_batch;       // 1 / samples in the batch
    float* partial;        // gridDim.x x NPART
};

__global__ void __launch_bounds__(128, 1) k_mlp_train(const TrainArgs A)
{
    extern __shared__ float sm[];
    float* X = sm;                  // 128 x 4
    float* Z1 = X + 128 * 4;        // 128 x TS
    float* Z2 = Z1 + 128 * TS;
    float* Z3 = Z2 + 128 * TS;
    float* Hs = Z3 + 128 * TS;
    float* W2 = Hs + 128 * TS;      // 64 x 64
    float* W3 = W2 + 64 * 64;
    float* W1 = W3 + 64 * 64;       // 64 x 4
    float* Bs = W1 + 64 * 4;        // b1, b2, b3, w4 (64 each)
    float* b4 = Bs + 4 * 64;        // 1
    float* DY = b4 + 1;             // 128
    float* LS = DY + 128;           // 128 (per-thread loss)
    const int t = threadIdx.x;
    for (int k = t; k < 64 * 64; k += 128) { W2[k] = A.params[O_W2 + k]; W3[k] = A.params[O_W3 + k]; }
    for (int k = t; k < 64 * 4; k += 128) W1[k] = A.params[O_W1 + k];
    if (t < 64) {
        Bs[t] = A.params[O_B1 + t];
        Bs[64 + t] = A.params[O_B2 + t];
        Bs[128 + t] = A.params[O_B3 + t];
        Bs[192 + t] = A.params[O_W4 + t];
    }
    if (t == 0) b4[0] = A.params[O_B4];
    __syncthreads();

    // gradient partials owned by this thread
    const int gn = t >> 1, gp = t & 1; // dW2/dW3 row gn, columns k = 2j + gp
    float gW3[32], gW2[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) { gW3[j] = 0.f; gW2[j] = 0.f; }
    float gb3 = 0.f, gb2 = 0.f, gb1 = 0.f, gW4 = 0.f, gb4 = 0.f, gW1a = 0.f, gW1b = 0.f, loss = 0.f;
    const int w1i0 = 2 * t, w1i1 = 2 * t + 1; // dW1 entries (n = idx / 4, k = idx % 4)

    for (int tile = 0; tile < A.tiles_per_cta; ++tile) {
        const long long bpos = ((long long)blockIdx.x * A.tiles_per_cta + tile) * 128 + t; // position in batch
        const bool valid = bpos < A.valid;
        float y = 0.f;
        {
            const unsigned long long p = (unsigned long long)(A.pos0 + bpos) & (unsigned long long)(A.nsamples - 1);
            const long long si = (long long)((p * A.perm_a + A.perm_b) & (unsigned long long)(A.nsamples - 1));
            const float4 f = A.feats[si];
            float x[4];
            mlp_inputs(f.x, f.y, f.z, f.w, x);
#pragma unroll
            for (int k = 0; k < 4; ++k) X[t * 4 + k] = x[k];
            y = A.targets[si];
        }
        // ---- forward (own row)
        float h[64];
#pragma unroll
        for (int n = 0; n < 64; ++n) {
            float z = Bs[n];
#pragma unroll
            for (int k = 0; k < 4; ++k) z = fmaf(W1[n * 4 + k], X[t * 4 + k], z);
            Z1[t * TS + n] = z;
            h[n] = silu_exact(z);
        }
#pragma unroll 1
        for (int layer = 0; layer < 2; ++layer) {
            const float* W = layer == 0 ? W2 : W3;
            const float* bb = Bs + 64 * (layer + 1);
            float* Zo = layer == 0 ? Z2 : Z3;
#pragma unroll 4
            for (int n = 0; n < 64; ++n) {
                float z = bb[n];
                const float4* wr = reinterpret_cast<const float4*>(W + n * 64);
#pragma unroll
                for (int k4 = 0; k4 < 16; ++k4) {
                    const float4 wv = wr[k4];
                    z = fmaf(wv.x, h[4 * k4], z);
                    z = fmaf(wv.y, h[4 * k4 + 1], z);
                    z = fmaf(wv.z, h[4 * k4 + 2], z);
                    z = fmaf(wv.w, h[4 * k4 + 3], z);
                }
                Zo[t * TS + n] = z;
            }
#pragma unroll
            for (int n = 0; n < 64; ++n) h[n] = silu_exact(Zo[t * TS + n]);
        }
        float out = b4[0];
#pragma unroll
        for (int k = 0; k < 64; ++k) out = fmaf(Bs[192 + k], h[k], out);
        const float r = valid ? out - y : 0.f;
        loss = fmaf(r, r, loss);
        DY[t] = 2.0f * r * A.inv_batch;
        __syncthreads();
        // ---- output layer gradients (fixed order over samples)
        if (t < 64) {
            float s = 0.f;
            for (int q = 0; q < 128; ++q) s = fmaf(DY[q], silu_exact(Z3[q * TS + t]), s);
            gW4 += s;
        } else if (t == 64) {
            float s = 0.f;
            for (int q = 0; q < 128; ++q) s += DY[q];
            gb4 += s;
        }
        __syncthreads();
        // ---- layer 3: dZ3 (in place), H2 = silu(Z2)
        {
            const float dy = DY[t];
#pragma unroll 8
            for (int k = 0; k < 64; ++k) {
                const float z3 = Z3[t * TS + k];
                Z3[t * TS + k] = dy * Bs[192 + k] * silu_grad(z3);
                Hs[t * TS + k] = silu_exact(Z2[t * TS + k]);
            }
        }
        __syncthreads();
        // dW3[gn][2j+gp] += sum_q dZ3[q][gn] H2[q][2j+gp]
        for (int q = 0; q < 128; ++q) {
            const float dz = Z3[q * TS + gn];
            if (gp == 0) gb3 += dz;
#pragma unroll
            for (int j = 0; j < 32; ++j) gW3[j] = fmaf(dz, Hs[q * TS + 2 * j + gp], gW3[j]);
        }
        // dH2 = W3^T dZ3 (own row) -> dZ2 in place
        {
            float dh[64];
#pragma unroll
            for (int k = 0; k < 64; ++k) dh[k] = 0.f;
#pragma unroll 2
            for (int n = 0; n < 64; ++n) {
                const float dz = Z3[t * TS + n];
                const float4* wr = reinterpret_cast<const float4*>(W3 + n * 64);
#pragma unroll
                for (int k4 = 0; k4 < 16; ++k4) {
                    const float4 wv = wr[k4];
                    dh[4 * k4] = fmaf(wv.x, dz, dh[4 * k4]);
                    dh[4 * k4 + 1] = fmaf(wv.y, dz, dh[4 * k4 + 1]);
                    dh[4 * k4 + 2] = fmaf(wv.z, dz, dh[4 * k4 + 2]);
                    dh[4 * k4 + 3] = fmaf(wv.w, dz, dh[4 * k4 + 3]);
                }
            }
#pragma unroll
            for (int k = 0; k < 64; ++k) Z2[t * TS + k] = dh[k] * silu_grad(Z2[t * TS + k]);
        }
        __syncthreads();
        // ---- layer 2: H1 = silu(Z1)
#pragma unroll 8
        for (int k = 0; k < 64; ++k) Hs[t * TS + k] = silu_exact(Z1[t * TS + k]);
        __syncthreads();
        for (int q = 0; q < 128; ++q) {
            const float dz = Z2[q * TS + gn];
            if (gp == 0) gb2 += dz;
#pragma unroll
            for (int j = 0; j < 32; ++j) gW2[j] = fmaf(dz, Hs[q * TS + 2 * j + gp], gW2[j]);
        }
        {
            float dh[64];
#pragma unroll
            for (int k = 0; k < 64; ++k) dh[k] = 0.f;
#pragma unroll 2
            for (int n = 0; n < 64; ++n) {
                const float dz = Z2[t * TS + n];
                const float4* wr = reinterpret_cast<const float4*>(W2 + n * 64);
#pragma unroll
                for (int k4 = 0; k4 < 16; ++k4) {
                    const float4 wv = wr[k4];
                    dh[4 * k4] = fmaf(wv.x, dz, dh[4 * k4]);
                    dh[4 * k4 + 1] = fmaf(wv.y, dz, dh[4 * k4 + 1]);
                    dh[4 * k4 + 2] = fmaf(wv.z, dz, dh[4 * k4 + 2]);
                    dh[4 * k4 + 3] = fmaf(wv.w, dz, dh[4 * k4 + 3]);
                }
            }
#pragma unroll
            for (int k = 0; k < 64; ++k) Z1[t * TS + k] = dh[k] * silu_grad(Z1[t * TS + k]);
        }
        __syncthreads();
        // ---- layer 1
        for (int q = 0; q < 128; ++q) {
            gW1a = fmaf(Z1[q * TS + (w1i0 >> 2)], X[q * 4 + (w1i0 & 3)], gW1a);
            gW1b = fmaf(Z1[q * TS + (w1i1 >> 2)], X[q * 4 + (w1i1 & 3)], gW1b);
            if (t < 64) gb1 += Z1[q * TS + t];
        }
        __syncthreads();
    }
    // ---- write this CTA's partials
    float* P = A.partial + (size_t)blockIdx.x * NPART;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
        P[O_W3 + gn * 64 + 2 * j + gp] = gW3[j];
        P[O_W2 + gn * 64 + 2 * j + gp] = gW2[j];
    }
    if (gp == 0) { P[O_B3 + gn] = gb3; P[O_B2 + gn] = gb2; }
    P[O_W1 + w1i0] = gW1a;
    P[O_W1 + w1i1] = gW1b;
    if (t < 64) { P[O_B1 + t] = gb1; P[O_W4 + t] = gW4; }
    if (t == 64) P[O_B4] = gb4;
    LS[t] = loss;
    __syncthreads();
    if (t == 0) {
        float s = 0.f;
        for (int q = 0; q < 128; ++q) s += LS[q];
        P[NPAR] = s;
    }
}

// Sum the partials in CTA order (deterministic), then one Adam step on the FP32 master
// parameters (Kingma and Ba 2015).  lr <= 0: only the gradient is written (checks).
__global__ void k_mlp_adam(float* params, float* m, float* v, const float* partial, int nparts, float* grad,
                           float* loss_out, float lr, float b1, float b2, float eps, float bc1, float bc2)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > NPAR) return;
    float g = 0.f;
    for (int c = 0; c < nparts; ++c) g += partial[(size_t)c * NPART + p];
    if (p == NPAR) { if (loss_out) *loss_out = g; return; }
    if (grad) grad[p] = g;
    if (lr <= 0.f) return;
    const float mm = b1 * m[p] + (1.f - b1) * g;
    const float vv = b2 * v[p] + (1.f - b2) * g * g;
    m[p] = mm;
    v[p] = vv;
    params[p] -= lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
}

// ---------------------------------------------------------------------------- deployment
// Offset of element (r, k) of a K-major BF16 operand with K columns in the no-swizzle
// canonical layout: 8 x 8 core matrices of 128 contiguous bytes (8 rows x 16 B),
// k-adjacent core matrices 128 B apart (leading byte offset), 8-row groups
// (K/8) * 128 B apart (stride byte offset).
__host__ __device__ inline int op_off(int r, int k, int K)
{
    return (r >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// A bias as the BF16 pair (hi, lo) that the tensor cores add (hi + lo = b to ~2^-17).
__device__ __forceinline__ float bias_hi(float b) { return bf16r(b); }
__device__ __forceinline__ float bias_lo(float b) { return bf16r(b - bf16r(b)); }

__global__ void k_mlp_deploy(const float* P, unsigned char* blob)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    // hidden layers prescaled by 1/2 (exact), so that the accumulators hold h = z/2 and
    // SiLU(z) = h + h tanh(h)
    if (i < 64 * 16) { // W1 as [hi | hi | lo | b1 hi, b1 lo, 0, 0] against inputs
                       // [x_hi | x_lo | x_hi | 1, 1, 0, 0]
        const int n = i / 16, k = i % 16, j = k & 3;
        const float w = 0.5f * P[O_W1 + n * 4 + j];
        const float hi = bf16r(w);
        const float b1 = 0.5f * P[O_B1 + n];
        const float v = k < 8 ? hi : (k < 12 ? w - hi : (k == 12 ? bias_hi(b1) : (k == 13 ? bias_lo(b1) : 0.f)));
        *reinterpret_cast<__nv_bfloat16*>(blob + DB_W1 + op_off(n, k, 16)) = __float2bfloat16_rn(v);
        // bias tiles of layers 2 and 3: (hi, lo) in columns 12 and 13, zero elsewhere
        const float b2 = 0.5f * P[O_B2 + n], b3 = 0.5f * P[O_B3 + n];
        const float v2 = k == 12 ? bias_hi(b2) : (k == 13 ? bias_lo(b2) : 0.f);
        const float v3 = k == 12 ? bias_hi(b3) : (k == 13 ? bias_lo(b3) : 0.f);
        *reinterpret_cast<__nv_bfloat16*>(blob + DB_B2 + op_off(n, k, 16)) = __float2bfloat16_rn(v2);
        *reinterpret_cast<__nv_bfloat16*>(blob + DB_B3 + op_off(n, k, 16)) = __float2bfloat16_rn(v3);
    }
    if (i < 64 * 64) {
        const int n = i / 64, k = i % 64;
        *reinterpret_cast<__nv_bfloat16*>(blob + DB_W2 + op_off(n, k, 64)) = __float2bfloat16_rn(0.5f * P[O_W2 + i]);
        *reinterpret_cast<__nv_bfloat16*>(blob + DB_W3 + op_off(n, k, 64)) = __float2bfloat16_rn(0.5f * P[O_W3 + i]);
    }
    float* F = reinterpret_cast<float*>(blob + DB_F);
    if (i < 64) {
        F[i] = 0.5f * P[O_B1 + i];
        F[64 + i] = 0.5f * P[O_B2 + i];
        F[128 + i] = 0.5f * P[O_B3 + i];
        F[192 + i] = bf16r(P[O_W4 + i]);
    }
    if (i == 0) F[256] = P[O_B4];
}

// ---------------------------------------------------------------------------- SIMT inference
// mode 0: FP32 weights and activations, exact SiLU (the training network);
// mode 1: the arithmetic of the tensor-core kernel (BF16 weights and activations, first
//         layer split three ways, FP32 accumulation, the deployed SiLU), for cross-checks.
// raw: out = the network's output y instead of B.
__global__ void k_mlp_infer_simt(const float* P, const float4* feats, long long n, int mode, int raw, float* out)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool q = mode == 1;
    auto R = [&](float v) { return q ? bf16r(v) : v; };
    auto S = [&](float z) { // deployed form: h = z/2 from prescaled weights, h + h tanh(h)
        if (!q) return silu_exact(z);
        const float h = 0.5f * z;
        return fmaf(h, tanh_approx(h), h);
    };
    const float4 f = feats[i];
    float x[4];
    mlp_inputs(f.x, f.y, f.z, f.w, x);
    float h[64], g[64];
    // BF16 split of the first layer (x_hi W_hi + x_lo W_hi + x_hi W_lo); BF16 weights and
    // activations elsewhere
    auto P2 = [&](float v) { return q ? bf16r(v) : v; };
    // hidden-layer biases as the tensor cores add them: hi + lo of the prescaled bias b/2
    auto Bq = [&](float b) { return q ? 2.0f * (bias_hi(0.5f * b) + bias_lo(0.5f * b)) : b; };
    for (int nn = 0; nn < 64; ++nn) {
        float z = 0.f;
        for (int k = 0; k < 4; ++k) {
            const float w = P[O_W1 + nn * 4 + k];
            if (q) {
                const float xh = bf16r(x[k]), xl = bf16r(x[k] - xh), wh = bf16r(w), wl = bf16r(w - wh);
                z = fmaf(wh, xh, z);
                z = fmaf(wh, xl, z);
                z = fmaf(wl, xh, z);
            } else {
                z = fmaf(w, x[k], z);
            }
        }
        h[nn] = P2(S(z + Bq(P[O_B1 + nn])));
    }
    for (int layer = 0; layer < 2; ++layer) {
        const int ow = layer == 0 ? O_W2 : O_W3, ob = layer == 0 ? O_B2 : O_B3;
        for (int nn = 0; nn < 64; ++nn) {
            float z = 0.f;
            for (int k = 0; k < 64; ++k) z = fmaf(R(P[ow + nn * 64 + k]), h[k], z);
            g[nn] = z + Bq(P[ob + nn]);
        }
        for (int nn = 0; nn < 64; ++nn) h[nn] = layer == 0 ? P2(S(g[nn])) : S(g[nn]);
    }
    float y = 0.f;
    for (int k = 0; k < 64; ++k) y = fmaf(R(P[O_W4 + k]), h[k], y);
    y += P[O_B4];
    out[i] = raw ? y : mlp_base(f.x, f.y, f.z) * fmaf(y, MLP_YINV, 1.0f);
}

// ---------------------------------------------------------------------------- tcgen05 helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (tcgen05): start address, leading and stride byte
// offsets (>> 4), fixed field 0b001 at bits 46-48, no swizzle.
__device__ __forceinline__ unsigned long long umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    unsigned long long d = 0;
    d |= (unsigned long long)((saddr & 0x3FFFFu) >> 4);
    d |= (unsigned long long)((lbo & 0x3FFFFu) >> 4) << 16;
    d |= (unsigned long long)((sbo & 0x3FFFFu) >> 4) << 32;
    d |= 1ull << 46;
    return d;
}
// Instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16 (bits 7-9,
// 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, unsigned long long adesc, unsigned long long bdesc,
                                          uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        :
        : "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t a, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: false if the phase did not complete within `limit` polls
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, int limit = 1 << 22)
{
    for (int it = 0; it < limit; ++it)
        if (mbar_try_wait(a, parity)) return true;
    return false;
}
// Failure-detection test hook (ik_mlp_test_stall): no MMA is issued and nothing is
// committed to the completion barrier, so its wait runs out after this many polls;
// no asynchronous tensor-core work is in flight when the kernel then gives up.
constexpr int TC_STALL_POLLS = 64;
// 32 lanes x 32 bits, 16 consecutive columns: thread l of warp w gets TMEM lane 32 w + l
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15])
                 :
                 : "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}
// packed FP32 pairs (f32x2 arithmetic): two columns of a row per instruction
typedef unsigned long long mlp_f2;
__device__ __forceinline__ mlp_f2 mlp_pk2(float a, float b)
{
    mlp_f2 r;
    asm("mov.b64 %0, {%1,%2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void mlp_up2(mlp_f2 r, float& a, float& b)
{
    asm("mov.b64 {%0,%1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ mlp_f2 mlp_fma2(mlp_f2 a, mlp_f2 b, mlp_f2 c)
{
    mlp_f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi)
{
    __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&p);
}

// ---------------------------------------------------------------------------- tcgen05 inference
// A CTA holds TC_WG warpgroups; each works through its own 128-row tiles (its own input
// and hidden operands, TMEM columns and completion barrier), and all of them share the
// deployed weights in shared memory -- more tiles in flight per SM than one tile per CTA.
#ifndef IK_TC_WG
#define IK_TC_WG 4
#endif
constexpr int TC_WG = IK_TC_WG;
constexpr int TC_THREADS = 128 * TC_WG;
// Shared memory layout of k_mlp_infer_tc (bytes, 1024-aligned pieces):
constexpr int TC_A0 = 0;                              // per warpgroup: 128 x 16 bf16 input operand   4096
constexpr int TC_H = TC_A0 + TC_WG * 128 * 16 * 2;    // per warpgroup: 128 x 64 bf16 hidden operand  16384
constexpr int TC_W = TC_H + TC_WG * 128 * 64 * 2;     // deployed blob (W1, W2, W3, bias tiles, floats)
constexpr int TC_BAR = TC_W + DB_BYTES;  // DB_BYTES is a multiple of 16: one barrier per warpgroup,
constexpr int TC_SMEM = TC_BAR + 64;     // the TMEM address and the abort flag
// The CTAs that fit an SM by shared memory (228 KB) hold 64 TMEM columns per warpgroup,
// at most 512 in all, so their allocations never wait on one another.
constexpr int TC_SMEM_LAUNCH = TC_SMEM;
constexpr int TC_CTAS_PER_SM = 233472 / (TC_SMEM_LAUNCH + 1024);
static_assert(TC_CTAS_PER_SM >= 1 && TC_CTAS_PER_SM * 64 * TC_WG <= 512, "TMEM columns of the resident CTAs");
static_assert(8 * TC_WG + 8 <= 64, "barrier area");
// CTAs of k_mlp_infer_tc resident per SM (shared memory bound): the records launch's grid
int mlp_tc_ctas_per_sm() { return TC_CTAS_PER_SM; }
constexpr uint32_t TC_COLS = 64 * TC_WG;

// Records of bonds that cross the support, written by the FP32 gather in surrogate
// mode: {M, mb, hh, B_fixed} in the gather's scaled units + {grid index, bond index}.
struct MlpRecArgs {
    const float4* rec;
    const int2* rid;
    const unsigned long long* count;  // records reserved (device)
    long long capacity;
    const float4* bonds;              // {hb, f'} bond records
    const unsigned char* table;       // per-bin use of the surrogate (1) or the fixed rule (0)
    float to_w;                       // scaled length -> units of w
    float w;
    int nc;                           // 3 (2D) or 6 (3D) components
    unsigned long long* corr;         // fixed-point accumulators, G x nc
    unsigned long long* fallbacks;    // += records that kept their fixed-point value
};

// Canonical surrogate coordinates of a record; returns the bin (or -1 outside the table).
__device__ __forceinline__ int mlp_record_coords(const float4 r, float to_w, float w, float& d, float& a, float& b)
{
    const float M = r.x, mb = r.y, hh = r.z;
    const float xi0 = mb / hh;
    const float d2 = fmaxf(M - mb * xi0, 0.0f);
    const float hl = sqrtf(hh);
    d = sqrtf(d2) * to_w;
    a = (-1.0f - xi0) * hl * to_w; // r_i
    b = (1.0f - xi0) * hl * to_w;  // r_j
    if (b < 0.0f) { a = -a; b = -b; }
    const int id = (int)(d * 4.0f), ia = (int)floorf((a + 3.0f) * 4.0f), ib = (int)(b * 4.0f);
    if (id < 0 || id >= 12 || ia < 0 || ia >= 24 || ib < 0 || ib >= 16) return -1;
    return (((w < 1.5f ? 0 : 1) * 12 + id) * 24 + ia) * 16 + ib;
}

// MODE 0: out[i] = surrogate B of feats[i] (units of w, un-normalised);
// MODE 1: IK records -> fixed-point stress corrections.
// stall != 0: the failure-detection test hook (TC_STALL_POLLS).  MODE 0 with raw != 0:
// out[i] = the network's output y instead of B.
template <int MODE>
__global__ void __launch_bounds__(TC_THREADS, TC_CTAS_PER_SM) k_mlp_infer_tc(const unsigned char* __restrict__ blob, const float4* feats,
                                                     long long n, float* out, MlpRecArgs R, int* status, int stall,
                                                     int raw)
{
    extern __shared__ __align__(1024) unsigned char tsm[];
    // t: this thread's row of its warpgroup's tile; warp: the warp within the CTA
    const int tid = threadIdx.x, wg = tid >> 7, t = tid & 127, warp = tid >> 5;
    unsigned char* sA0 = tsm + TC_A0 + wg * (128 * 16 * 2);
    unsigned char* sH = tsm + TC_H + wg * (128 * 64 * 2);
    unsigned char* sW = tsm + TC_W;
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(tsm + TC_BAR) + wg;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(tsm + TC_BAR + 8 * TC_WG);
    int* abort_flag = reinterpret_cast<int*>(tsm + TC_BAR + 8 * TC_WG + 4);
    // the warpgroup's own barrier (named barrier wg + 1; 0 is __syncthreads)
    auto wg_sync = [&]() { asm volatile("bar.sync %0, 128;" ::"r"(wg + 1) : "memory"); };

    // stage the deployed weights; zero the input operands (columns 4..15 stay zero)
    for (int k = tid; k < DB_BYTES / 16; k += TC_THREADS)
        reinterpret_cast<uint4*>(sW)[k] = reinterpret_cast<const uint4*>(blob)[k];
    for (int k = tid; k < TC_WG * 128 * 16 * 2 / 16; k += TC_THREADS)
        reinterpret_cast<uint4*>(tsm + TC_A0)[k] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        for (int w = 0; w < TC_WG; ++w) mbar_init(smem_u32(reinterpret_cast<unsigned long long*>(tsm + TC_BAR) + w), 1);
        *abort_flag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(TC_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem_base = *tslot;
    const uint32_t tmem = tmem_base + 64u * (uint32_t)wg;        // the warpgroup's columns
    const uint32_t tl = tmem + ((uint32_t)(32 * (warp & 3)) << 16); // this warp's TMEM lanes
    const float* F = reinterpret_cast<const float*>(sW + (DB_F));
    const uint32_t aA0 = smem_u32(sA0), aH = smem_u32(sH), aW1 = smem_u32(sW + DB_W1),
                   aW2 = smem_u32(sW + DB_W2), aW3 = smem_u32(sW + DB_W3), aB2 = smem_u32(sW + DB_B2),
                   aB3 = smem_u32(sW + DB_B3), aBar = smem_u32(bar);
    constexpr uint32_t ID = idesc_bf16(128, 64);
    uint32_t phase = 0;

    long long total = n;
    if (MODE == 1) {
        total = (long long)*R.count;
        if (total > R.capacity) total = R.capacity;
    }
    const long long ntiles = (total + 127) / 128;
    // a row's inputs are loaded one tile ahead, so that their latency hides under the
    // previous tile's MMAs and epilogues
    float4 next_f = make_float4(0.f, 0.f, 0.f, 0.f);
    int2 next_id = make_int2(-1, 0);
    auto fetch = [&](long long tl_) {
        const long long r_ = tl_ * 128 + t;
        next_id = make_int2(-1, 0);
        if (tl_ < ntiles && r_ < total) {
            if (MODE == 0) {
                next_f = feats[r_];
            } else {
                next_f = R.rec[r_];
                next_id = R.rid[r_];
            }
        }
    };
    const long long tile0 = (long long)blockIdx.x * TC_WG + wg, tstep = (long long)gridDim.x * TC_WG;
    fetch(tile0);
    for (long long tile = tile0; tile < ntiles; tile += tstep) {
        const long long row = tile * 128 + t;
        const float4 cur_f = next_f;
        const int2 cur_id = next_id;
        fetch(tile + tstep);
        bool valid = row < total;
        float fd = 0.f, fa = 0.f, fb = 0.f, fw = R.w, bfix = 0.f;
        int g = -1, bin = -1;
        float4 bd = make_float4(0.f, 0.f, 0.f, 0.f); // MODE 1: the bond's record, for the coefficient
        bool use = false;                           // MODE 1: the bin uses the network
        if (MODE == 0) {
            if (valid) { fd = cur_f.x; fa = cur_f.y; fb = cur_f.z; fw = cur_f.w; }
        } else if (valid) {
            g = cur_id.x;
            valid = g >= 0;
            if (valid) {
                bin = mlp_record_coords(cur_f, R.to_w, R.w, fd, fa, fb);
                bfix = cur_f.w;
                // issued now, used after the MMAs
                bd = __ldg(R.bonds + cur_id.y);
                use = bin >= 0 && __ldg(R.table + bin) != 0;
            }
        }
        // Gauss-Legendre-4 baseline on the clipped segment (as mlp_base, exp via ex2.approx)
        float base;
        {
            const float tc = sqrtf(fmaxf(9.0f - fd * fd, 0.0f));
            const float l = fb - fa;
            const float s1 = l > 0.0f ? fminf(fmaxf((tc - fa) / l, 0.0f), 1.0f) : 0.0f;
            const float h = 0.5f * s1 * l, mm = fa + h, d2 = fd * fd;
            auto ex = [&](float tt) {
                float r;
                asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(-0.72134752044448170f * fmaf(tt, tt, d2)));
                return r;
            };
            const float sum = (float)GL4W1 * (ex(fmaf(-h, (float)GL4X1, mm)) + ex(fmaf(h, (float)GL4X1, mm))) +
                              (float)GL4W0 * (ex(fmaf(-h, (float)GL4X0, mm)) + ex(fmaf(h, (float)GL4X0, mm)));
            base = 0.5f * s1 * sum;
        }
        {
            // inputs as [x_hi | x_lo | x_hi | 1, 1, 0, 0] against W1 as [hi | hi | lo | b1 hi,
            // b1 lo, 0, 0]; the ones also multiply the bias tiles of layers 2 and 3
            float x[4], xl[4];
            mlp_inputs(fd, fa, fb, fw, x);
#pragma unroll
            for (int k = 0; k < 4; ++k) { const float hi = bf16r(x[k]); xl[k] = x[k] - hi; x[k] = hi; }
            const uint4 c0 = make_uint4(pack_bf16x2(x[0], x[1]), pack_bf16x2(x[2], x[3]),
                                        pack_bf16x2(xl[0], xl[1]), pack_bf16x2(xl[2], xl[3]));
            const uint4 c1 = make_uint4(pack_bf16x2(x[0], x[1]), pack_bf16x2(x[2], x[3]), pack_bf16x2(1.0f, 1.0f), 0u);
            *reinterpret_cast<uint4*>(sA0 + op_off(t, 0, 16)) = c0;
            *reinterpret_cast<uint4*>(sA0 + op_off(t, 8, 16)) = c1;
        }
        fence_async_smem();
        fence_before();
        wg_sync();
        if (*abort_flag) break;
#pragma unroll 1
        for (int layer = 0; layer < 3; ++layer) {
            if (t == 0 && !stall) {
                fence_after();
                if (layer == 0) {
                    umma_bf16(tmem, umma_desc(aA0, 128, 256), umma_desc(aW1, 128, 256), ID, 0u);
                } else {
                    // h (K = 64) against W: four MMAs of K = 16; then the bias: the input
                    // operand's ones against the layer's bias tile
                    const uint32_t aw = layer == 1 ? aW2 : aW3, ab = layer == 1 ? aB2 : aB3;
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk)
                        umma_bf16(tmem, umma_desc(aH + kk * 256, 128, 1024), umma_desc(aw + kk * 256, 128, 1024), ID,
                                  kk > 0 ? 1u : 0u);
                    umma_bf16(tmem, umma_desc(aA0, 128, 256), umma_desc(ab, 128, 256), ID, 1u);
                }
                umma_commit(aBar);
            }
            if (!mbar_wait(aBar, phase, stall ? TC_STALL_POLLS : 1 << 22)) {
                atomicOr(status, IK_ST_MMA_TIMEOUT);
                *abort_flag = 1;
            }
            phase ^= 1u;
            fence_after();
            if (layer < 2) {
                // SiLU -> BF16 operand of the next layer (own row); the accumulators hold
                // h = z/2 with the bias (prescaled weights), SiLU = h + h tanh(h), two
                // columns per packed FP32 instruction
#pragma unroll
                for (int c16 = 0; c16 < 4; ++c16) {
                    float v[16];
                    tmem_ld16(tl + 16 * c16, v);
                    uint32_t ph[8];
#pragma unroll
                    for (int k = 0; k < 16; k += 2) {
                        const mlp_f2 h2 = mlp_pk2(v[k], v[k + 1]);
                        float a0, a1;
                        mlp_up2(mlp_fma2(h2, mlp_pk2(tanh_approx(v[k]), tanh_approx(v[k + 1])), h2), a0, a1);
                        ph[k / 2] = pack_bf16x2(a0, a1);
                    }
#pragma unroll
                    for (int h8 = 0; h8 < 2; ++h8) {
                        const int k0 = 16 * c16 + 8 * h8;
                        *reinterpret_cast<uint4*>(sH + op_off(t, k0, 64)) =
                            make_uint4(ph[4 * h8], ph[4 * h8 + 1], ph[4 * h8 + 2], ph[4 * h8 + 3]);
                    }
                }
                fence_async_smem();
                fence_before();
                wg_sync();
                if (*abort_flag) break;
            } else {
                // output layer on the CUDA cores: y = w4 . silu(z3 + b3) + b4 (w4 in BF16,
                // SiLU in FP32), column pairs in packed FP32
                mlp_f2 y2 = mlp_pk2(0.f, 0.f);
#pragma unroll
                for (int c16 = 0; c16 < 4; ++c16) {
                    float v[16];
                    tmem_ld16(tl + 16 * c16, v);
#pragma unroll
                    for (int k = 0; k < 16; k += 4) {
                        const float4 w4 = *reinterpret_cast<const float4*>(F + 192 + 16 * c16 + k);
                        const mlp_f2 h2 = mlp_pk2(v[k], v[k + 1]), g2 = mlp_pk2(v[k + 2], v[k + 3]);
                        const mlp_f2 s2 = mlp_fma2(h2, mlp_pk2(tanh_approx(v[k]), tanh_approx(v[k + 1])), h2);
                        const mlp_f2 t2 = mlp_fma2(g2, mlp_pk2(tanh_approx(v[k + 2]), tanh_approx(v[k + 3])), g2);
                        y2 = mlp_fma2(s2, mlp_pk2(w4.x, w4.y), y2);
                        y2 = mlp_fma2(t2, mlp_pk2(w4.z, w4.w), y2);
                    }
                }
                float ya, yb;
                mlp_up2(y2, ya, yb);
                const float y = F[256] + (ya + yb);
                fence_before();
                const float Bs = base * fmaf(y, MLP_YINV, 1.0f);
                bool fell_back = false;
                if (MODE == 0) {
                    if (valid) out[row] = raw ? y : Bs;
                } else if (valid) {
                    // the gather's units: B integrates over [-1, 1] (twice the [0, 1] value)
                    const float Bv = use ? 2.0f * Bs : bfix;
                    fell_back = !use;
                    const float fx = bd.w * bd.x, fy = bd.w * bd.y;
                    auto add = [&](int c, float coef) {
                        const long long v = __float2ll_rn(Bv * coef * 4294967296.0f);
                        atomicAdd(R.corr + (size_t)g * R.nc + c, (unsigned long long)v);
                    };
                    add(0, fx * bd.x);
                    add(1, fy * bd.y);
                    if (R.nc == 3) {
                        add(2, fx * bd.y);
                    } else {
                        const float fz = bd.w * bd.z;
                        add(2, fz * bd.z);
                        add(3, fx * bd.y);
                        add(4, fx * bd.z);
                        add(5, fy * bd.z);
                    }
                }
                if (MODE == 1 && R.fallbacks) { // one atomic per warp
                    const unsigned fb = __ballot_sync(0xffffffffu, fell_back);
                    if ((t & 31) == 0 && fb) atomicAdd(R.fallbacks, (unsigned long long)__popc(fb));
                }
            }
        }
        // an abort raised in the last layer is seen after the next tile's barrier
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(TC_COLS)
                     : "memory");
    }
}

// ---------------------------------------------------------------------------- host side
struct MBuf {
    void* p = nullptr;
    size_t bytes = 0;
    MBuf() = default;
    MBuf(const MBuf&) = delete;
    MBuf& operator=(const MBuf&) = delete;
    ~MBuf() { if (p) cudaFree(p); }
    int ensure(size_t need)
    {
        if (need <= bytes && p) return IK_OK;
        if (p) { cudaFree(p); p = nullptr; bytes = 0; }
        size_t b = std::max<size_t>(need, 256);
        if (cudaMalloc(&p, b) != cudaSuccess) { cudaGetLastError(); return IK_ERR_NOMEM; }
        bytes = b;
        return IK_OK;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

struct ik_mlp {
    int device = 0;
    int sm_count = 0;
    cudaStream_t st = nullptr;
    MBuf params, am, av, partial, grad, loss, blob, table, status;
    MBuf feats, targets, labels;  // training set
    MBuf efeats, eout;            // evaluation scratch
    long long nsamples = 0;
    bool initialised = false, deployed = false, validated = false;
    long long steps = 0;
    double last_loss = 0.0;
    MlpGL gl{};
    int stall = 0; // failure-detection test hook (ik_mlp_test_stall)
};

static int mfail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    ik_internal_set_error(buf);
    return code;
}
#define MCK(x)                                                                                         \
    do {                                                                                               \
        cudaError_t e_ = (x);                                                                          \
        if (e_ != cudaSuccess) return mfail(IK_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_));        \
    } while (0)
#define MENS(buf, n)                                                                                   \
    do {                                                                                               \
        if ((buf).ensure(n)) return mfail(IK_ERR_NOMEM, "device allocation of %zu bytes failed", (size_t)(n)); \
    } while (0)

static int mcheck(ik_mlp* m)
{
    if (!m) return mfail(IK_ERR_ARG, "null surrogate handle");
    MCK(cudaSetDevice(m->device));
    return IK_OK;
}

static int deploy(ik_mlp* m)
{
    MENS(m->blob, DB_BYTES);
    k_mlp_deploy<<<(64 * 64 + 255) / 256, 256, 0, m->st>>>(m->params.as<float>(), m->blob.as<unsigned char>());
    MCK(cudaGetLastError());
    m->deployed = true;
    return IK_OK;
}

static int gen_samples(ik_mlp* m, long long n, unsigned long long seed, MBuf& f, MBuf& y, MBuf* lab)
{
    MENS(f, sizeof(float4) * (size_t)std::max<long long>(n, 1));
    MENS(y, sizeof(float) * (size_t)std::max<long long>(n, 1));
    MBuf tmp;
    MBuf& L = lab ? *lab : tmp;
    MENS(L, sizeof(double) * (size_t)std::max<long long>(n, 1));
    if (n > 0) {
        k_mlp_samples<<<(unsigned)((n + 127) / 128), 128, 0, m->st>>>(n, seed, m->gl, f.as<float4>(),
                                                                      L.as<double>(), y.as<float>());
        MCK(cudaGetLastError());
    }
    if (!lab) MCK(cudaStreamSynchronize(m->st));
    return IK_OK;
}

static int run_tc(ik_mlp* m, long long n, const float4* f, float* out, int raw = 0)
{
    if (!m->deployed) if (int r = deploy(m)) return r;
    MENS(m->status, sizeof(int));
    MCK(cudaMemsetAsync(m->status.p, 0, sizeof(int), m->st));
    MCK(cudaFuncSetAttribute(k_mlp_infer_tc<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_LAUNCH));
    const long long tiles = (n + 127) / 128;
    const int blocks = (int)std::min<long long>(std::max<long long>((tiles + TC_WG - 1) / TC_WG, 1),
                                                (long long)m->sm_count * TC_CTAS_PER_SM);
    MlpRecArgs none{};
    k_mlp_infer_tc<0><<<blocks, TC_THREADS, TC_SMEM_LAUNCH, m->st>>>(m->blob.as<unsigned char>(), f, n, out, none,
                                                               m->status.as<int>(), m->stall, raw);
    MCK(cudaGetLastError());
    int st = 0;
    MCK(cudaMemcpyAsync(&st, m->status.p, sizeof(int), cudaMemcpyDeviceToHost, m->st));
    MCK(cudaStreamSynchronize(m->st));
    if (st & IK_ST_MMA_TIMEOUT) return mfail(IK_ERR_TIMEOUT, "tensor-core wait gave up (status %d)", st);
    return IK_OK;
}

// bin of canonical surrogate coordinates (host copy of mlp_record_coords' binning)
static int host_bin(float d, float a, float b, float w)
{
    const int id = (int)(d * 4.0f), ia = (int)std::floor((a + 3.0f) * 4.0f), ib = (int)(b * 4.0f);
    if (id < 0 || id >= 12 || ia < 0 || ia >= 24 || ib < 0 || ib >= 16) return -1;
    return (((w < 1.5f ? 0 : 1) * 12 + id) * 24 + ia) * 16 + ib;
}

// ---- internal entry points used by the IK context (ik_api.cu)
const unsigned char* ik_mlp_internal_blob(ik_mlp* m) { return m && m->deployed ? m->blob.as<unsigned char>() : nullptr; }
const unsigned char* ik_mlp_internal_table(ik_mlp* m) { return m && m->validated ? m->table.as<unsigned char>() : nullptr; }

cudaError_t launch_mlp_records(ik_mlp* m, const float4* rec, const int2* rid, const unsigned long long* count,
                               long long capacity, const float4* bonds, float to_w, float w, int nc,
                               unsigned long long* corr, unsigned long long* fallbacks, int* status, int blocks,
                               cudaStream_t st)
{
    cudaError_t e = cudaFuncSetAttribute(k_mlp_infer_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         TC_SMEM_LAUNCH);
    if (e != cudaSuccess) return e;
    MlpRecArgs R{};
    R.rec = rec;
    R.rid = rid;
    R.count = count;
    R.capacity = capacity;
    R.bonds = bonds;
    R.table = m->table.as<unsigned char>();
    R.to_w = to_w;
    R.w = w;
    R.nc = nc;
    R.corr = corr;
    R.fallbacks = fallbacks;
    k_mlp_infer_tc<1><<<blocks, TC_THREADS, TC_SMEM_LAUNCH, st>>>(m->blob.as<unsigned char>(), nullptr, 0, nullptr, R,
                                                            status, m->stall, 0);
    return cudaGetLastError();
}

void ik_gl_rule(int n, double* x, double* w);

extern "C" {

int ik_mlp_create(ik_mlp** out, int device)
{
    if (!out) return mfail(IK_ERR_ARG, "null output pointer");
    *out = nullptr;
    MCK(cudaSetDevice(device));
    ik_mlp* m = new ik_mlp();
    m->device = device;
    cudaDeviceGetAttribute(&m->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking) != cudaSuccess) {
        delete m;
        return mfail(IK_ERR_CUDA, "stream creation failed");
    }
    ik_gl_rule(10, m->gl.x10, m->gl.w10);
    ik_gl_rule(20, m->gl.x20, m->gl.w20);
    *out = m;
    return IK_OK;
}

int ik_mlp_destroy(ik_mlp* m)
{
    if (!m) return IK_OK;
    cudaSetDevice(m->device);
    if (m->st) { cudaStreamSynchronize(m->st); cudaStreamDestroy(m->st); }
    delete m;
    return IK_OK;
}

int ik_mlp_samples(ik_mlp* m, int64_t n, uint64_t seed, float* feats, double* labels)
{
    if (int r = mcheck(m)) return r;
    if (n < 0 || (n > 0 && (!feats || !labels))) return mfail(IK_ERR_ARG, "bad sample arguments");
    MBuf f, y, L;
    if (int r = gen_samples(m, n, seed, f, y, &L)) return r;
    if (n > 0) {
        MCK(cudaMemcpyAsync(feats, f.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, m->st));
        MCK(cudaMemcpyAsync(labels, L.p, sizeof(double) * n, cudaMemcpyDeviceToHost, m->st));
    }
    MCK(cudaStreamSynchronize(m->st));
    return IK_OK;
}

int ik_mlp_set_params(ik_mlp* m, const float* p, int64_t n)
{
    if (int r = mcheck(m)) return r;
    if (!p || n != NPAR) return mfail(IK_ERR_ARG, "expected %d parameters", NPAR);
    MENS(m->params, sizeof(float) * NPAR);
    MENS(m->am, sizeof(float) * NPAR);
    MENS(m->av, sizeof(float) * NPAR);
    MCK(cudaMemcpyAsync(m->params.p, p, sizeof(float) * NPAR, cudaMemcpyHostToDevice, m->st));
    MCK(cudaMemsetAsync(m->am.p, 0, sizeof(float) * NPAR, m->st));
    MCK(cudaMemsetAsync(m->av.p, 0, sizeof(float) * NPAR, m->st));
    m->initialised = true;
    m->validated = false;
    m->steps = 0;
    if (int r = deploy(m)) return r;
    MCK(cudaStreamSynchronize(m->st));
    return IK_OK;
}

int ik_mlp_get_params(ik_mlp* m, float* p, int64_t n)
{
    if (int r = mcheck(m)) return r;
    if (!p || n != NPAR) return mfail(IK_ERR_ARG, "expected %d parameters", NPAR);
    if (!m->initialised) return mfail(IK_ERR_STATE, "surrogate has no parameters yet");
    MCK(cudaMemcpyAsync(p, m->params.p, sizeof(float) * NPAR, cudaMemcpyDeviceToHost, m->st));
    MCK(cudaStreamSynchronize(m->st));
    return IK_OK;
}

int ik_mlp_num_params(void) { return NPAR; }

int ik_mlp_init(ik_mlp* m, uint64_t seed)
{
    if (int r = mcheck(m)) return r;
    // Kaiming-uniform weights (fan-in), zero biases; host-side SplitMix64
    std::vector<float> p(NPAR, 0.0f);
    unsigned long long s = seed;
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        unsigned long long z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](int off, int count, int fan_in) {
        const double lim = std::sqrt(6.0 / fan_in);
        for (int k = 0; k < count; ++k) p[off + k] = (float)((2.0 * next() - 1.0) * lim);
    };
    fill(O_W1, H * NIN, NIN);
    fill(O_W2, H * H, H);
    fill(O_W3, H * H, H);
    fill(O_W4, H, H);
    return ik_mlp_set_params(m, p.data(), NPAR);
}

int ik_mlp_grad(ik_mlp* m, int64_t n, const float* feats, const float* targets, float* grad, double* loss)
{
    if (int r = mcheck(m)) return r;
    if (!m->initialised) return mfail(IK_ERR_STATE, "surrogate has no parameters (ik_mlp_init)");
    if (n < 1 || n > (1 << 20) || (n & (n - 1)) || !feats || !targets || !grad)
        return mfail(IK_ERR_ARG, "gradient batch must be a power of two in [1, 2^20]");
    MBuf f, y, part, g, l;
    MENS(f, sizeof(float4) * n);
    MENS(y, sizeof(float) * n);
    const int ctas = (int)((n + 127) / 128);
    MENS(part, sizeof(float) * NPART * ctas);
    MENS(g, sizeof(float) * NPAR);
    MENS(l, sizeof(float));
    MCK(cudaMemcpyAsync(f.p, feats, sizeof(float4) * n, cudaMemcpyHostToDevice, m->st));
    MCK(cudaMemcpyAsync(y.p, targets, sizeof(float) * n, cudaMemcpyHostToDevice, m->st));
    TrainArgs A{};
    A.params = m->params.as<float>();
    A.feats = f.as<float4>();
    A.targets = y.as<float>();
    A.nsamples = n;
    A.pos0 = 0;
    A.perm_a = 1;
    A.perm_b = 0;
    A.tiles_per_cta = 1;
    A.valid = n;
    A.inv_batch = 1.0f / (float)n;
    A.partial = part.as<float>();
    MCK(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TRAIN_SMEM));
    k_mlp_train<<<ctas, 128, TRAIN_SMEM, m->st>>>(A);
    MCK(cudaGetLastError());
    k_mlp_adam<<<(NPAR + 1 + 255) / 256, 256, 0, m->st>>>(nullptr, nullptr, nullptr, part.as<float>(), ctas,
                                                          g.as<float>(), l.as<float>(), 0.f, 0.f, 0.f, 0.f, 1.f, 1.f);
    MCK(cudaGetLastError());
    float lh = 0.f;
    MCK(cudaMemcpyAsync(grad, g.p, sizeof(float) * NPAR, cudaMemcpyDeviceToHost, m->st));
    MCK(cudaMemcpyAsync(&lh, l.p, sizeof(float), cudaMemcpyDeviceToHost, m->st));
    MCK(cudaStreamSynchronize(m->st));
    if (loss) *loss = lh / (double)n;
    return IK_OK;
}

int ik_mlp_train(ik_mlp* m, int64_t nsamples, int epochs, int ctas, double lr, uint64_t seed, double* loss_hist,
                 int64_t hist_len)
{
    if (int r = mcheck(m)) return r;
    if (nsamples < 1024 || (nsamples & (nsamples - 1)) || nsamples > (1ll << 26))
        return mfail(IK_ERR_ARG, "nsamples must be a power of two in [2^10, 2^26]");
    if (epochs < 1 || ctas < 1 || ctas > 4096 || !(lr > 0.0)) return mfail(IK_ERR_ARG, "bad training arguments");
    if (!m->initialised) if (int r = ik_mlp_init(m, seed ^ 0x5DEECE66Dull)) return r;
    if (m->nsamples != nsamples) {
        if (int r = gen_samples(m, nsamples, seed, m->feats, m->targets, &m->labels)) return r;
        m->nsamples = nsamples;
    }
    const long long batch = (long long)ctas * 128;
    const long long steps_per_epoch = (nsamples + batch - 1) / batch;
    const long long total = steps_per_epoch * epochs;
    MENS(m->partial, sizeof(float) * NPART * ctas);
    MENS(m->loss, sizeof(float) * std::max<long long>(total, 1));
    MCK(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TRAIN_SMEM));
    const float b1 = 0.9f, b2 = 0.999f;
    unsigned long long ps = seed * 0x2545F4914F6CDD1Dull + 1;
    for (int e = 0; e < epochs; ++e) {
        ps = ps * 6364136223846793005ull + 1442695040888963407ull;
        const unsigned long long pa = (ps >> 16) | 1ull, pb = ps >> 7;
        for (long long s = 0; s < steps_per_epoch; ++s) {
            const long long step = (long long)e * steps_per_epoch + s;
            TrainArgs A{};
            A.params = m->params.as<float>();
            A.feats = m->feats.as<float4>();
            A.targets = m->targets.as<float>();
            A.nsamples = nsamples;
            A.pos0 = s * batch;
            A.perm_a = pa;
            A.perm_b = pb;
            A.tiles_per_cta = 1;
            A.valid = batch;
            A.inv_batch = 1.0f / (float)batch;
            A.partial = m->partial.as<float>();
            k_mlp_train<<<ctas, 128, TRAIN_SMEM, m->st>>>(A);
            MCK(cudaGetLastError());
            // cosine decay to lr / 100
            const double frac = (double)step / (double)std::max<long long>(total - 1, 1);
            const double lrs = lr * (0.01 + 0.99 * 0.5 * (1.0 + std::cos(3.14159265358979323846 * frac)));
            const long long tstep = m->steps + 1;
            const float bc1 = (float)(1.0 - std::pow((double)b1, (double)tstep));
            const float bc2 = (float)(1.0 - std::pow((double)b2, (double)tstep));
            k_mlp_adam<<<(NPAR + 1 + 255) / 256, 256, 0, m->st>>>(m->params.as<float>(), m->am.as<float>(),
                                                                  m->av.as<float>(), m->partial.as<float>(), ctas,
                                                                  nullptr, m->loss.as<float>() + step, (float)lrs, b1,
                                                                  b2, 1e-8f, bc1, bc2);
            MCK(cudaGetLastError());
            ++m->steps;
        }
    }
    std::vector<float> lh((size_t)total);
    MCK(cudaMemcpyAsync(lh.data(), m->loss.p, sizeof(float) * total, cudaMemcpyDeviceToHost, m->st));
    MCK(cudaStreamSynchronize(m->st));
    if (loss_hist)
        for (int64_t k = 0; k < hist_len && k < total; ++k) loss_hist[k] = lh[(size_t)k] / (double)batch;
    m->last_loss = lh.empty() ? 0.0 : lh.back() / (double)batch;
    m->validated = false;
    return deploy(m);
}

int ik_mlp_test_stall(ik_mlp* m, int on)
{
    if (int r = mcheck(m)) return r;
    m->stall = on ? 1 : 0;
    return IK_OK;
}

int ik_mlp_eval(ik_mlp* m, int64_t n, const float* feats, float* out, int kernel)
{
    if (int r = mcheck(m)) return r;
    if (!m->initialised) return mfail(IK_ERR_STATE, "surrogate has no parameters");
    const int raw = (kernel & IK_MLP_EVAL_RAW) ? 1 : 0;
    kernel &= ~IK_MLP_EVAL_RAW;
    if (n < 0 || (n > 0 && (!feats || !out)) || kernel < 0 || kernel > 2)
        return mfail(IK_ERR_ARG, "bad evaluation arguments");
    if (n == 0) return IK_OK;
    MENS(m->efeats, sizeof(float4) * n);
    MENS(m->eout, sizeof(float) * n);
    MCK(cudaMemcpyAsync(m->efeats.p, feats, sizeof(float4) * n, cudaMemcpyHostToDevice, m->st));
    if (kernel == 0) {
        if (int r = run_tc(m, n, m->efeats.as<float4>(), m->eout.as<float>(), raw)) return r;
    } else {
        k_mlp_infer_simt<<<(unsigned)((n + 127) / 128), 128, 0, m->st>>>(m->params.as<float>(), m->efeats.as<float4>(),
                                                                         n, kernel == 1 ? 1 : 0, raw,
                                                                         m->eout.as<float>());
        MCK(cudaGetLastError());
    }
    MCK(cudaMemcpyAsync(out, m->eout.p, sizeof(float) * n, cudaMemcpyDeviceToHost, m->st));
    MCK(cudaStreamSynchronize(m->st));
    return IK_OK;
}

int ik_mlp_validate(ik_mlp* m, int64_t n, uint64_t seed, double tol, double* coverage, double* max_err,
                    double* rms_err, double* bin_err, int64_t nbins)
{
    if (int r = mcheck(m)) return r;
    if (!m->initialised) return mfail(IK_ERR_STATE, "surrogate has no parameters");
    if (n < 1 || n > (1ll << 26) || !(tol >= 0.0)) return mfail(IK_ERR_ARG, "bad validation arguments");
    MBuf f, y, L, o;
    if (int r = gen_samples(m, n, seed, f, y, &L)) return r;
    MENS(o, sizeof(float) * n);
    if (int r = run_tc(m, n, f.as<float4>(), o.as<float>())) return r;
    std::vector<float4> hf((size_t)n);
    std::vector<double> hl((size_t)n);
    std::vector<float> ho((size_t)n);
    MCK(cudaMemcpyAsync(hf.data(), f.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, m->st));
    MCK(cudaMemcpyAsync(hl.data(), L.p, sizeof(double) * n, cudaMemcpyDeviceToHost, m->st));
    MCK(cudaMemcpyAsync(ho.data(), o.p, sizeof(float) * n, cudaMemcpyDeviceToHost, m->st));
    MCK(cudaStreamSynchronize(m->st));
    constexpr int NB = 2 * 12 * 24 * 16;
    std::vector<double> be(NB, 0.0);
    std::vector<long long> bc(NB, 0);
    double mx = 0.0, ss = 0.0;
    for (long long i = 0; i < n; ++i) {
        const double e = std::fabs((double)ho[(size_t)i] - hl[(size_t)i]);
        mx = std::max(mx, e);
        ss += e * e;
        const int b = host_bin(hf[(size_t)i].x, hf[(size_t)i].y, hf[(size_t)i].z, hf[(size_t)i].w);
        if (b >= 0) { be[(size_t)b] = std::max(be[(size_t)b], e); ++bc[(size_t)b]; }
    }
    std::vector<unsigned char> tab(NB, 0);
    long long covered_samples = 0;
    for (int b = 0; b < NB; ++b)
        if (bc[(size_t)b] >= 8 && be[(size_t)b] <= tol) { tab[(size_t)b] = 1; covered_samples += bc[(size_t)b]; }
    MENS(m->table, NB);
    MCK(cudaMemcpyAsync(m->table.p, tab.data(), NB, cudaMemcpyHostToDevice, m->st));
    MCK(cudaStreamSynchronize(m->st));
    m->validated = true;
    if (coverage) *coverage = (double)covered_samples / (double)n;
    if (max_err) *max_err = mx;
    if (rms_err) *rms_err = std::sqrt(ss / (double)n);
    if (bin_err)
        for (int64_t k = 0; k < nbins && k < NB; ++k) bin_err[k] = bc[(size_t)k] ? be[(size_t)k] : -1.0;
    return IK_OK;
}

} // extern "C"
