// ik_api.cu -- C ABI of the GB300 Irving-Kirkwood engine (declared in include/ik_gb300.h):
// context, device buffers, geometry/bin set-up and the per-frame launch sequence.
#include "ik_kernels.h"
#include "../../include/ik_gb300.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <atomic>
#include <vector>

#include <nvtx3/nvToolsExt.h>

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(e_ == cudaErrorMemoryAllocation ? IK_ERR_NOMEM : IK_ERR_CUDA,     \
                        "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                        \
    } while (0)

// bumped by every device allocation: a captured graph holds buffer addresses
static std::atomic<int64_t> g_alloc_epoch{0};

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept
    {
        if (this != &o) { if (p) cudaFree(p); p = o.p; bytes = o.bytes; o.p = nullptr; o.bytes = 0; }
        return *this;
    }
    ~DevBuf() { if (p) cudaFree(p); }
    int ensure(size_t need)
    {
        if (need <= bytes && p) return IK_OK;
        if (p) { cudaFree(p); p = nullptr; bytes = 0; }
        size_t b = std::max<size_t>(need, 256);
        ++g_alloc_epoch;
        cudaError_t e = cudaMalloc(&p, b);
        if (e != cudaSuccess) {
            p = nullptr;
            return fail(IK_ERR_NOMEM, "cudaMalloc(%zu) failed: %s", b, cudaGetErrorString(e));
        }
        bytes = b;
        return IK_OK;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

#define ENS(buf, n) do { int r_ = (buf).ensure(n); if (r_) return r_; } while (0)

// NVTX ranges around the host-side phases (upload, cell list, bonds, gather, finish,
// download): a profiler's timeline shows which phase enqueued which launches.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};
// Consecutive phases of one function: next() closes the open range and opens another.
struct NvtxPhases {
    bool open = false;
    void next(const char* name)
    {
        if (open) nvtxRangePop();
        nvtxRangePushA(name);
        open = true;
    }
    ~NvtxPhases() { if (open) nvtxRangePop(); }
};

// Box, grid and the binning derived from them.  The context holds one; a slot with a
// geometry of its own (frames of different boxes in one batch) holds another, swapped
// in while that slot is processed.
struct Geo {
    double boxsize[3] = {0, 0, 0}, origin[3] = {0, 0, 0};
    bool box_set = false;
    std::vector<double> grid_h;
    int64_t G = 0;
    DevBuf grid_d;
    IkGeom geom{};
    bool geom_valid = false;
    int bw[3] = {1, 1, 1}, reach[3] = {0, 0, 0};
    int nitems = 0;
    DevBuf gpts_d, items_d;
    std::vector<float4> gpts_h; // host copies (the fused batch concatenates them)
    std::vector<int4> items_h;
};

struct Slot {
    int64_t n = 0;
    bool has_geo = false; // own box + grid (ik_set_slot_geometry)
    Geo geo;
    bool has_vel = false, has_mass = false;
    double dmax = 0.0;
    DevBuf pos, vel, mass, diam;
    DevBuf disp; // displacements for the elastic virial field (ik_upload_displacement)
    DevBuf stage32; // FP32 upload staging (ik_upload_frame_f32)
    bool has_disp = false;
    DevBuf vir, kin, ela;
    int last_prec = -1, last_fields = 0;
    DevBuf counters; // 5 x u64: bonds, pairs, triples, surrogate records, surrogate fallbacks
    cudaEvent_t done = nullptr; // completion of the slot's last computation (on its lane)
    bool done_recorded = false;
    cudaEvent_t d2h_done = nullptr; // completion of the slot's last field download
    bool d2h_recorded = false;
    Slot() = default;
    Slot(Slot&&) = default;
    Slot& operator=(Slot&&) = default;
};

// A lane: one stream and one set of per-frame work buffers.  Frames computed on
// different lanes overlap on the GPU.
struct Lane {
    cudaStream_t st = nullptr;
    cudaEvent_t last = nullptr;
    DevBuf cell_of, rank, cell_count, cell_start, sorted, prec, kin, diam32;
    DevBuf bonds32, nb32, bonds64, nb64, pos64, bonds_tmp, boff, bsum, bsum_cells, relhi, rello, plo;
    DevBuf work_counter;
    DevBuf vir2, kin2; // double-float outputs of the FP32 gather
    DevBuf mlp_rec, mlp_rid, mlp_count, corr; // surrogate records and fixed-point corrections
    DevBuf eb64, ec64, eb32, ec32, enb, ecnt;  // elastic-field bond records, scratch counters
};
constexpr int IK_LANES = 8;

// A fused batch: the frames of ik_compute_batch concatenated (particles, cells, grid
// points, work items in batch order) so that every stage runs once over the batch.
// Built on the host when the batch, a slot's size or geometry, or a setting changes.
struct FusedBatch {
    IkBatchLaunch b{};
    int nitems = 0;
    long long gtot = 0;
    DevBuf slots, p_offs, c_offs, v_offs, items, item_slot, gpts, grid;
    DevBuf cell_of, rank, cell_count, cell_start, sorted, bsum, relhi, rello, prec, plo, pos64, kin, diam32, tmp, nb;
    DevBuf vir2, kin2, work;
    // host-mapped copies of a fused ik_compute_batch_io (IK_TUNE_IO_MAPPED): the frames'
    // uploads and the fields' downloads, one launch_io_copy each
    DevBuf io_up, io_dn;
    int n_up = 0, n_dn = 0;
    long long w_up = 0, w_dn = 0;
};

// A computation not yet confirmed by ik_synchronize (re-run after a capacity growth),
// with the host outputs its fields are being downloaded into (re-issued after a re-run).
struct PendingOp {
    int slot, prec, fields;
    double* out[3] = {nullptr, nullptr, nullptr}; // virial, kinetic, elastic
};

// Host buffers of one frame of ik_compute_batch_io.
struct IoFrame {
    const double *pos = nullptr, *vel = nullptr, *mass = nullptr, *diam = nullptr;
    double* out[3] = {nullptr, nullptr, nullptr};
};

} // namespace

struct ik_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int sm_count = 0;
    int flags = 0;
    // configuration
    int dim = 0;
    Geo geo; // box, grid, binning (swapped with a slot's own while it is processed)
    IkPot pot{};
    double scaled_rcut = 0.0;
    bool pot_set = false;
    IkCG cg{};
    bool cg_set = false;
    IkGL gl{};
    double cg_width_param = 0.0;
    double max_rcut = 0.0;
    bool max_rcut_set = false;
    // per-frame work buffers live in the lanes
    Lane lanes[IK_LANES];
    int next_lane = 0;
    cudaEvent_t fork = nullptr;
    cudaStream_t d2h = nullptr; // field downloads (ik_download_field_async): full-duplex with uploads
    cudaEvent_t d2h_last = nullptr;
    DevBuf status, maxnb;
    DevBuf bsum_q; // scan scratch of the neighbour queries (main stream)
    int maxb = 0, halo_cap = 0;
    int maxbe = 0;      // elastic-field records per particle (neighbours within max_rcut)
    DevBuf maxnbe;
    // neighbour-query scratch
    DevBuf q_cell_of, q_rank, q_count, q_start, q_sorted, q_cnt, q_offs, q_idx, q_flag;
    DevBuf th_partial, th_out; // global thermodynamic observables (ik_compute_thermo)
    std::vector<Slot> slots;
    std::vector<PendingOp> pending;
    ik_mlp* mlp = nullptr; // learned bond-integral surrogate (IK_QUAD_MLP)
    // tuning of the FP32 gather (0 = default)
    int tune_bin_points = 0, tune_blocks_per_sm = 0;
    int tune_fused = 1;     // ik_compute_batch: fused batches where eligible (IK_TUNE_FUSED_BATCH)
    FusedBatch fused;
    bool batch_fused = false; // the recorded batch graph is a fused batch
    bool in_batch = false; // enqueueing a batch: frames share the GPU (default 1 gather CTA per SM)
    long long mlp_cap = 0;  // record capacity per lane
    // CUDA-graph replay of ik_compute_batch
    bool capturing = false;
    int captured_lanes = 0;
    cudaGraphExec_t batch_exec = nullptr;
    std::vector<int> batch_slots;
    int batch_prec = -1, batch_fields = 0, batch_maxb = 0, batch_halo = 0, batch_maxbe = 0;
    int64_t batch_geom_version = -1, batch_slot_version = -1;
    int64_t geom_version = 0, slot_version = 0, config_version = 0;
    int64_t batch_config_version = -1, batch_alloc_epoch = -1;
    int64_t batch_launches = 0;
    // CUDA-graph replay of ik_compute_batch_io (copies from and to host inside the graph)
    cudaGraphExec_t io_exec = nullptr;
    std::vector<int64_t> io_key;
    int64_t io_launches = 0;
    const IoFrame* io_cur = nullptr; // frame whose copies enqueue() adds to its lane
    // a fused ik_compute_batch_io: sub-batches of frames, each a fused batch, whose copies
    // overlap the other sub-batches' computation (IK_TUNE_IO_BATCHES: their number)
    std::vector<FusedBatch> fused_io;
    std::vector<cudaEvent_t> io_ev; // per sub-batch: uploads done, computation done
    int tune_io_batches = 0, tune_io_mapped = 0;
    bool io_fused = false, io_mapped = false;
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    int64_t launches = 0;
    float timing[4] = {0, 0, 0, 0};
};

// ---------------------------------------------------------------------------
namespace {

void gl_rule(int n, double* x, double* w)
{
    // Newton iteration on the Legendre three-term recurrence.
    for (int k = 0; k < n; ++k) {
        long double z = cosl(3.14159265358979323846264338327950288L * (k + 0.75L) / (n + 0.5L));
        long double pp = 1.0L;
        for (int it = 0; it < 100; ++it) {
            long double p0 = 1.0L, p1 = z;
            for (int j = 2; j <= n; ++j) {
                long double p2 = ((2.0L * j - 1.0L) * z * p1 - (j - 1.0L) * p0) / j;
                p0 = p1; p1 = p2;
            }
            if (n == 1) { p1 = z; p0 = 1.0L; }
            pp = n * (z * p1 - p0) / (z * z - 1.0L);
            long double dz = p1 / pp;
            z -= dz;
            if (fabsl(dz) < 1e-19L) break;
        }
        long double p0 = 1.0L, p1 = z;
        for (int j = 2; j <= n; ++j) {
            long double p2 = ((2.0L * j - 1.0L) * z * p1 - (j - 1.0L) * p0) / j;
            p0 = p1; p1 = p2;
        }
        if (n == 1) { p1 = z; p0 = 1.0L; }
        pp = n * (z * p1 - p0) / (z * z - 1.0L);
        x[n - 1 - k] = (double)z;
        w[n - 1 - k] = (double)(2.0L / ((1.0L - z * z) * pp * pp));
    }
    if (n % 2 == 1) x[n / 2] = 0.0;
}

// Gauss-Kronrod 7/15 rule (the rule of gsl_integration_qag key 1).  The Kronrod nodes
// are the zeros of the Stieltjes polynomial E_8(x) = x^8 + a6 x^6 + a4 x^4 + a2 x^2 + a0,
// fixed by orthogonality to x^k (k = 1, 3, 5, 7; the even k vanish by parity) under the
// weight P_7 on [-1, 1] (Kronrod 1965); they interlace with the Gauss nodes, which locates
// each for bisection.  The 15 weights make the rule exact on x^(2m), m = 0..7 (degree 22
// with the odd powers).  Long double throughout; computed once.
static IkGK make_gk15()
{
    typedef long double LD;
    // P_7(x) = (429 x^7 - 693 x^5 + 315 x^3 - 35 x) / 16: moments M(q) = int P_7 x^q, q odd
    const LD p7[4] = {-35.0L / 16, 315.0L / 16, -693.0L / 16, 429.0L / 16}; // x^1, x^3, x^5, x^7
    auto mom = [&](int q) {
        LD m = 0;
        for (int t = 0; t < 4; ++t) m += p7[t] * 2.0L / (LD)(q + 2 * t + 1 + 1);
        return m;
    };
    // sum_e c_e M(k + e) = -M(k + 8) over e = 0, 2, 4, 6 (coefficients a0, a2, a4, a6), k odd
    LD A[4][5];
    for (int r = 0; r < 4; ++r) {
        const int k = 2 * r + 1;
        for (int e = 0; e < 4; ++e) A[r][e] = mom(k + 2 * e);
        A[r][4] = -mom(k + 8);
    }
    for (int col = 0; col < 4; ++col) {
        int piv = col;
        for (int r = col + 1; r < 4; ++r)
            if (fabsl(A[r][col]) > fabsl(A[piv][col])) piv = r;
        for (int t = 0; t < 5; ++t) std::swap(A[col][t], A[piv][t]);
        for (int r = 0; r < 4; ++r) {
            if (r == col) continue;
            const LD f = A[r][col] / A[col][col];
            for (int t = col; t < 5; ++t) A[r][t] -= f * A[col][t];
        }
    }
    LD a[4];
    for (int e = 0; e < 4; ++e) a[e] = A[e][4] / A[e][e];
    auto E8 = [&](LD x) {
        const LD y = x * x;
        return (((y + a[3]) * y + a[2]) * y + a[1]) * y + a[0];
    };
    double gx[7], gw[7];
    gl_rule(7, gx, gw);
    const LD edges[5] = {0.0L, (LD)gx[4], (LD)gx[5], (LD)gx[6], 1.0L};
    LD nodes[8];
    nodes[0] = 0.0L;
    for (int r = 0; r < 4; ++r) {
        LD lo = edges[r], hi = edges[r + 1];
        const bool neg_lo = E8(lo) < 0;
        for (int it = 0; it < 128; ++it) {
            const LD mid = 0.5L * (lo + hi);
            if ((E8(mid) < 0) == neg_lo) lo = mid;
            else hi = mid;
        }
        nodes[2 * r + 1] = 0.5L * (lo + hi);
        if (r < 3) nodes[2 * r + 2] = (LD)gx[4 + r];
    }
    // weights: w0 [m == 0] + 2 sum_i w_i x_i^(2m) = 2 / (2m + 1), m = 0..7
    LD W[8][9];
    for (int m = 0; m < 8; ++m) {
        for (int t = 0; t < 8; ++t) W[m][t] = t == 0 ? (m == 0 ? 1.0L : 0.0L) : 2.0L * powl(nodes[t], 2 * m);
        W[m][8] = 2.0L / (2 * m + 1);
    }
    for (int col = 0; col < 8; ++col) {
        int piv = col;
        for (int r = col + 1; r < 8; ++r)
            if (fabsl(W[r][col]) > fabsl(W[piv][col])) piv = r;
        for (int t = 0; t < 9; ++t) std::swap(W[col][t], W[piv][t]);
        for (int r = 0; r < 8; ++r) {
            if (r == col) continue;
            const LD f = W[r][col] / W[col][col];
            for (int t = col; t < 9; ++t) W[r][t] -= f * W[col][t];
        }
    }
    IkGK g;
    for (int t = 0; t < 8; ++t) {
        g.x[t] = (double)nodes[t];
        g.wk[t] = (double)(W[t][8] / W[t][t]);
    }
    for (int t = 0; t < 4; ++t) g.wg[t] = gw[3 + t];
    return g;
}
static const IkGK& gk15()
{
    static const IkGK g = make_gk15();
    return g;
}

int check_ctx(ik_ctx* c)
{
    if (!c) return fail(IK_ERR_ARG, "null context");
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return fail(IK_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    return IK_OK;
}

int nc_of(int dim, int c) { return c < dim ? 1 : 0; }

// (Re)build the cell geometry and the grid binning for the current box, cut-offs and grid.
int ensure_geometry(ik_ctx* c)
{
    if (c->geo.geom_valid) return IK_OK;
    IkGeom g{};
    g.dim = c->dim;
    const double R = c->cg.rcut;
    for (int a = 0; a < 3; ++a) {
        g.L[a] = c->geo.boxsize[a];
        g.lo[a] = -0.5 * c->geo.boxsize[a] - c->geo.origin[a];
        g.periodic[a] = nc_of(c->dim, a);
        int nc = 1;
        if (g.periodic[a]) {
            if (!(2.0 * c->max_rcut < g.L[a]) || !(2.0 * R < g.L[a]))
                return fail(IK_ERR_BOX,
                            "cut-off too large for the periodic box: max_rcut=%g, R_cg=%g, L[%d]=%g "
                            "(need 2*cutoff < L)", c->max_rcut, R, a, g.L[a]);
            nc = (int)std::floor(g.L[a] / c->max_rcut);
            if (nc < 1) nc = 1;
            if (nc > (1 << 20)) nc = 1 << 20;
        }
        g.nc[a] = nc;
        g.cw[a] = g.L[a] / nc;
        g.invL[a] = 1.0 / g.L[a];
        g.reach_bond[a] = 1;
        g.all_bond[a] = (nc < 3) ? 1 : 0;
    }
    if (c->dim == 2) { g.lo[2] = -0.5 * c->geo.boxsize[2] - c->geo.origin[2]; g.cw[2] = g.L[2]; }
    for (int a = 0; a < 3; ++a) {
        g.cwhi[a] = (float)g.cw[a];
        g.cwlo[a] = (float)(g.cw[a] - (double)g.cwhi[a]);
    }
    long long ncell = (long long)g.nc[0] * g.nc[1] * g.nc[2];
    if (ncell > (1LL << 30)) return fail(IK_ERR_UNSUPPORTED, "too many cells (%lld)", ncell);
    g.ncell = (int)ncell;

    // halo reach and bin width for the FP32 gather
    double cellvol = 1.0, boxvol = 1.0;
    for (int a = 0; a < c->dim; ++a) { cellvol *= g.cw[a]; boxvol *= g.L[a]; }
    double pts_per_cell = c->geo.G > 0 ? (double)c->geo.G * cellvol / boxvol : 1.0;
    double target = c->tune_bin_points > 0 ? (double)c->tune_bin_points : (c->dim == 2 ? 20.0 : 24.0);
    int bwv = (int)std::lround(std::pow(std::max(target / std::max(pts_per_cell, 1e-9), 1.0), 1.0 / c->dim));
    bwv = std::max(1, std::min(bwv, 8));
    for (int a = 0; a < 3; ++a) {
        if (a < c->dim) {
            c->geo.reach[a] = (int)std::ceil(R / g.cw[a]);
            if (c->geo.reach[a] < 1) c->geo.reach[a] = 1;
            c->geo.bw[a] = std::min(bwv, g.nc[a]);
        } else {
            c->geo.reach[a] = 0;
            c->geo.bw[a] = 1;
        }
    }
    c->geo.geom = g;

    // ---- bin the grid points (host, once per box/grid)
    const int D = c->dim;
    int nb[3] = {1, 1, 1};
    for (int a = 0; a < D; ++a) nb[a] = (g.nc[a] + c->geo.bw[a] - 1) / c->geo.bw[a];
    const double spacing = std::pow(boxvol / std::max<int64_t>(c->geo.G, 1), 1.0 / D);
    struct Key { int64_t bin; uint64_t morton; int64_t idx; double w[3]; int cell0[3]; };
    std::vector<Key> keys((size_t)c->geo.G);
    for (int64_t i = 0; i < c->geo.G; ++i) {
        Key k{};
        k.idx = i;
        int bcoord[3] = {0, 0, 0};
        uint32_t qv[3] = {0, 0, 0};
        for (int a = 0; a < 3; ++a) {
            double x = c->geo.grid_h[3 * i + a];
            if (a < D) {
                double t = (x - g.lo[a]) / g.L[a];
                t -= std::floor(t);
                double xw = g.lo[a] + t * g.L[a];
                int cell = (int)(t * g.nc[a]);
                cell = std::max(0, std::min(cell, g.nc[a] - 1));
                bcoord[a] = cell / c->geo.bw[a];
                k.cell0[a] = bcoord[a] * c->geo.bw[a];
                k.w[a] = xw - (g.lo[a] + k.cell0[a] * g.cw[a]);
                double qq = std::floor(k.w[a] / spacing);
                qv[a] = (uint32_t)std::max(0.0, std::min(qq, 1023.0));
            } else {
                k.cell0[a] = 0;
                k.w[a] = x; // non-periodic axis: absolute (2D z is 0)
            }
        }
        // bins in Morton order: consecutive work items are spatial neighbours, so the
        // warps of a CTA (which take consecutive items) share halo particles and bond
        // records in L1
        int64_t bm = 0;
        for (int b = 0; b < 21; ++b)
            for (int a = 0; a < D; ++a) bm |= (int64_t)((bcoord[a] >> b) & 1) << (b * D + a);
        k.bin = bm;
        uint64_t m = 0;
        for (int b = 0; b < 10; ++b)
            for (int a = 0; a < D; ++a) m |= (uint64_t)((qv[a] >> b) & 1u) << (b * D + a);
        k.morton = m;
        keys[(size_t)i] = k;
    }
    std::sort(keys.begin(), keys.end(), [](const Key& x, const Key& y) {
        if (x.bin != y.bin) return x.bin < y.bin;
        if (x.morton != y.morton) return x.morton < y.morton;
        return x.idx < y.idx;
    });
    const float kappa = c->cg.kappa;
    std::vector<float4> gpts((size_t)std::max<int64_t>(c->geo.G, 1));
    for (int64_t k = 0; k < c->geo.G; ++k) {
        const Key& kk = keys[(size_t)k];
        float4 v;
        v.x = (float)(kappa * kk.w[0]);
        v.y = (float)(kappa * kk.w[1]);
        v.z = D == 3 ? (float)(kappa * kk.w[2]) : 0.f;
        int gi = (int)kk.idx;
        std::memcpy(&v.w, &gi, 4);
        gpts[(size_t)k] = v;
    }
    // work items: ranges of groups inside a bin, sized for >= ~4 items per warp slot
    int64_t nbins_used = 0;
    for (int64_t k = 0; k < c->geo.G; ++k) if (k == 0 || keys[(size_t)k].bin != keys[(size_t)k - 1].bin) ++nbins_used;
    int64_t total_groups = 0;
    {
        int64_t s = 0;
        for (int64_t k = 1; k <= c->geo.G; ++k)
            if (k == c->geo.G || keys[(size_t)k].bin != keys[(size_t)k - 1].bin) { total_groups += (k - s + IK_P - 1) / IK_P; s = k; }
    }
    int64_t warps = (int64_t)c->sm_count * 16;
    int64_t want_items = std::max<int64_t>(4 * warps, nbins_used);
    int gi_max = (int)std::max<int64_t>(1, (total_groups + want_items - 1) / want_items);
    std::vector<int4> items;
    {
        int64_t s = 0;
        for (int64_t k = 1; k <= c->geo.G; ++k) {
            if (k == c->geo.G || keys[(size_t)k].bin != keys[(size_t)k - 1].bin) {
                const Key& kk = keys[(size_t)s];
                for (int64_t t = s; t < k; t += (int64_t)gi_max * IK_P)
                    items.push_back(make_int4(kk.cell0[0], kk.cell0[1], kk.cell0[2], (int)t));
                s = k;
            }
        }
        items.push_back(make_int4(0, 0, 0, (int)c->geo.G));
    }
    c->geo.nitems = (int)items.size() - 1;
    c->geo.gpts_h = gpts;
    c->geo.items_h = items;
    ENS(c->geo.gpts_d, gpts.size() * sizeof(float4));
    ENS(c->geo.items_d, items.size() * sizeof(int4));
    CK(cudaMemcpy(c->geo.gpts_d.p, gpts.data(), gpts.size() * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->geo.items_d.p, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice));
    c->geo.geom_valid = true;
    ++c->geom_version;
    return IK_OK;
}

int ensure_ready(ik_ctx* c)
{
    if (!c->geo.box_set) return fail(IK_ERR_STATE, "box not set (ik_set_box)");
    if (!c->pot_set) return fail(IK_ERR_STATE, "pair potential not set");
    if (!c->cg_set) return fail(IK_ERR_STATE, "coarse-graining function not set");
    if (c->geo.G <= 0) return fail(IK_ERR_STATE, "grid not set (ik_set_grid)");
    if (!c->max_rcut_set) return fail(IK_ERR_STATE, "max_rcut unknown: upload a frame or call ik_set_max_rcut");
    return IK_OK;
}

// Cell list for a slot into (cell_of, rank, count, start, sorted) buffers.
int build_cells(ik_ctx* c, Slot& s, const IkGeom& g, cudaStream_t st, DevBuf& cell_of, DevBuf& rank,
                DevBuf& count, DevBuf& start, DevBuf& sorted, DevBuf& bsum, DevBuf* relhi = nullptr,
                DevBuf* rello = nullptr)
{
    int n = (int)s.n;
    ENS(cell_of, sizeof(int) * std::max(n, 1));
    ENS(rank, sizeof(int) * std::max(n, 1));
    ENS(count, sizeof(int) * (g.ncell + 1));
    ENS(start, sizeof(int) * (g.ncell + 1));
    ENS(sorted, sizeof(int) * std::max(n, 1));
    ENS(bsum, sizeof(int) * ((g.ncell + 4095) / 4096 + 1));
    CK(cudaMemsetAsync(count.p, 0, sizeof(int) * (g.ncell + 1), st));
    if (n > 0) {
        if (relhi) {
            ENS(*relhi, sizeof(float4) * std::max(n, 1));
            ENS(*rello, sizeof(float4) * std::max(n, 1));
            CK(launch_bin32(s.pos.as<double>(), n, g, cell_of.as<int>(), rank.as<int>(), count.as<int>(),
                            relhi->as<float4>(), rello->as<float4>(), c->status.as<int>(), st));
        } else {
            k_bin<<<(n + 255) / 256, 256, 0, st>>>(s.pos.as<double>(), n, g, cell_of.as<int>(), rank.as<int>(),
                                                   count.as<int>(), c->status.as<int>());
            CK(cudaGetLastError());
        }
    }
    CK(launch_scan(count.as<int>(), g.ncell, start.as<int>(), bsum.as<int>(), st));
    if (n > 0) {
        k_scatter<<<(n + 255) / 256, 256, 0, st>>>(cell_of.as<int>(), rank.as<int>(), start.as<int>(), n,
                                                   sorted.as<int>());
        CK(cudaGetLastError());
    }
    return IK_OK;
}

int mode_ok(ik_ctx* c, int precision)
{
    if (c->cg.mode == IK_QUAD_FIXEDPOINT) return IK_OK;
    if (c->cg.mode == IK_QUAD_EXACT) {
        if (precision != IK_PREC_FP64 && c->cg.kind != IK_CG_GAUSSIAN)
            return fail(IK_ERR_UNSUPPORTED, "the exact bond integral runs on the FP32 path for the Gaussian kernel only");
        return IK_OK;
    }
    if (c->cg.mode == IK_QUAD_CLIPPED) {
        if (precision != IK_PREC_FP32 || c->cg.kind != IK_CG_GAUSSIAN)
            return fail(IK_ERR_UNSUPPORTED, "the clipped closed form runs on the FP32 path for the Gaussian kernel only");
        return IK_OK;
    }
    if (c->cg.mode == IK_QUAD_ADAPTIVE) {
        if (precision != IK_PREC_FP64)
            return fail(IK_ERR_UNSUPPORTED, "the adaptive bond integral runs on the FP64 path");
        return IK_OK;
    }
    if (c->cg.mode == IK_QUAD_MLP) {
        if (precision != IK_PREC_FP32) return fail(IK_ERR_UNSUPPORTED, "the learned surrogate runs on the FP32 path");
        if (!c->mlp || !ik_mlp_internal_blob(c->mlp) || !ik_mlp_internal_table(c->mlp))
            return fail(IK_ERR_STATE, "quadrature mode mlp needs a trained and validated surrogate (ik_set_mlp)");
        return IK_OK;
    }
    return fail(IK_ERR_UNSUPPORTED, "quadrature mode %d is not available on the GPU path yet", c->cg.mode);
}

int slot_ok(ik_ctx* c, int slot)
{
    if (slot < 0 || slot >= (int)c->slots.size()) return fail(IK_ERR_ARG, "slot %d out of range", slot);
    return IK_OK;
}

// Elastic-field bond records of slot s on lane L (k_bonds64e); the cell list is built.
int elastic_bonds(ik_ctx* c, Slot& s, Lane& L, const IkGeom& g, int n)
{
    const int D = c->dim, NC = D == 2 ? 3 : 6, CW = D == 2 ? 1 : 2;
    if (!s.has_disp) return fail(IK_ERR_STATE, "the elastic field needs displacements (ik_upload_displacement)");
    if (c->maxbe == 0) c->maxbe = D == 2 ? 32 : 63;
    if ((size_t)std::max(n, 1) * (size_t)c->maxbe >= ((size_t)1 << 25))
        return fail(IK_ERR_UNSUPPORTED, "elastic field: n * %d neighbour records exceed 2^25", c->maxbe);
    const size_t nrec = (size_t)c->maxbe * std::max(n, 1);
    ENS(s.ela, sizeof(double) * NC * std::max<int64_t>(c->geo.G, 1));
    ENS(L.eb64, sizeof(IkB64) * nrec);
    ENS(L.ec64, sizeof(double) * NC * nrec);
    ENS(L.eb32, sizeof(float4) * nrec);
    ENS(L.ec32, sizeof(float4) * CW * nrec);
    ENS(L.enb, sizeof(int) * (std::max(n, 1) + 1));
    if (n > 0) {
        k_bonds64e<<<(n + 127) / 128, 128, 0, L.st>>>(g, c->pot, c->cg.kappa, n, L.sorted.as<int>(),
                                                      L.cell_of.as<int>(), s.pos.as<double>(), s.disp.as<double>(),
                                                      s.diam.as<double>(), L.cell_start.as<int>(),
                                                      L.eb64.as<IkB64>(), L.ec64.as<double>(), L.eb32.as<float4>(),
                                                      L.ec32.as<float4>(), c->maxbe, L.enb.as<int>(),
                                                      c->status.as<int>(), c->maxnbe.as<int>());
        CK(cudaGetLastError());
        c->launches += 1;
    } else if (c->geo.G > 0) {
        CK(cudaMemsetAsync(s.ela.p, 0, sizeof(double) * NC * c->geo.G, L.st));
    }
    return IK_OK;
}

GatherGeo gather_geo(ik_ctx* c);
void gather_rule(ik_ctx* c, GatherArgs32& a);

int enqueue(ik_ctx* c, int slot, int prec, int fields)
{
    Slot& s = c->slots[(size_t)slot];
    Lane& L = c->lanes[c->next_lane];
    c->next_lane = (c->next_lane + 1) % IK_LANES;
    // fork from the main stream (uploads), and after the slot's previous computation
    CK(cudaEventRecord(c->fork, c->stream));
    CK(cudaStreamWaitEvent(L.st, c->fork, 0));
    if (s.done_recorded && !c->capturing) CK(cudaStreamWaitEvent(L.st, s.done, 0));
    if (s.d2h_recorded && !c->capturing) CK(cudaStreamWaitEvent(L.st, s.d2h_done, 0)); // outputs being read
    const IkGeom& g = c->geo.geom;
    const int D = c->dim, NC = D == 2 ? 3 : 6;
    const int n = (int)s.n;
    NvtxPhases nv;
    if (c->io_cur && n > 0) { // ik_compute_batch_io: this frame's inputs, copied on its lane
        nv.next("ik upload");
        const IoFrame& io = *c->io_cur;
        CK(cudaMemcpyAsync(s.pos.p, io.pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, L.st));
        CK(cudaMemcpyAsync(s.diam.p, io.diam, sizeof(double) * n, cudaMemcpyHostToDevice, L.st));
        if (io.vel) CK(cudaMemcpyAsync(s.vel.p, io.vel, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, L.st));
        if (io.mass) CK(cudaMemcpyAsync(s.mass.p, io.mass, sizeof(double) * n, cudaMemcpyHostToDevice, L.st));
        if (prec != IK_PREC_FP32) { // the FP32 path's binning and packing make these tests themselves
            k_validate<<<(n + 255) / 256, 256, 0, L.st>>>(s.pos.as<double>(), s.diam.as<double>(), n, c->dim,
                                                          c->status.as<int>());
            CK(cudaGetLastError());
            c->launches += 1;
        }
    }
    bool timing = (c->flags & IK_FLAG_TIMING) != 0 && !c->capturing;
    if (timing) CK(cudaEventRecord(c->ev[0], L.st));
    ENS(s.vir, sizeof(double) * NC * c->geo.G);
    ENS(s.kin, sizeof(double) * NC * c->geo.G);
    ENS(s.counters, sizeof(unsigned long long) * 5);
    CK(cudaMemsetAsync(s.counters.p, 0, sizeof(unsigned long long) * 5, L.st));
    if (!(fields & IK_FIELD_KINETIC)) CK(cudaMemsetAsync(s.kin.p, 0, sizeof(double) * NC * c->geo.G, L.st));
    if (!(fields & IK_FIELD_VIRIAL)) CK(cudaMemsetAsync(s.vir.p, 0, sizeof(double) * NC * c->geo.G, L.st));
    nv.next("ik cells");
    int r = build_cells(c, s, g, L.st, L.cell_of, L.rank, L.cell_count, L.cell_start, L.sorted, L.bsum_cells,
                        prec == IK_PREC_FP32 ? &L.relhi : nullptr, prec == IK_PREC_FP32 ? &L.rello : nullptr);
    if (r) return r;
    const int scan_launches = g.ncell <= 65536 ? 1 : 2;
    c->launches += (n > 0 ? 2 : 0) + scan_launches; // bin, scan, scatter
    ENS(L.prec, sizeof(IkPRec) * std::max(n, 1));
    ENS(L.kin, sizeof(float4) * 2 * std::max(n, 1));
    ENS(L.diam32, sizeof(float) * std::max(n, 1));
    if (g.ncell > 0 && prec != IK_PREC_FP32) { // sort ids inside each cell: deterministic order
        k_cell_sort_pack<<<(g.ncell + 127) / 128, 128, 0, L.st>>>(
            g, L.cell_start.as<int>(), L.sorted.as<int>(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
            nullptr, 0);
        CK(cudaGetLastError());
        c->launches += 1;
    }
    unsigned long long* cnt = s.counters.as<unsigned long long>();
    if (prec == IK_PREC_FP32) {
        ENS(L.pos64, sizeof(IkB64) * std::max(n, 1));
        ENS(L.plo, sizeof(float4) * std::max(n, 1));
        // per-cell sort + pack in one launch
        CK(launch_sort_pack32(g, L.cell_start.as<int>(), L.sorted.as<int>(), L.relhi.as<float4>(),
                              L.rello.as<float4>(), s.pos.as<double>(), s.has_vel ? s.vel.as<double>() : nullptr,
                              s.has_mass ? s.mass.as<double>() : nullptr, s.diam.as<double>(), L.prec.as<IkPRec>(),
                              L.plo.as<float4>(), L.pos64.as<IkB64>(), L.kin.as<float4>(), L.diam32.as<float>(),
                              c->status.as<int>(), L.st));
        c->launches += g.ncell > 0 ? 1 : 0;
        if (timing) CK(cudaEventRecord(c->ev[1], L.st));
        // bond records at a fixed stride of maxb per particle; compacted to CSR only
        // when the staged (offset << 6 | count) word would not hold the offsets
        const bool stride = (size_t)std::max(n, 1) * (size_t)c->maxb < ((size_t)1 << 25) &&
                            !(c->flags & IK_FLAG_CSR_BONDS);
        nv.next("ik bonds");
        ENS(L.bonds_tmp, sizeof(float4) * (size_t)c->maxb * std::max(n, 1));
        ENS(L.nb32, sizeof(int) * (std::max(n, 1) + 1));
        const bool main_pass = (fields & (IK_FIELD_VIRIAL | IK_FIELD_KINETIC)) != 0;
        if (main_pass) {
            CK(launch_bonds32(D, g, c->pot, c->cg.kappa, n, L.prec.as<IkPRec>(), L.diam32.as<float>(),
                              L.cell_start.as<int>(), L.plo.as<float4>(), L.pos64.as<IkB64>(),
                              L.bonds_tmp.as<float4>(), c->maxb, L.nb32.as<int>(), c->status.as<int>(),
                              c->maxnb.as<int>(), stride ? cnt : nullptr, L.st));
            c->launches += n > 0 ? 1 : 0;
        }
        if (!stride && main_pass) {
            ENS(L.bonds32, sizeof(float4) * (size_t)c->maxb * std::max(n, 1));
            ENS(L.boff, sizeof(int) * (std::max(n, 1) + 1));
            ENS(L.bsum, sizeof(int) * ((std::max(n, 1) + 4095) / 4096 + 1));
            CK(launch_scan(L.nb32.as<int>(), n, L.boff.as<int>(), L.bsum.as<int>(), L.st));
            CK(launch_bond_compact(n, c->maxb, L.nb32.as<int>(), L.boff.as<int>(), L.bonds_tmp.as<float4>(),
                                   L.bonds32.as<float4>(), cnt, L.st));
            c->launches += (n <= 65536 ? 1 : 2) + (n > 0 ? 1 : 0);
        }
        const float4* bonds = stride ? L.bonds_tmp.as<float4>() : L.bonds32.as<float4>();
        if (timing) CK(cudaEventRecord(c->ev[2], L.st));
        nv.next("ik gather");
        GatherArgs32 a{};
        a.geo = gather_geo(c);
        gather_rule(c, a);
        a.prec = L.prec.as<IkPRec>();
        a.pos64 = L.pos64.as<IkB64>();
        a.cell_start = L.cell_start.as<int>();
        a.boff = stride ? nullptr : L.boff.as<int>();
        a.nprec = n;
        a.nb = L.nb32.as<int>();
        a.bonds = bonds;
        a.maxb = c->maxb;
        a.kin = L.kin.as<float4>();
        a.gpts = c->geo.gpts_d.as<float4>();
        a.grid = c->geo.grid_d.as<double>();
        a.items = c->geo.items_d.as<int4>();
        a.nitems = c->geo.nitems;
        a.halo_cap = c->halo_cap;
        a.qcap = 32 * (std::min(c->maxb, 63) + 1); // <= 63 bonds per staged entry
        double norm = c->cg.kind == IK_CG_MOLLIFIER ? c->cg.mollifier_norm : c->cg.norm;
        ENS(L.vir2, sizeof(float2) * NC * (size_t)c->geo.G);
        ENS(L.kin2, sizeof(float2) * NC * (size_t)c->geo.G);
        a.out_vir = L.vir2.as<float2>();
        a.out_kin = L.kin2.as<float2>();
        a.fields = fields & (s.has_vel ? 3 : 1);
        if ((fields & IK_FIELD_KINETIC) && !s.has_vel)
            CK(cudaMemsetAsync(s.kin.p, 0, sizeof(double) * NC * c->geo.G, L.st));
        a.work_counter = L.work_counter.as<int>();
        a.status = c->status.as<int>();
        a.cnt_pairs = cnt + 1;
        a.cnt_triples = cnt + 2;
        CK(cudaMemsetAsync(L.work_counter.p, 0, sizeof(int), L.st));
        const bool mlp = c->cg.mode == IK_QUAD_MLP && (a.fields & 1);
        // without surrogate corrections to add the gather writes the FP64 fields itself
        a.direct64 = mlp ? 0 : 1;
        a.out64_vir = (a.fields & 1) ? s.vir.as<double>() : nullptr;
        a.out64_kin = (a.fields & 2) ? s.kin.as<double>() : nullptr;
        a.s64_vir = 0.5 * norm;
        a.s64_kin = norm;
        if (mlp) {
            if (c->mlp_cap == 0) c->mlp_cap = std::max<long long>(1 << 20, 128LL * c->geo.G);
            ENS(L.mlp_rec, sizeof(float4) * (size_t)c->mlp_cap);
            ENS(L.mlp_rid, sizeof(int2) * (size_t)c->mlp_cap);
            ENS(L.mlp_count, sizeof(unsigned long long));
            ENS(L.corr, sizeof(unsigned long long) * NC * (size_t)c->geo.G);
            CK(cudaMemsetAsync(L.mlp_count.p, 0, sizeof(unsigned long long), L.st));
            CK(cudaMemsetAsync(L.corr.p, 0, sizeof(unsigned long long) * NC * (size_t)c->geo.G, L.st));
            a.mlp_rec = L.mlp_rec.as<float4>();
            a.mlp_rid = L.mlp_rid.as<int2>();
            a.mlp_count = L.mlp_count.as<unsigned long long>();
            a.mlp_cap = c->mlp_cap;
            a.cnt_records = cnt + 3;
        }
        const size_t stage_bytes = D == 3 ? 20 : 16; // float4 (+ the index word in 3D) per staged entry
        size_t smem = (size_t)IK_WARPS_GATHER * ((size_t)c->halo_cap * stage_bytes + (size_t)a.qcap * 4);
        // one frame alone: two CTAs per SM fill the GPU; frames of a batch on several lanes
        // run side by side, and one CTA per SM each measured faster (8330 -> 8620 frames/s)
        const int bps = c->tune_blocks_per_sm > 0 ? c->tune_blocks_per_sm : (c->in_batch ? 1 : 2);
        int blocks = std::min(c->geo.nitems, c->sm_count * bps);
        if (blocks > 0 && main_pass) {
            const int qm = mlp ? 1 : (c->cg.mode == IK_QUAD_CLIPPED ? 2 : (c->cg.mode == IK_QUAD_EXACT ? 3 : 0));
            CK(launch_gather32(a, c->cg.kind, (c->flags & IK_FLAG_LANE_KAHAN) != 0 && qm == 0, qm, blocks,
                               32 * IK_WARPS_GATHER, smem, L.st));
            c->launches += 1;
        }
        if (mlp) { // the surrogate on the tensor cores for the recorded bonds
            const double to_w = std::sqrt(2.0 / 1.4426950408889634);
            CK(launch_mlp_records(c->mlp, L.mlp_rec.as<float4>(), L.mlp_rid.as<int2>(),
                                  L.mlp_count.as<unsigned long long>(), c->mlp_cap, bonds,
                                  (float)to_w, (float)c->cg.width, NC, L.corr.as<unsigned long long>(),
                                  cnt + 4, c->status.as<int>(), c->sm_count * mlp_tc_ctas_per_sm(), L.st));
            c->launches += 1;
        }
        // FP64 finish: ((double)hi + (double)lo) * normalisation (0.5 of the GL map for the
        // virial), with the surrogate's corrections (otherwise done by the gather)
        if (!a.direct64) {
            nv.next("ik finish");
            CK(launch_pairs_to_f64(L.vir2.as<float2>(), mlp ? L.corr.as<unsigned long long>() : nullptr,
                                   (a.fields & 1) ? s.vir.as<double>() : nullptr, 0.5 * norm, L.kin2.as<float2>(),
                                   (a.fields & 2) ? s.kin.as<double>() : nullptr, norm, (long long)NC * c->geo.G,
                                   L.st));
            c->launches += (c->geo.G > 0 && a.fields) ? 1 : 0;
        }
        if (fields & IK_FIELD_ELASTIC) { // the elastic virial field: same staging, elastic records
            nv.next("ik elastic");
            if (int r2 = elastic_bonds(c, s, L, g, n)) return r2;
            GatherArgs32 e = a;
            e.boff = nullptr;
            e.nb = L.enb.as<int>();
            e.bonds = L.eb32.as<float4>();
            e.bcoef = L.ec32.as<float4>();
            e.maxb = c->maxbe;
            e.qcap = 32 * (std::min(c->maxbe, 63) + 1);
            e.fields = IK_FIELD_VIRIAL;
            e.direct64 = 1; // the gather writes the FP64 elastic field itself
            e.out64_vir = s.ela.as<double>();
            e.out64_kin = nullptr;
            e.s64_vir = 0.5 * norm;
            e.mlp_rec = nullptr;
            e.mlp_rid = nullptr;
            e.mlp_count = nullptr;
            e.cnt_records = nullptr;
            ENS(L.ecnt, sizeof(unsigned long long) * 2);
            e.cnt_pairs = L.ecnt.as<unsigned long long>();
            e.cnt_triples = e.cnt_pairs + 1;
            CK(cudaMemsetAsync(L.work_counter.p, 0, sizeof(int), L.st));
            const size_t esmem = (size_t)IK_WARPS_GATHER * ((size_t)c->halo_cap * stage_bytes + (size_t)e.qcap * 4);
            if (blocks > 0) {
                CK(launch_gather32(e, c->cg.kind, false, 0, blocks, 32 * IK_WARPS_GATHER, esmem, L.st));
                c->launches += 1;
            }
        }
    } else {
        if (timing) CK(cudaEventRecord(c->ev[1], L.st));
        nv.next("ik bonds");
        ENS(L.bonds64, sizeof(IkB64) * (size_t)c->maxb * std::max(n, 1));
        ENS(L.nb64, sizeof(int) * std::max(n, 1));
        const bool main_pass = (fields & (IK_FIELD_VIRIAL | IK_FIELD_KINETIC)) != 0;
        if (n > 0 && main_pass) {
            k_bonds64<<<(n + 127) / 128, 128, 0, L.st>>>(
                g, c->pot, n, L.sorted.as<int>(), L.cell_of.as<int>(), s.pos.as<double>(), s.diam.as<double>(),
                L.cell_start.as<int>(), L.bonds64.as<IkB64>(), c->maxb, L.nb64.as<int>(), c->status.as<int>(),
                c->maxnb.as<int>());
            CK(cudaGetLastError());
        }
        if (timing) CK(cudaEventRecord(c->ev[2], L.st));
        nv.next("ik gather");
        GatherArgs64 a{};
        a.g = g;
        a.cg = c->cg;
        for (int k = 0; k < 3; ++k) {
            a.reach[k] = c->geo.reach[k];
            a.all[k] = (k < D && 2 * c->geo.reach[k] + 1 >= g.nc[k]) ? 1 : 0;
        }
        a.nq = c->gl.n;
        for (int k = 0; k < c->gl.n; ++k) { a.xs[k] = 0.5 + 0.5 * c->gl.x[k]; a.ws[k] = c->gl.w[k]; }
        a.gk = gk15();
        a.status = c->status.as<int>();
        a.sorted = L.sorted.as<int>();
        a.cell_start = L.cell_start.as<int>();
        a.pos = s.pos.as<double>();
        a.vel = s.has_vel ? s.vel.as<double>() : nullptr;
        a.mass = s.has_mass ? s.mass.as<double>() : nullptr;
        a.nb = L.nb64.as<int>();
        a.bonds = L.bonds64.as<IkB64>();
        a.maxb = c->maxb;
        a.grid = c->geo.grid_d.as<double>();
        a.ngrid = c->geo.G;
        a.out_vir = s.vir.as<double>();
        a.out_kin = s.kin.as<double>();
        a.fields = fields;
        if ((fields & IK_FIELD_KINETIC) && !s.has_vel)
            CK(cudaMemsetAsync(s.kin.p, 0, sizeof(double) * NC * c->geo.G, L.st));
        if (main_pass) {
            CK(launch_gather64(a, L.st));
            c->launches += (n > 0 ? 1 : 0) + (c->geo.G > 0 ? 1 : 0);
        }
        if (fields & IK_FIELD_ELASTIC) { // the elastic virial field
            nv.next("ik elastic");
            if (int r2 = elastic_bonds(c, s, L, g, n)) return r2;
            GatherArgs64 e = a;
            e.bonds = L.eb64.as<IkB64>();
            e.nb = L.enb.as<int>();
            e.ecoef = L.ec64.as<double>();
            e.maxb = c->maxbe;
            e.out_vir = s.ela.as<double>();
            e.out_kin = nullptr;
            e.fields = IK_FIELD_VIRIAL;
            CK(launch_gather64(e, L.st));
            c->launches += c->geo.G > 0 ? 1 : 0;
        }
    }
    if (c->io_cur && c->geo.G > 0) { // ik_compute_batch_io: this frame's fields to the host
        nv.next("ik download");
        const DevBuf* src[3] = {&s.vir, &s.kin, &s.ela};
        for (int f = 0; f < 3; ++f)
            if (c->io_cur->out[f] && (fields & (1 << f)))
                CK(cudaMemcpyAsync(c->io_cur->out[f], src[f]->p, sizeof(double) * NC * c->geo.G,
                                   cudaMemcpyDeviceToHost, L.st));
    }
    if (timing) CK(cudaEventRecord(c->ev[3], L.st));
    s.last_prec = prec;
    s.last_fields = fields;
    if (!s.done) CK(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
    if (c->capturing) { // the lane rejoins the main stream at the end of the capture
        c->captured_lanes |= 1 << (int)(&L - c->lanes);
        return IK_OK;
    }
    CK(cudaEventRecord(s.done, L.st));
    s.done_recorded = true;
    CK(cudaEventRecord(L.last, L.st));
    return IK_OK;
}

// Settings that every binning depends on (cut-offs, kappa, bin size) changed.
void invalidate_geometry(ik_ctx* c);

// The FP32 gather's geometry of the current box and binning (ensure_geometry done).
GatherGeo gather_geo(ik_ctx* c)
{
    const IkGeom& g = c->geo.geom;
    const int D = c->dim;
    GatherGeo G{};
    G.g = g;
    for (int k = 0; k < 3; ++k) {
        G.cws[k] = (float)(c->cg.kappa * g.cw[k]);
        G.bw[k] = c->geo.bw[k];
        G.reach[k] = c->geo.reach[k];
    }
    // cull the staged halo to the particles within R of the bin's box where that drops
    // a fifth or more of it (3D: a bin of one cell with a reach of one; the kernel
    // culls in 3D only -- 2D bins of several cells lose ~12 %, less than the second
    // pass over their particles costs)
    double stagedv = 1.0, nearv = 1.0, side[3] = {0, 0, 0};
    for (int k = 0; k < D; ++k) {
        side[k] = c->geo.bw[k] * g.cw[k];
        stagedv *= side[k] + 2.0 * c->geo.reach[k] * g.cw[k];
    }
    const double R = c->cg.rcut, PI = 3.14159265358979323846;
    if (D == 2) nearv = side[0] * side[1] + 2.0 * R * (side[0] + side[1]) + PI * R * R;
    else nearv = side[0] * side[1] * side[2] + 2.0 * R * (side[0] * side[1] + side[1] * side[2] + side[0] * side[2]) +
                 PI * R * R * (side[0] + side[1] + side[2]) + 4.0 / 3.0 * PI * R * R * R;
    G.cull = nearv < 0.8 * stagedv ? 1 : 0;
    return G;
}

// The coarse-graining constants and the Gauss-Legendre rule of the FP32 gather.
void gather_rule(ik_ctx* c, GatherArgs32& a)
{
    a.kappa = c->cg.kappa;
    a.R2s = c->cg.R2s;
    a.margin = 1e-4f * c->cg.R2s;
    a.R2 = c->cg.rcutsq;
    a.npairs = c->gl.npairs;
    a.w0 = c->gl.w0;
    for (int k = 0; k < 32; ++k) {
        a.xi2[k] = c->gl.t[k] * c->gl.t[k];
        a.m2xi[k] = -2.0f * c->gl.t[k];
        a.w[k] = c->gl.wt[k];
    }
}

void invalidate_geometry(ik_ctx* c)
{
    c->geo.geom_valid = false;
    for (Slot& s : c->slots) s.geo.geom_valid = false;
}

// Swaps a slot's own geometry (if any) into the context for the scope.
struct GeoSwap {
    ik_ctx* c;
    Slot* s = nullptr;
    GeoSwap(ik_ctx* c_, int slot) : c(c_)
    {
        if (slot >= 0 && slot < (int)c->slots.size() && c->slots[(size_t)slot].has_geo) {
            s = &c->slots[(size_t)slot];
            std::swap(c->geo, s->geo);
        }
    }
    ~GeoSwap() { if (s) std::swap(c->geo, s->geo); }
    GeoSwap(const GeoSwap&) = delete;
    GeoSwap& operator=(const GeoSwap&) = delete;
};

// ---- fused batches -----------------------------------------------------------
// A batch runs fused (every stage once over all its frames) when it computes the
// virial and/or kinetic field on the FP32 path with the fixed-point rule of order 4 or
// 5, every slot's bond records fit the per-frame staged-entry word (n maxb < 2^25, at
// most 63 bonds per particle), and no slot appears twice.  Otherwise its frames run on
// the lanes (one launch sequence per frame), as with fused batches turned off.
bool fused_eligible(ik_ctx* c, const std::vector<int>& slots, int prec, int fields)
{
    if (!c->tune_fused || prec != IK_PREC_FP32 || (fields & ~(IK_FIELD_VIRIAL | IK_FIELD_KINETIC)) || !fields)
        return false;
    if (c->cg.mode != IK_QUAD_FIXEDPOINT || c->gl.npairs != 2 || c->maxb > 63) return false;
    if (c->flags & (IK_FLAG_CSR_BONDS | IK_FLAG_TIMING)) return false;
    std::vector<int> sorted(slots);
    std::sort(sorted.begin(), sorted.end());
    if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end()) return false;
    long long ptot = 0;
    for (int k : slots) {
        const int64_t n = c->slots[(size_t)k].n;
        if ((size_t)std::max<int64_t>(n, 1) * (size_t)c->maxb >= ((size_t)1 << 25)) return false;
        ptot += n;
    }
    return ptot < (1LL << 30);
}

// Concatenates the slots' frames, cells, grids and work items (host, then one upload of
// each array) into F and sizes its batch-wide work buffers.  Not during a capture.
int fused_build(ik_ctx* c, const std::vector<int>& slots, FusedBatch& F)
{
    const int D = c->dim, NC = D == 2 ? 3 : 6, S = (int)slots.size();
    std::vector<IkBatchSlot> hs((size_t)S);
    std::vector<int> po((size_t)S + 1), co((size_t)S + 1);
    std::vector<long long> vo((size_t)S + 1);
    std::vector<int4> items;
    std::vector<int> islot;
    std::vector<float4> gp;
    std::vector<double> gr;
    long long P = 0, Cc = 0, Gt = 0;
    for (int k = 0; k < S; ++k) {
        GeoSwap gs(c, slots[(size_t)k]);
        Slot& s = c->slots[(size_t)slots[(size_t)k]];
        const IkGeom& g = c->geo.geom;
        const int64_t G = c->geo.G;
        ENS(s.vir, sizeof(double) * NC * std::max<int64_t>(G, 1));
        ENS(s.kin, sizeof(double) * NC * std::max<int64_t>(G, 1));
        ENS(s.counters, sizeof(unsigned long long) * 5);
        IkBatchSlot& b = hs[(size_t)k];
        b.geo = gather_geo(c);
        b.geo.c_off = (int)Cc;
        b.geo.p_off = (int)P;
        b.geo.cnt = s.counters.as<unsigned long long>();
        b.pos = s.pos.as<double>();
        b.vel = s.has_vel ? s.vel.as<double>() : nullptr;
        b.mass = s.has_mass ? s.mass.as<double>() : nullptr;
        b.diam = s.diam.as<double>();
        b.out_vir = s.vir.as<double>();
        b.out_kin = s.kin.as<double>();
        b.n = (int)s.n;
        b.ncell = g.ncell;
        b.allax = 0;
        for (int a = 0; a < D; ++a) b.allax |= (g.all_bond[a] && g.nc[a] > 1) ? 1 : 0;
        b.G = G;
        b.g_off = Gt;
        po[(size_t)k] = (int)P;
        co[(size_t)k] = (int)Cc;
        vo[(size_t)k] = Gt * NC;
        // one work item per bin: the frame's items split a bin so that a frame alone fills
        // the GPU; a batch has enough bins, and a whole bin stages its halo once
        for (int j = 0; j < c->geo.nitems; ++j) {
            int4 it = c->geo.items_h[(size_t)j];
            if (j > 0) {
                const int4& pv = c->geo.items_h[(size_t)j - 1];
                if (pv.x == it.x && pv.y == it.y && pv.z == it.z) continue;
            }
            it.w += (int)Gt;
            items.push_back(it);
            islot.push_back(k);
        }
        for (int64_t j = 0; j < G; ++j) {
            float4 v = c->geo.gpts_h[(size_t)j];
            int gi;
            std::memcpy(&gi, &v.w, 4);
            gi += (int)Gt;
            std::memcpy(&v.w, &gi, 4);
            gp.push_back(v);
        }
        gr.insert(gr.end(), c->geo.grid_h.begin(), c->geo.grid_h.begin() + 3 * G);
        P += s.n;
        Cc += g.ncell;
        Gt += G;
        if (P >= (1LL << 30) || Cc >= (1LL << 30) || Gt >= (1LL << 30))
            return fail(IK_ERR_UNSUPPORTED, "fused batch too large (particles, cells or grid points >= 2^30)");
    }
    po[(size_t)S] = (int)P;
    co[(size_t)S] = (int)Cc;
    vo[(size_t)S] = Gt * NC;
    items.push_back(make_int4(0, 0, 0, (int)Gt));
    F.nitems = (int)items.size() - 1;
    F.gtot = Gt;
    auto up = [&](DevBuf& d, const void* h, size_t bytes) -> int {
        ENS(d, std::max<size_t>(bytes, 16));
        if (bytes) CK(cudaMemcpy(d.p, h, bytes, cudaMemcpyHostToDevice));
        return IK_OK;
    };
    if (int r = up(F.slots, hs.data(), sizeof(IkBatchSlot) * hs.size())) return r;
    if (int r = up(F.p_offs, po.data(), sizeof(int) * po.size())) return r;
    if (int r = up(F.c_offs, co.data(), sizeof(int) * co.size())) return r;
    if (int r = up(F.v_offs, vo.data(), sizeof(long long) * vo.size())) return r;
    if (int r = up(F.items, items.data(), sizeof(int4) * items.size())) return r;
    if (int r = up(F.item_slot, islot.data(), sizeof(int) * islot.size())) return r;
    if (int r = up(F.gpts, gp.data(), sizeof(float4) * gp.size())) return r;
    if (int r = up(F.grid, gr.data(), sizeof(double) * gr.size())) return r;
    const size_t np = (size_t)std::max<long long>(P, 1), nc1 = (size_t)Cc + 1;
    ENS(F.cell_of, sizeof(int) * np);
    ENS(F.rank, sizeof(int) * np);
    ENS(F.sorted, sizeof(int) * np);
    ENS(F.nb, sizeof(int) * np);
    ENS(F.cell_count, sizeof(int) * nc1);
    ENS(F.cell_start, sizeof(int) * nc1);
    ENS(F.bsum, sizeof(int) * (nc1 / 4096 + 2));
    ENS(F.relhi, sizeof(float4) * np);
    ENS(F.rello, sizeof(float4) * np);
    ENS(F.prec, sizeof(IkPRec) * np);
    ENS(F.plo, sizeof(float4) * np);
    ENS(F.pos64, sizeof(IkB64) * np);
    ENS(F.kin, sizeof(float4) * (D == 3 ? 2 : 1) * np);
    ENS(F.diam32, sizeof(float) * np);
    ENS(F.tmp, sizeof(float4) * (size_t)c->maxb * np);
    ENS(F.vir2, sizeof(float2) * NC * (size_t)std::max<long long>(Gt, 1));
    ENS(F.kin2, sizeof(float2) * NC * (size_t)std::max<long long>(Gt, 1));
    ENS(F.work, sizeof(int));
    IkBatchLaunch& b = F.b;
    b.slots = F.slots.as<IkBatchSlot>();
    b.p_offs = F.p_offs.as<int>();
    b.c_offs = F.c_offs.as<int>();
    b.v_offs = F.v_offs.as<long long>();
    b.nslots = S;
    b.ptot = (int)P;
    b.ctot = (int)Cc;
    b.vtot = Gt * NC;
    b.cell_of = F.cell_of.as<int>();
    b.rank = F.rank.as<int>();
    b.cell_count = F.cell_count.as<int>();
    b.cell_start = F.cell_start.as<int>();
    b.sorted = F.sorted.as<int>();
    b.bsum = F.bsum.as<int>();
    b.relhi = F.relhi.as<float4>();
    b.rello = F.rello.as<float4>();
    b.prec = F.prec.as<IkPRec>();
    b.plo = F.plo.as<float4>();
    b.pos64 = F.pos64.as<IkB64>();
    b.kin = F.kin.as<float4>();
    b.diam32 = F.diam32.as<float>();
    b.tmp = F.tmp.as<float4>();
    b.nb = F.nb.as<int>();
    b.maxb = c->maxb;
    b.status = c->status.as<int>();
    b.maxnb = c->maxnb.as<int>();
    return IK_OK;
}

// The launches of the fused batch F on stream st (fused_build done).  timing: events
// ev[0] before the preparation, ev[1] = ev[2] after it, ev[3] after the gather.
int fused_enqueue(ik_ctx* c, FusedBatch& F, int fields, cudaStream_t st, bool timing = false)
{
    NvtxRange nvr("ik fused batch");
    const IkBatchLaunch& b = F.b;
    const int D = c->dim;
    if (timing) CK(cudaEventRecord(c->ev[0], st));
    CK(cudaMemsetAsync(b.cell_count, 0, sizeof(int) * ((size_t)b.ctot + 1), st));
    CK(cudaMemsetAsync(F.work.p, 0, sizeof(int), st));
    CK(launch_batch_prepare(b, D, c->pot, c->cg.kappa, st));
    if (timing) {
        CK(cudaEventRecord(c->ev[1], st));
        CK(cudaEventRecord(c->ev[2], st));
    }
    c->launches += 1 + (b.ctot <= 65536 ? 1 : 2) + (b.ptot > 0 ? 1 : 0) + (b.ctot > 0 ? 1 : 0) + (b.ptot > 0 ? 1 : 0);
    GatherArgs32 a{};
    a.geo.g.dim = D; // the slots carry their own geometry
    gather_rule(c, a);
    a.prec = b.prec;
    a.pos64 = b.pos64;
    a.cell_start = b.cell_start;
    a.boff = nullptr;
    a.nprec = b.ptot;
    a.nb = b.nb;
    a.bonds = b.tmp;
    a.maxb = c->maxb;
    a.kin = b.kin;
    a.gpts = F.gpts.as<float4>();
    a.grid = F.grid.as<double>();
    a.items = F.items.as<int4>();
    a.nitems = F.nitems;
    a.halo_cap = c->halo_cap;
    a.qcap = 32 * (std::min(c->maxb, 63) + 1);
    a.out_vir = F.vir2.as<float2>();
    a.out_kin = F.kin2.as<float2>();
    a.fields = fields & (IK_FIELD_VIRIAL | IK_FIELD_KINETIC);
    const double norm = c->cg.kind == IK_CG_MOLLIFIER ? c->cg.mollifier_norm : c->cg.norm;
    // both fields: the gather writes each slot's FP64 fields itself; one field: the
    // finish also writes the other as zeros
    a.direct64 = a.fields == (IK_FIELD_VIRIAL | IK_FIELD_KINETIC) ? 1 : 0;
    a.s64_vir = 0.5 * norm;
    a.s64_kin = norm;
    a.work_counter = F.work.as<int>();
    a.status = c->status.as<int>();
    a.slots = b.slots;
    a.item_slot = F.item_slot.as<int>();
    const size_t stage_bytes = D == 3 ? 20 : 16;
    const size_t smem = (size_t)IK_WARPS_GATHER * ((size_t)c->halo_cap * stage_bytes + (size_t)a.qcap * 4);
    // every frame's items in one launch: two CTAs per SM by default, as a frame alone
    const int bps = c->tune_blocks_per_sm > 0 ? c->tune_blocks_per_sm : 2;
    const int blocks = std::min(F.nitems, c->sm_count * bps);
    if (blocks > 0) {
        CK(launch_gather32_batch(a, c->cg.kind, (c->flags & IK_FLAG_LANE_KAHAN) != 0, blocks, 32 * IK_WARPS_GATHER,
                                 smem, st));
        c->launches += 1;
    }
    if (timing) CK(cudaEventRecord(c->ev[3], st));
    if (!a.direct64) {
        CK(launch_batch_finish(b, a.out_vir, a.out_kin, 0.5 * norm, norm, fields, st));
        c->launches += b.vtot > 0 ? 1 : 0;
    }
    return IK_OK;
}

// Checks, geometry and capacities of one slot, then its launches.
int prepare_enqueue(ik_ctx* c, int slot, int prec, int fields)
{
    GeoSwap gs(c, slot);
    if (int r = ensure_ready(c)) return r;
    if (int r = mode_ok(c, prec)) return r;
    if ((fields & IK_FIELD_ELASTIC) && prec == IK_PREC_FP32 &&
        (c->cg.mode == IK_QUAD_EXACT || c->cg.mode == IK_QUAD_CLIPPED))
        return fail(IK_ERR_UNSUPPORTED, "the elastic field on the FP32 path uses the fixed-point rule only");
    if (int r = ensure_geometry(c)) return r;
    if (c->maxb == 0) c->maxb = c->dim == 2 ? IK_MAXB_2D : IK_MAXB_3D;
    if (c->halo_cap == 0) c->halo_cap = 384; // staged particles per warp (grows on overflow)
    return enqueue(c, slot, prec, fields);
}

// The sub-batches of a fused ik_compute_batch_io: contiguous runs of the batch's frames with
// about equal particle counts, IK_TUNE_IO_BATCHES of them, never more than the frames.
// Returns the runs' boundaries (first 0, last count).
std::vector<int> io_split(ik_ctx* c, const int* slots, int count)
{
    long long ptot = 0;
    for (int k = 0; k < count; ++k) ptot += c->slots[(size_t)slots[k]].n;
    const int nsub = std::max(1, std::min(c->tune_io_batches, count));
    std::vector<int> cut{0};
    long long acc = 0;
    for (int k = 0; k + 1 < count && (int)cut.size() < nsub; ++k) {
        acc += c->slots[(size_t)slots[k]].n;
        const long long b = (long long)cut.size(); // the boundary this frame may close
        if (acc * nsub >= ptot * b) cut.push_back(k + 1);
    }
    cut.push_back(count);
    return cut;
}

// At least n completion events for the sub-batches of a fused ik_compute_batch_io (created
// before a capture).
int io_events(ik_ctx* c, int n)
{
    while ((int)c->io_ev.size() < n) {
        cudaEvent_t e = nullptr;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        c->io_ev.push_back(e);
    }
    return IK_OK;
}

// The device's view of a page-locked host array (null when it has none).
const void* host_mapped(const void* p)
{
    if (!p) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// The descriptor tables of host-mapped copies (IK_TUNE_IO_MAPPED) for the sub-batches of a
// fused ik_compute_batch_io (fused_build of each done): per frame its positions (checked),
// diameters (checked), velocities and masses into the slot's buffers; per frame each
// requested field out of the slot's buffer.  Returns false (nothing built) when an array
// has no device view, so that the copies stay on the copy engines.
bool io_build_mapped(ik_ctx* c, const int* slots, const std::vector<IoFrame>& fr, const std::vector<int>& cut,
                     int fields, int* err)
{
    *err = IK_OK;
    const int NC = c->dim == 2 ? 3 : 6, nsub = (int)cut.size() - 1;
    std::vector<std::vector<IkIoCopy>> ups((size_t)nsub), dns((size_t)nsub);
    for (int b = 0; b < nsub; ++b)
        for (int k = cut[(size_t)b]; k < cut[(size_t)b + 1]; ++k) {
            Slot& s = c->slots[(size_t)slots[k]];
            const IoFrame& io = fr[(size_t)k];
            const long long n = s.n;
            // one copy: host array -> device buffer (up) or device buffer -> host array
            auto add = [&](bool up, const void* src, void* dst, long long words, int check) {
                if (words <= 0) return true;
                const void* ms = up ? host_mapped(src) : src;
                const void* md = up ? dst : host_mapped(dst);
                if (!ms || !md) return false;
                IkIoCopy d{};
                d.src = static_cast<const long long*>(ms);
                d.dst = static_cast<long long*>(const_cast<void*>(md));
                d.words = words;
                d.check = check;
                d.dim = c->dim;
                (up ? ups : dns)[(size_t)b].push_back(d);
                return true;
            };
            if (!add(true, io.pos, s.pos.p, 3 * n, 1) || !add(true, io.diam, s.diam.p, n, 2) ||
                (io.vel && !add(true, io.vel, s.vel.p, 3 * n, 0)) || (io.mass && !add(true, io.mass, s.mass.p, n, 0)))
                return false;
            int64_t G = 0;
            { GeoSwap gs(c, slots[k]); G = c->geo.G; }
            const DevBuf* src[2] = {&s.vir, &s.kin};
            for (int f = 0; f < 2; ++f)
                if (io.out[f] && (fields & (1 << f)) && !add(false, src[f]->p, io.out[f], (long long)NC * G, 0))
                    return false;
        }
    for (int b = 0; b < nsub; ++b) {
        FusedBatch& F = c->fused_io[(size_t)b];
        for (int dir = 0; dir < 2; ++dir) {
            std::vector<IkIoCopy>& v = dir ? dns[(size_t)b] : ups[(size_t)b];
            long long off = 0;
            for (IkIoCopy& d : v) { d.off = off; off += d.words; }
            DevBuf& buf = dir ? F.io_dn : F.io_up;
            if ((*err = buf.ensure(std::max<size_t>(v.size(), 1) * sizeof(IkIoCopy)))) return false;
            if (!v.empty() && cudaMemcpy(buf.p, v.data(), v.size() * sizeof(IkIoCopy), cudaMemcpyHostToDevice) != cudaSuccess) {
                *err = fail(IK_ERR_CUDA, "descriptor upload failed");
                return false;
            }
            (dir ? F.n_dn : F.n_up) = (int)v.size();
            (dir ? F.w_dn : F.w_up) = off;
        }
    }
    return true;
}

// The launches and copies of a fused ik_compute_batch_io, to be captured (fused_build of
// every sub-batch and io_events done).  Lane 0 uploads the frames in batch order (copies
// only: a kernel there would wait for the SMs that a persistent gather holds, and the next
// uploads behind it); lanes 1 and 2 take the sub-batches in turn, each a fused batch
// (whose binning and packing validate the frames) started once its frames are on the
// device (the preparation of one overlaps the end of the previous gather); lane 3
// downloads a sub-batch's fields as soon as it is computed.  The copies of the other sub-batches overlap every computation
// but the first upload and the last download.
int fused_io_enqueue(ik_ctx* c, const int* slots, const std::vector<IoFrame>& fr, const std::vector<int>& cut,
                     int fields, bool mapped)
{
    const int NC = c->dim == 2 ? 3 : 6, nsub = (int)cut.size() - 1;
    cudaStream_t up = c->lanes[0].st, dn = c->lanes[3].st;
    CK(cudaEventRecord(c->fork, c->stream));
    for (int l = 0; l < 4; ++l) CK(cudaStreamWaitEvent(c->lanes[l].st, c->fork, 0));
    c->captured_lanes |= 0xF;
    if (mapped) {
        // host-mapped copies (io_build_mapped done): a sub-batch's uploads with their
        // validation, its fused batch and its downloads, on lanes 1 and 2 in turn
        for (int b = 0; b < nsub; ++b) {
            FusedBatch& F = c->fused_io[(size_t)b];
            cudaStream_t cs = c->lanes[1 + (b & 1)].st;
            CK(launch_io_copy(F.io_up.as<IkIoCopy>(), F.n_up, F.w_up, c->status.as<int>(), c->sm_count, cs));
            c->launches += F.w_up > 0 ? 1 : 0;
            if (int r = fused_enqueue(c, F, fields, cs)) return r;
            CK(launch_io_copy(F.io_dn.as<IkIoCopy>(), F.n_dn, F.w_dn, c->status.as<int>(), c->sm_count, cs));
            c->launches += F.w_dn > 0 ? 1 : 0;
        }
        return IK_OK;
    }
    for (int b = 0; b < nsub; ++b) {
        NvtxRange nvr("ik upload");
        for (int k = cut[(size_t)b]; k < cut[(size_t)b + 1]; ++k) {
            Slot& s = c->slots[(size_t)slots[k]];
            const IoFrame& io = fr[(size_t)k];
            const int n = (int)s.n;
            if (n == 0) continue;
            CK(cudaMemcpyAsync(s.pos.p, io.pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, up));
            CK(cudaMemcpyAsync(s.diam.p, io.diam, sizeof(double) * n, cudaMemcpyHostToDevice, up));
            if (io.vel) CK(cudaMemcpyAsync(s.vel.p, io.vel, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, up));
            if (io.mass) CK(cudaMemcpyAsync(s.mass.p, io.mass, sizeof(double) * n, cudaMemcpyHostToDevice, up));
        }
        CK(cudaEventRecord(c->io_ev[(size_t)(2 * b)], up));
        cudaStream_t cs = c->lanes[1 + (b & 1)].st;
        CK(cudaStreamWaitEvent(cs, c->io_ev[(size_t)(2 * b)], 0));
        if (int r = fused_enqueue(c, c->fused_io[(size_t)b], fields, cs)) return r;
        CK(cudaEventRecord(c->io_ev[(size_t)(2 * b + 1)], cs));
        CK(cudaStreamWaitEvent(dn, c->io_ev[(size_t)(2 * b + 1)], 0));
        for (int k = cut[(size_t)b]; k < cut[(size_t)b + 1]; ++k) {
            Slot& s = c->slots[(size_t)slots[k]];
            int64_t G = 0;
            { GeoSwap gs(c, slots[k]); G = c->geo.G; }
            if (G == 0) continue;
            const DevBuf* src[2] = {&s.vir, &s.kin};
            for (int f = 0; f < 2; ++f)
                if (fr[(size_t)k].out[f] && (fields & (1 << f)))
                    CK(cudaMemcpyAsync(fr[(size_t)k].out[f], src[f]->p, sizeof(double) * NC * G,
                                       cudaMemcpyDeviceToHost, dn));
        }
    }
    return IK_OK;
}

} // namespace

// Lets entry points defined in other translation units report through ik_last_error().
void ik_internal_set_error(const char* msg) { g_err = msg; }
void ik_gl_rule(int n, double* x, double* w) { gl_rule(n, x, w); }

int ik_gk15_rule(double x[8], double wk[8], double wg[4])
{
    if (!x || !wk || !wg) return fail(IK_ERR_ARG, "null output");
    const IkGK& g = gk15();
    for (int k = 0; k < 8; ++k) { x[k] = g.x[k]; wk[k] = g.wk[k]; }
    for (int k = 0; k < 4; ++k) wg[k] = g.wg[k];
    return IK_OK;
}

// ===========================================================================
extern "C" {

const char* ik_last_error(void) { return g_err.c_str(); }
int ik_version(void) { return 100; }

int ik_create(ik_ctx** out, int device)
{
    if (!out) return fail(IK_ERR_ARG, "null output pointer");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(IK_ERR_CUDA, "no CUDA device available (%s)", cudaGetErrorString(e));
    if (device < 0 || device >= ndev) return fail(IK_ERR_ARG, "device %d out of range (%d devices)", device, ndev);
    ik_ctx* c = new ik_ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess) { delete c; return fail(IK_ERR_CUDA, "cudaSetDevice failed"); }
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, device);
    c->sm_count = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return fail(IK_ERR_CUDA, "cudaStreamCreate failed");
    }
    if (cudaStreamCreateWithFlags(&c->d2h, cudaStreamNonBlocking) != cudaSuccess) {
        cudaStreamDestroy(c->stream);
        delete c;
        return fail(IK_ERR_CUDA, "cudaStreamCreate failed");
    }
    for (auto& ev : c->ev) cudaEventCreate(&ev);
    cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c->d2h_last, cudaEventDisableTiming);
    for (Lane& L : c->lanes) {
        if (cudaStreamCreateWithFlags(&L.st, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&L.last, cudaEventDisableTiming) != cudaSuccess) {
            ik_destroy(c);
            return fail(IK_ERR_CUDA, "stream/event creation failed");
        }
        cudaEventRecord(L.last, L.st);
    }
    c->slots.resize(1);
    int r;
    if ((r = c->status.ensure(sizeof(int))) || (r = c->maxnb.ensure(sizeof(int))) ||
        (r = c->maxnbe.ensure(sizeof(int)))) {
        ik_destroy(c);
        return r;
    }
    for (Lane& L : c->lanes)
        if ((r = L.work_counter.ensure(sizeof(int)))) {
            ik_destroy(c);
            return r;
        }
    cudaMemset(c->status.p, 0, sizeof(int));
    cudaMemset(c->maxnb.p, 0, sizeof(int));
    cudaMemset(c->maxnbe.p, 0, sizeof(int));
    *out = c;
    return IK_OK;
}

int ik_destroy(ik_ctx* c)
{
    if (!c) return IK_OK;
    cudaSetDevice(c->device);
    for (Lane& L : c->lanes) if (L.st) cudaStreamSynchronize(L.st);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->d2h) cudaStreamSynchronize(c->d2h);
    for (auto& ev : c->ev) if (ev) cudaEventDestroy(ev);
    if (c->batch_exec) cudaGraphExecDestroy(c->batch_exec);
    if (c->io_exec) cudaGraphExecDestroy(c->io_exec);
    if (c->fork) cudaEventDestroy(c->fork);
    for (cudaEvent_t e : c->io_ev) cudaEventDestroy(e);
    if (c->d2h_last) cudaEventDestroy(c->d2h_last);
    for (Slot& s : c->slots) {
        if (s.done) cudaEventDestroy(s.done);
        if (s.d2h_done) cudaEventDestroy(s.d2h_done);
    }
    for (Lane& L : c->lanes) {
        if (L.last) cudaEventDestroy(L.last);
        if (L.st) cudaStreamDestroy(L.st);
    }
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->d2h) cudaStreamDestroy(c->d2h);
    delete c;
    return IK_OK;
}

int ik_set_box(ik_ctx* c, int dim, const double boxsize[3], const double origin[3])
{
    if (int r = check_ctx(c)) return r;
    ++c->config_version; // captured batch graphs hold the old settings
    if (dim != 2 && dim != 3) return fail(IK_ERR_ARG, "dim must be 2 or 3 (got %d)", dim);
    if (!boxsize) return fail(IK_ERR_ARG, "null boxsize");
    double b[3] = {boxsize[0], boxsize[1], boxsize[2]};
    double o[3] = {origin ? origin[0] : 0.0, origin ? origin[1] : 0.0, origin ? origin[2] : 0.0};
    if (dim == 2) { b[2] = 1.0; o[2] = 0.0; } // SimBox.cc:34-40
    for (int a = 0; a < dim; ++a)
        if (!(b[a] > 0.0) || !std::isfinite(b[a])) return fail(IK_ERR_ARG, "box edge %d must be > 0 (got %g)", a, b[a]);
    bool same = c->geo.box_set && c->dim == dim;
    for (int a = 0; a < 3 && same; ++a) same = (c->geo.boxsize[a] == b[a] && c->geo.origin[a] == o[a]);
    if (!same) {
        c->dim = dim;
        for (int a = 0; a < 3; ++a) { c->geo.boxsize[a] = b[a]; c->geo.origin[a] = o[a]; }
        c->geo.geom_valid = false;
        c->geo.box_set = true;
        if (c->cg_set) { // the Gaussian normalisation depends on dim
            int r = ik_set_cgfunc(c, c->cg.kind, c->cg.mode, c->cg.order, c->cg.rcut, c->cg_width_param);
            if (r) return r;
        }
    }
    return IK_OK;
}

// Parameter counts and layouts of the reference's models (potential/__init__.py and the
// constructors of potential/*.h): LJ [eps, vareps]; Poly10 [v0, eps, c0, c1, c2, c3];
// PolyYukawa [v0, kappa, eps, c0, c1, c2]; the others [v0, eps, c0, c1, c2].
int ik_potential_nparams(int kind)
{
    switch (kind) {
    case IK_POT_LJ: case IK_POT_FSLJ: return 2;
    case IK_POT_POLY10: case IK_POT_POLYYUKAWA: return 6;
    case IK_POT_POLY12: case IK_POT_POLY106: case IK_POT_POLY18: case IK_POT_POLYLJ: return 5;
    default: return -1;
    }
}

int ik_set_potential(ik_ctx* c, int kind, double scaled_rcut, const double* params, int nparams)
{
    if (int r = check_ctx(c)) return r;
    const int need = ik_potential_nparams(kind);
    if (need < 0) return fail(IK_ERR_ARG, "unknown pair potential kind %d", kind);
    if (!params) return fail(IK_ERR_ARG, "null params");
    if (nparams < need) return fail(IK_ERR_ARG, "pair potential kind %d needs %d parameters (got %d)", kind, need, nparams);
    if (!(scaled_rcut > 0.0) || !std::isfinite(scaled_rcut)) return fail(IK_ERR_ARG, "scaled_rcut must be > 0");
    ++c->config_version; // captured batch graphs hold the old settings
    IkPot p{};
    p.kind = kind;
    p.rcutsq = scaled_rcut * scaled_rcut;
    if (need == 2) {
        p.v0 = params[0];
        p.eps = params[1];
    } else if (kind == IK_POT_POLYYUKAWA) {
        p.v0 = params[0]; p.kappa = params[1]; p.eps = params[2];
        p.c0 = params[3]; p.c1 = params[4]; p.c2 = params[5];
    } else {
        p.v0 = params[0]; p.eps = params[1];
        p.c0 = params[2]; p.c1 = params[3]; p.c2 = params[4];
        if (kind == IK_POT_POLY10) p.c3 = params[5];
    }
    p.max_rcut_sq = c->max_rcut * c->max_rcut;
    c->pot = p;
    c->scaled_rcut = scaled_rcut;
    c->pot_set = true;
    return IK_OK;
}

int ik_set_potential_poly12(ik_ctx* c, double scaled_rcut, const double params[5])
{
    return ik_set_potential(c, IK_POT_POLY12, scaled_rcut, params, 5);
}

int ik_set_cgfunc(ik_ctx* c, int kind, int mode, int order, double rcut, double width)
{
    if (int r = check_ctx(c)) return r;
    ++c->config_version; // captured batch graphs hold the old settings
    if (kind < 0 || kind > 3) return fail(IK_ERR_ARG, "unknown coarse-graining kind %d", kind);
    if (mode < 0 || mode > 4) return fail(IK_ERR_ARG, "unknown quadrature mode %d", mode);
    if (!(rcut > 0.0) || !std::isfinite(rcut)) return fail(IK_ERR_ARG, "rcut must be > 0");
    if (mode == IK_QUAD_MLP && kind != IK_CG_GAUSSIAN)
        return fail(IK_ERR_UNSUPPORTED, "the learned surrogate covers the Gaussian kernel only");
    if (mode == IK_QUAD_CLIPPED && kind != IK_CG_GAUSSIAN)
        return fail(IK_ERR_UNSUPPORTED, "the clipped closed form covers the Gaussian kernel only");
    if ((mode == IK_QUAD_FIXEDPOINT || mode == IK_QUAD_MLP || mode == IK_QUAD_EXACT || mode == IK_QUAD_CLIPPED) &&
        (order < 1 || order > 64))
        return fail(IK_ERR_ARG, "Gauss-Legendre order must be in [1, 64] (got %d)", order);
    if (kind == IK_CG_GAUSSIAN && !(width > 0.0)) return fail(IK_ERR_ARG, "Gaussian width must be > 0");
    const double PI = 3.14159265358979323846;
    int dim = c->dim ? c->dim : 2;
    IkCG& cg = c->cg;
    int old_kind = cg.kind;
    double old_rcut = cg.rcut;
    cg.kind = kind;
    cg.mode = mode;
    cg.order = order;
    cg.rcut = rcut;
    cg.rcutsq = rcut * rcut;
    cg.width = kind == IK_CG_GAUSSIAN ? width : 0.0;
    c->cg_width_param = width;
    switch (kind) {
    case IK_CG_OCTIC: cg.norm = 15.0 / (8 * PI * cg.rcutsq); break;
    case IK_CG_GAUSSIAN: {
        double w2 = width * width;
        cg.norm = dim == 3 ? 1.0 / ((2.0 * PI * w2) * std::sqrt(2.0 * PI * w2)) : 1.0 / (2.0 * PI * w2);
        break;
    }
    case IK_CG_RECT: cg.norm = 1 / (PI * cg.rcutsq); break;
    default: {
        double rn = width > 0.0 ? width : rcut; // Mollifier keeps its construction radius
        cg.mollifier_norm = 13.46842098743079272180855772032086697297031125109170011102 / (2.0 * PI * rn * rn);
        cg.norm = cg.mollifier_norm;
    }
    }
    if (kind == IK_CG_GAUSSIAN) {
        cg.kappa = (float)std::sqrt(1.4426950408889634 / (2.0 * width * width));
        cg.R2s = (float)((double)cg.kappa * cg.kappa * cg.rcutsq);
    } else {
        cg.kappa = (float)(1.0 / rcut);
        cg.R2s = 1.0f;
    }
    if (mode == IK_QUAD_FIXEDPOINT || mode == IK_QUAD_MLP || mode == IK_QUAD_EXACT || mode == IK_QUAD_CLIPPED) {
        // GL-n: the rule itself, the surrogate's (or the clipped closed form's) rule for
        // the bonds inside the support, or (FP64 exact mode) the rule on the clipped
        // interval, at least 5 points (20 for the mollifier)
        IkGL& gl = c->gl;
        if (mode == IK_QUAD_EXACT) order = std::max(order, kind == IK_CG_MOLLIFIER ? 20 : 5);
        gl.n = order;
        gl_rule(order, gl.x, gl.w);
        gl.npairs = order / 2;
        gl.w0 = (order % 2) ? (float)gl.w[order / 2] : 0.f;
        for (int k = 0; k < 32; ++k) { gl.t[k] = 0.f; gl.wt[k] = 0.f; }
        for (int k = 0; k < gl.npairs; ++k) {
            gl.t[k] = (float)gl.x[order - 1 - k];
            gl.wt[k] = (float)gl.w[order - 1 - k];
        }
    }
    if (!c->cg_set || old_kind != kind || old_rcut != rcut) invalidate_geometry(c);
    if (kind == IK_CG_GAUSSIAN) invalidate_geometry(c); // kappa changes gpts
    c->cg_set = true;
    return IK_OK;
}

int ik_set_adaptive(ik_ctx* c, int neval, double relerr, double abserr)
{
    if (int r = check_ctx(c)) return r;
    ++c->config_version; // captured batch graphs hold the old settings
    c->cg.neval = neval;
    c->cg.relerr = relerr;
    c->cg.abserr = abserr;
    return IK_OK;
}

int ik_set_max_rcut(ik_ctx* c, double max_rcut)
{
    if (int r = check_ctx(c)) return r;
    ++c->config_version; // captured batch graphs hold the old settings
    if (!(max_rcut > 0.0) || !std::isfinite(max_rcut)) return fail(IK_ERR_ARG, "max_rcut must be > 0");
    if (!c->max_rcut_set || c->max_rcut != max_rcut) invalidate_geometry(c);
    c->max_rcut = max_rcut;
    c->max_rcut_set = true;
    c->pot.max_rcut_sq = max_rcut * max_rcut;
    return IK_OK;
}

int ik_get_max_rcut(ik_ctx* c, double* out)
{
    if (int r = check_ctx(c)) return r;
    if (!out) return fail(IK_ERR_ARG, "null output");
    if (!c->max_rcut_set) return fail(IK_ERR_STATE, "max_rcut not set yet");
    *out = c->max_rcut;
    return IK_OK;
}

int ik_set_grid(ik_ctx* c, int64_t g, const double* xyz)
{
    if (int r = check_ctx(c)) return r;
    ++c->config_version; // captured batch graphs hold the old settings
    if (g < 0 || (g > 0 && !xyz)) return fail(IK_ERR_ARG, "bad grid arguments");
    if (g > (int64_t)1 << 30) return fail(IK_ERR_UNSUPPORTED, "grid too large");
    for (int64_t i = 0; i < 3 * g; ++i)
        if (!std::isfinite(xyz[i])) return fail(IK_ERR_ARG, "grid coordinate %lld is not finite", (long long)i);
    c->geo.grid_h.assign(xyz, xyz + 3 * g);
    c->geo.G = g;
    ENS(c->geo.grid_d, sizeof(double) * 3 * std::max<int64_t>(g, 1));
    if (g > 0) CK(cudaMemcpy(c->geo.grid_d.p, xyz, sizeof(double) * 3 * g, cudaMemcpyHostToDevice));
    c->geo.geom_valid = false;
    return IK_OK;
}

int ik_set_slot_geometry(ik_ctx* c, int slot, int dim, const double boxsize[3], const double origin[3], int64_t g,
                         const double* xyz)
{
    if (int r = check_ctx(c)) return r;
    if (int r = slot_ok(c, slot)) return r;
    if (dim != 2 && dim != 3) return fail(IK_ERR_ARG, "dim must be 2 or 3 (got %d)", dim);
    if (c->dim != 0 && c->dim != dim) return fail(IK_ERR_ARG, "dim %d differs from the context's %d", dim, c->dim);
    if (!boxsize) return fail(IK_ERR_ARG, "null box");
    for (int a = 0; a < 3; ++a)
        if (!(boxsize[a] > 0.0) || !std::isfinite(boxsize[a])) return fail(IK_ERR_ARG, "box lengths must be > 0");
    if (g < 1 || g > ((int64_t)1 << 30) || !xyz) return fail(IK_ERR_ARG, "bad grid arguments");
    for (int64_t i = 0; i < 3 * g; ++i)
        if (!std::isfinite(xyz[i])) return fail(IK_ERR_ARG, "grid coordinate %lld is not finite", (long long)i);
    Slot& s = c->slots[(size_t)slot];
    if (s.done_recorded) CK(cudaEventSynchronize(s.done)); // the slot's grid may be in use
    if (c->dim == 0) { // the first geometry fixes the context's dimension
        c->dim = dim;
        if (c->cg_set) {
            int r = ik_set_cgfunc(c, c->cg.kind, c->cg.mode, c->cg.order, c->cg.rcut, c->cg_width_param);
            if (r) return r;
        }
    }
    Geo& G = s.geo;
    for (int a = 0; a < 3; ++a) { G.boxsize[a] = boxsize[a]; G.origin[a] = origin ? origin[a] : 0.0; }
    G.box_set = true;
    G.grid_h.assign(xyz, xyz + 3 * g);
    G.G = g;
    ENS(G.grid_d, sizeof(double) * 3 * g);
    CK(cudaMemcpy(G.grid_d.p, xyz, sizeof(double) * 3 * g, cudaMemcpyHostToDevice));
    G.geom_valid = false;
    s.has_geo = true;
    ++c->slot_version;
    ++c->config_version;
    return IK_OK;
}

int ik_reserve_slots(ik_ctx* c, int nslots)
{
    if (int r = check_ctx(c)) return r;
    ++c->config_version; // captured batch graphs hold the old settings
    if (nslots < 1 || nslots > 65536) return fail(IK_ERR_ARG, "nslots out of range");
    if (int r = ik_synchronize(c)) return r;
    if ((int)c->slots.size() < nslots) c->slots.resize((size_t)nslots);
    return IK_OK;
}

// Frame upload from FP64 or FP32 host arrays (FP32: one staging copy, widened on the GPU).
static int upload_impl(ik_ctx* c, int slot, int64_t n, const void* pos, const void* vel, const void* mass,
                       const void* diam, bool f32)
{
    NvtxRange nvr("ik upload");
    if (int r = check_ctx(c)) return r;
    if (int r = slot_ok(c, slot)) return r;
    if (n < 0 || n >= (1 << 25)) return fail(IK_ERR_ARG, "particle count %lld out of range (max 2^25 - 1)", (long long)n);
    if (n > 0 && (!pos || !diam)) return fail(IK_ERR_ARG, "positions and diameters are required");
    if (!c->geo.box_set && !c->slots[(size_t)slot].has_geo)
        return fail(IK_ERR_STATE, "box not set (ik_set_box or ik_set_slot_geometry)");
    double dmax = 0.0;
    if (!c->max_rcut_set) // Calculator.h:41-45 freezes max_rcut from the first frame
        for (int64_t i = 0; i < n; ++i)
            dmax = std::max(dmax, f32 ? (double)((const float*)diam)[i] : ((const double*)diam)[i]);
    Slot& s = c->slots[(size_t)slot];
    if (s.done_recorded) CK(cudaStreamWaitEvent(c->stream, s.done, 0)); // inputs still in use
    const void* old_ptrs[4] = {s.pos.p, s.diam.p, s.vel.p, s.mass.p};
    const bool old_vel = s.has_vel, old_mass = s.has_mass;
    ENS(s.pos, sizeof(double) * 3 * std::max<int64_t>(n, 1));
    ENS(s.diam, sizeof(double) * std::max<int64_t>(n, 1));
    s.has_vel = vel != nullptr;
    s.has_mass = mass != nullptr;
    if (vel) ENS(s.vel, sizeof(double) * 3 * std::max<int64_t>(n, 1));
    if (mass) ENS(s.mass, sizeof(double) * std::max<int64_t>(n, 1));
    if (n > 0 && !f32) {
        CK(cudaMemcpyAsync(s.pos.p, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(s.diam.p, diam, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        if (vel) CK(cudaMemcpyAsync(s.vel.p, vel, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->stream));
        if (mass) CK(cudaMemcpyAsync(s.mass.p, mass, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    } else if (n > 0) { // staging layout: pos 3n | vel 3n | mass n | diam n floats
        ENS(s.stage32, sizeof(float) * 8 * n);
        float* st = s.stage32.as<float>();
        CK(cudaMemcpyAsync(st, pos, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, c->stream));
        if (vel) CK(cudaMemcpyAsync(st + 3 * n, vel, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, c->stream));
        if (mass) CK(cudaMemcpyAsync(st + 6 * n, mass, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(st + 7 * n, diam, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream));
        k_widen_frame<<<(int)((n + 255) / 256), 256, 0, c->stream>>>(st, (int)n, s.pos.as<double>(),
                                                                     vel ? s.vel.as<double>() : nullptr,
                                                                     mass ? s.mass.as<double>() : nullptr,
                                                                     s.diam.as<double>());
        CK(cudaGetLastError());
    }
    if (n > 0) { // device-side validation; reported by ik_synchronize
        k_validate<<<(int)((n + 255) / 256), 256, 0, c->stream>>>(s.pos.as<double>(), s.diam.as<double>(), (int)n,
                                                                  c->dim, c->status.as<int>());
        CK(cudaGetLastError());
    }
    if (s.n != n || old_ptrs[0] != s.pos.p || old_ptrs[1] != s.diam.p || old_ptrs[2] != s.vel.p ||
        old_ptrs[3] != s.mass.p || old_vel != s.has_vel || old_mass != s.has_mass)
        ++c->slot_version; // sizes or buffers changed: captured graphs are stale
    s.n = n;
    s.dmax = dmax;
    if (!c->max_rcut_set && n > 0 && c->pot_set) {
        double m = c->scaled_rcut * dmax;
        ik_set_max_rcut(c, m > dmax ? m : dmax); // Calculator.h:41-45
    }
    return IK_OK;
}

int ik_upload_frame(ik_ctx* c, int slot, int64_t n, const double* pos, const double* vel, const double* mass,
                    const double* diam)
{
    return upload_impl(c, slot, n, pos, vel, mass, diam, false);
}

int ik_upload_frame_f32(ik_ctx* c, int slot, int64_t n, const float* pos, const float* vel, const float* mass,
                        const float* diam)
{
    return upload_impl(c, slot, n, pos, vel, mass, diam, true);
}

int ik_upload_displacement(ik_ctx* c, int slot, int64_t n, const double* disp)
{
    if (int r = check_ctx(c)) return r;
    if (int r = slot_ok(c, slot)) return r;
    Slot& s = c->slots[(size_t)slot];
    if (n != s.n) return fail(IK_ERR_ARG, "displacements for %lld particles, the slot holds %lld", (long long)n, (long long)s.n);
    if (n > 0 && !disp) return fail(IK_ERR_ARG, "null displacements");
    for (int64_t i = 0; i < 3 * n; ++i)
        if (!std::isfinite(disp[i])) return fail(IK_ERR_ARG, "displacement %lld is not finite", (long long)(i / 3));
    if (s.done_recorded) CK(cudaStreamWaitEvent(c->stream, s.done, 0)); // the old ones may be in use
    const void* old = s.disp.p;
    ENS(s.disp, sizeof(double) * 3 * std::max<int64_t>(n, 1));
    if (n > 0) CK(cudaMemcpyAsync(s.disp.p, disp, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->stream));
    if (!s.has_disp || old != s.disp.p) ++c->slot_version; // captured graphs hold the old buffer
    s.has_disp = true;
    return IK_OK;
}

int ik_set_frame(ik_ctx* c, int64_t n, const double* pos, const double* vel, const double* mass,
                 const double* diam)
{
    return ik_upload_frame(c, 0, n, pos, vel, mass, diam);
}

int ik_compute_slot(ik_ctx* c, int slot, int precision, int fields)
{
    if (int r = check_ctx(c)) return r;
    if (int r = slot_ok(c, slot)) return r;
    if (precision != IK_PREC_FP64 && precision != IK_PREC_FP32) return fail(IK_ERR_ARG, "unknown precision %d", precision);
    if (fields < 1 || fields > 7) return fail(IK_ERR_ARG, "fields mask must be in [1, 7]");
    c->pending.push_back({slot, precision, fields});
    if (int r = prepare_enqueue(c, slot, precision, fields)) { c->pending.pop_back(); return r; }
    return IK_OK;
}

int ik_compute_batch(ik_ctx* c, const int* slots, int count, int precision, int fields)
{
    NvtxRange nvr("ik compute_batch");
    if (int r = check_ctx(c)) return r;
    if (count < 1 || !slots) return fail(IK_ERR_ARG, "empty batch");
    for (int k = 0; k < count; ++k) if (int r = slot_ok(c, slots[k])) return r;
    if (precision != IK_PREC_FP64 && precision != IK_PREC_FP32) return fail(IK_ERR_ARG, "unknown precision %d", precision);
    if (fields < 1 || fields > 7) return fail(IK_ERR_ARG, "fields mask must be in [1, 7]");
    for (int k = 0; k < count; ++k) { // every slot ready, its geometry current
        GeoSwap gs(c, slots[k]);
        if (int r = ensure_ready(c)) return r;
        if (int r = mode_ok(c, precision)) return r;
        if (int r = ensure_geometry(c)) return r;
    }
    if (c->maxb == 0) c->maxb = c->dim == 2 ? IK_MAXB_2D : IK_MAXB_3D;
    if (c->halo_cap == 0) c->halo_cap = 384; // staged particles per warp (grows on overflow)
    std::vector<int> key(slots, slots + count);
    const bool reuse = c->batch_exec && key == c->batch_slots && c->batch_prec == precision &&
                       c->batch_fields == fields && c->batch_maxb == c->maxb && c->batch_halo == c->halo_cap &&
                       c->batch_maxbe == c->maxbe &&
                       c->batch_geom_version == c->geom_version && c->batch_slot_version == c->slot_version &&
                       c->batch_config_version == c->config_version && c->batch_alloc_epoch == g_alloc_epoch.load() &&
                       !(c->flags & IK_FLAG_TIMING);
    if (!reuse) {
        // first run of this batch: plain launches (sizes every buffer, checks capacities);
        // frames take the lanes from lane 0 here and in the capture, so that the capture
        // finds every buffer it uses sized (an allocation there leaves the graph unused)
        c->next_lane = 0;
        c->in_batch = true;
        for (int k = 0; k < count; ++k) {
            c->pending.push_back({slots[k], precision, fields});
            if (int r = prepare_enqueue(c, slots[k], precision, fields)) { c->in_batch = false; return r; }
        }
        c->in_batch = false;
        if (int r = ik_synchronize(c)) return r;
        if (c->flags & IK_FLAG_TIMING) return IK_OK;
        // then capture the batch as one graph: fused (every stage once over the batch) where
        // eligible, else the same per-frame sequence (lanes fork from and join the main stream)
        const bool fused = fused_eligible(c, key, precision, fields);
        if (fused) {
            if (int r = fused_build(c, key, c->fused)) return r;
        }
        if (c->batch_exec) { cudaGraphExecDestroy(c->batch_exec); c->batch_exec = nullptr; }
        if (c->io_exec) { cudaGraphExecDestroy(c->io_exec); c->io_exec = nullptr; } // versions below are ours now
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
        const int64_t launches_before = c->launches;
        const int64_t epoch_before = g_alloc_epoch.load();
        c->capturing = true;
        c->captured_lanes = 0;
        int rr = IK_OK;
        c->next_lane = 0;
        c->in_batch = true;
        if (fused) rr = fused_enqueue(c, c->fused, fields, c->stream);
        for (int k = 0; k < count && rr == IK_OK && !fused; ++k) rr = prepare_enqueue(c, slots[k], precision, fields);
        c->in_batch = false;
        for (int l = 0; l < IK_LANES && rr == IK_OK; ++l)
            if (c->captured_lanes & (1 << l)) {
                if (cudaEventRecord(c->lanes[l].last, c->lanes[l].st) != cudaSuccess ||
                    cudaStreamWaitEvent(c->stream, c->lanes[l].last, 0) != cudaSuccess)
                    rr = fail(IK_ERR_CUDA, "joining a lane during capture failed");
            }
        c->capturing = false;
        c->batch_launches = c->launches - launches_before;
        c->launches = launches_before; // captured, not launched
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
        if (rr != IK_OK) { if (graph) cudaGraphDestroy(graph); return rr; }
        if (e != cudaSuccess) return fail(IK_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&c->batch_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) { c->batch_exec = nullptr; return fail(IK_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e)); }
        c->batch_slots = key;
        c->batch_fused = fused;
        c->batch_prec = precision;
        c->batch_fields = fields;
        c->batch_maxb = c->maxb;
        c->batch_halo = c->halo_cap;
        c->batch_maxbe = c->maxbe;
        c->batch_geom_version = c->geom_version;
        c->batch_slot_version = c->slot_version;
        c->batch_config_version = c->config_version;
        // an allocation during the capture (none is expected) leaves the graph unused
        c->batch_alloc_epoch = g_alloc_epoch.load() == epoch_before ? epoch_before : -2;
        return IK_OK; // the first call's results come from the plain launches
    }
    // replay: after everything already enqueued on the lanes and the slots' downloads
    if (int r = ik_wait_all(c)) return r;
    for (int k = 0; k < count; ++k) {
        Slot& s = c->slots[(size_t)slots[k]];
        if (s.d2h_recorded) CK(cudaStreamWaitEvent(c->stream, s.d2h_done, 0));
    }
    for (int k = 0; k < count; ++k) c->pending.push_back({slots[k], precision, fields});
    CK(cudaGraphLaunch(c->batch_exec, c->stream));
    for (int k = 0; k < count; ++k) {
        Slot& s = c->slots[(size_t)slots[k]];
        CK(cudaEventRecord(s.done, c->stream));
        s.done_recorded = true;
        s.last_prec = precision;
        s.last_fields = fields;
    }
    c->launches += c->batch_launches;
    return IK_OK;
}

int ik_time_fused_batch(ik_ctx* c, const int* slots, int count, int fields, float* ms4)
{
    NvtxRange nvr("ik time_fused_batch");
    if (int r = check_ctx(c)) return r;
    if (count < 1 || !slots || !ms4) return fail(IK_ERR_ARG, "empty batch or null output");
    for (int k = 0; k < count; ++k) if (int r = slot_ok(c, slots[k])) return r;
    for (int k = 0; k < count; ++k) {
        GeoSwap gs(c, slots[k]);
        if (int r = ensure_ready(c)) return r;
        if (int r = mode_ok(c, IK_PREC_FP32)) return r;
        if (int r = ensure_geometry(c)) return r;
    }
    if (c->maxb == 0) c->maxb = c->dim == 2 ? IK_MAXB_2D : IK_MAXB_3D;
    if (c->halo_cap == 0) c->halo_cap = 384;
    std::vector<int> key(slots, slots + count);
    // eligibility of the batch itself, whatever the timing flag and the schedule setting
    const int saved_flags = c->flags, saved_fused = c->tune_fused;
    c->flags &= ~IK_FLAG_TIMING;
    c->tune_fused = 1;
    const bool ok = fused_eligible(c, key, IK_PREC_FP32, fields);
    c->flags = saved_flags;
    c->tune_fused = saved_fused;
    if (!ok) return fail(IK_ERR_UNSUPPORTED, "this batch cannot run fused");
    if (int r = ik_wait_all(c)) return r;
    if (int r = fused_build(c, key, c->fused)) return r;
    ++c->config_version; // the fused buffers were rebuilt: a recorded batch graph re-records
    for (int k = 0; k < count; ++k) c->pending.push_back({slots[k], IK_PREC_FP32, fields});
    if (int r = fused_enqueue(c, c->fused, fields, c->stream, true)) return r;
    if (int r = ik_synchronize(c)) return r;
    CK(cudaEventElapsedTime(&ms4[0], c->ev[0], c->ev[1]));
    CK(cudaEventElapsedTime(&ms4[1], c->ev[1], c->ev[2]));
    CK(cudaEventElapsedTime(&ms4[2], c->ev[2], c->ev[3]));
    CK(cudaEventElapsedTime(&ms4[3], c->ev[0], c->ev[3]));
    return IK_OK;
}

static bool host_pinned(const void* p)
{
    if (!p) return true;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

int ik_compute_batch_io(ik_ctx* c, const int* slots, int count, int precision, int fields, const int64_t* n,
                        const double* const* pos, const double* const* vel, const double* const* mass,
                        const double* const* diam, double* const* out)
{
    NvtxRange nvr("ik compute_batch_io");
    if (int r = check_ctx(c)) return r;
    if (count < 1 || !slots || !n || !pos || !diam || !out) return fail(IK_ERR_ARG, "empty batch or null array");
    if (precision != IK_PREC_FP64 && precision != IK_PREC_FP32) return fail(IK_ERR_ARG, "unknown precision %d", precision);
    if (fields < 1 || fields > 7) return fail(IK_ERR_ARG, "fields mask must be in [1, 7]");
    std::vector<IoFrame> fr((size_t)count);
    std::vector<int64_t> key;
    key.reserve((size_t)count * 9 + 2);
    key.push_back(precision);
    key.push_back(fields);
    for (int k = 0; k < count; ++k) {
        if (int r = slot_ok(c, slots[k])) return r;
        for (int j = 0; j < k; ++j)
            if (slots[j] == slots[k]) return fail(IK_ERR_ARG, "slot %d appears twice in the batch", slots[k]);
        if (n[k] < 0 || n[k] >= (1 << 25)) return fail(IK_ERR_ARG, "particle count %lld out of range", (long long)n[k]);
        IoFrame& f = fr[(size_t)k];
        f.pos = pos[k];
        f.diam = diam[k];
        f.vel = vel ? vel[k] : nullptr;
        f.mass = mass ? mass[k] : nullptr;
        for (int q = 0; q < 3; ++q) f.out[q] = (fields & (1 << q)) ? out[3 * k + q] : nullptr;
        if (n[k] > 0 && (!f.pos || !f.diam)) return fail(IK_ERR_ARG, "frame %d: positions and diameters are required", k);
        const void* ptrs[7] = {f.pos, f.diam, f.vel, f.mass, f.out[0], f.out[1], f.out[2]};
        key.push_back(slots[k]);
        key.push_back(n[k]);
        for (const void* p : ptrs) key.push_back((int64_t)(intptr_t)p);
    }
    if (key != c->io_key) // new buffers: page-locked? (checked once per set of buffers)
        for (int k = 0; k < count; ++k) {
            const IoFrame& f = fr[(size_t)k];
            const void* ptrs[7] = {f.pos, f.diam, f.vel, f.mass, f.out[0], f.out[1], f.out[2]};
            for (const void* p : ptrs)
                if (!host_pinned(p)) return fail(IK_ERR_ARG, "frame %d: host buffers must be page-locked", k);
        }
    const bool reuse = c->io_exec && key == c->io_key && c->batch_maxb == c->maxb && c->batch_halo == c->halo_cap &&
                       c->batch_maxbe == c->maxbe && c->batch_geom_version == c->geom_version &&
                       c->batch_slot_version == c->slot_version && c->batch_config_version == c->config_version &&
                       c->batch_alloc_epoch == g_alloc_epoch.load() && !(c->flags & IK_FLAG_TIMING);
    if (!reuse) {
        // plain path: uploads (sizes every buffer), computations, capacity checks, downloads
        for (int k = 0; k < count; ++k) {
            const IoFrame& f = fr[(size_t)k];
            if (int r = ik_upload_frame(c, slots[k], n[k], f.pos, f.vel, f.mass, f.diam)) return r;
        }
        c->next_lane = 0; // the same lanes here and in the capture (see ik_compute_batch)
        c->in_batch = true;
        for (int k = 0; k < count; ++k) {
            c->pending.push_back({slots[k], precision, fields});
            if (int r = prepare_enqueue(c, slots[k], precision, fields)) { c->in_batch = false; return r; }
        }
        c->in_batch = false;
        if (int r = ik_synchronize(c)) return r;
        for (int k = 0; k < count; ++k) {
            int64_t G = 0;
            { GeoSwap gs(c, slots[k]); G = c->geo.G; }
            for (int q = 0; q < 3; ++q)
                if (fr[(size_t)k].out[q])
                    if (int r = ik_download_field_async(c, slots[k], 1 << q, fr[(size_t)k].out[q], G * (c->dim == 2 ? 3 : 6)))
                        return r;
        }
        if (int r = ik_synchronize(c)) return r;
        if (c->flags & IK_FLAG_TIMING) return IK_OK;
        // record: an eligible batch as fused sub-batches whose copies overlap each other's
        // computation, else per frame on its lane, host -> device copies, the kernels,
        // device -> host
        const bool fused =
            c->tune_io_batches > 0 && fused_eligible(c, std::vector<int>(slots, slots + count), precision, fields);
        std::vector<int> cut;
        bool mapped = false;
        if (fused) {
            cut = io_split(c, slots, count);
            const int nsub = (int)cut.size() - 1;
            if ((int)c->fused_io.size() < nsub) c->fused_io.resize((size_t)nsub);
            for (int b = 0; b < nsub; ++b)
                if (int r = fused_build(c, std::vector<int>(slots + cut[(size_t)b], slots + cut[(size_t)b + 1]),
                                        c->fused_io[(size_t)b]))
                    return r;
            if (int r = io_events(c, 2 * nsub)) return r;
            int err = IK_OK;
            mapped = c->tune_io_mapped && io_build_mapped(c, slots, fr, cut, fields, &err);
            if (err) return err;
        }
        if (c->io_exec) { cudaGraphExecDestroy(c->io_exec); c->io_exec = nullptr; }
        if (c->batch_exec) { cudaGraphExecDestroy(c->batch_exec); c->batch_exec = nullptr; } // versions below are ours now
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
        const int64_t launches_before = c->launches;
        const int64_t epoch_before = g_alloc_epoch.load();
        c->capturing = true;
        c->captured_lanes = 0;
        int rr = IK_OK;
        c->next_lane = 0;
        c->in_batch = true;
        if (fused) rr = fused_io_enqueue(c, slots, fr, cut, fields, mapped);
        for (int k = 0; k < count && rr == IK_OK && !fused; ++k) {
            c->io_cur = &fr[(size_t)k];
            rr = prepare_enqueue(c, slots[k], precision, fields);
        }
        c->io_cur = nullptr;
        c->in_batch = false;
        for (int l = 0; l < IK_LANES && rr == IK_OK; ++l)
            if (c->captured_lanes & (1 << l)) {
                if (cudaEventRecord(c->lanes[l].last, c->lanes[l].st) != cudaSuccess ||
                    cudaStreamWaitEvent(c->stream, c->lanes[l].last, 0) != cudaSuccess)
                    rr = fail(IK_ERR_CUDA, "joining a lane during capture failed");
            }
        c->capturing = false;
        c->io_launches = c->launches - launches_before;
        c->launches = launches_before;
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
        if (rr != IK_OK) { if (graph) cudaGraphDestroy(graph); return rr; }
        if (e != cudaSuccess) return fail(IK_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&c->io_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) { c->io_exec = nullptr; return fail(IK_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e)); }
        c->io_key = key;
        c->io_fused = fused;
        c->io_mapped = mapped;
        c->batch_maxb = c->maxb;
        c->batch_halo = c->halo_cap;
        c->batch_maxbe = c->maxbe;
        c->batch_geom_version = c->geom_version;
        c->batch_slot_version = c->slot_version;
        c->batch_config_version = c->config_version;
        c->batch_alloc_epoch = g_alloc_epoch.load() == epoch_before ? epoch_before : -2;
        return IK_OK; // the first call's results come from the plain path
    }
    // replay after everything already enqueued and every download of these slots
    if (int r = ik_wait_all(c)) return r;
    for (int k = 0; k < count; ++k) {
        Slot& s = c->slots[(size_t)slots[k]];
        if (s.d2h_recorded) CK(cudaStreamWaitEvent(c->stream, s.d2h_done, 0));
    }
    for (int k = 0; k < count; ++k) {
        PendingOp op{slots[k], precision, fields};
        for (int q = 0; q < 3; ++q) op.out[q] = fr[(size_t)k].out[q];
        c->pending.push_back(op);
    }
    CK(cudaGraphLaunch(c->io_exec, c->stream));
    for (int k = 0; k < count; ++k) {
        Slot& s = c->slots[(size_t)slots[k]];
        CK(cudaEventRecord(s.done, c->stream));
        s.done_recorded = true;
        s.last_prec = precision;
        s.last_fields = fields;
    }
    c->launches += c->io_launches;
    return IK_OK;
}

int ik_synchronize(ik_ctx* c)
{
    NvtxRange nvr("ik synchronize");
    if (int r = check_ctx(c)) return r;
    for (int attempt = 0; attempt < 4; ++attempt) {
        for (Lane& L : c->lanes) CK(cudaStreamSynchronize(L.st));
        CK(cudaStreamSynchronize(c->stream));
        CK(cudaStreamSynchronize(c->d2h));
        int st = 0, mx = 0;
        CK(cudaMemcpy(&st, c->status.p, sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(&mx, c->maxnb.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (st == 0) { c->pending.clear(); return IK_OK; }
        CK(cudaMemset(c->status.p, 0, sizeof(int)));
        if (st & IK_ST_BAD_INPUT) {
            c->pending.clear();
            return fail(IK_ERR_ARG, "invalid frame: a position is not finite, a diameter is not > 0, or a 2D "
                                    "frame has z != 0");
        }
        bool grow = false;
        if (st & IK_ST_BOND_OVERFLOW) {
            int mxe = 0;
            CK(cudaMemcpy(&mxe, c->maxnbe.p, sizeof(int), cudaMemcpyDeviceToHost));
            if (mx > c->maxb) {
                if (mx > IK_MAXB_LIMIT) { c->pending.clear(); return fail(IK_ERR_CAPACITY, "a particle has %d force-active bonds (max %d)", mx, IK_MAXB_LIMIT); }
                c->maxb = mx;
            }
            if (mxe > c->maxbe) {
                if (mxe > IK_MAXB_LIMIT) { c->pending.clear(); return fail(IK_ERR_CAPACITY, "a particle has %d neighbours within max_rcut (max %d for the elastic field)", mxe, IK_MAXB_LIMIT); }
                c->maxbe = mxe;
            }
            grow = true;
        }
        if (st & IK_ST_MMA_TIMEOUT) { c->pending.clear(); return fail(IK_ERR_TIMEOUT, "a tensor-core wait gave up"); }
        if (st & IK_ST_BOND_RANGE) {
            c->pending.clear();
            return fail(IK_ERR_CAPACITY, "a frame has 2^25 or more force-active bond records, more than the FP32 "
                                         "gather addresses; use the FP64 path or smaller frames");
        }
        if (st & IK_ST_QUAD_FAIL) {
            c->pending.clear();
            return fail(IK_ERR_QUADRATURE, "adaptive bond integral: tolerance not met within %d subintervals",
                        std::min(std::max(c->cg.neval, 1), IK_QAG_MAXSUB));
        }
        if (st & IK_ST_MLP_OVERFLOW) {
            if (c->mlp_cap >= (1LL << 31)) { c->pending.clear(); return fail(IK_ERR_CAPACITY, "surrogate record buffer cannot grow"); }
            c->mlp_cap *= 2;
            grow = true;
        }
        if (st & IK_ST_HALO_OVERFLOW) {
            // the per-warp stage lives in the CTA's dynamic shared memory (227 KB at most)
            const int qcap = 32 * (std::min(std::max(c->maxb, c->maxbe), 63) + 1);
            const int limit = (int)((227 * 1024 / IK_WARPS_GATHER - 4 * qcap - 64) / 20) & ~31;
            if (c->halo_cap >= limit) { c->pending.clear(); return fail(IK_ERR_CAPACITY, "a cell holds more particles than the halo buffer (%d)", c->halo_cap); }
            c->halo_cap = std::min(2 * c->halo_cap, limit);
            grow = true;
        }
        if (!grow) { c->pending.clear(); return fail(IK_ERR_CUDA, "device status 0x%x", st); }
        std::vector<PendingOp> ops = c->pending;
        for (const PendingOp& op : ops) {
            if (int r = prepare_enqueue(c, op.slot, op.prec, op.fields)) { c->pending.clear(); return r; }
            // downloads of the first attempt copied an incomplete result: copy again
            for (int f = 0; f < 3; ++f)
                if (op.out[f]) {
                    int64_t G = 0;
                    { GeoSwap gs(c, op.slot); G = c->geo.G; }
                    if (int r = ik_download_field_async(c, op.slot, 1 << f, op.out[f], G * (c->dim == 2 ? 3 : 6))) {
                        c->pending.clear();
                        return r;
                    }
                }
        }
    }
    c->pending.clear();
    return fail(IK_ERR_CAPACITY, "capacity growth did not converge");
}

int ik_compute(ik_ctx* c, int precision, int fields)
{
    if (int r = ik_compute_slot(c, 0, precision, fields)) return r;
    return ik_synchronize(c);
}

int ik_get_field(ik_ctx* c, int slot, int field, double* out, int64_t count)
{
    NvtxRange nvr("ik download");
    if (int r = check_ctx(c)) return r;
    if (int r = slot_ok(c, slot)) return r;
    GeoSwap gs(c, slot);
    if (field != IK_FIELD_VIRIAL && field != IK_FIELD_KINETIC && field != IK_FIELD_ELASTIC)
        return fail(IK_ERR_ARG, "unknown field %d", field);
    if (int r = ik_synchronize(c)) return r;
    Slot& s = c->slots[(size_t)slot];
    if (s.last_prec < 0) return fail(IK_ERR_STATE, "slot %d has not been computed", slot);
    const int D = c->dim, NC = D == 2 ? 3 : 6;
    if (count != c->geo.G * D * D) return fail(IK_ERR_ARG, "output needs %lld doubles (got %lld)", (long long)(c->geo.G * D * D), (long long)count);
    std::vector<double> tmp((size_t)(NC * c->geo.G));
    const DevBuf& src = field == IK_FIELD_VIRIAL ? s.vir : (field == IK_FIELD_KINETIC ? s.kin : s.ela);
    if (c->geo.G > 0) CK(cudaMemcpy(tmp.data(), src.p, sizeof(double) * NC * c->geo.G, cudaMemcpyDeviceToHost));
    static const int map2[3][2] = {{0, 0}, {1, 1}, {0, 1}};
    static const int map3[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
    for (int64_t g = 0; g < c->geo.G; ++g) {
        double* o = out + g * D * D;
        for (int k = 0; k < NC; ++k) {
            int a = D == 2 ? map2[k][0] : map3[k][0], b = D == 2 ? map2[k][1] : map3[k][1];
            double v = tmp[(size_t)(g * NC + k)];
            o[a + D * b] = v;
            o[b + D * a] = v;
        }
    }
    return IK_OK;
}

// Cell grid of cut-off `radius` over the current box (ik_get_neighbors, ik_compute_thermo).
static int query_geometry(ik_ctx* c, double radius, IkGeom& g)
{
    g = IkGeom{};
    g.dim = c->dim;
    for (int a = 0; a < 3; ++a) {
        g.L[a] = c->geo.boxsize[a];
        g.lo[a] = -0.5 * c->geo.boxsize[a] - c->geo.origin[a];
        g.periodic[a] = nc_of(c->dim, a);
        int nc = 1;
        if (g.periodic[a]) {
            if (!(2.0 * radius < g.L[a])) return fail(IK_ERR_BOX, "radius %g >= half the box edge %g", radius, g.L[a]);
            nc = std::max(1, (int)std::floor(g.L[a] / radius));
        }
        g.nc[a] = nc;
        g.cw[a] = g.L[a] / nc;
        g.invL[a] = 1.0 / g.L[a];
        g.reach_bond[a] = 1;
        g.all_bond[a] = nc < 3 ? 1 : 0;
    }
    g.ncell = g.nc[0] * g.nc[1] * g.nc[2];
    return IK_OK;
}

int ik_compute_thermo(ik_ctx* c, int slot, double* out, int64_t count)
{
    if (int r = check_ctx(c)) return r;
    if (int r = slot_ok(c, slot)) return r;
    GeoSwap gs(c, slot);
    if (!c->geo.box_set) return fail(IK_ERR_STATE, "box not set");
    if (!c->pot_set) return fail(IK_ERR_STATE, "pair potential not set");
    if (!c->max_rcut_set) return fail(IK_ERR_STATE, "max_rcut unknown: upload a frame or call ik_set_max_rcut");
    const int D = c->dim, D2 = D * D;
    const int64_t need = 1 + 3 * D2 + D2 * D2;
    if (!out || count < need) return fail(IK_ERR_ARG, "output needs %lld values", (long long)need);
    Slot& s = c->slots[(size_t)slot];
    const int n = (int)s.n;
    IkGeom g;
    if (int r = query_geometry(c, c->max_rcut, g)) return r;
    if (s.done_recorded) CK(cudaStreamWaitEvent(c->stream, s.done, 0));
    if (int r = build_cells(c, s, g, c->stream, c->q_cell_of, c->q_rank, c->q_count, c->q_start, c->q_sorted,
                            c->bsum_q))
        return r;
    if (g.ncell > 0)
        k_cell_sort_pack<<<(g.ncell + 127) / 128, 128, 0, c->stream>>>(g, c->q_start.as<int>(), c->q_sorted.as<int>(),
                                                                       nullptr, nullptr, nullptr, nullptr, nullptr,
                                                                       nullptr, nullptr, 0);
    const int nq = ik_thermo_nq(D), nblocks = (n + 127) / 128;
    ENS(c->th_partial, sizeof(double) * (size_t)nq * std::max(nblocks, 1));
    ENS(c->th_out, sizeof(double) * nq);
    const double vol = D == 2 ? g.L[0] * g.L[1] : g.L[0] * g.L[1] * g.L[2]; // SimBox.cc:15-22
    IkPot pot = c->pot;
    pot.max_rcut_sq = c->max_rcut * c->max_rcut;
    CK(launch_thermo64(g, pot, n, c->q_sorted.as<int>(), c->q_cell_of.as<int>(), s.pos.as<double>(),
                       s.has_vel ? s.vel.as<double>() : nullptr, s.has_mass ? s.mass.as<double>() : nullptr,
                       s.diam.as<double>(), s.has_disp ? s.disp.as<double>() : nullptr, c->q_start.as<int>(),
                       c->th_partial.as<double>(), nblocks, 1 / vol, c->th_out.as<double>(), c->stream));
    c->launches += (g.ncell > 0 ? 1 : 0) + (nblocks > 0 ? 1 : 0) + 1;
    std::vector<double> h((size_t)nq);
    CK(cudaMemcpyAsync(h.data(), c->th_out.p, sizeof(double) * nq, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    // {energy, virial, elastic, kinetic} as they are; the Born tensor from its symmetric
    // components (enumerated i <= j <= k <= l as on the device)
    for (int k = 0; k < 1 + 3 * D2; ++k) out[k] = h[(size_t)k];
    int sym[3][3][3][3];
    int u = 1 + 3 * D2;
    for (int a = 0; a < D; ++a)
        for (int b = a; b < D; ++b)
            for (int k = b; k < D; ++k)
                for (int l = k; l < D; ++l) sym[a][b][k][l] = u++;
    for (int l = 0; l < D; ++l)
        for (int k = 0; k < D; ++k)
            for (int j = 0; j < D; ++j)
                for (int i = 0; i < D; ++i) {
                    int t[4] = {i, j, k, l};
                    std::sort(t, t + 4);
                    out[1 + 3 * D2 + i + D * (j + D * (k + D * l))] = h[(size_t)sym[t[0]][t[1]][t[2]][t[3]]];
                }
    return IK_OK;
}

int ik_get_neighbors(ik_ctx* c, int slot, double radius, int64_t* offs, int32_t* idx, int64_t idx_capacity,
                     int64_t* nnz)
{
    if (int r = check_ctx(c)) return r;
    if (int r = slot_ok(c, slot)) return r;
    GeoSwap gs(c, slot);
    if (!c->geo.box_set) return fail(IK_ERR_STATE, "box not set");
    if (!(radius > 0.0)) return fail(IK_ERR_ARG, "radius must be > 0");
    if (!offs || !nnz) return fail(IK_ERR_ARG, "null output");
    Slot& s = c->slots[(size_t)slot];
    int n = (int)s.n;
    IkGeom g;
    if (int r = query_geometry(c, radius, g)) return r;
    if (s.done_recorded) CK(cudaStreamWaitEvent(c->stream, s.done, 0));
    if (int r = build_cells(c, s, g, c->stream, c->q_cell_of, c->q_rank, c->q_count, c->q_start, c->q_sorted,
                            c->bsum_q))
        return r;
    if (g.ncell > 0)
        k_cell_sort_pack<<<(g.ncell + 127) / 128, 128, 0, c->stream>>>(g, c->q_start.as<int>(), c->q_sorted.as<int>(),
                                                                       nullptr, nullptr, nullptr, nullptr, nullptr,
                                                                       nullptr, nullptr, 0);
    ENS(c->q_cnt, sizeof(int) * (n + 1));
    ENS(c->q_offs, sizeof(int) * (n + 1));
    double r2 = radius * radius;
    CK(launch_neigh(false, g, n, r2, c->q_sorted.as<int>(), c->q_cell_of.as<int>(), s.pos.as<double>(),
                    c->q_start.as<int>(), c->q_cnt.as<int>(), nullptr, nullptr, c->stream));
    k_scan<<<1, 1024, 0, c->stream>>>(c->q_cnt.as<int>(), n, c->q_offs.as<int>());
    std::vector<int> ho((size_t)n + 1);
    CK(cudaMemcpyAsync(ho.data(), c->q_offs.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    int64_t total = ho[(size_t)n];
    *nnz = total;
    for (int i = 0; i <= n; ++i) offs[i] = ho[(size_t)i];
    if (!idx) return IK_OK;
    if (idx_capacity < total) return fail(IK_ERR_ARG, "idx capacity %lld < %lld", (long long)idx_capacity, (long long)total);
    ENS(c->q_idx, sizeof(int) * std::max<int64_t>(total, 1));
    CK(launch_neigh(true, g, n, r2, c->q_sorted.as<int>(), c->q_cell_of.as<int>(), s.pos.as<double>(),
                    c->q_start.as<int>(), nullptr, c->q_offs.as<int>(), c->q_idx.as<int>(), c->stream));
    if (total > 0) CK(cudaMemcpyAsync(idx, c->q_idx.p, sizeof(int) * total, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return IK_OK;
}

int ik_get_neighbors_point(ik_ctx* c, int slot, const double point[3], double radius, int32_t* ids,
                           int64_t capacity, int64_t* count)
{
    if (int r = check_ctx(c)) return r;
    if (int r = slot_ok(c, slot)) return r;
    GeoSwap gs(c, slot);
    if (!c->geo.box_set) return fail(IK_ERR_STATE, "box not set");
    if (!point || !count) return fail(IK_ERR_ARG, "null argument");
    Slot& s = c->slots[(size_t)slot];
    int n = (int)s.n;
    IkGeom g{};
    g.dim = c->dim;
    for (int a = 0; a < 3; ++a) {
        g.L[a] = c->geo.boxsize[a];
        g.lo[a] = -0.5 * c->geo.boxsize[a] - c->geo.origin[a];
        g.periodic[a] = nc_of(c->dim, a);
    }
    ENS(c->q_flag, std::max(n, 1));
    if (n > 0) {
        k_point_query<<<(n + 255) / 256, 256, 0, c->stream>>>(g, n, s.pos.as<double>(), point[0], point[1], point[2],
                                                             radius * radius, c->q_flag.as<unsigned char>());
        CK(cudaGetLastError());
    }
    std::vector<unsigned char> f((size_t)std::max(n, 1));
    if (n > 0) CK(cudaMemcpyAsync(f.data(), c->q_flag.p, n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    int64_t k = 0;
    for (int i = 0; i < n; ++i)
        if (f[(size_t)i]) {
            if (ids && k < capacity) ids[k] = i;
            ++k;
        }
    *count = k;
    if (ids && k > capacity) return fail(IK_ERR_ARG, "capacity %lld < %lld", (long long)capacity, (long long)k);
    return IK_OK;
}

int ik_eval_pair(ik_ctx* c, int64_t m, const double* rij, const double* di, const double* dj, double* force_divr,
                 double* energy)
{
    if (int r = check_ctx(c)) return r;
    if (!c->pot_set) return fail(IK_ERR_STATE, "pair potential not set");
    if (m < 0 || (m > 0 && (!rij || !di || !dj || !force_divr || !energy))) return fail(IK_ERR_ARG, "bad arguments");
    if (m == 0) return IK_OK;
    DevBuf b;
    ENS(b, sizeof(double) * 7 * m);
    double* d = b.as<double>();
    CK(cudaMemcpyAsync(d, rij, sizeof(double) * 3 * m, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(d + 3 * m, di, sizeof(double) * m, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(d + 4 * m, dj, sizeof(double) * m, cudaMemcpyHostToDevice, c->stream));
    k_eval_pair<<<(int)((m + 127) / 128), 128, 0, c->stream>>>(c->pot, (int)m, d, d + 3 * m, d + 4 * m, d + 5 * m,
                                                                d + 6 * m);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(force_divr, d + 5 * m, sizeof(double) * m, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(energy, d + 6 * m, sizeof(double) * m, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return IK_OK;
}

int ik_eval_bond(ik_ctx* c, int64_t m, const double* x, const double* ri, const double* rij, double* bond,
                 double* delta)
{
    if (int r = check_ctx(c)) return r;
    if (!c->cg_set) return fail(IK_ERR_STATE, "coarse-graining function not set");
    if (m < 0 || (m > 0 && (!x || !ri || !rij || !bond || !delta))) return fail(IK_ERR_ARG, "bad arguments");
    if (m == 0) return IK_OK;
    DevBuf b;
    ENS(b, sizeof(double) * 11 * m);
    double* d = b.as<double>();
    CK(cudaMemcpyAsync(d, x, sizeof(double) * 3 * m, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(d + 3 * m, ri, sizeof(double) * 3 * m, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(d + 6 * m, rij, sizeof(double) * 3 * m, cudaMemcpyHostToDevice, c->stream));
    double xs[64], ws[64];
    for (int k = 0; k < c->gl.n; ++k) { xs[k] = 0.5 + 0.5 * c->gl.x[k]; ws[k] = c->gl.w[k]; }
    CK(cudaMemsetAsync(c->status.p, 0, sizeof(int), c->stream));
    CK(launch_eval_bond(c->cg, c->dim ? c->dim : 2, xs, ws, c->gl.n, gk15(), c->status.as<int>(), (int)m, d,
                        d + 3 * m, d + 6 * m, d + 9 * m, d + 10 * m, c->stream));
    CK(cudaMemcpyAsync(bond, d + 9 * m, sizeof(double) * m, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(delta, d + 10 * m, sizeof(double) * m, cudaMemcpyDeviceToHost, c->stream));
    int st = 0;
    CK(cudaMemcpyAsync(&st, c->status.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (st & IK_ST_QUAD_FAIL)
        return fail(IK_ERR_QUADRATURE, "adaptive bond integral: tolerance not met within %d subintervals",
                    std::min(std::max(c->cg.neval, 1), IK_QAG_MAXSUB));
    return IK_OK;
}

int ik_set_mlp(ik_ctx* c, ik_mlp* m)
{
    if (int r = check_ctx(c)) return r;
    ++c->config_version; // captured batch graphs hold the old settings
    c->mlp = m;
    return IK_OK;
}

int ik_set_tuning(ik_ctx* c, int param, int value)
{
    if (int r = check_ctx(c)) return r;
    ++c->config_version; // captured batch graphs hold the old settings
    switch (param) {
    case IK_TUNE_BIN_POINTS:
        if (value < 0 || value > 4096) return fail(IK_ERR_ARG, "bin points must be in [0, 4096]");
        c->tune_bin_points = value;
        invalidate_geometry(c);
        return IK_OK;
    case IK_TUNE_BLOCKS_PER_SM:
        if (value < 0 || value > 16) return fail(IK_ERR_ARG, "blocks per SM must be in [0, 16]");
        c->tune_blocks_per_sm = value;
        return IK_OK;
    case IK_TUNE_HALO_CAP:
        if (value < 0 || value > 1024) return fail(IK_ERR_ARG, "halo capacity must be in [0, 1024]");
        c->halo_cap = (value + 31) & ~31; // whole warps of entries (the per-warp layout needs a multiple of 4)
        return IK_OK;
    case IK_TUNE_FUSED_BATCH:
        if (value != 0 && value != 1) return fail(IK_ERR_ARG, "fused batches: 0 or 1");
        c->tune_fused = value;
        return IK_OK;
    case IK_TUNE_IO_BATCHES:
        if (value < 0 || value > 64) return fail(IK_ERR_ARG, "sub-batches must be in [0, 64]");
        c->tune_io_batches = value;
        return IK_OK;
    case IK_TUNE_IO_MAPPED:
        if (value != 0 && value != 1) return fail(IK_ERR_ARG, "host-mapped copies: 0 or 1");
        c->tune_io_mapped = value;
        return IK_OK;
    default:
        return fail(IK_ERR_ARG, "unknown tuning parameter %d", param);
    }
}

// Time the host-I/O batch under each schedule of its copies, keep the fastest.
int ik_autotune_batch_io(ik_ctx* c, const int* slots, int count, int precision, int fields, const int64_t* n,
                         const double* const* pos, const double* const* vel, const double* const* mass,
                         const double* const* diam, double* const* out, int reps, int* best_io_batches,
                         float* best_ms)
{
    NvtxRange nvr("ik autotune_batch_io");
    if (int r = check_ctx(c)) return r;
    if (reps < 1 || reps > 1000) return fail(IK_ERR_ARG, "reps must be in [1, 1000]");
    // candidates: per frame on the lanes (at the batch's CTAs per SM and at the lanes'
    // default), fused sub-batches with their copies on the copy engines, and fused
    // sub-batches with host-mapped copies (both when the batch can run fused)
    struct Cand { int nb, mapped, lanes_default; };
    static const Cand cands[] = {{0, 0, 0}, {0, 0, 1}, {2, 0, 0}, {4, 0, 0}, {8, 0, 0}, {16, 0, 0}, {32, 0, 0},
                                 {1, 1, 0}, {2, 1, 0}, {4, 1, 0}};
    const int io0 = c->tune_io_batches, map0 = c->tune_io_mapped, bps0 = c->tune_blocks_per_sm;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); return fail(IK_ERR_CUDA, "event creation failed"); }
    float best = 1e30f;
    int bi = io0, bm = map0, bk = bps0, rc = IK_OK;
    bool fused_ok = c->tune_fused != 0, mapped_ok = true;
    std::vector<std::array<int, 3>> tried;
    for (const Cand& cd : cands) {
        if (rc != IK_OK) break;
        const int nb = std::min(cd.nb, count), bps = cd.lanes_default ? 0 : bps0;
        if (cd.lanes_default && bps0 == 0) continue;
        if (nb > 0 && (!fused_ok || (cd.mapped && !mapped_ok))) continue;
        const std::array<int, 3> key{nb, cd.mapped, bps};
        if (std::find(tried.begin(), tried.end(), key) != tried.end()) continue;
        tried.push_back(key);
        if ((rc = ik_set_tuning(c, IK_TUNE_IO_BATCHES, nb)) || (rc = ik_set_tuning(c, IK_TUNE_IO_MAPPED, cd.mapped)) ||
            (rc = ik_set_tuning(c, IK_TUNE_BLOCKS_PER_SM, bps)) ||
            (rc = ik_compute_batch_io(c, slots, count, precision, fields, n, pos, vel, mass, diam, out)) ||
            (rc = ik_compute_batch_io(c, slots, count, precision, fields, n, pos, vel, mass, diam, out)) ||
            (rc = ik_synchronize(c)))
            break;
        if (nb > 0 && !c->io_fused) { fused_ok = false; continue; } // the batch cannot run fused
        if (cd.mapped && !c->io_mapped) { mapped_ok = false; continue; } // an array has no device view
        if (cudaEventRecord(e0, c->stream) != cudaSuccess) { rc = fail(IK_ERR_CUDA, "event record failed"); break; }
        for (int t = 0; t < reps && rc == IK_OK; ++t)
            rc = ik_compute_batch_io(c, slots, count, precision, fields, n, pos, vel, mass, diam, out);
        if (rc) break;
        float ms = 0.f;
        if (cudaEventRecord(e1, c->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) { rc = fail(IK_ERR_CUDA, "event timing failed"); break; }
        if ((rc = ik_synchronize(c))) break;
        ms /= (float)reps;
        if (ms < best) { best = ms; bi = nb; bm = cd.mapped; bk = bps; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (int r = ik_set_tuning(c, IK_TUNE_IO_BATCHES, bi)) return r;
    if (int r = ik_set_tuning(c, IK_TUNE_IO_MAPPED, bm)) return r;
    if (int r = ik_set_tuning(c, IK_TUNE_BLOCKS_PER_SM, bk)) return r;
    if (best_io_batches) *best_io_batches = bi;
    if (best_ms) *best_ms = best;
    return IK_OK;
}

// Time the batch under each candidate (bin points x CTAs per SM), keep the fastest.
int ik_autotune_batch(ik_ctx* c, const int* slots, int count, int precision, int fields, int reps,
                      int* best_bin_points, int* best_blocks_per_sm, float* best_ms)
{
    if (int r = check_ctx(c)) return r;
    if (reps < 1 || reps > 1000) return fail(IK_ERR_ARG, "reps must be in [1, 1000]");
    if (precision != IK_PREC_FP32) return fail(IK_ERR_ARG, "the autotuner tunes the FP32 path");
    // candidates: the schedule (fused batch or one launch sequence per frame on the
    // lanes), the work-item bin size, persistent CTAs per SM, staged halo per warp
    static const int bins_2d[] = {12, 16, 20, 25, 36};
    static const int bins_3d[] = {16, 24, 48, 96};
    static const int blocks[] = {1, 2};
    static const int halos[] = {256, 384, 512};
    const int* bins = c->dim == 3 ? bins_3d : bins_2d;
    const int nbins = c->dim == 3 ? 4 : 5;
    const int halo_min = c->halo_cap > 384 ? c->halo_cap : 0; // a halo grown by an overflow stays grown
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); return fail(IK_ERR_CUDA, "event creation failed"); }
    float best = 1e30f;
    int bb = 0, bk = 0, bh = c->halo_cap, bf = c->tune_fused, rc = IK_OK;
    for (int fu = 1; fu >= 0 && rc == IK_OK; --fu)
        for (int i = 0; i < nbins && rc == IK_OK; ++i)
            for (int k = 0; k < 2 && rc == IK_OK; ++k)
                for (int h = 0; h < 3 && rc == IK_OK; ++h) {
                    const int hv = std::max(halos[h], halo_min);
                    if (h > 0 && hv == std::max(halos[h - 1], halo_min)) continue;
                    if ((rc = ik_set_tuning(c, IK_TUNE_FUSED_BATCH, fu)) ||
                        (rc = ik_set_tuning(c, IK_TUNE_BIN_POINTS, bins[i])) ||
                        (rc = ik_set_tuning(c, IK_TUNE_BLOCKS_PER_SM, blocks[k])) ||
                        (rc = ik_set_tuning(c, IK_TUNE_HALO_CAP, hv)) ||
                        (rc = ik_compute_batch(c, slots, count, precision, fields)) || // plain run + graph recording
                        (rc = ik_compute_batch(c, slots, count, precision, fields)) || (rc = ik_wait_all(c)))
                        break;
                    if (cudaEventRecord(e0, c->stream) != cudaSuccess) { rc = fail(IK_ERR_CUDA, "event record failed"); break; }
                    for (int t = 0; t < reps && rc == IK_OK; ++t) rc = ik_compute_batch(c, slots, count, precision, fields);
                    if (rc || (rc = ik_wait_all(c))) break;
                    float ms = 0.f;
                    if (cudaEventRecord(e1, c->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) { rc = fail(IK_ERR_CUDA, "event timing failed"); break; }
                    if ((rc = ik_synchronize(c))) break;
                    ms /= (float)reps;
                    if (ms < best) { best = ms; bb = bins[i]; bk = blocks[k]; bh = c->halo_cap; bf = fu; }
                }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (int r = ik_set_tuning(c, IK_TUNE_FUSED_BATCH, bf)) return r;
    if (int r = ik_set_tuning(c, IK_TUNE_BIN_POINTS, bb)) return r;
    if (int r = ik_set_tuning(c, IK_TUNE_BLOCKS_PER_SM, bk)) return r;
    if (int r = ik_set_tuning(c, IK_TUNE_HALO_CAP, bh)) return r;
    if (best_bin_points) *best_bin_points = bb;
    if (best_blocks_per_sm) *best_blocks_per_sm = bk;
    if (best_ms) *best_ms = best;
    return IK_OK;
}
int ik_get_tuning(ik_ctx* c, int param, int* value)
{
    if (int r = check_ctx(c)) return r;
    if (!value) return fail(IK_ERR_ARG, "null output");
    switch (param) {
    case IK_TUNE_BIN_POINTS: *value = c->tune_bin_points; return IK_OK;
    case IK_TUNE_BLOCKS_PER_SM: *value = c->tune_blocks_per_sm; return IK_OK;
    case IK_TUNE_HALO_CAP: *value = c->halo_cap; return IK_OK;
    case IK_TUNE_FUSED_BATCH: *value = c->tune_fused; return IK_OK;
    case IK_TUNE_IO_BATCHES: *value = c->tune_io_batches; return IK_OK;
    case IK_TUNE_IO_MAPPED: *value = c->tune_io_mapped; return IK_OK;
    default: return fail(IK_ERR_ARG, "unknown tuning parameter %d", param);
    }
}

int ik_set_flags(ik_ctx* c, int flags)
{
    if (int r = check_ctx(c)) return r;
    ++c->config_version; // captured batch graphs hold the old settings
    c->flags = flags;
    return IK_OK;
}

int ik_get_timing(ik_ctx* c, float* ms4)
{
    if (int r = check_ctx(c)) return r;
    if (!ms4) return fail(IK_ERR_ARG, "null output");
    if (!(c->flags & IK_FLAG_TIMING)) return fail(IK_ERR_STATE, "timing flag not set");
    CK(cudaEventSynchronize(c->ev[3]));
    CK(cudaEventElapsedTime(&ms4[0], c->ev[0], c->ev[1]));
    CK(cudaEventElapsedTime(&ms4[1], c->ev[1], c->ev[2]));
    CK(cudaEventElapsedTime(&ms4[2], c->ev[2], c->ev[3]));
    CK(cudaEventElapsedTime(&ms4[3], c->ev[0], c->ev[3]));
    return IK_OK;
}

int ik_wait_all(ik_ctx* c)
{
    if (int r = check_ctx(c)) return r;
    for (Lane& L : c->lanes) {
        CK(cudaEventRecord(L.last, L.st));
        CK(cudaStreamWaitEvent(c->stream, L.last, 0));
    }
    CK(cudaEventRecord(c->d2h_last, c->d2h));
    CK(cudaStreamWaitEvent(c->stream, c->d2h_last, 0));
    return IK_OK;
}

int ik_get_launch_count(ik_ctx* c, int64_t* out)
{
    if (int r = check_ctx(c)) return r;
    if (!out) return fail(IK_ERR_ARG, "null output");
    *out = c->launches;
    return IK_OK;
}

int ik_get_stream(ik_ctx* c, void** stream)
{
    if (int r = check_ctx(c)) return r;
    if (!stream) return fail(IK_ERR_ARG, "null output");
    *stream = (void*)c->stream;
    return IK_OK;
}

int ik_download_field_async(ik_ctx* c, int slot, int field, double* host_out, int64_t count)
{
    NvtxRange nvr("ik download");
    if (int r = check_ctx(c)) return r;
    if (int r = slot_ok(c, slot)) return r;
    GeoSwap gs(c, slot);
    if (field != IK_FIELD_VIRIAL && field != IK_FIELD_KINETIC && field != IK_FIELD_ELASTIC)
        return fail(IK_ERR_ARG, "unknown field %d", field);
    const int NC = c->dim == 2 ? 3 : 6;
    if (!host_out || count != c->geo.G * NC) return fail(IK_ERR_ARG, "output needs %lld doubles", (long long)(c->geo.G * NC));
    Slot& s = c->slots[(size_t)slot];
    const DevBuf& src = field == IK_FIELD_VIRIAL ? s.vir : (field == IK_FIELD_KINETIC ? s.kin : s.ela);
    if (!src.p) return fail(IK_ERR_STATE, "slot %d has not been computed", slot);
    // on the download stream, after the slot's computation: uploads of other frames
    // (context stream) and computations (lanes) proceed meanwhile
    if (s.done_recorded) CK(cudaStreamWaitEvent(c->d2h, s.done, 0));
    if (c->geo.G > 0) CK(cudaMemcpyAsync(host_out, src.p, sizeof(double) * NC * c->geo.G, cudaMemcpyDeviceToHost, c->d2h));
    if (!s.d2h_done) CK(cudaEventCreateWithFlags(&s.d2h_done, cudaEventDisableTiming));
    CK(cudaEventRecord(s.d2h_done, c->d2h));
    s.d2h_recorded = true;
    // a computation of this slot still to be confirmed: re-download if it is re-run
    for (auto it = c->pending.rbegin(); it != c->pending.rend(); ++it)
        if (it->slot == slot) { it->out[field == IK_FIELD_VIRIAL ? 0 : (field == IK_FIELD_KINETIC ? 1 : 2)] = host_out; break; }
    return IK_OK;
}

int ik_measure_fp32_peak(int device, double* tflops)
{
    if (!tflops) return fail(IK_ERR_ARG, "null output");
    CK(cudaSetDevice(device));
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, device));
    int blocks = prop.multiProcessorCount * 8, threads = 256, iters = 4096;
    float* out = nullptr;
    CK(cudaMalloc(&out, sizeof(float) * blocks * threads));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(a);
        cudaError_t e = launch_fma_probe(blocks, threads, iters, out);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        if (e != cudaSuccess) { cudaFree(out); return fail(IK_ERR_CUDA, "probe launch: %s", cudaGetErrorString(e)); }
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (rep > 0 && ms < best) best = ms; // first launch is warm-up
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    double flop = 2.0 * IK_FMA_PROBE_CHAINS * (double)iters * blocks * threads;
    *tflops = flop / (best * 1e-3) / 1e12;
    return IK_OK;
}

int ik_get_counters(ik_ctx* c, int slot, int64_t* out3)
{
    if (int r = check_ctx(c)) return r;
    if (int r = slot_ok(c, slot)) return r;
    if (!out3) return fail(IK_ERR_ARG, "null output");
    if (int r = ik_synchronize(c)) return r;
    Slot& s = c->slots[(size_t)slot];
    unsigned long long h[4] = {0, 0, 0, 0};
    if (s.counters.p) CK(cudaMemcpy(h, s.counters.p, sizeof h, cudaMemcpyDeviceToHost));
    out3[0] = (int64_t)h[0];
    out3[1] = (int64_t)h[1];
    out3[2] = (int64_t)h[2];
    return IK_OK;
}

int ik_get_mlp_records(ik_ctx* c, int slot, int64_t* out)
{
    if (int r = check_ctx(c)) return r;
    if (int r = slot_ok(c, slot)) return r;
    if (!out) return fail(IK_ERR_ARG, "null output");
    if (int r = ik_synchronize(c)) return r;
    Slot& s = c->slots[(size_t)slot];
    unsigned long long h[4] = {0, 0, 0, 0};
    if (s.counters.p) CK(cudaMemcpy(h, s.counters.p, sizeof h, cudaMemcpyDeviceToHost));
    *out = (int64_t)h[3];
    return IK_OK;
}

int ik_get_mlp_fallbacks(ik_ctx* c, int slot, int64_t* out)
{
    if (int r = check_ctx(c)) return r;
    if (int r = slot_ok(c, slot)) return r;
    if (!out) return fail(IK_ERR_ARG, "null output");
    if (int r = ik_synchronize(c)) return r;
    Slot& s = c->slots[(size_t)slot];
    unsigned long long h[5] = {0, 0, 0, 0, 0};
    if (s.counters.p && s.counters.bytes >= sizeof h) CK(cudaMemcpy(h, s.counters.p, sizeof h, cudaMemcpyDeviceToHost));
    *out = (int64_t)h[4];
    return IK_OK;
}

} // extern "C"
