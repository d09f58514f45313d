// ik_noalloc.cu -- ik_compute_fp64_noalloc: the plain FP64 Irving-Kirkwood computation
// for callers that must not allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is unavailable or forbidden -- inside
// a host callback or a real-time loop that may not block on the allocator, in a
// process whose device memory is owned by another framework's pool, or under a
// memory budget fixed at start-up.  Such callers bring their own input and output
// buffers; this entry point brings the rest.
//
// All scratch (cell list, sorted particle ids, FP64 bond records, status words)
// lives in one file-scope __device__ array of IK_NOALLOC_SCRATCH_BYTES (about 4.3 MB).
// Every GPU that loads the library holds that array until the process exits.  Calls
// share it: two calls that overlap on the GPU (different streams, or different host
// threads on the same device) race on it and must be serialised by the caller.  The
// array keeps the previous call's contents; everything that must start at zero is
// cleared on the caller's stream at the start of each call.
//
// The first call on each device looks up the array's device address
// (cudaGetSymbolAddress, with that device current); make that first call before any
// stream capture on the device.
#include "ik_kernels.h"
#include "../../include/ik_gb300.h"

#include <cmath>
#include <cstdio>
#include <mutex>

namespace {

constexpr int NA_MAX_N = 4096;       // particles
constexpr int NA_MAX_CELLS = 16384;  // cell-list cells
constexpr int NA_MAXB = 32;          // force-active bonds per particle
constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t OFF_STATUS = 0;
constexpr size_t OFF_MAXNB = 256;
constexpr size_t OFF_COUNT = 512;
constexpr size_t OFF_START = OFF_COUNT + align256(sizeof(int) * (NA_MAX_CELLS + 1));
constexpr size_t OFF_CELLOF = OFF_START + align256(sizeof(int) * (NA_MAX_CELLS + 1));
constexpr size_t OFF_RANK = OFF_CELLOF + align256(sizeof(int) * NA_MAX_N);
constexpr size_t OFF_SORTED = OFF_RANK + align256(sizeof(int) * NA_MAX_N);
constexpr size_t OFF_NB = OFF_SORTED + align256(sizeof(int) * NA_MAX_N);
constexpr size_t OFF_BONDS = OFF_NB + align256(sizeof(int) * NA_MAX_N);
constexpr size_t IK_NOALLOC_SCRATCH_BYTES = OFF_BONDS + sizeof(IkB64) * (size_t)NA_MAX_N * NA_MAXB;

} // namespace

static __device__ __align__(256) unsigned char ik_noalloc_scratch[IK_NOALLOC_SCRATCH_BYTES];

namespace {

int na_fail(int code, const char* msg)
{
    char buf[512];
    snprintf(buf, sizeof buf, "ik_compute_fp64_noalloc: %s", msg);
    ik_internal_set_error(buf); // reported by ik_last_error()
    return code;
}

constexpr int NA_MAX_DEVICES = 64;
unsigned char* na_ptr[NA_MAX_DEVICES] = {nullptr};
std::mutex na_mutex;

// Device address of the scratch array on the current device (set up once per device).
int na_scratch(unsigned char** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return na_fail(IK_ERR_CUDA, "cudaGetDevice failed");
    if (dev < 0 || dev >= NA_MAX_DEVICES) return na_fail(IK_ERR_UNSUPPORTED, "device index too large");
    std::lock_guard<std::mutex> lk(na_mutex);
    if (!na_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, ik_noalloc_scratch);
        if (e != cudaSuccess || !p) return na_fail(IK_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed");
        na_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = na_ptr[dev];
    return IK_OK;
}

void na_gl_rule(int n, double* x, double* w)
{
    // Gauss-Legendre nodes/weights on [-1,1]: Newton on the three-term recurrence.
    for (int k = 0; k < n; ++k) {
        long double z = cosl(3.14159265358979323846264338327950288L * (k + 0.75L) / (n + 0.5L)), pp = 1.0L;
        for (int it = 0; it < 100; ++it) {
            long double p0 = 1.0L, p1 = z;
            for (int j = 2; j <= n; ++j) { long double p2 = ((2.0L * j - 1.0L) * z * p1 - (j - 1.0L) * p0) / j; p0 = p1; p1 = p2; }
            pp = n * (z * p1 - p0) / (z * z - 1.0L);
            long double dz = p1 / pp;
            z -= dz;
            if (fabsl(dz) < 1e-19L) break;
        }
        long double p0 = 1.0L, p1 = z;
        for (int j = 2; j <= n; ++j) { long double p2 = ((2.0L * j - 1.0L) * z * p1 - (j - 1.0L) * p0) / j; p0 = p1; p1 = p2; }
        pp = n * (z * p1 - p0) / (z * z - 1.0L);
        x[n - 1 - k] = (double)z;
        w[n - 1 - k] = (double)(2.0L / ((1.0L - z * z) * pp * pp));
    }
    if (n % 2 == 1) x[n / 2] = 0.0;
}

} // namespace

extern "C" int ik_compute_fp64_noalloc(int dim, const double boxsize[3], const double origin[3],
                                       double scaled_rcut, const double params[5], double max_rcut,
                                       int cg_kind, int gl_order, double cg_rcut, double cg_width,
                                       int64_t n, const double* d_pos, const double* d_diam,
                                       const double* d_vel, const double* d_mass, int64_t g,
                                       const double* d_grid, double* d_virial, double* d_kinetic,
                                       void* stream_handle)
{
    // ---- arguments
    if (dim != 2 && dim != 3) return na_fail(IK_ERR_ARG, "dim must be 2 or 3");
    if (!boxsize || !params) return na_fail(IK_ERR_ARG, "null boxsize or params");
    if (n < 0 || n > NA_MAX_N) {
        char m[128];
        snprintf(m, sizeof m, "n = %lld particles exceeds the maximum of %d", (long long)n, NA_MAX_N);
        return na_fail(IK_ERR_CAPACITY, m);
    }
    if (g < 0 || g > (1LL << 30)) return na_fail(IK_ERR_ARG, "grid size out of range");
    if ((n > 0 && (!d_pos || !d_diam)) || (g > 0 && (!d_grid || !d_virial)))
        return na_fail(IK_ERR_ARG, "null device pointer");
    if (cg_kind < 0 || cg_kind > 3) return na_fail(IK_ERR_ARG, "unknown coarse-graining kind");
    if (gl_order < 1 || gl_order > 64) return na_fail(IK_ERR_ARG, "Gauss-Legendre order must be in [1, 64]");
    if (!(cg_rcut > 0.0) || !(max_rcut > 0.0) || !(scaled_rcut > 0.0)) return na_fail(IK_ERR_ARG, "cut-offs must be > 0");
    if (cg_kind == IK_CG_GAUSSIAN && !(cg_width > 0.0)) return na_fail(IK_ERR_ARG, "Gaussian width must be > 0");
    cudaStream_t st = static_cast<cudaStream_t>(stream_handle);
    unsigned char* base = nullptr;
    if (int r = na_scratch(&base)) return r;

    // ---- geometry (SimBox bounds; cells of width >= max_rcut, at most NA_MAX_CELLS)
    IkGeom geo{};
    geo.dim = dim;
    for (int a = 0; a < 3; ++a) {
        double L = (dim == 2 && a == 2) ? 1.0 : boxsize[a];
        double o = origin ? ((dim == 2 && a == 2) ? 0.0 : origin[a]) : 0.0;
        geo.L[a] = L;
        geo.lo[a] = -0.5 * L - o;
        geo.periodic[a] = a < dim ? 1 : 0;
        if (!(L > 0.0)) return na_fail(IK_ERR_ARG, "box edges must be > 0");
        if (geo.periodic[a] && (!(2.0 * max_rcut < L) || !(2.0 * cg_rcut < L)))
            return na_fail(IK_ERR_BOX, "a cut-off is >= half the periodic box");
        geo.nc[a] = geo.periodic[a] ? (int)std::max(1.0, std::floor(L / max_rcut)) : 1;
    }
    while ((long long)geo.nc[0] * geo.nc[1] * geo.nc[2] > NA_MAX_CELLS) {
        int a = (geo.nc[0] >= geo.nc[1] && geo.nc[0] >= geo.nc[2]) ? 0 : (geo.nc[1] >= geo.nc[2] ? 1 : 2);
        geo.nc[a] = (geo.nc[a] + 1) / 2; // wider cells: still >= max_rcut
    }
    for (int a = 0; a < 3; ++a) {
        geo.cw[a] = geo.L[a] / geo.nc[a];
        geo.reach_bond[a] = 1;
        geo.all_bond[a] = geo.nc[a] < 3 ? 1 : 0;
    }
    geo.ncell = geo.nc[0] * geo.nc[1] * geo.nc[2];

    IkPot pot{};
    pot.rcutsq = scaled_rcut * scaled_rcut;
    pot.v0 = params[0]; pot.eps = params[1]; pot.c0 = params[2]; pot.c1 = params[3]; pot.c2 = params[4];
    pot.max_rcut_sq = max_rcut * max_rcut;

    const double PI = 3.14159265358979323846;
    GatherArgs64 a{};
    a.g = geo;
    IkCG& cg = a.cg;
    cg.kind = cg_kind;
    cg.mode = IK_QUAD_FIXEDPOINT;
    cg.order = gl_order;
    cg.rcut = cg_rcut;
    cg.rcutsq = cg_rcut * cg_rcut;
    cg.width = cg_kind == IK_CG_GAUSSIAN ? cg_width : 0.0;
    if (cg_kind == IK_CG_OCTIC) cg.norm = 15.0 / (8 * PI * cg.rcutsq);
    else if (cg_kind == IK_CG_GAUSSIAN) {
        double w2 = cg_width * cg_width;
        cg.norm = dim == 3 ? 1.0 / ((2.0 * PI * w2) * std::sqrt(2.0 * PI * w2)) : 1.0 / (2.0 * PI * w2);
    } else if (cg_kind == IK_CG_RECT) cg.norm = 1 / (PI * cg.rcutsq);
    else {
        double rn = cg_width > 0.0 ? cg_width : cg_rcut;
        cg.mollifier_norm = 13.46842098743079272180855772032086697297031125109170011102 / (2.0 * PI * rn * rn);
        cg.norm = cg.mollifier_norm;
    }
    for (int k = 0; k < 3; ++k) {
        a.reach[k] = k < dim ? (int)std::ceil(cg_rcut / geo.cw[k]) : 0;
        if (k < dim && a.reach[k] < 1) a.reach[k] = 1;
        a.all[k] = (k < dim && 2 * a.reach[k] + 1 >= geo.nc[k]) ? 1 : 0;
    }
    double gx[64], gw[64];
    na_gl_rule(gl_order, gx, gw);
    a.nq = gl_order;
    for (int k = 0; k < gl_order; ++k) { a.xs[k] = 0.5 + 0.5 * gx[k]; a.ws[k] = gw[k]; }

    // ---- scratch views
    int* status = reinterpret_cast<int*>(base + OFF_STATUS);
    int* maxnb = reinterpret_cast<int*>(base + OFF_MAXNB);
    int* count = reinterpret_cast<int*>(base + OFF_COUNT);
    int* start = reinterpret_cast<int*>(base + OFF_START);
    int* cell_of = reinterpret_cast<int*>(base + OFF_CELLOF);
    int* rank = reinterpret_cast<int*>(base + OFF_RANK);
    int* sorted = reinterpret_cast<int*>(base + OFF_SORTED);
    int* nb = reinterpret_cast<int*>(base + OFF_NB);
    IkB64* bonds = reinterpret_cast<IkB64*>(base + OFF_BONDS);
    const int maxb = NA_MAXB;

#define NA_CK(call)                                                                        \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) return na_fail(IK_ERR_CUDA, cudaGetErrorString(e_));        \
    } while (0)

    // ---- clear what must start at zero, then the launch sequence of the plain path
    NA_CK(cudaMemsetAsync(status, 0, sizeof(int), st));
    NA_CK(cudaMemsetAsync(maxnb, 0, sizeof(int), st));
    NA_CK(cudaMemsetAsync(count, 0, sizeof(int) * (geo.ncell + 1), st));
    const int nn = (int)n;
    if (nn > 0) {
        k_validate<<<(nn + 255) / 256, 256, 0, st>>>(d_pos, d_diam, nn, dim, status);
        k_bin<<<(nn + 255) / 256, 256, 0, st>>>(d_pos, nn, geo, cell_of, rank, count, status);
    }
    k_scan<<<1, 1024, 0, st>>>(count, geo.ncell, start);
    if (nn > 0) k_scatter<<<(nn + 255) / 256, 256, 0, st>>>(cell_of, rank, start, nn, sorted);
    k_cell_sort_pack<<<(geo.ncell + 127) / 128, 128, 0, st>>>(geo, start, sorted, nullptr, nullptr, nullptr, nullptr,
                                                              nullptr, nullptr, nullptr, 0);
    if (nn > 0)
        k_bonds64<<<(nn + 127) / 128, 128, 0, st>>>(geo, pot, nn, sorted, cell_of, d_pos, d_diam, start, bonds, maxb,
                                                    nb, status, maxnb);
    NA_CK(cudaGetLastError());
    a.sorted = sorted;
    a.cell_start = start;
    a.pos = d_pos;
    a.vel = d_vel;
    a.mass = d_mass;
    a.nb = nb;
    a.bonds = bonds;
    a.maxb = maxb;
    a.grid = d_grid;
    a.ngrid = g;
    a.out_vir = d_virial;
    a.out_kin = d_kinetic;
    a.fields = IK_FIELD_VIRIAL | (d_kinetic && d_vel ? IK_FIELD_KINETIC : 0);
    if (d_kinetic && !d_vel && g > 0)
        NA_CK(cudaMemsetAsync(d_kinetic, 0, sizeof(double) * (dim == 2 ? 3 : 6) * g, st));
    if (g > 0) NA_CK(launch_gather64(a, st));
    NA_CK(cudaStreamSynchronize(st));
    int hs = 0;
    NA_CK(cudaMemcpy(&hs, status, sizeof(int), cudaMemcpyDeviceToHost));
    if (hs & IK_ST_BAD_INPUT)
        return na_fail(IK_ERR_ARG, "invalid frame: a position is not finite, a diameter is not > 0, or a 2D frame has z != 0");
    if (hs & IK_ST_BOND_OVERFLOW) return na_fail(IK_ERR_CAPACITY, "a particle has more than 32 force-active bonds");
    return IK_OK;
#undef NA_CK
}
