// ik_noalloc.cu -- ik_compute_fp64_noalloc: the plain FP64 Irving-Kirkwood computation
// for callers that cannot allocate device memory.
//
// Who needs it: a process whose device memory is owned by another framework's pool
// (a caching allocator that has reserved the device, where a cudaMalloc from this
// library would fail or fragment it), a service under a device-memory budget fixed at
// start-up, and code that must not enter cudaMalloc because cudaMalloc may wait for
// work on other streams of the device.  Such callers bring their own input and output
// buffers; this entry point brings the rest.
//
// The call is synchronous: it makes CUDA runtime calls (cudaMemsetAsync, kernel
// launches, cudaMemcpyAsync, cudaStreamSynchronize) and returns once the caller's
// stream has finished.  It must not be called from a stream callback or a host
// function (cudaLaunchHostFunc), where CUDA calls are not permitted.
//
// All scratch (cell list, sorted particle ids, FP64 bond records, status words)
// lives in one file-scope __device__ array of IK_NOALLOC_SCRATCH_BYTES (about 4.3 MB).
// Every GPU that loads the library holds that array until the process exits.  Calls
// share it: two calls that overlap on the GPU (different streams, or different host
// threads on the same device) race on it and must be serialised by the caller.  The
// array keeps the previous call's contents; everything that must start at zero is
// cleared on the caller's stream at the start of each call.
//
// The array's address belongs to a CUDA context.  The first call in each context (for
// the usual primary context: the first call on each device) looks it up with
// cudaGetSymbolAddress, with that context current, and caches it under the context's
// unique id; make that first call before any stream capture in the context.
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

// Scratch addresses by CUDA context.  A context id (cuCtxGetId) is unique for the
// life of the process, so a context created after cudaDeviceReset -- even at a reused
// handle -- gets a set-up of its own.
constexpr int NA_MAX_CONTEXTS = 64;
struct NaEntry { unsigned long long ctx_id; unsigned char* ptr; };
NaEntry na_cache[NA_MAX_CONTEXTS];
int na_cached = 0;
std::mutex na_mutex;
typedef int (*na_ctx_current_fn)(void** ctx);
typedef int (*na_ctx_id_fn)(void* ctx, unsigned long long* id);
na_ctx_current_fn na_ctx_current = nullptr;
na_ctx_id_fn na_ctx_id = nullptr;

// Device address of the scratch array in the current context (set up once per context).
int na_scratch(unsigned char** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return na_fail(IK_ERR_CUDA, "cudaGetDevice failed");
    std::lock_guard<std::mutex> lk(na_mutex);
    if (!na_ctx_current || !na_ctx_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return na_fail(IK_ERR_CUDA, "the driver's context queries (cuCtxGetCurrent, cuCtxGetId) are unavailable");
        na_ctx_current = reinterpret_cast<na_ctx_current_fn>(f1);
        na_ctx_id = reinterpret_cast<na_ctx_id_fn>(f2);
    }
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (na_ctx_current(&ctx) != 0) return na_fail(IK_ERR_CUDA, "cuCtxGetCurrent failed");
    if (!ctx) { // no context on this thread yet: the device's primary context
        if (cudaSetDevice(dev) != cudaSuccess || na_ctx_current(&ctx) != 0 || !ctx)
            return na_fail(IK_ERR_CUDA, "no CUDA context could be made current");
    }
    if (na_ctx_id(ctx, &id) != 0) return na_fail(IK_ERR_CUDA, "cuCtxGetId failed");
    for (int k = 0; k < na_cached; ++k)
        if (na_cache[k].ctx_id == id) { *out = na_cache[k].ptr; return IK_OK; }
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, ik_noalloc_scratch);
    if (e != cudaSuccess || !p) return na_fail(IK_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed");
    if (na_cached == NA_MAX_CONTEXTS) na_cached = 0; // full: start over (set-ups are redone on demand)
    na_cache[na_cached++] = NaEntry{id, static_cast<unsigned char*>(p)};
    *out = static_cast<unsigned char*>(p);
    return IK_OK;
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
    ik_gl_rule(gl_order, gx, gw);
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
    int hs = 0; // the status word, read on the caller's stream (not the legacy default stream)
    NA_CK(cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    if (hs & IK_ST_BAD_INPUT)
        return na_fail(IK_ERR_ARG, "invalid frame: a position is not finite, a diameter is not > 0, or a 2D frame has z != 0");
    if (hs & IK_ST_BOND_OVERFLOW) return na_fail(IK_ERR_CAPACITY, "a particle has more than 32 force-active bonds");
    return IK_OK;
#undef NA_CK
}
