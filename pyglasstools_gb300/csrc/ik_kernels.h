// ik_kernels.h -- kernel argument blocks and launcher prototypes shared by the
// .cu translation units of the GB300 Irving-Kirkwood engine.
#pragma once
#include "ik_common.cuh"

// ---- cells / bonds (ik_cells.cu) -------------------------------------------
__global__ void k_bin(const double* pos, int n, IkGeom g, int* cell_of, int* rank, int* cell_count,
                      int* status);
__global__ void k_scan(const int* in, int n, int* out);
__global__ void k_widen_frame(const float* st, int n, double* pos, double* vel, double* mass, double* diam);
__global__ void k_scatter(const int* cell_of, const int* rank, const int* cell_start, int n, int* sorted);
__global__ void k_cell_sort_pack(IkGeom g, const int* cell_start, int* sorted, const double* pos,
                                 const double* vel, const double* mass, const double* diam,
                                 IkPRec* prec, float4* kin, float* diam32, int want_pack);
// ---- tuned-path preparation (ik_bonds.cu) ---------------------------------
// both also make k_validate's tests (positions in the binning, diameters in the packing),
// reported as IK_ST_BAD_INPUT in status
cudaError_t launch_bin32(const double* pos, int n, IkGeom g, int* cell_of, int* rank, int* cell_count, float4* relhi,
                         float4* rello, int* status, cudaStream_t st);
cudaError_t launch_sort_pack32(IkGeom g, const int* cell_start, int* sorted, const float4* relhi, const float4* rello,
                               const double* pos, const double* vel, const double* mass, const double* diam,
                               IkPRec* prec, float4* plo, IkB64* pos64, float4* kin, float* diam32, int* status,
                               cudaStream_t st);
// nbond_total (may be null): += force-active directed bonds
cudaError_t launch_bonds32(int dim, IkGeom g, IkPot pot, float kappa, int n, const IkPRec* prec,
                            const float* diam32, const int* cell_start, const float4* plo, const IkB64* pos64,
                            float4* tmp, int maxb, int* nb, int* status, int* maxnb,
                            unsigned long long* nbond_total, cudaStream_t st);
cudaError_t launch_bond_compact(int n, int maxb, const int* nb, const int* boff, const float4* tmp, float4* bonds,
                                unsigned long long* nbond_total, cudaStream_t st);
// exclusive scan of n ints into out[0..n]; bsum needs ceil(n / 4096) ints
cudaError_t launch_scan(const int* in, int n, int* out, int* bsum, cudaStream_t st);
__global__ void k_bonds64(IkGeom g, IkPot pot, int n, const int* sorted, const int* cell_of,
                          const double* pos, const double* diam, const int* cell_start, IkB64* bonds,
                          int maxb, int* nb, int* status, int* maxnb);
__global__ void k_bonds64e(IkGeom g, IkPot pot, float kappa, int n, const int* sorted, const int* cell_of,
                           const double* pos, const double* disp, const double* diam, const int* cell_start,
                           IkB64* b64, double* c64, float4* b32, float4* c32, int maxb, int* nb, int* status,
                           int* maxnb);
cudaError_t launch_neigh(bool fill, IkGeom g, int n, double r2cut, const int* sorted, const int* cell_of,
                         const double* pos, const int* cell_start, int* count, const int* offs, int* idx,
                         cudaStream_t st);
__global__ void k_point_query(IkGeom g, int n, const double* pos, double px, double py, double pz,
                              double r2cut, unsigned char* flag);
__global__ void k_validate(const double* pos, const double* diam, int n, int dim, int* status);
// One copy of a host-mapped batch copy (launch_io_copy): `words` 8-byte words from src to
// dst, the copy's first word at `off` in the launch's concatenation; check: 0 none,
// 1 positions (n x 3: finite, z == 0 in 2D), 2 diameters (finite, > 0) -- k_validate's
// tests, made while copying.
struct IkIoCopy {
    const long long* src;
    long long* dst;
    long long words, off;
    int check, dim;
};
// Every copy of `d` (n descriptors, `total` words, none empty, contiguous offsets) in one
// kernel whose threads read and write through the device's view of page-locked host
// memory; failed checks set IK_ST_BAD_INPUT in status.
cudaError_t launch_io_copy(const IkIoCopy* d, int n, long long total, int* status, int sm_count, cudaStream_t st);
__global__ void k_eval_pair(IkPot pot, int m, const double* rij, const double* di, const double* dj,
                            double* f, double* en);

// ---- FP32 tuned gather (ik_gather32.cu) ------------------------------------
// The geometry the gather needs per frame (per slot in a fused batch).
struct GatherGeo {
    IkGeom g;
    float cws[3];          // kappa * cell width
    int bw[3];             // bin width (cells) per axis
    int reach[3];          // halo reach (cells) per axis; 0 on non-periodic axes
    int cull;              // stage only particles within R of the bin's box
    int c_off;             // fused batch: the slot's first cell in the batch's cell list (else 0)
    int p_off;             // fused batch: the slot's first particle in the batch (else 0)
    unsigned long long* cnt; // fused batch: the slot's 5 counters (bonds, pairs, triples, records, fallbacks)
};
// A slot of a fused batch (ik_compute_batch with every stage batch-wide): its gather
// geometry, inputs, outputs and extents in the batch's concatenated arrays.
struct IkBatchSlot {
    GatherGeo geo;
    const double *pos, *vel, *mass, *diam; // the slot's frame (vel / mass may be null)
    double *out_vir, *out_kin;             // FP64 fields, G x NC (null: not requested)
    int n, ncell, allax;                   // allax: some axis has fewer than three cells
    long long G, g_off;                    // grid points; first grid point in the batch
};
struct GatherArgs32 {
    GatherGeo geo;
    float kappa, R2s, margin;
    double R2;             // FP64 R^2 for the boundary re-check
    // Gauss-Legendre in symmetric form: nodes +-xi_k (k < npairs) with weights w_k,
    // centre weight w0; xi2 = xi^2, m2xi = -2 xi
    int npairs;
    float w0, xi2[32], m2xi[32], w[32];
    // particle data (cell order)
    const IkPRec* prec;
    const IkB64* pos64;    // raw FP64 positions in cell order
    const int* cell_start;
    const int* boff;       // CSR offsets of the bond records (n + 1), or null: records of
                           // particle q at q * maxb (fixed stride), nb[q] of them
    int nprec;             // particles of the frame (boff[nprec] = its bond records)
    const int* nb;
    const float4* bonds;   // {kappa r_ij / 2, 2 forceDivR / kappa^2}
    const float4* bcoef;   // elastic field: the bond's stress coefficient (NC floats in
                           // 1 or 2 float4) instead of f' h (x) h; null otherwise
    int maxb;
    const float4* kin;
    // grid
    const float4* gpts;    // bin-ordered {ux,uy,uz, bits(grid index)}
    const double* grid;    // original FP64 grid (g x 3)
    const int4* items;     // {cx0, cy0, cz0, gstart}; items[nitems].w = end
    int nitems;
    int halo_cap, qcap;
    float2* out_vir;       // unscaled double-float pairs (hi, lo), g x NC
    float2* out_kin;
    // direct64: the item's last chunk writes each field value as FP64,
    // ((double)hi + (double)lo) * scale, into out64_vir / out64_kin (a fused batch: into
    // its slot's fields) instead of a pair for a separate finish; out_vir / out_kin then
    // only carry the partial sums between the chunks of an item
    int direct64;
    double* out64_vir;
    double* out64_kin;
    double s64_vir, s64_kin;
    int fields;
    int* work_counter;
    int* status;
    unsigned long long* cnt_pairs;
    unsigned long long* cnt_triples;
    // fused batch: per item its slot (item_slot), per slot its geometry (slots[s].geo);
    // particle, bond, grid and output indices are the batch's
    const IkBatchSlot* slots;
    const int* item_slot;
    // surrogate mode: bonds crossing the edge of the support go to records instead of
    // the fixed-point sum ({M, mb, hh, B_fixed} + {grid index, bond index})
    float4* mlp_rec;
    int2* mlp_rid;
    unsigned long long* mlp_count;  // records reserved (chunks of IK_MLP_CHUNK)
    long long mlp_cap;
    unsigned long long* cnt_records;
};
#define IK_MLP_CHUNK 2048
// a.bcoef != null: elastic coefficients.  launch_gather32 passes the elastic field and
// maxb > 63 on to launch_gather32_aux (variants in the second translation unit), and
// the closed-form modes to launch_gather32_exact (a third).  qm: the quadrature mode --
// 0 fixed-point rule, 1 surrogate records, 2 closed form on bonds crossing the edge of
// the support, 3 closed form on every bond (1-3: Gaussian kernel; 1: plain lane sums).
cudaError_t launch_gather32(const GatherArgs32& a, int kind, bool kahan, int qm, int blocks, int threads,
                            size_t smem, cudaStream_t st);
cudaError_t launch_gather32_aux(const GatherArgs32& a, int kind, bool kahan, int qm, int blocks, int threads,
                                size_t smem, cudaStream_t st);
cudaError_t launch_gather32_exact(const GatherArgs32& a, int kind, bool kahan, int qm, int blocks, int threads,
                                  size_t smem, cudaStream_t st);
// vir = ((double)hi + (double)lo + corr * 2^-32) * svir   (corr: fixed point, may be null),
// kin = ((double)hi + (double)lo) * skin; a null output is skipped.  One launch.
cudaError_t launch_pairs_to_f64(const float2* vin, const unsigned long long* corr, double* vout, double svir,
                                const float2* kin, double* kout, double skin, long long count, cudaStream_t st);

// ---- fused batches (ik_batch.cu, ik_gather32_batch.cu) ------------------------
// Device arrays of a fused batch: the slots, the offsets of their particles, cells and
// field values in the batch, and the batch-wide work buffers of the preparation.
struct IkBatchLaunch {
    const IkBatchSlot* slots;
    const int* p_offs;          // nslots + 1: first particle of each slot, ptot last
    const int* c_offs;          // nslots + 1: first cell
    const long long* v_offs;    // nslots + 1: first field value (grid point x NC)
    int nslots, ptot, ctot;
    long long vtot;
    int *cell_of, *rank, *cell_count, *cell_start, *sorted, *bsum;
    float4 *relhi, *rello;
    IkPRec* prec;
    float4* plo;
    IkB64* pos64;
    float4* kin;
    float* diam32;
    float4* tmp;                // bond records, maxb per particle
    int* nb;
    int maxb;
    int *status, *maxnb;
};
// bin, scan, scatter, sort + pack, bonds over the whole batch (5 or 6 launches)
cudaError_t launch_batch_prepare(const IkBatchLaunch& b, int dim, const IkPot& pot, float kappa, cudaStream_t st);
// the batch's double-float sums into each slot's FP64 fields (1 launch)
cudaError_t launch_batch_finish(const IkBatchLaunch& b, const float2* vir2, const float2* kin2, double svir,
                                double skin, int fields, cudaStream_t st);
// the FP32 gather over the work items of every slot (a.slots, a.item_slot set); the
// fixed-point rule with two symmetric node pairs (Gauss-Legendre order 4 or 5)
cudaError_t launch_gather32_batch(const GatherArgs32& a, int kind, bool kahan, int blocks, int threads, size_t smem,
                                  cudaStream_t st);

// ---- FP64 plain gather (ik_gather64.cu) ------------------------------------
struct GatherArgs64 {
    IkGeom g;
    IkCG cg;
    int reach[3];
    int all[3];
    int nq;
    double xs[64], ws[64];  // GL nodes mapped to [0,1] (s) and their [-1,1] weights
    IkGK gk;                // adaptive mode: the GK15 rule
    int* status;            // adaptive mode: IK_ST_QUAD_FAIL on a missed tolerance
    const int* sorted;
    const int* cell_start;
    const double* pos;
    const double* vel;
    const double* mass;
    const int* nb;
    const IkB64* bonds;
    const double* ecoef;   // elastic field: NC FP64 coefficients per bond record, or null
    int maxb;
    const double* grid;
    int64_t ngrid;
    double* out_vir;
    double* out_kin;
    int fields;
};
cudaError_t launch_gather64(const GatherArgs64& a, cudaStream_t st);

// ---- scalar bond evaluations (ik_gather64.cu) ------------------------------
cudaError_t launch_eval_bond(const IkCG& cg, int dim, const double* xs, const double* ws, int nq,
                             const IkGK& gk, int* status, int m, const double* x, const double* ri,
                             const double* rij, double* bond, double* delta, cudaStream_t st);

// ---- global thermodynamic observables (ik_cells.cu) --------------------------
// per-block partials (nblocks x ik_thermo_nq(dim)) -> out[ik_thermo_nq(dim)] =
// {energy, virial D x D, elastic D x D, kinetic D x D, Born symmetric components} / vol
int ik_thermo_nq(int dim);
cudaError_t launch_thermo64(const IkGeom& g, const IkPot& pot, int n, const int* sorted, const int* cell_of,
                            const double* pos, const double* vel, const double* mass, const double* diam,
                            const double* disp, const int* cell_start, double* partial, int nblocks,
                            double inv_vol, double* out, cudaStream_t st);

// ---- FP32 FMA throughput probe (ik_cells.cu) --------------------------------
#define IK_FMA_PROBE_CHAINS 8
cudaError_t launch_fma_probe(int blocks, int threads, int iters, float* out);

// ---- learned bond-integral surrogate (ik_mlp.cu) ----------------------------
struct ik_mlp;
const unsigned char* ik_mlp_internal_blob(ik_mlp* m);   // deployed BF16 weights (null if none)
const unsigned char* ik_mlp_internal_table(ik_mlp* m);  // per-bin use table (null if not validated)
// records {M, mb, hh, B_fixed} + {grid index, bond index} -> fixed-point corrections (2^-32);
// fallbacks += records that kept their fixed-point value (bin not validated or outside the table)
cudaError_t launch_mlp_records(ik_mlp* m, const float4* rec, const int2* rid, const unsigned long long* count,
                               long long capacity, const float4* bonds, float to_w, float w, int nc,
                               unsigned long long* corr, unsigned long long* fallbacks, int* status, int blocks,
                               cudaStream_t st);
int mlp_tc_ctas_per_sm(); // resident CTAs per SM of the tensor-core kernel (its grid: SMs x this)

// ---- shared host helpers (ik_api.cu) -----------------------------------------
void ik_internal_set_error(const char* msg);
void ik_gl_rule(int n, double* x, double* w);  // n-point Gauss-Legendre on [-1, 1]
