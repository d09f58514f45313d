/*
 * ik_gb300.h -- C ABI of the GB300 (sm_103a) Irving-Kirkwood stress-field engine.
 *
 * One context = one GPU stream, one box, one pair potential, one coarse-graining
 * function, one grid and any number of resident frame slots.  All pointers are
 * HOST pointers unless the name says _device.  Every call returns an int status
 * (IK_OK = 0, negative on error); ik_last_error() gives the message of the last
 * failing call on the calling thread.  No call aborts the process and no kernel
 * traps: device-side failures are reported through status words.
 *
 * Each entry point cites the reference interface it replaces (paths relative to
 * the pyglasstools repository).
 */
#ifndef IK_GB300_H
#define IK_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------- */
#define IK_OK             0
#define IK_ERR_ARG       -1  /* bad argument (size mismatch, NaN, unknown enum) */
#define IK_ERR_CUDA      -2  /* a CUDA runtime call failed */
#define IK_ERR_STATE     -3  /* call out of order (e.g. compute before set_grid) */
#define IK_ERR_BOX       -4  /* a cut-off is >= half the periodic box */
#define IK_ERR_CAPACITY  -5  /* a fixed-capacity buffer overflowed and could not grow */
#define IK_ERR_TIMEOUT   -6  /* a bounded device-side wait gave up */
#define IK_ERR_NOMEM     -7  /* device allocation failed */
#define IK_ERR_UNSUPPORTED -8
#define IK_ERR_QUADRATURE -9 /* an adaptive bond integral missed its tolerance (GSL would abort) */

/* ---- enums ------------------------------------------------------------------ */
enum ik_cg_kind { IK_CG_OCTIC = 0, IK_CG_GAUSSIAN = 1, IK_CG_RECT = 2, IK_CG_MOLLIFIER = 3 };
enum ik_quad_mode { IK_QUAD_FIXEDPOINT = 0, IK_QUAD_ADAPTIVE = 1, IK_QUAD_EXACT = 2,
                    IK_QUAD_MLP = 3, IK_QUAD_CLIPPED = 4 };
enum ik_precision { IK_PREC_FP64 = 0,   /* plain path: FP64 throughout */
                    IK_PREC_FP32 = 1 }; /* tuned path: FP32 pair arithmetic, compensated
                                           accumulation, FP64 min-image/selection/final */
enum ik_field { IK_FIELD_VIRIAL = 1, IK_FIELD_KINETIC = 2,
                IK_FIELD_ELASTIC = 4 }; /* ElasticVirialStressField (needs displacements) */

typedef struct ik_ctx ik_ctx;

/* Message of the last failing call on this thread ("" if none). */
const char* ik_last_error(void);
/* ABI version (major * 10000 + minor * 100 + patch). */
int ik_version(void);

/* Create / destroy a context on CUDA device `device`.
 * Replaces: construction of IrvingKirkwood (irvingkirkwood/IrvingKirkwood.h:12-18)
 * and the MPI Communicator it holds (MPIInterface.h:58). */
int ik_create(ik_ctx** out, int device);
int ik_destroy(ik_ctx* ctx);

/* Box: SimBox(boxsize, origin, dim) semantics -- bounds [-L/2 - origin, L/2 - origin],
 * periodic in x, y and (3D only) z.  Replaces SimBox::SimBox (SimBox.cc:25-45). */
int ik_set_box(ik_ctx* ctx, int dim, const double boxsize[3], const double origin[3]);

/* Pair potentials: the eight ShortRangePairPotential<Model> types the reference exports
 * (potential/module-potential.cpp:13-34), params in the reference's own order:
 *   IK_POT_POLY12      PairPotentialPoly12          {v0, eps, c0, c1, c2}      Polydisperse12.h
 *   IK_POT_LJ          PairPotentialLJ              {eps, vareps}              LennardJones.h:6-88
 *   IK_POT_FSLJ        PairPotentialForceShiftedLJ  {eps, vareps}              LennardJones.h:91-125
 *   IK_POT_POLY10      PairPotentialPoly10          {v0, eps, c0, c1, c2, c3}  Polydisperse10.h
 *   IK_POT_POLY106     PairPotentialPoly106         {v0, eps, c0, c1, c2}      Polydisperse106.h
 *   IK_POT_POLY18      PairPotentialPoly18          {v0, eps, c0, c1, c2}      Polydisperse18.h
 *   IK_POT_POLYLJ      PairPotentialPolyLJ          {v0, eps, c0, c1, c2}      PolydisperseLJ.h
 *   IK_POT_POLYYUKAWA  PairPotentialPolyYukawa      {v0, kappa, eps, c0, c1, c2} PolydisperseYukawa.h
 * The force (computeForceDivR) is evaluated in FP64 in the reference's expression order
 * on the FP64 path (bit-identical to the CPU restatement; Yukawa within 2 ulp through
 * exp) and in FP32 on the FP32 path; the set of force-active bonds is the FP64 one on
 * both paths.  Replaces ShortRangePairPotential<Model> (potential/PairPotential.h:69-123). */
enum ik_pot_kind { IK_POT_POLY12 = 0, IK_POT_LJ = 1, IK_POT_FSLJ = 2, IK_POT_POLY10 = 3,
                   IK_POT_POLY106 = 4, IK_POT_POLY18 = 5, IK_POT_POLYLJ = 6, IK_POT_POLYYUKAWA = 7 };
int ik_set_potential(ik_ctx* ctx, int kind, double scaled_rcut, const double* params, int nparams);
/* Number of parameters of a kind (-1: unknown kind). */
int ik_potential_nparams(int kind);
/* = ik_set_potential(ctx, IK_POT_POLY12, scaled_rcut, params, 5). */
int ik_set_potential_poly12(ik_ctx* ctx, double scaled_rcut, const double params[5]);

/* Coarse-graining function.  rcut = support radius R (Gaussian: cut * width);
 * width = Gaussian standard deviation (Mollifier: the radius its normalisation was
 * built with); order = Gauss-Legendre points for IK_QUAD_FIXEDPOINT.  Modes on the GPU:
 * IK_QUAD_FIXEDPOINT (both paths); IK_QUAD_EXACT (FP64 path: the segment clipped to the
 * support, erf closed form for the Gaussian, GL on the clipped interval otherwise; FP32
 * path, Gaussian only: the clipped erf closed form for every bond, in FP32);
 * IK_QUAD_MLP (FP32 path, Gaussian: the attached surrogate on bonds that cross the edge
 * of the support, GL-order elsewhere and as its fallback); IK_QUAD_CLIPPED (FP32 path,
 * Gaussian: the clipped erf closed form on the bonds that cross the edge of the support
 * -- the bonds the surrogate stands in for -- and GL-order elsewhere); the closed-form and
 * surrogate modes keep plain per-lane sums (IK_FLAG_LANE_KAHAN is not applied) and do
 * not cover the elastic field on the FP32 path; IK_QUAD_ADAPTIVE (FP64 path:
 * QUADPACK's QAG with the GK15 rule per bond integral, as gsl_integration_qag key 1, at
 * most min(neval, 64) subintervals; a missed tolerance is reported as IK_ERR_QUADRATURE by
 * ik_synchronize / ik_eval_bond).
 * Replaces FixedPointCGFunc<...>(order, rcut) / AdaptiveCGFunc<...>(neval, relerr,
 * abserr, rcut) (irvingkirkwood/cgfunc/CoarseGrainFunction.h:56-134). */
int ik_set_cgfunc(ik_ctx* ctx, int kind, int mode, int order, double rcut, double width);
/* Adaptive-mode tolerances (AdaptiveCGFunc(neval, relerr, abserr, rcut)). */
int ik_set_adaptive(ik_ctx* ctx, int neval, double relerr, double abserr);
/* The Gauss-Kronrod 7/15 rule of the adaptive mode on [-1, 1] (host only): x[0] = 0 and
 * the positive nodes ascending (Kronrod nodes at odd slots, Gauss-7 nodes at even),
 * Kronrod weights wk, Gauss weights wg of the nodes 0, x[2], x[4], x[6]. */
int ik_gk15_rule(double x[8], double wk[8], double wg[4]);

/* Neighbour cut-off max_rcut; frozen like Calculator::max_rcut (Calculator.h:41-45).
 * If never set, the first uploaded frame fixes it to max(scaled_rcut*dmax, dmax). */
int ik_set_max_rcut(ik_ctx* ctx, double max_rcut);
int ik_get_max_rcut(ik_ctx* ctx, double* out);

/* Grid points (g x 3, FP64).  Replaces the gridpoints argument of
 * IrvingKirkwood::compute (IrvingKirkwood.h:21,74) and
 * CoarseGrainedField::addGridpoints (CoarseGrainedField.h:18-21). */
int ik_set_grid(ik_ctx* ctx, int64_t g, const double* xyz);

/* Frame slots.  pos/vel: n x 3 FP64 (vel may be NULL -> 0), mass: n (NULL -> 1),
 * diam: n.  Replaces ParticleSystem(simbox, N, d, m, pos, vel)
 * (ParticleSystem.cc:3-30) and IrvingKirkwood::setSystemData (Calculator.h:50-53).
 * Slot 0 is the default frame.  The copy is asynchronous on the context stream
 * from pinned host memory and synchronous otherwise. */
int ik_reserve_slots(ik_ctx* ctx, int nslots);
/* A box and grid of the slot's own (frames of different sizes in one batch): the
 * slot's computations use them instead of the context's ik_set_box / ik_set_grid,
 * and its fields have g grid points.  Same meaning as SimBox::SimBox (SimBox.cc:25-45)
 * and the ikcalculator grid (irvingkirkwood/__init__.py:44-51), per frame. */
/* The same upload from FP32 host arrays, as GSD files store them (particles/position,
 * velocity, mass, diameter: float32): one staging copy of half the bytes, widened to
 * FP64 on the GPU (exactly).  Replaces the list conversion of data_gsd.update
 * (utils.py:85-101) feeding ParticleSystem. */
int ik_upload_frame_f32(ik_ctx* ctx, int slot, int64_t n, const float* pos, const float* vel, const float* mass,
                        const float* diam);

/* Per-particle displacements u (n x 3, the slot's particle order) for the elastic
 * virial field IK_FIELD_ELASTIC: per neighbour pair within max_rcut,
 * 0.5 * bond * (f(|r+u_ij|) (r+u_ij)(x)(r+u_ij) - f(|r|) r(x)r), u_ij = u_j - u_i.
 * Replaces ParticleSystem::setDisplacement (ParticleSystem.cc:60-67) feeding
 * ElasticVirialStress (ListofCommonObservables.h:86-122) in ElasticVirialStressField
 * (irvingkirkwood/module-irvingkirkwood.cpp:10-11). */
int ik_upload_displacement(ik_ctx* ctx, int slot, int64_t n, const double* disp);
int ik_set_slot_geometry(ik_ctx* ctx, int slot, int dim, const double boxsize[3], const double origin[3],
                         int64_t g, const double* xyz);
int ik_upload_frame(ik_ctx* ctx, int slot, int64_t n, const double* pos, const double* vel,
                    const double* mass, const double* diam);
int ik_set_frame(ik_ctx* ctx, int64_t n, const double* pos, const double* vel,
                 const double* mass, const double* diam); /* = upload to slot 0 */

/* Enqueue the IK computation of a slot (cell list, bonds, gather) on the context
 * stream; results stay in HBM in the slot's field buffers.  fields: IK_FIELD_* mask.
 * Replaces IrvingKirkwood::compute (IrvingKirkwood.h:74-110). */
int ik_compute_slot(ik_ctx* ctx, int slot, int precision, int fields);
/* Compute `count` slots as one batch.  The first call with a given slot list runs
 * the slots with ordinary launches (sizing every buffer) and records the same
 * sequence as a CUDA graph; later calls with the same slots, precision and fields
 * replay that graph with a single launch (re-recorded automatically after a frame's
 * size, the box, the grid or a capacity changes).  Asynchronous like ik_compute_slot.
 * Replaces the per-frame loop of pyglasstools.analyze (pyglasstools/__init__.py:107-138)
 * over IrvingKirkwood::compute for resident frames. */
int ik_compute_batch(ik_ctx* ctx, const int* slots, int count, int precision, int fields);

/* Wait for all of the context's work; reports device-side status words.  (Slots are
 * computed on several internal streams so that consecutive frames overlap.) */
int ik_synchronize(ik_ctx* ctx);
/* Make the context's main stream (ik_get_stream) wait, on the device, for all work
 * enqueued so far; no host synchronisation.  For timing with events on that stream. */
int ik_wait_all(ik_ctx* ctx);
/* ik_compute_slot(0) + ik_synchronize. */
int ik_compute(ik_ctx* ctx, int precision, int fields);

/* Field download: out = g x dim x dim FP64, column-major per grid point
 * (element (a,b) at g*dim*dim + a + dim*b), matching the Eigen::Tensor<double,2>
 * storage behind CoarseGrainedField::gettostring (CoarseGrainedField.h:160-183). */
int ik_get_field(ik_ctx* ctx, int slot, int field, double* out, int64_t count);

/* Candidate neighbour list within `radius` (FP64 minimum image, |r_ij|^2 < radius^2,
 * j != i, j ascending): CSR offs[n+1], idx[nnz].  Call with idx == NULL to get nnz.
 * Replaces ParticleSystem::getNeighborsDistance / the Aboria euclidean_search
 * around particles (ParticleSystem.cc:183-195, IrvingKirkwood.h:93-95). */
int ik_get_neighbors(ik_ctx* ctx, int slot, double radius, int64_t* offs, int32_t* idx,
                     int64_t idx_capacity, int64_t* nnz);
/* Particles within `radius` of a point, ascending ids.
 * Replaces ParticleSystem::getNeighbors (ParticleSystem.cc:171-181). */
int ik_get_neighbors_point(ik_ctx* ctx, int slot, const double point[3], double radius,
                           int32_t* ids, int64_t capacity, int64_t* count);

/* Per-pair scalar kernels on the device for API parity with
 * PairPotential::getPairForceDivR / getPairEnergy and
 * CoarseGrainFunction::getDeltaFunc / getBondFunc (PairPotential.h:98-113,
 * CoarseGrainFunction.h:78-88).  Arrays of m queries; rij/x/ri: m x 3. */
int ik_eval_pair(ik_ctx* ctx, int64_t m, const double* rij, const double* di,
                 const double* dj, double* force_divr, double* energy);
int ik_eval_bond(ik_ctx* ctx, int64_t m, const double* x, const double* ri,
                 const double* rij, double* bond, double* delta);

/* Timing of the last ik_compute_slot on the stream (ms per stage, CUDA events):
 * [0] cells, [1] bonds, [2] gather, [3] total.  Needs IK_TIMING in ik_set_flags. */
#define IK_FLAG_TIMING 1
/* FP32 path: Kahan-compensated per-lane sums (the combination of the lane partials
 * of every grid point is always compensated; per-lane sums are plain by default). */
#define IK_FLAG_LANE_KAHAN 2
#define IK_FLAG_CSR_BONDS 4 /* FP32 path: compact the bond records to CSR even when the
                               fixed-stride layout fits (the layout used for n * maxb >= 2^25) */
int ik_set_flags(ik_ctx* ctx, int flags);
int ik_get_timing(ik_ctx* ctx, float* ms4);

/* The context's CUDA stream (a cudaStream_t), for callers that time or order
 * work against it (e.g. CUDA events recorded on this stream). */
int ik_get_stream(ik_ctx* ctx, void** stream);

/* One batch with host I/O, replayed as one CUDA graph: for each slots[k], frame k is
 * copied from page-locked host memory (n[k] particles; pos[k] n x 3 and diam[k] required,
 * vel[k] n x 3 and mass[k] optional -- vel / mass themselves may be null), computed
 * (`fields`), and every requested field written to page-locked host memory
 * out[3k + f] (f = 0 virial, 1 kinetic, 2 elastic; g x NC FP64 as in
 * ik_download_field_async; null = not copied).  The copies and kernels of a frame run on
 * one engine lane, so the uploads, computations and downloads of different frames
 * overlap; or, with IK_TUNE_IO_BATCHES = n >= 1 and a batch that can run fused (see
 * IK_TUNE_FUSED_BATCH), the batch runs as n fused sub-batches: one stream uploads the
 * frames in order, each sub-batch is computed once its frames are on the device, and its
 * fields are downloaded as soon as it is done, so that the copies of the other
 * sub-batches overlap its computation.  The first call (and any call after a change of slots, sizes, pointers or
 * settings) runs the plain path and records the graph; later calls replay it, reading the
 * host inputs' current contents.  The graph holds the host arrays' addresses (page-locked
 * status is checked when they change): an array freed and replaced by another at the same
 * address must be page-locked too, as the replay copies from and to it (host-mapped
 * copies: through the device's view of it).  Outputs are complete after ik_synchronize (which copies
 * them again if a capacity growth re-ran a frame).  Slots must be distinct.  Elastic
 * fields use the displacements of ik_upload_displacement. */
int ik_compute_batch_io(ik_ctx* ctx, const int* slots, int count, int precision, int fields,
                        const int64_t* n, const double* const* pos, const double* const* vel,
                        const double* const* mass, const double* const* diam, double* const* out);

/* Autotuner of ik_compute_batch_io (no reference counterpart; arguments as there): times
 * `reps` CUDA-graph replays of the batch, host copies included (CUDA events on the
 * context's stream), for each schedule of its copies -- per frame on the lanes at the
 * current CTAs per SM and at the lanes' default, and, for a batch that can run fused, 2, 4,
 * 8, 16 and 32 fused sub-batches with their copies on the copy engines and 1, 2 and 4 with
 * host-mapped copies (at most one sub-batch per frame) -- and keeps the fastest
 * (IK_TUNE_IO_BATCHES, IK_TUNE_IO_MAPPED, IK_TUNE_BLOCKS_PER_SM).  Tune the resident batch first
 * (ik_autotune_batch): the sub-batches run with its settings.  The host outputs hold the
 * batch's fields afterwards. */
int ik_autotune_batch_io(ik_ctx* ctx, const int* slots, int count, int precision, int fields,
                         const int64_t* n, const double* const* pos, const double* const* vel,
                         const double* const* mass, const double* const* diam, double* const* out,
                         int reps, int* best_io_batches, float* best_ms);

/* Asynchronous download of a slot's field in compact form: g x NC FP64 with
 * NC = 3 (xx, yy, xy) in 2D or 6 (xx, yy, zz, xy, xz, yz) in 3D.  The copy runs on a
 * download stream of its own after the slot's computation, so that it overlaps the
 * uploads of other frames and their computations; the slot's next computation waits for
 * it.  host_out should be pinned for the copy to overlap; it is complete after
 * ik_synchronize. */
int ik_download_field_async(ik_ctx* ctx, int slot, int field, double* host_out, int64_t count);

/* Measured FP32 FMA throughput of `device` (TFLOP/s, 2 FLOP per FMA) from a
 * dependent-chain-free FFMA loop over all SMs; the roofline denominator of the
 * FP32 gather.  Diagnostic: no reference counterpart. */
int ik_measure_fp32_peak(int device, double* tflops);

/* No-allocation variant of the plain FP64 computation (ik_compute with IK_PREC_FP64),
 * for callers that cannot call cudaMalloc: processes whose device memory belongs to
 * another framework's pool, services under a device-memory budget fixed at start-up,
 * and code that must not enter cudaMalloc because it can wait for other streams' work.
 * No counterpart in the reference.  Allocates nothing: the caller passes DEVICE
 * pointers for inputs (d_pos n x 3, d_diam n, optional d_vel n x 3 and d_mass n,
 * d_grid g x 3) and outputs (d_virial and optional d_kinetic, each g x NC FP64 with
 * NC = 3 in 2D (xx, yy, xy) or 6 in 3D (xx, yy, zz, xy, xz, yz)); all scratch is a
 * static device array of about 4.3 MB that every GPU loading the library holds until
 * exit.  Limits: n <= 4096 particles (larger n is rejected with IK_ERR_CAPACITY), at
 * most 32 force-active bonds per particle (IK_ERR_CAPACITY after the run).  Runs on
 * `stream` (a cudaStream_t; NULL = default stream).  The call is synchronous: it makes
 * CUDA runtime calls and returns after that stream has finished, so it must not be
 * made from a stream callback or a host function (cudaLaunchHostFunc).  The first
 * call in each CUDA context (the first call on each device, for the primary context)
 * sets up the scratch address; make it before any stream capture.  Calls share the
 * scratch array: calls that overlap on the GPU race and must be serialised by the
 * caller.  Box, potential and coarse-graining arguments mean what they mean in
 * ik_set_box, ik_set_potential_poly12, ik_set_max_rcut and ik_set_cgfunc
 * (fixed-point mode). */
int ik_compute_fp64_noalloc(int dim, const double boxsize[3], const double origin[3],
                            double scaled_rcut, const double params[5], double max_rcut,
                            int cg_kind, int gl_order, double cg_rcut, double cg_width,
                            int64_t n, const double* d_pos, const double* d_diam,
                            const double* d_vel, const double* d_mass, int64_t g,
                            const double* d_grid, double* d_virial, double* d_kinetic,
                            void* stream);

/* Global thermodynamic observables of a slot's frame: ThermoCalculator::compute
 * (thermo/ThermoCalculator.h:68-90) with every observable of thermo/module-thermo.cpp:7-20.
 * Unique pairs i < j within max_rcut, r_ij = r_i - r_j (the reference's p_j.dx()), and the
 * particles' kinetic terms, all divided by the box volume (SimBox::vol).  out (FP64, count
 * >= IK_THERMO_SIZE(dim)): [0] potential energy; then virial, elastic virial (zero unless a
 * displacement was uploaded) and kinetic stress, dim x dim each at index a + dim*b; then
 * the Born tensor, dim^4 at index i + dim*(j + dim*(k + dim*l)).  FP64, deterministic,
 * synchronous.  Replaces ThermoCalculator::compute + the Global* ThermoProperty classes. */
#define IK_THERMO_SIZE(dim) (1 + 3 * (dim) * (dim) + (dim) * (dim) * (dim) * (dim))
int ik_compute_thermo(ik_ctx* ctx, int slot, double* out, int64_t count);

/* Number of kernels this context has launched since it was created. */
int ik_get_launch_count(ik_ctx* ctx, int64_t* out);

/* Counters of the last computation: [0] force-active directed bonds,
 * [1] accepted (grid, particle) pairs, [2] active (grid, i, j) triples (FP32 path). */
int ik_get_counters(ik_ctx* ctx, int slot, int64_t* out3);
/* Tuning of the FP32 gather (no reference counterpart).  0 restores the default (except
 * IK_TUNE_FUSED_BATCH, where 0 turns fused batches off).
 *   IK_TUNE_BIN_POINTS     target grid points per work item (bin of cells)
 *   IK_TUNE_BLOCKS_PER_SM  persistent CTAs launched per SM (default: 2 for a frame computed alone and
 *                          for a fused batch, 1 for the frames of a batch that run side by side on
 *                          the engine lanes)
 *   IK_TUNE_HALO_CAP       staged halo particles per warp (grows on overflow)
 *   IK_TUNE_FUSED_BATCH    1 (default): ik_compute_batch runs an eligible batch fused -- every
 *                          stage once over all its frames (bin, scan, scatter, sort + pack,
 *                          bonds, one persistent gather over every frame's work items,
 *                          finish: 7 to 8 kernel launches per batch, recorded as one CUDA
 *                          graph); 0: one launch sequence per frame on the lanes.  Eligible:
 *                          FP32 path, virial and/or kinetic field, fixed-point rule of order
 *                          4 or 5, n * (bonds per particle) < 2^25 per slot, no slot twice
 *   IK_TUNE_IO_BATCHES     ik_compute_batch_io: 0 (default): each frame's copies and kernels on
 *                          one engine lane; n >= 1, for a batch that can run fused (fused
 *                          batches on): n fused sub-batches -- contiguous runs of frames with
 *                          about equal particle counts, never more than the frames -- whose
 *                          host copies overlap the other sub-batches' computation
 *   IK_TUNE_IO_MAPPED      with IK_TUNE_IO_BATCHES >= 1: 0 (default): the copies on the copy
 *                          engines, one per array; 1: each sub-batch's uploads (with the
 *                          frames' validation) and downloads as one kernel each, reading and
 *                          writing the device's view of the page-locked host arrays, on the
 *                          sub-batch's stream -- no per-array copy cost, for batches of
 *                          many small frames (arrays without a device view: copy engines) */
#define IK_TUNE_BIN_POINTS 1
#define IK_TUNE_BLOCKS_PER_SM 2
#define IK_TUNE_HALO_CAP 3
#define IK_TUNE_FUSED_BATCH 4
#define IK_TUNE_IO_BATCHES 5
#define IK_TUNE_IO_MAPPED 6
int ik_set_tuning(ik_ctx* ctx, int param, int value);
int ik_get_tuning(ik_ctx* ctx, int param, int* value);
/* Diagnostic (no reference counterpart): runs the batch once fused, without a graph,
 * with CUDA events around its stages, and returns ms4 = {preparation (bin, scan,
 * scatter, sort + pack, bonds), 0, the persistent gather over every frame, both}.  The
 * slots' fields are computed as by ik_compute_batch.  IK_ERR_UNSUPPORTED for a batch
 * that cannot run fused (see IK_TUNE_FUSED_BATCH). */
int ik_time_fused_batch(ik_ctx* ctx, const int* slots, int count, int fields, float* ms4);
/* Autotuner: times ik_compute_batch over the given slots (`reps` CUDA-graph replays per
 * candidate, CUDA events on the context's stream) for each candidate schedule (fused
 * batch or per-frame lanes) x bin size x CTAs per SM x staged halo per warp, keeps the
 * fastest (all four settings, readable with ik_get_tuning) and reports the bin size,
 * CTAs per SM and time.  FP32 path only. */
int ik_autotune_batch(ik_ctx* ctx, const int* slots, int count, int precision, int fields, int reps,
                      int* best_bin_points, int* best_blocks_per_sm, float* best_ms);

/* Bonds the last surrogate-mode computation of `slot` handed to the network (crossing
 * the edge of the support; each falls back on its fixed-point value outside the
 * validated bins).  No reference counterpart. */
int ik_get_mlp_records(ik_ctx* ctx, int slot, int64_t* out);

/* ---- learned bond-integral surrogate -------------------------------------------
 * No reference counterpart: a small network (4 -> 64 -> 64 -> 64 -> 1, SiLU) that
 * stands in for the quadrature of the bond integral (cgfunc/CoarseGrainFunction.h:85-88
 * fixed point, :124-127 adaptive) of a Gaussian kernel truncated at 3 widths, on the
 * bonds that cross the kernel's support.  Units of the width w throughout:
 *   B(d, a, b) = int_0^1 exp(-(d^2 + (a + s (b - a))^2) / 2) [inside r < 3] ds,
 * d = distance of the grid point from the bond's line, a / b = signed positions of the
 * inside / outside end along it (b > 0).  Inputs x = (sqrt(1 - (d/3)^2), a/4, b/4,
 * 2 (w - 1.5)); output y with B = base (1 + y / 1e4), base = four-point Gauss-Legendre
 * on the part of the bond inside the support (the fraction s1 = (t_c - a)/(b - a),
 * t_c = sqrt(9 - d^2)): the network learns the scaled residual of that rule, whose
 * relative error is below 1e-4 here, so its own error reaches B scaled down by 1e4.
 * Trained on the GPU in FP32 (own forward,
 * backward and Adam kernels) on labels from adaptive quadrature; deployed in BF16 on
 * the tensor cores (tcgen05, FP32 accumulation).  A per-bin table from validation
 * decides where the network replaces the fixed-point rule (max error <= tol).
 * Parameters: W1[64][4], b1[64], W2[64][64], b2[64], W3[64][64], b3[64], w4[64], b4. */
typedef struct ik_mlp ik_mlp;
int ik_mlp_create(ik_mlp** out, int device);
int ik_mlp_destroy(ik_mlp* m);
int ik_mlp_num_params(void);                                       /* 8705 */
int ik_mlp_init(ik_mlp* m, uint64_t seed);                          /* fan-in uniform weights */
int ik_mlp_set_params(ik_mlp* m, const float* params, int64_t n);
int ik_mlp_get_params(ik_mlp* m, float* params, int64_t n);
/* n seeded samples of the crossing-bond domain: feats n x {d, a, b, w}, labels B (FP64) */
int ik_mlp_samples(ik_mlp* m, int64_t n, uint64_t seed, float* feats, double* labels);
/* gradient of the mean squared error of y over a batch (n a power of two) */
int ik_mlp_grad(ik_mlp* m, int64_t n, const float* feats, const float* targets, float* grad, double* loss);
/* Adam on nsamples (power of two) generated samples; loss_hist gets the per-step loss */
int ik_mlp_train(ik_mlp* m, int64_t nsamples, int epochs, int ctas, double lr, uint64_t seed,
                 double* loss_hist, int64_t hist_len);
/* B of n feature rows; kernel 0 = tensor cores (BF16), 1 = CUDA cores BF16, 2 = FP32;
 * kernel | IK_MLP_EVAL_RAW: the network's output y = (B / base - 1) * 1e4 instead of B */
#define IK_MLP_EVAL_RAW 4
int ik_mlp_eval(ik_mlp* m, int64_t n, const float* feats, float* out, int kernel);
/* error of the deployed network on n fresh samples; builds the per-bin use table:
 * bins of (w, d, a, b) with >= 8 samples and max |B_net - B_label| <= tol */
int ik_mlp_validate(ik_mlp* m, int64_t n, uint64_t seed, double tol, double* coverage, double* max_err,
                    double* rms_err, double* bin_err, int64_t nbins);
/* Failure-detection test hook (no reference counterpart; the reference's quadrature
 * failures abort the process through GSL's default handler, cgfunc/Quadrature.h:47-49,
 * and its exception hook calls MPI_Abort, pyglasstools/__init__.py:26-35).  With
 * on != 0 the tensor-core inference kernels of this surrogate issue no MMA and wait for
 * its completion with a poll limit of 64: the wait runs out, the kernel frees its
 * tensor memory and returns, and the call reports IK_ERR_TIMEOUT (ik_mlp_eval,
 * ik_mlp_validate; ik_synchronize for an IK computation in surrogate mode), with the
 * CUDA context left usable.  on = 0 restores normal operation. */
int ik_mlp_test_stall(ik_mlp* m, int on);
/* Attach a validated surrogate to a context; used by ik_set_cgfunc(.., IK_QUAD_MLP, ..)
 * on the FP32 path.  The caller keeps the surrogate alive while attached. */
int ik_set_mlp(ik_ctx* ctx, ik_mlp* m);
/* Records of the slot's last computation in surrogate mode that kept their fixed-point
 * value (their bin was not validated within the tolerance, or lies outside the table);
 * ik_get_mlp_records gives all records. */
int ik_get_mlp_fallbacks(ik_ctx* ctx, int slot, int64_t* out);

#ifdef __cplusplus
}
#endif
#endif /* IK_GB300_H */
