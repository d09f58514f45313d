/*
 * ik_oracle.h -- CPU FP64 restatement of pyglasstools' Irving-Kirkwood (IK)
 * stress-field path.  TEST INFRASTRUCTURE ONLY: the oracle is the checker for
 * the CUDA path and the timed CPU baseline; the product never calls it.
 *
 * Parity status: the reference's IK loop (IrvingKirkwood.h) needs Aboria, Eigen,
 * GSL and MPI, none of which is present, so the loop itself cannot be run here:
 * parity of the FIELD is unpinned by the reference.  The pair force and the
 * coarse-graining kernels ARE pinned: oracle/build_ref.sh compiles
 * pyglasstools/potential/Polydisperse12.h and the cgfunc/CGFunc*.h headers from
 * the reference tree and tests/test_oracle_pins.py checks the restatement
 * against them bit for bit (plus committed golden vectors for machines without
 * the reference tree).  Quadrature is pinned by exactness on polynomials and by
 * closed forms (octic polynomial, truncated-Gaussian erf form).
 */
#ifndef IK_ORACLE_H
#define IK_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { IKOR_CG_OCTIC = 0, IKOR_CG_GAUSSIAN = 1, IKOR_CG_RECT = 2, IKOR_CG_MOLLIFIER = 3 };
enum { IKOR_QUAD_FIXED = 0, IKOR_QUAD_ADAPTIVE = 1, IKOR_QUAD_EXACT = 2 };

typedef struct {
    int dim;            /* 2 or 3 */
    double L[3];        /* box edge lengths (SimBox::boxsize) */
    double lo[3];       /* lower bound (SimBox::lowerbound) */
    int periodic[3];    /* 1 = periodic (x, y always; z only in 3D) */
} ikor_box;

/* The eight pair models of potential/module-potential.cpp:13-34. */
enum { IKOR_POT_POLY12 = 0, IKOR_POT_LJ = 1, IKOR_POT_FSLJ = 2, IKOR_POT_POLY10 = 3,
       IKOR_POT_POLY106 = 4, IKOR_POT_POLY18 = 5, IKOR_POT_POLYLJ = 6, IKOR_POT_POLYYUKAWA = 7 };

/* Pair potential in a common layout: v0 = energy scale (LJ: eps), eps = non-additivity
 * (LJ: vareps), c0..c3 smoothing coefficients (c3: Poly10), kappa (Yukawa). */
typedef struct {
    double scaled_rcut; /* r~_c: cut-off in units of sigma_ij */
    double v0, eps, c0, c1, c2;
    int kind;           /* IKOR_POT_* */
    double c3, kappa;
} ikor_pot;

typedef struct {
    int kind;           /* IKOR_CG_* */
    int mode;           /* IKOR_QUAD_* */
    int order;          /* Gauss-Legendre points (fixed mode) */
    double rcut;        /* support radius R (Gaussian: cut * width) */
    double width;       /* Gaussian standard deviation w (unused otherwise) */
    double epsabs, epsrel; /* adaptive mode tolerances */
    int limit;          /* adaptive mode: max subintervals */
} ikor_cg;

/* Gauss-Legendre nodes/weights on [-1,1] (Newton on the three-term recurrence). */
void ikor_gl_rule(int n, double* x, double* w);

/* computeForceDivR / computeEnergy of every model; computeStiffness of Polydisperse12. */
double ikor_force_divr(const ikor_pot* p, double rsq, double di, double dj);
double ikor_pair_energy(const ikor_pot* p, double rsq, double di, double dj);
double ikor_bond_stiffness(const ikor_pot* p, double rsq, double di, double dj);

/* Coarse-graining kernel Delta(dr_sq) for a d-dimensional system. */
double ikor_delta(const ikor_cg* cg, int dim, double dr_sq);
/* Bond integral  B = int_0^1 Delta(|x - (ri + s rij)|^2) ds. */
double ikor_bond(const ikor_cg* cg, int dim, const double x[3], const double ri[3], const double rij[3]);

/* max_rcut = max(scaled_rcut * d_max, d_max)  (Calculator.h:41-45). */
double ikor_max_rcut(double scaled_rcut, int64_t n, const double* diam);

/* Minimum-image displacement b - a (FP64, no contraction). */
void ikor_min_image(const ikor_box* box, const double a[3], const double b[3], double out[3]);

/* Candidate neighbour list: for every i all j != i with |minimg(r_j - r_i)|^2 < radius^2,
 * j ascending.  offs has n+1 entries; idx must hold offs[n] entries (call once with
 * idx == NULL to size it).  Returns the total count. */
int64_t ikor_neighbors(const ikor_box* box, int64_t n, const double* pos, double radius,
                       int64_t* offs, int32_t* idx);

/* The IK gather (IrvingKirkwood::compute restated).  pos/vel: n x 3, diam/mass: n.
 * vel/mass may be NULL (kinetic field then zero).  grid: g x 3.
 * virial/kinetic: g x dim x dim, column-major per grid point (index a + dim*b).
 * nthreads <= 0: OpenMP default.  Returns 0 or a negative error. */
/* The same gather with the elastic virial field of ElasticVirialStressField
 * (ListofCommonObservables.h:86-122 through VirialStress::compute_cg, :72-82): per pair
 * 0.5 * bond * (f(|r+u|) (r+u)(x)(r+u) - f(|r|) r(x)r), u = disp_j - disp_i, over the
 * neighbours within max_rcut of the undisplaced frame.  disp: n x 3. */
int ikor_compute_elastic(const ikor_box* box, int64_t n, const double* pos, const double* disp,
                         const double* diam, const ikor_pot* pot, const ikor_cg* cg,
                         double max_rcut, int64_t g0, int64_t g1, const double* grid,
                         double* virial, double* elastic, int nthreads);

int ikor_compute(const ikor_box* box, int64_t n, const double* pos, const double* vel,
                 const double* mass, const double* diam, const ikor_pot* pot,
                 const ikor_cg* cg, double max_rcut, int64_t g, const double* grid,
                 double* virial, double* kinetic, int nthreads);

/* Same loop restricted to grid points [g0, g1) (used for bounded CPU samples). */
int ikor_compute_range(const ikor_box* box, int64_t n, const double* pos, const double* vel,
                       const double* mass, const double* diam, const ikor_pot* pot,
                       const ikor_cg* cg, double max_rcut, int64_t g0, int64_t g1,
                       const double* grid, double* virial, double* kinetic, int nthreads);

/* Global virial sum_{i<j} F_ij (x) r_ij (ThermoCalculator.h:68-90, not divided by volume). */
void ikor_global_virial(const ikor_box* box, int64_t n, const double* pos, const double* diam,
                        const ikor_pot* pot, double max_rcut, double* out /* dim x dim */);
/* OpenMP threads of the oracle's parallel regions after asking for `requested` (0: the
 * default); 1 without OpenMP. */
int ikor_threads(int requested);

/* Global thermodynamic observables (ThermoCalculator::compute); out holds
 * 1 + 3 dim^2 + dim^4 values: energy, virial, elastic virial, kinetic stress, Born tensor,
 * all divided by the box volume. */
void ikor_global_thermo(const ikor_box* box, int64_t n, const double* pos, const double* vel, const double* mass,
                        const double* diam, const double* disp, const ikor_pot* pot, double max_rcut, double* out);

#ifdef __cplusplus
}
#endif
#endif
