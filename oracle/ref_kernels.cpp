// Shim that exposes the reference's own pair-force and coarse-graining kernel
// classes through a C ABI so the oracle's restatement can be pinned against
// them.  It includes the reference headers from the reference tree at build
// time (include paths passed by build_ref.sh); no reference source is copied here.
#include <cmath>
#include <vector>
#include "Polydisperse12.h"
#include "Polydisperse10.h"
#include "Polydisperse106.h"
#include "Polydisperse18.h"
#include "PolydisperseLJ.h"
#include "PolydisperseYukawa.h"
#include "LennardJones.h"
#include "CGFuncOctic.h"
#include "CGFuncRect.h"
#include "CGFuncMollifier.h"

namespace {
// ShortRangePairPotential<Model>::getPairForceDivR / getPairEnergy
// (potential/PairPotential.h:98-113): a non-const model built from rsq and
// scaled_rcut^2, so the force-shifted LJ's own computeForceDivR is the one called.
template <class M>
double force_of(double rsq, double rc, const double* prm, int np, double di, double dj)
{
    std::vector<double> p(prm, prm + np);
    M m(rsq, rc * rc, p);
    return m.computeForceDivR(di, dj);
}
template <class M>
double energy_of(double rsq, double rc, const double* prm, int np, double di, double dj)
{
    std::vector<double> p(prm, prm + np);
    M m(rsq, rc * rc, p);
    return m.computeEnergy(di, dj);
}
template <class M>
double stiffness_of(double rsq, double rc, const double* prm, int np, double di, double dj)
{
    std::vector<double> p(prm, prm + np);
    M m(rsq, rc * rc, p);
    return m.computeStiffness(di, dj);
}
}  // namespace

extern "C" {
double ref_poly12_force_divr(double rsq, double scaled_rcut, const double* prm, double di, double dj)
{
    return force_of<Polydisperse12>(rsq, scaled_rcut, prm, 5, di, dj);
}
double ref_poly12_energy(double rsq, double scaled_rcut, const double* prm, double di, double dj)
{
    return energy_of<Polydisperse12>(rsq, scaled_rcut, prm, 5, di, dj);
}
double ref_poly12_stiffness(double rsq, double scaled_rcut, const double* prm, double di, double dj)
{
    std::vector<double> p(prm, prm + 5);
    Polydisperse12 m(rsq, scaled_rcut * scaled_rcut, p);
    return m.computeStiffness(di, dj);
}
// kind: 0 Poly12, 1 LJ, 2 force-shifted LJ, 3 Poly10, 4 Poly106, 5 Poly18, 6 PolyLJ, 7 PolyYukawa
double ref_pot_force_divr(int kind, double rsq, double rc, const double* prm, int np, double di, double dj)
{
    switch (kind) {
    case 1: return force_of<LennardJones>(rsq, rc, prm, np, di, dj);
    case 2: return force_of<ForceShiftedLennardJones>(rsq, rc, prm, np, di, dj);
    case 3: return force_of<Polydisperse10>(rsq, rc, prm, np, di, dj);
    case 4: return force_of<Polydisperse106>(rsq, rc, prm, np, di, dj);
    case 5: return force_of<Polydisperse18>(rsq, rc, prm, np, di, dj);
    case 6: return force_of<PolydisperseLJ>(rsq, rc, prm, np, di, dj);
    case 7: return force_of<PolydisperseYukawa>(rsq, rc, prm, np, di, dj);
    default: return force_of<Polydisperse12>(rsq, rc, prm, np, di, dj);
    }
}
double ref_pot_energy(int kind, double rsq, double rc, const double* prm, int np, double di, double dj)
{
    switch (kind) {
    case 1: return energy_of<LennardJones>(rsq, rc, prm, np, di, dj);
    case 2: return energy_of<ForceShiftedLennardJones>(rsq, rc, prm, np, di, dj);
    case 3: return energy_of<Polydisperse10>(rsq, rc, prm, np, di, dj);
    case 4: return energy_of<Polydisperse106>(rsq, rc, prm, np, di, dj);
    case 5: return energy_of<Polydisperse18>(rsq, rc, prm, np, di, dj);
    case 6: return energy_of<PolydisperseLJ>(rsq, rc, prm, np, di, dj);
    case 7: return energy_of<PolydisperseYukawa>(rsq, rc, prm, np, di, dj);
    default: return energy_of<Polydisperse12>(rsq, rc, prm, np, di, dj);
    }
}
double ref_pot_stiffness(int kind, double rsq, double rc, const double* prm, int np, double di, double dj)
{
    switch (kind) {
    case 1: return stiffness_of<LennardJones>(rsq, rc, prm, np, di, dj);
    case 2: return stiffness_of<ForceShiftedLennardJones>(rsq, rc, prm, np, di, dj);
    case 3: return stiffness_of<Polydisperse10>(rsq, rc, prm, np, di, dj);
    case 4: return stiffness_of<Polydisperse106>(rsq, rc, prm, np, di, dj);
    case 5: return stiffness_of<Polydisperse18>(rsq, rc, prm, np, di, dj);
    case 6: return stiffness_of<PolydisperseLJ>(rsq, rc, prm, np, di, dj);
    case 7: return stiffness_of<PolydisperseYukawa>(rsq, rc, prm, np, di, dj);
    default: return stiffness_of<Polydisperse12>(rsq, rc, prm, np, di, dj);
    }
}
double ref_octic(double rcut, double dr_sq) { Octic f(rcut); return f.compute(dr_sq); }
double ref_rect(double rcut, double dr_sq) { Rect f(rcut); return f.compute(dr_sq); }
double ref_mollifier(double rcut, double dr_sq) { Mollifier f(rcut); return f.compute(dr_sq); }
}
