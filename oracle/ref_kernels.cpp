// Shim that exposes the reference's own pair-force and coarse-graining kernel
// classes through a C ABI so the oracle's restatement can be pinned against
// them.  It includes the reference headers from the reference tree at build
// time (paths passed by build_ref.sh); no reference source is copied here.
#include <cmath>
#include <vector>
#include REF_POLY12_H
#include REF_OCTIC_H
#include REF_RECT_H
#include REF_MOLLIFIER_H

extern "C" {
double ref_poly12_force_divr(double rsq, double scaled_rcut, const double* prm, double di, double dj)
{
    std::vector<double> p(prm, prm + 5);
    Polydisperse12 m(rsq, scaled_rcut * scaled_rcut, p);
    return m.computeForceDivR(di, dj);
}
double ref_poly12_energy(double rsq, double scaled_rcut, const double* prm, double di, double dj)
{
    std::vector<double> p(prm, prm + 5);
    Polydisperse12 m(rsq, scaled_rcut * scaled_rcut, p);
    return m.computeEnergy(di, dj);
}
double ref_poly12_stiffness(double rsq, double scaled_rcut, const double* prm, double di, double dj)
{
    std::vector<double> p(prm, prm + 5);
    Polydisperse12 m(rsq, scaled_rcut * scaled_rcut, p);
    return m.computeStiffness(di, dj);
}
double ref_octic(double rcut, double dr_sq) { Octic f(rcut); return f.compute(dr_sq); }
double ref_rect(double rcut, double dr_sq) { Rect f(rcut); return f.compute(dr_sq); }
double ref_mollifier(double rcut, double dr_sq) { Mollifier f(rcut); return f.compute(dr_sq); }
}
