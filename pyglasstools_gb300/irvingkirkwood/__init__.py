R"""Irving-Kirkwood coarse-grained fields (pyglasstools/irvingkirkwood/__init__.py).

``ikcalculator(cgfunc, dx, precision=None)`` builds the reference's lattice grid
(linspace(-L/2, L/2, int(L/dx)) per axis, endpoints included) and computes the
registered fields on the GPU.  ``precision="fp64"`` selects the plain FP64 kernels,
"fp32" the tuned path (FP32 pair arithmetic, compensated accumulation, FP64 selection
and final sums); the default is "fp32", or "fp64" for an adaptive or exact bond
integral (those run on the FP64 path).
"""
import numpy as np

import pyglasstools_gb300
from pyglasstools_gb300 import _core, comm, rank, size, solvers_list

_irvingkirkwood = _core._irvingkirkwood


def initialize_field(names, dim, gridpoints):
    """Field objects for the requested names (irvingkirkwood/__init__.py:8-32)."""
    list_obs = {}
    n = len(gridpoints)
    if any("virialstress" in s for s in names):
        if any("elastic" in s for s in names):
            cls = (_irvingkirkwood.ElasticVirialStressField2D if dim == 2
                   else _irvingkirkwood.ElasticVirialStressField3D)
            list_obs['elasticvirialstress'] = cls("elasticvirialstress", "2-TENSOR", False, n)
            list_obs['elasticvirialstress'].addGridpoints(gridpoints)
        if all("elastic" in s for s in names) is False:
            cls = _irvingkirkwood.VirialStressField2D if dim == 2 else _irvingkirkwood.VirialStressField3D
            list_obs['virialstress'] = cls("virialstress", "2-TENSOR", False, n)
            list_obs['virialstress'].addGridpoints(gridpoints)
    if any("kineticstress" in s for s in names):
        cls = _irvingkirkwood.KineticStressField2D if dim == 2 else _irvingkirkwood.KineticStressField3D
        list_obs['kineticstress'] = cls("kineticstress", "2-TENSOR", True, n)
        list_obs['kineticstress'].addGridpoints(gridpoints)
    return list_obs


def lattice_gridpoints(L, dx, dim=2):
    """The reference's grid: nmax = int(L/dx) points per axis over [-L/2, L/2]."""
    nmax = int(L / dx)
    points = np.linspace(-L / 2.0, +L / 2.0, nmax)
    if dim == 2:
        gx, gy = np.meshgrid(points, points, indexing="ij")
        return np.stack([gx.ravel(), gy.ravel(), np.zeros(gx.size)], axis=1)
    gx, gy, gz = np.meshgrid(points, points, points, indexing="ij")
    return np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1)


def _default_precision(cgfunc, precision):
    """FP32 (the tuned path) unless the bond integral is adaptive or exact (FP64 path)."""
    if precision is not None:
        return precision
    return "fp64" if cgfunc._getCGFunc().mode in ("adaptive", "exact") else "fp32"


class ikcalculator(object):
    def __init__(self, cgfunc, dx, precision=None):
        self.cgfunc = cgfunc
        self.manager = _core._pyglasstools.Manager()
        self.coordmode = "cartesian"
        sysdata = pyglasstools_gb300.get_sysdata()
        L = sysdata.pysimbox.boxsize[0]
        self.gridpoints = lattice_gridpoints(L, dx, sysdata.pysimbox.dim)
        self.gridsize = len(self.gridpoints)
        self.calculator = _irvingkirkwood.IrvingKirkwood(
            sysdata.cppparticledata, pyglasstools_gb300.get_potential().cpppairpotential,
            cgfunc._getCGFunc(), comm)
        self.calculator.setPrecision(_default_precision(cgfunc, precision))
        solvers_list.append(self)

    def add_observables(self, observables):
        for name in observables:
            self.calculator.addObservable(observables[name])

    def run(self):
        self.calculator.compute(self.gridpoints)

    def update(self, frame_num):
        pyglasstools_gb300.update_sysdata(frame_num)
        self.calculator.setSystemData(pyglasstools_gb300.get_sysdata().cppparticledata)


def polar_gridpoints(center=(0.0, 0.0, 0.0), spacingtype="normal", rmax=10, rmin=0, dr=0.1, dlnr=0.05):
    """The radialcalculator grid (irvingkirkwood/__init__.py:83-127): the centre, then
    rings of radius r (linspace(0, rmax, int(rmax/dr))[1:], or log-spaced) with
    int(2 pi r / dr) points at theta = linspace(0, 2 pi, .) each.  Returns
    (gridpoints, gridid, r, theta)."""
    center = np.asarray(center, dtype=np.float64)
    if spacingtype == "normal":
        r = np.linspace(0, rmax, int(rmax / dr))[1:]
    elif spacingtype == "log":
        r = np.exp(np.linspace(np.log(rmin), np.log(rmax), int((np.log(rmax) - np.log(rmin)) / dlnr)))
    else:
        raise ValueError("spacingtype must be 'normal' or 'log'")
    gridid, globalr, globaltheta, points = [0.0], [0.0], [0.0], [center]
    for i in range(len(r)):
        dtheta = dr / r[i]
        theta = np.linspace(0, 2 * np.pi, int(2 * np.pi / dtheta))
        x = r[i] * np.cos(theta)
        y = r[i] * np.sin(theta)
        gridid.extend([i + 1.0] * len(theta))
        globalr.extend([r[i]] * len(theta))
        globaltheta.extend(theta.tolist())
        points.extend(np.stack([x, y, np.zeros(len(theta))], axis=1) + center)
    return (np.asarray(points, dtype=np.float64).reshape(-1, 3), np.asarray(gridid), np.asarray(globalr),
            np.asarray(globaltheta))


class radialcalculator(object):
    """Fields on a polar grid around ``center`` (irvingkirkwood/__init__.py:80-166); the
    same IrvingKirkwood computation as ikcalculator, on these grid points."""

    def __init__(self, cgfunc, center=np.array([0, 0, 0]), spacingtype="normal", rmax=10, rmin=0, dr=0.1,
                 dlnr=0.05, precision=None):
        self.cgfunc = cgfunc
        self.manager = _core._pyglasstools.Manager()
        self.coordmode = "polar"
        self.center = np.asarray(center, dtype=np.float64)
        self.gridpoints, self.gridid, self.globalr, self.globaltheta = polar_gridpoints(
            self.center, spacingtype, rmax, rmin, dr, dlnr)
        self.gridsize = len(self.gridpoints)
        sysdata = pyglasstools_gb300.get_sysdata()
        self.calculator = _irvingkirkwood.IrvingKirkwood(
            sysdata.cppparticledata, pyglasstools_gb300.get_potential().cpppairpotential,
            cgfunc._getCGFunc(), comm)
        self.calculator.setPrecision(_default_precision(cgfunc, precision))
        solvers_list.append(self)

    def set_center(self, center):
        self.center = center
        self.gridpoints[0:] += center

    def add_observables(self, observables):
        for name in observables:
            self.calculator.addObservable(observables[name])

    def run(self):
        self.calculator.compute(self.gridpoints)

    def update(self, frame_num):
        pyglasstools_gb300.update_sysdata(frame_num)
        self.calculator.setSystemData(pyglasstools_gb300.get_sysdata().cppparticledata)
