R"""Irving-Kirkwood coarse-grained fields (pyglasstools/irvingkirkwood/__init__.py).

``ikcalculator(cgfunc, dx, precision="fp32")`` builds the reference's lattice grid
(linspace(-L/2, L/2, int(L/dx)) per axis, endpoints included) and computes the
registered fields on the GPU.  ``precision="fp64"`` selects the plain FP64 kernels;
the default "fp32" is the tuned path (FP32 pair arithmetic, compensated
accumulation, FP64 selection and final sums).
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


class ikcalculator(object):
    def __init__(self, cgfunc, dx, precision="fp32"):
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
        self.calculator.setPrecision(precision)
        solvers_list.append(self)

    def add_observables(self, observables):
        for name in observables:
            self.calculator.addObservable(observables[name])

    def run(self):
        self.calculator.compute(self.gridpoints)

    def update(self, frame_num):
        pyglasstools_gb300.update_sysdata(frame_num)
        self.calculator.setSystemData(pyglasstools_gb300.get_sysdata().cppparticledata)
