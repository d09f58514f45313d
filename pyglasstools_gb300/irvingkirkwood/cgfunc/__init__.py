R"""Coarse-graining functions (pyglasstools/irvingkirkwood/cgfunc/__init__.py).

``octic``, ``rect`` and ``mollifier`` keep the reference's constructor
(``rcut``, ``mode`` in {"fixedpoint", "adaptive"}, ``order`` | ``relerr``,
``abserr``, ``maxiter``).  ``gaussian(width, cut=3.0, ...)`` is new: a Gaussian of
standard deviation ``width`` truncated at ``cut * width`` and normalised as
(2 pi w^2)^(-dim/2) (not renormalised for the truncation).
"""
from pyglasstools_gb300 import _core

_cgfunc = _core._cgfunc


class basecgfunc(object):
    def _getCGFunc(self):
        return self.cgfunc

    def set_rcut(self, rcut):
        self.cgfunc.setRcut(rcut)

    def get_rcut(self):
        return self.cgfunc.getRcut()

    def get_deltafunc(self, x, ri):
        return self.cgfunc.getDeltaFunc(x, ri)

    def get_objfunc(self, s, x, ri, rij):
        return self.cgfunc.getObjFunc(s, x, ri, rij)

    def get_bondfunc(self, x, ri, rij):
        return self.cgfunc.getBondFunc(x, ri, rij)


def _make(kind, rcut, mode, kwargs):
    if mode == "fixedpoint":
        if "order" not in kwargs:
            raise TypeError("mode='fixedpoint' needs order=")
        return getattr(_cgfunc, f"CGFunc{kind}FixedPoint")(int(kwargs["order"]), float(rcut))
    if mode == "adaptive":
        for k in ("relerr", "abserr", "maxiter"):
            if k not in kwargs:
                raise TypeError(f"mode='adaptive' needs {k}=")
        return getattr(_cgfunc, f"CGFunc{kind}Adaptive")(int(kwargs["maxiter"]), float(kwargs["relerr"]),
                                                         float(kwargs["abserr"]), float(rcut))
    raise NameError("Coarse-graining mode not recognized: 'fixedpoint' and 'adaptive' are available")


class octic(basecgfunc):
    R"""15/(8 pi R^2) (1 - 2 (r/R)^4 + (r/R)^8) for r < R (CGFuncOctic.h)."""

    def __init__(self, rcut=2.5, mode=None, **kwargs):
        self.cgfunc = _make("Octic", rcut, mode, kwargs)


class rect(basecgfunc):
    R"""1/(pi R^2) for r < R (CGFuncRect.h)."""

    def __init__(self, rcut=2.5, mode=None, **kwargs):
        self.cgfunc = _make("Rect", rcut, mode, kwargs)


class mollifier(basecgfunc):
    R"""C1/(2 pi R^2) exp(-1/(1 - r^2/R^2)) for r < R (CGFuncMollifier.h)."""

    def __init__(self, rcut=2.5, mode=None, **kwargs):
        self.cgfunc = _make("Mollifier", rcut, mode, kwargs)


class gaussian(basecgfunc):
    R"""(2 pi w^2)^(-dim/2) exp(-r^2/(2 w^2)) for r < cut*w (new)."""

    def __init__(self, width=2.0, cut=3.0, mode="fixedpoint", **kwargs):
        if mode == "fixedpoint":
            order = int(kwargs.get("order", 5))
            self.cgfunc = _cgfunc.CGFuncGaussianFixedPoint(order, float(width), float(cut))
        elif mode == "adaptive":
            for k in ("relerr", "abserr", "maxiter"):
                if k not in kwargs:
                    raise TypeError(f"mode='adaptive' needs {k}=")
            self.cgfunc = _cgfunc.CGFuncGaussianAdaptive(int(kwargs["maxiter"]), float(kwargs["relerr"]),
                                                         float(kwargs["abserr"]), float(width), float(cut))
        else:
            raise NameError("Coarse-graining mode not recognized: 'fixedpoint' and 'adaptive' are available")
        self.width = width
        self.cut = cut
