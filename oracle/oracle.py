"""ctypes front-end of the FP64 CPU oracle (oracle/ik_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py``.  The product (``pyglasstools_gb300``) never
imports this module.

Parity: the reference's IK field cannot be produced here (its loop needs Aboria,
Eigen, GSL and MPI), so field parity is *unpinned by the reference*; the force
and kernel formulas are pinned bit-for-bit against the reference headers built
by ``oracle/build_ref.sh`` (tests/test_oracle_pins.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

CG_KIND = {"octic": 0, "gaussian": 1, "rect": 2, "mollifier": 3}
QUAD_MODE = {"fixedpoint": 0, "adaptive": 1, "exact": 2}


class Box(C.Structure):
    _fields_ = [("dim", C.c_int), ("L", C.c_double * 3), ("lo", C.c_double * 3),
                ("periodic", C.c_int * 3)]


POT_KIND = {"poly12": 0, "lj": 1, "fslj": 2, "poly10": 3, "poly106": 4, "poly18": 5, "polylj": 6,
            "polyyukawa": 7}


class Pot(C.Structure):
    """ikor_pot: v0 = energy scale (LJ: eps), eps = non-additivity (LJ: vareps)."""
    _fields_ = [("scaled_rcut", C.c_double), ("v0", C.c_double), ("eps", C.c_double),
                ("c0", C.c_double), ("c1", C.c_double), ("c2", C.c_double),
                ("kind", C.c_int), ("c3", C.c_double), ("kappa", C.c_double)]



class CG(C.Structure):
    _fields_ = [("kind", C.c_int), ("mode", C.c_int), ("order", C.c_int),
                ("rcut", C.c_double), ("width", C.c_double), ("epsabs", C.c_double),
                ("epsrel", C.c_double), ("limit", C.c_int)]


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        L.ikor_gl_rule.argtypes = [C.c_int, dp, dp]
        L.ikor_gk15_rule.argtypes = [dp, dp, dp]
        for f in ("ikor_force_divr", "ikor_pair_energy", "ikor_bond_stiffness"):
            getattr(L, f).argtypes = [C.POINTER(Pot), C.c_double, C.c_double, C.c_double]
            getattr(L, f).restype = C.c_double
        L.ikor_delta.argtypes = [C.POINTER(CG), C.c_int, C.c_double]
        L.ikor_delta.restype = C.c_double
        L.ikor_bond.argtypes = [C.POINTER(CG), C.c_int, dp, dp, dp]
        L.ikor_bond.restype = C.c_double
        L.ikor_max_rcut.argtypes = [C.c_double, C.c_int64, dp]
        L.ikor_max_rcut.restype = C.c_double
        L.ikor_neighbors.argtypes = [C.POINTER(Box), C.c_int64, dp, C.c_double,
                                     C.POINTER(C.c_int64), C.POINTER(C.c_int32)]
        L.ikor_neighbors.restype = C.c_int64
        L.ikor_compute_range.argtypes = [C.POINTER(Box), C.c_int64, dp, dp, dp, dp,
                                         C.POINTER(Pot), C.POINTER(CG), C.c_double,
                                         C.c_int64, C.c_int64, dp, dp, dp, C.c_int]
        L.ikor_compute_range.restype = C.c_int
        L.ikor_compute_elastic.argtypes = [C.POINTER(Box), C.c_int64, dp, dp, dp, C.POINTER(Pot),
                                           C.POINTER(CG), C.c_double, C.c_int64, C.c_int64, dp, dp, dp,
                                           C.c_int]
        L.ikor_compute_elastic.restype = C.c_int
        L.ikor_global_virial.argtypes = [C.POINTER(Box), C.c_int64, dp, dp, C.POINTER(Pot),
                                         C.c_double, dp]
        L.ikor_threads.argtypes = [C.c_int]
        L.ikor_threads.restype = C.c_int
        L.ikor_global_thermo.argtypes = [C.POINTER(Box), C.c_int64, dp, dp, dp, dp, dp, C.POINTER(Pot),
                                         C.c_double, dp]
        _LIB = L
    return _LIB


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def make_box(dim, L, origin=(0.0, 0.0, 0.0)):
    """SimBox(boxsize, origin, dim) bounds: lo = -L/2 - origin (SimBox.cc:48-52);
    z non-periodic in 2D (SimBox.cc:34-40)."""
    L = np.broadcast_to(np.asarray(L, dtype=np.float64), (3,)).copy()
    if dim == 2:
        L[2] = 1.0 if L[2] == 0 else L[2]
    b = Box()
    b.dim = dim
    for c in range(3):
        b.L[c] = float(L[c])
        b.lo[c] = -0.5 * float(L[c]) - float(origin[c])
        b.periodic[c] = 1 if (c < dim) else 0
    return b


def make_poly12(v0=1.0, eps=0.2, rcut=1.25):
    """pyglasstools.potential.polydisperse12 coefficients (potential/__init__.py:81-86)."""
    return make_potential("poly12", rcut, [v0, eps, -28.0 * v0 / rcut ** 12, 48.0 * v0 / rcut ** 14,
                                           -21.0 * v0 / rcut ** 16])


def make_potential(kind, rcut, params):
    """A pair model from the reference's parameter list (potential/__init__.py:58-146):
    lj/fslj [eps, vareps]; poly10 [v0, eps, c0, c1, c2, c3]; polyyukawa
    [v0, kappa, eps, c0, c1, c2]; poly12/poly106/poly18/polylj [v0, eps, c0, c1, c2]."""
    p = Pot()
    p.kind = POT_KIND[kind]
    p.scaled_rcut = rcut
    q = [float(v) for v in params]
    if kind in ("lj", "fslj"):
        p.v0, p.eps = q[0], q[1]
    elif kind == "polyyukawa":
        p.v0, p.kappa, p.eps, p.c0, p.c1, p.c2 = q[:6]
    else:
        p.v0, p.eps, p.c0, p.c1, p.c2 = q[:5]
        if kind == "poly10":
            p.c3 = q[5]
    return p


def potential_params(kind, **kw):
    """The parameter list the reference's Python constructor builds for a model
    (potential/__init__.py:58-146), defaults as there (LJ: eps=1, vareps=0, rcut=2.5)."""
    import math
    if kind in ("lj", "fslj"):
        return kw.get("rcut", 2.5), [kw.get("eps", 1.0), kw.get("vareps", 0.0)]
    if kind == "poly12":
        v0, eps, rc = kw.get("v0", 1.0), kw.get("eps", 0.2), kw.get("rcut", 1.25)
        return rc, [v0, eps, -28.0 * v0 / rc ** 12, 48.0 * v0 / rc ** 14, -21.0 * v0 / rc ** 16]
    if kind == "poly18":
        v0, eps, rc = kw.get("v0", 1.0), kw.get("eps", 0.0), kw.get("rcut", 1.25)
        return rc, [v0, eps, -55.0 * v0 / rc ** 18, 99.0 * v0 / rc ** 20, -45.0 * v0 / rc ** 22]
    if kind == "polylj":
        v0, eps, rc = kw.get("v0", 1.0), kw.get("eps", 0.2), kw.get("rcut", 2.5)
        return rc, [v0, eps, -28.0 * v0 / rc ** 12 + 10.0 / rc ** 6, 48.0 * v0 / rc ** 14 - 15.0 / rc ** 8,
                    -21.0 * v0 / rc ** 16 + 6.0 / rc ** 10]
    if kind == "poly10":
        v0, eps, rc = kw.get("v0", 1.0), kw.get("eps", 0.0416667), kw.get("rcut", 1.48)
        return rc, [v0, eps, -56.0 * v0 / rc ** 10, 140.0 * v0 / rc ** 12, -120.0 * v0 / rc ** 14,
                    35.0 * v0 / rc ** 16]
    if kind == "poly106":
        v0, eps, rc = kw.get("v0", 1.0), kw.get("eps", 0.1), kw.get("rcut", 3.0)
        return rc, [v0, eps, (-21 + 10 * rc ** 4) * v0 / rc ** 10, -((5 * (-7 + 3 * rc ** 4) * v0) / rc ** 12),
                    (3 * (-5 + 2 * rc ** 4) * v0) / rc ** 14]
    if kind == "polyyukawa":
        v0, eps, rc, k = kw.get("v0", 10.0), kw.get("eps", 0.0), kw.get("rcut", 4.0), kw.get("kappa", 1.0)
        e = math.exp(-k * rc)
        return rc, [v0, k, eps, -((e * (15 + 7 * k * rc + k ** 2 * rc ** 2) * v0) / (8 * rc)),
                    (e * (5 + 5 * k * rc + k ** 2 * rc ** 2) * v0) / (4 * rc ** 3),
                    -((e * (3 + 3 * k * rc + k ** 2 * rc ** 2) * v0) / (8 * rc ** 5))]
    raise KeyError(kind)


def make_cg(kind="octic", rcut=2.0, mode="fixedpoint", order=5, width=0.0,
            epsabs=1e-10, epsrel=1e-10, limit=1000):
    c = CG()
    c.kind = CG_KIND[kind]
    c.mode = QUAD_MODE[mode]
    c.order = order
    c.rcut = rcut
    c.width = width
    c.epsabs = epsabs
    c.epsrel = epsrel
    c.limit = limit
    return c


def gl_rule(n):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().ikor_gl_rule(n, _dp(x), _dp(w))
    return x, w


def gk15_rule():
    x = np.zeros(8)
    wk = np.zeros(8)
    wg = np.zeros(4)
    lib().ikor_gk15_rule(_dp(x), _dp(wk), _dp(wg))
    return x, wk, wg


def force_divr(pot, rsq, di, dj):
    return lib().ikor_force_divr(C.byref(pot), rsq, di, dj)


def pair_energy(pot, rsq, di, dj):
    return lib().ikor_pair_energy(C.byref(pot), rsq, di, dj)


def bond_stiffness(pot, rsq, di, dj):
    return lib().ikor_bond_stiffness(C.byref(pot), rsq, di, dj)


def delta(cg, dim, dr_sq):
    return lib().ikor_delta(C.byref(cg), dim, dr_sq)


def bond(cg, dim, x, ri, rij):
    x = np.ascontiguousarray(x, dtype=np.float64)
    ri = np.ascontiguousarray(ri, dtype=np.float64)
    rij = np.ascontiguousarray(rij, dtype=np.float64)
    return lib().ikor_bond(C.byref(cg), dim, _dp(x), _dp(ri), _dp(rij))


def max_rcut(scaled_rcut, diam):
    diam = np.ascontiguousarray(diam, dtype=np.float64)
    return lib().ikor_max_rcut(scaled_rcut, len(diam), _dp(diam))


def neighbors(box, pos, radius):
    """Candidate CSR (offs, idx) with j ascending; pos is n x 3."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    n = len(pos)
    offs = np.zeros(n + 1, dtype=np.int64)
    L = lib()
    nnz = L.ikor_neighbors(C.byref(box), n, _dp(pos), radius,
                           offs.ctypes.data_as(C.POINTER(C.c_int64)), None)
    idx = np.zeros(max(nnz, 1), dtype=np.int32)
    L.ikor_neighbors(C.byref(box), n, _dp(pos), radius,
                     offs.ctypes.data_as(C.POINTER(C.c_int64)),
                     idx.ctypes.data_as(C.POINTER(C.c_int32)))
    return offs, idx[:nnz]


def compute(box, pos, diam, pot, cg, grid, vel=None, mass=None, max_rc=None,
            g0=0, g1=None, nthreads=0):
    """Run the IK gather over grid points [g0, g1).  Returns (virial, kinetic), each
    (g1-g0) x dim x dim with [g, a, b] = T_ab (symmetric)."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    diam = np.ascontiguousarray(diam, dtype=np.float64)
    grid = np.ascontiguousarray(grid, dtype=np.float64)
    n = len(pos)
    if g1 is None:
        g1 = len(grid)
    if max_rc is None:
        max_rc = max_rcut(pot.scaled_rcut, diam)
    D = box.dim
    vir = np.zeros((g1 - g0) * D * D)
    kin = np.zeros((g1 - g0) * D * D)
    if vel is not None and mass is not None:
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        vp, mp = _dp(vel), _dp(mass)
    else:
        vp = mp = None
    rc = lib().ikor_compute_range(C.byref(box), n, _dp(pos), vp, mp, _dp(diam), C.byref(pot),
                                  C.byref(cg), max_rc, g0, g1, _dp(grid), _dp(vir), _dp(kin),
                                  nthreads)
    if rc != 0:
        raise ValueError(f"oracle compute failed ({rc}): box too small for the cut-offs")
    # column-major per grid point: index a + D*b -> [g, b, a]; symmetric so same
    vir = vir.reshape(g1 - g0, D, D).transpose(0, 2, 1).copy()
    kin = kin.reshape(g1 - g0, D, D).transpose(0, 2, 1).copy()
    return vir, kin


def compute_elastic(box, pos, disp, diam, pot, cg, grid, max_rc=None, g0=0, g1=None, nthreads=0):
    """Virial and elastic virial fields (ElasticVirialStressField) over grid points [g0, g1);
    disp: per-particle displacements (n x 3).  Returns (virial, elastic), [g, a, b]."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    disp = np.ascontiguousarray(disp, dtype=np.float64)
    diam = np.ascontiguousarray(diam, dtype=np.float64)
    grid = np.ascontiguousarray(grid, dtype=np.float64)
    n = len(pos)
    if g1 is None:
        g1 = len(grid)
    if max_rc is None:
        max_rc = max_rcut(pot.scaled_rcut, diam)
    D = box.dim
    vir = np.zeros((g1 - g0) * D * D)
    ela = np.zeros((g1 - g0) * D * D)
    rc = lib().ikor_compute_elastic(C.byref(box), n, _dp(pos), _dp(disp), _dp(diam), C.byref(pot), C.byref(cg),
                                    max_rc, g0, g1, _dp(grid), _dp(vir), _dp(ela), nthreads)
    if rc != 0:
        raise ValueError(f"oracle compute failed ({rc}): box too small for the cut-offs")
    vir = vir.reshape(g1 - g0, D, D).transpose(0, 2, 1).copy()
    ela = ela.reshape(g1 - g0, D, D).transpose(0, 2, 1).copy()
    return vir, ela


def global_virial(box, pos, diam, pot, max_rc=None):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    diam = np.ascontiguousarray(diam, dtype=np.float64)
    if max_rc is None:
        max_rc = max_rcut(pot.scaled_rcut, diam)
    D = box.dim
    out = np.zeros(D * D)
    lib().ikor_global_virial(C.byref(box), len(pos), _dp(pos), _dp(diam), C.byref(pot),
                             max_rc, _dp(out))
    return out.reshape(D, D).T.copy()


def threads(requested=0):
    """OpenMP threads the oracle's parallel loops run on (1 without OpenMP)."""
    return int(lib().ikor_threads(int(requested)))


def global_thermo(box, pos, diam, pot, vel=None, mass=None, disp=None, max_rc=None):
    """ThermoCalculator::compute: dict of the global observables divided by the volume:
    potentialenergy (scalar), virialstress, elasticvirialstress, kineticstress (D x D,
    [a, b]), borntensor (D x D x D x D, [i, j, k, l])."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    diam = np.ascontiguousarray(diam, dtype=np.float64)
    if max_rc is None:
        max_rc = max_rcut(pot.scaled_rcut, diam)
    D = box.dim
    out = np.zeros(1 + 3 * D * D + D ** 4)
    arr = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (vel, mass, disp)]
    ptr = [None if a is None else _dp(a) for a in arr]
    lib().ikor_global_thermo(C.byref(box), len(pos), _dp(pos), ptr[0], ptr[1], _dp(diam), ptr[2], C.byref(pot),
                             max_rc, _dp(out))
    return unpack_thermo(out, D)


def unpack_thermo(out, D):
    """Split the flat layout [energy | virial | elastic | kinetic | Born] (column-major
    tensors: index a + D b, i + D (j + D (k + D l)))."""
    D2 = D * D
    t = lambda k: out[1 + k * D2:1 + (k + 1) * D2].reshape(D, D).T.copy()
    return {"potentialenergy": float(out[0]), "virialstress": t(0), "elasticvirialstress": t(1),
            "kineticstress": t(2), "borntensor": out[1 + 3 * D2:].reshape(D, D, D, D).transpose(3, 2, 1, 0).copy()}


# ---- reference kernels compiled from the reference tree (oracle/_ref) --------
def ref_lib():
    """The reference's own pair models and Octic/Rect/Mollifier, or None when
    oracle/_ref was not built (no reference tree on this machine)."""
    path = os.path.join(_HERE, "_ref", "libref_kernels.so")
    if not os.path.exists(path):
        return None
    try:
        L = C.CDLL(path)
    except OSError:
        return None
    dp = C.POINTER(C.c_double)
    for f in ("ref_poly12_force_divr", "ref_poly12_energy", "ref_poly12_stiffness"):
        getattr(L, f).argtypes = [C.c_double, C.c_double, dp, C.c_double, C.c_double]
        getattr(L, f).restype = C.c_double
    for f in ("ref_pot_force_divr", "ref_pot_energy", "ref_pot_stiffness"):
        getattr(L, f).argtypes = [C.c_int, C.c_double, C.c_double, dp, C.c_int, C.c_double, C.c_double]
        getattr(L, f).restype = C.c_double
    for f in ("ref_octic", "ref_rect", "ref_mollifier"):
        getattr(L, f).argtypes = [C.c_double, C.c_double]
        getattr(L, f).restype = C.c_double
    return L
