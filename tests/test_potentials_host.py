"""Host-side tests of the pair-potential front-end (no GPU): the Python constructors of
the eight models build the reference's parameter lists (potential/__init__.py:58-146),
getRcut follows Model::computeRcut on the host, and the C ABI reports argument errors.
"""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture
def potmod():
    import pyglasstools_gb300 as pg
    import pyglasstools_gb300.potential as pot
    pg.reset()
    yield pot
    pg.reset()


CASES = [
    ("polydisperse12", "poly12", dict(v0=1.0, eps=0.2, rcut=1.25), "PairPotentialPoly12"),
    ("polydisperse18", "poly18", dict(v0=1.0, eps=0.0, rcut=1.25), "PairPotentialPoly18"),
    ("polydisperselj", "polylj", dict(v0=1.0, eps=0.2, rcut=2.5), "PairPotentialPolyLJ"),
    ("polydisperse10", "poly10", dict(v0=1.0, eps=0.0416667, rcut=1.48), "PairPotentialPoly10"),
    ("polydisperse106", "poly106", dict(v0=1.0, eps=0.1, rcut=3.0), "PairPotentialPoly106"),
    ("polydisperseyukawa", "polyyukawa", dict(v0=10.0, eps=0.0, rcut=4.0, kappa=1.0),
     "PairPotentialPolyYukawa"),
]


@pytest.mark.parametrize("cls,kind,kw,cpp", CASES)
def test_constructors_build_reference_parameter_lists(potmod, oracle, cls, kind, kw, cpp):
    p = getattr(potmod, cls)(**kw)
    rc, want = oracle.potential_params(kind, **kw)
    assert type(p.cpppairpotential).__name__ == cpp
    assert p.get_scaledrcut() == rc
    np.testing.assert_array_equal(p.get_params(), want)
    # named parameters
    p.set_params(0.5, "eps")
    assert p.get_params("eps") == 0.5
    assert p.get_params()[p.dict_params["eps"]] == 0.5


@pytest.mark.parametrize("mode,cpp", [("truncated", "PairPotentialLJ"),
                                      ("force-shifted", "PairPotentialForceShiftedLJ")])
def test_lj_modes(potmod, mode, cpp):
    p = potmod.lj(eps=1.0, vareps=0.1, rcut=2.5, mode=mode)
    assert type(p.cpppairpotential).__name__ == cpp
    assert p.get_potentialname() == "lennard-jones+" + mode
    assert p.get_params() == [1.0, 0.1]
    # the reference's table maps both names to index 0 (potential/__init__.py:74)
    assert p.dict_params == {"eps": 0, "vareps": 0}


def test_lj_mode_errors(potmod):
    with pytest.raises(NameError):
        potmod.lj(eps=1.0, vareps=0.0, rcut=2.5)
    with pytest.raises(NameError):
        potmod.lj(eps=1.0, vareps=0.0, rcut=2.5, mode="smoothed")


@pytest.mark.parametrize("cls,kw,epsidx", [("polydisperse12", {}, 1), ("polydisperseyukawa", {"eps": 0.1}, 2),
                                           ("polydisperse106", {}, 1)])
def test_getrcut_is_compute_rcut(potmod, cls, kw, epsidx):
    p = getattr(potmod, cls)(**kw)
    rc = p.get_scaledrcut()
    eps = p.get_params()[epsidx]
    rng = np.random.default_rng(1)
    for _ in range(50):
        di, dj = rng.uniform(0.7, 1.7, 2)
        s = 0.5 * (di + dj) * (1 - eps * abs(di - dj))
        assert p.cpppairpotential.getRcut(np.zeros(3), di, dj) == rc * rc * s * s


def test_force_shifted_lj_rcut_uses_vareps(potmod):
    """ForceShiftedLennardJones inherits LennardJones::computeRcut (LennardJones.h:77-81)."""
    p = potmod.lj(eps=1.0, vareps=0.2, rcut=2.5, mode="force-shifted")
    di, dj = 0.8, 1.4
    s = 0.5 * (di + dj) * (1 - 0.2 * abs(di - dj))
    assert p.cpppairpotential.getRcut(np.zeros(3), di, dj) == 2.5 * 2.5 * s * s


def test_too_few_parameters_raise(potmod):
    from pyglasstools_gb300 import _core
    p = _core._potential.PairPotentialPoly10(1.48, [1.0, 0.0, 1.0])
    with pytest.raises(ValueError):
        p.getRcut(np.zeros(3), 1.0, 1.0)


def test_c_abi_parameter_counts_and_errors():
    from pyglasstools_gb300 import ikabi
    L = ikabi.lib()
    assert [L.ik_potential_nparams(k) for k in range(8)] == [5, 2, 2, 6, 5, 5, 5, 6]
    assert L.ik_potential_nparams(8) == -1 and L.ik_potential_nparams(-1) == -1
    prm = (C.c_double * 6)(1, 0, 0, 0, 0, 0)
    assert L.ik_set_potential(None, 0, 1.25, prm, 5) != 0  # null context
