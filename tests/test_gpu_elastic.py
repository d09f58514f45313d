"""GPU parity of the elastic virial field (ElasticVirialStressField: the reference's
ElasticVirialStress, ListofCommonObservables.h:86-122, through VirialStress::compute_cg)
against the FP64 oracle.  Tolerances as for the virial: FP64 <= 1e-12, FP32 <= 1e-5
relative L2 per component (the per-bond coefficients are formed in FP64)."""
import numpy as np
import pytest

from conftest import rel_l2, uniq

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ik():
    from pyglasstools_gb300 import ikabi
    return ikabi


def _gpu(ik, dim, f, grid, cg, prec, disp, fields, max_rc):
    with ik.IKContext() as c:
        c.set_box(dim, [f.L, f.L, f.L if dim == 3 else 1.0])
        c.set_poly12()
        c.set_cgfunc(**cg)
        c.set_max_rcut(max_rc)
        c.set_grid(grid)
        c.set_frame(f.pos, f.diam, f.vel, f.mass)
        if disp is not None:
            c.upload_displacement(disp)
        c.compute(prec, fields)
        out = {}
        for name, fl in (("vir", ik.FIELD_VIRIAL), ("kin", ik.FIELD_KINETIC), ("ela", ik.FIELD_ELASTIC)):
            if fields & fl:
                out[name] = c.get_field(fl)
        return out


def _disp(f, dim, scale, seed):
    u = np.random.default_rng(seed).normal(0.0, scale, f.pos.shape)
    if dim == 2:
        u[:, 2] = 0.0
    return u


@pytest.mark.parametrize("dim,cg,n,nmax", [
    (2, dict(kind="octic", rcut=2.0, mode="fixedpoint", order=5), 2500, 40),
    (2, dict(kind="gaussian", rcut=6.0, mode="fixedpoint", order=5, width=2.0), 2500, 32),
    (3, dict(kind="octic", rcut=2.0, mode="fixedpoint", order=5), 1500, 10),
])
def test_elastic_field_vs_oracle(ik, oracle, dim, cg, n, nmax):
    from pyglasstools_gb300 import synth
    f = synth.make_frame(n, dim=dim, seed=81)
    grid = synth.lattice_grid(f.L, nmax, dim)
    u = _disp(f, dim, 0.02, 5)
    box = oracle.make_box(dim, [f.L, f.L, f.L if dim == 3 else 1.0])
    pot = oracle.make_poly12()
    ocg = oracle.make_cg(cg["kind"], rcut=cg["rcut"], mode="fixedpoint", order=5, width=cg.get("width", 0.0))
    max_rc = oracle.max_rcut(1.25, f.diam)
    want_v, want_e = oracle.compute_elastic(box, f.pos, u, f.diam, pot, ocg, grid, max_rc=max_rc)
    for prec, tol in (("fp64", 1e-12), ("fp32", 1e-5)):
        got = _gpu(ik, dim, f, grid, cg, prec, u, ik.FIELD_VIRIAL | ik.FIELD_KINETIC | ik.FIELD_ELASTIC, max_rc)
        err_e = rel_l2(uniq(got["ela"]), uniq(want_e))
        err_v = rel_l2(uniq(got["vir"]), uniq(want_v))
        assert np.all(err_e <= tol), (prec, err_e)
        assert np.all(err_v <= tol), (prec, err_v)
        # the elastic field alone equals the one computed with the other fields
        alone = _gpu(ik, dim, f, grid, cg, prec, u, ik.FIELD_ELASTIC, max_rc)
        np.testing.assert_array_equal(alone["ela"], got["ela"])


def test_zero_displacement_gives_zero_field_and_errors(ik):
    from pyglasstools_gb300 import synth
    f = synth.make_frame(1200, dim=2, seed=82)
    grid = synth.lattice_grid(f.L, 16, 2)
    cg = dict(kind="octic", rcut=2.0, mode="fixedpoint", order=5)
    for prec in ("fp64", "fp32"):
        got = _gpu(ik, 2, f, grid, cg, prec, np.zeros_like(f.pos), ik.FIELD_ELASTIC, 1.25 * 1.62)
        assert np.all(got["ela"] == 0.0)
    with pytest.raises(ik.IKError):
        _gpu(ik, 2, f, grid, cg, "fp32", None, ik.FIELD_ELASTIC, 1.25 * 1.62)  # no displacements
    with ik.IKContext() as c:
        c.set_box(2, [f.L, f.L, 1.0])
        c.set_frame(f.pos, f.diam)
        with pytest.raises(ik.IKError):
            c.upload_displacement(np.zeros((5, 3)))                          # wrong size


def test_elastic_field_through_the_pybind_classes(ik, oracle):
    """ElasticVirialStressField2D with ParticleSystem.setDisplacement and
    IrvingKirkwood.compute (the reference's module-irvingkirkwood.cpp classes)."""
    from pyglasstools_gb300 import synth
    from pyglasstools_gb300._core import _irvingkirkwood as K, _pyglasstools as P, _potential as Pot, _cgfunc as CG
    f = synth.make_frame(900, dim=2, seed=83)
    grid = synth.lattice_grid(f.L, 12, 2)
    u = _disp(f, 2, 0.03, 9)
    box = P.SimBox(np.array([f.L, f.L, 1.0]), np.zeros(3), 2)
    sys = P.ParticleSystem(box, len(f.pos), f.diam, f.mass, f.pos, f.vel)
    sys.setDisplacement(u)
    rc = 1.25
    pot = Pot.PairPotentialPoly12(rc, [1.0, 0.2, -28.0 / rc ** 12, 48.0 / rc ** 14, -21.0 / rc ** 16])
    cg = CG.CGFuncOcticFixedPoint(5, 2.0)
    calc = K.IrvingKirkwood(sys, pot, cg, P.Communicator())
    calc.setPrecision("fp64")
    fld = K.ElasticVirialStressField2D("elasticvirialstress", "2-TENSOR", False, len(grid))
    fld.addGridpoints(grid)
    calc.addObservable(fld)
    calc.compute(grid)
    got = fld.values()
    obox = oracle.make_box(2, [f.L, f.L, 1.0])
    _, want = oracle.compute_elastic(obox, f.pos, u, f.diam, oracle.make_poly12(), oracle.make_cg("octic", rcut=2.0),
                                     grid, max_rc=calc.max_rcut)
    assert np.all(rel_l2(uniq(got), uniq(want)) <= 1e-12)


def test_elastic_field_with_polydisperse_yukawa_vs_oracle(ik, oracle):
    """The elastic field with another pair model (PolydisperseYukawa, rcut 4: ~130
    neighbours within max_rcut per particle, past the 63 of one staged entry): both paths
    against the oracle."""
    from pyglasstools_gb300 import synth
    f = synth.make_frame(1500, dim=2, seed=83)
    grid = synth.lattice_grid(f.L, 24, 2)
    u = _disp(f, 2, 0.02, 7)
    rc, prm = oracle.potential_params("polyyukawa")
    box = oracle.make_box(2, [f.L, f.L, 1.0])
    ocg = oracle.make_cg("octic", rcut=2.0, mode="fixedpoint", order=5)
    max_rc = oracle.max_rcut(rc, f.diam)
    _, want_e = oracle.compute_elastic(box, f.pos, u, f.diam, oracle.make_potential("polyyukawa", rc, prm), ocg, grid,
                                       max_rc=max_rc)
    for prec, tol in (("fp64", 1e-12), ("fp32", 1e-5)):
        with ik.IKContext() as c:
            c.set_box(2, [f.L, f.L, 1.0])
            c.set_potential("polyyukawa", rc, prm)
            c.set_cgfunc("octic", 2.0, order=5)
            c.set_max_rcut(max_rc)
            c.set_grid(grid)
            c.set_frame(f.pos, f.diam, f.vel, f.mass)
            c.upload_displacement(u)
            c.compute(prec, ik.FIELD_ELASTIC)
            got = c.get_field(ik.FIELD_ELASTIC)
        assert np.all(rel_l2(uniq(got), uniq(want_e)) <= tol), prec
