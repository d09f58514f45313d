"""GPU tests of the closed-form bond integrals of the truncated Gaussian on the FP32 path:
quadrature mode "exact" (every bond: the segment clipped to the support, error
functions along it) and mode "clipped" (the closed form on the bonds whose far end
lies outside the support -- the bonds the learned surrogate stands in for -- and
Gauss-Legendre elsewhere).  The oracle is the FP64 exact mode of the CPU restatement
(the clipped interval, erf closed form), which stands in for the reference's adaptive
quadrature of the same integral (AdaptiveCGFunc::getBondFunc,
irvingkirkwood/cgfunc/CoarseGrainFunction.h:124-127, cgfunc/Quadrature.h:47-49).

Tolerances: the FP32 tolerances of the parity tests (relative L2 per component
<= 1e-5, max |error| / max |T| <= 1e-4); the clipped mode at width 2, where Gauss-
Legendre-5 on bonds inside the support is exact far below FP32 rounding.
"""
import numpy as np
import pytest

from conftest import rel_l2, uniq

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5
FP32_MAX_TOL = 1e-4


def _gpu(ik, dim, f, grid, mode, width, cut=3.0, prec="fp32", fields=None):
    with ik.IKContext() as c:
        c.set_box(dim, [f.L, f.L, f.L if dim == 3 else 1.0])
        c.set_poly12()
        c.set_cgfunc("gaussian", cut * width, mode=mode, order=5, width=width)
        c.set_grid(grid)
        c.set_frame(f.pos, f.diam, f.vel, f.mass)
        if fields is None:
            c.compute(prec)
        else:
            c.compute(prec, fields)
        return c.get_field(ik.FIELD_VIRIAL), c.get_field(ik.FIELD_KINETIC), c.get_max_rcut()


def _exact_oracle(oracle, dim, f, grid, width, max_rc, cut=3.0):
    box = oracle.make_box(dim, [f.L, f.L, f.L if dim == 3 else 1.0])
    cg = oracle.make_cg("gaussian", rcut=cut * width, mode="exact", order=5, width=width)
    return oracle.compute(box, f.pos, f.diam, oracle.make_poly12(), cg, grid, vel=f.vel, mass=f.mass, max_rc=max_rc)


def _check(got, want, what):
    g, w = uniq(got), uniq(want)
    err = rel_l2(g, w)
    m = np.max(np.abs(g - w), axis=0) / np.max(np.abs(w), axis=0)
    assert np.all(err <= FP32_TOL), f"{what}: rel L2 {err}"
    assert np.all(m <= FP32_MAX_TOL), f"{what}: max-abs/max {m}"
    return err


@pytest.mark.parametrize("width", [2.0, 1.0])
def test_fp32_exact_mode_vs_oracle_2d(oracle, width):
    from pyglasstools_gb300 import ikabi as ik, synth
    f = synth.make_frame(3000, dim=2, seed=81)
    grid = synth.lattice_grid(f.L, 48, 2)
    v, k, max_rc = _gpu(ik, 2, f, grid, "exact", width)
    ov, ok = _exact_oracle(oracle, 2, f, grid, width, max_rc)
    _check(v, ov, f"exact w={width} virial")
    # the kinetic term has no bond integral: the same as the fixed-point rule's
    _check(k, ok, f"exact w={width} kinetic")


def test_fp32_exact_mode_vs_oracle_3d(oracle):
    from pyglasstools_gb300 import ikabi as ik, synth
    f = synth.make_frame(4000, dim=3, seed=82)
    grid = synth.lattice_grid(f.L, 12, 3)
    v, k, max_rc = _gpu(ik, 3, f, grid, "exact", 1.0, cut=2.5)
    ov, ok = _exact_oracle(oracle, 3, f, grid, 1.0, max_rc, cut=2.5)
    _check(v, ov, "3d exact virial")
    _check(k, ok, "3d exact kinetic")


def test_fp32_clipped_mode_vs_oracle_and_gain_over_rule(oracle):
    from pyglasstools_gb300 import ikabi as ik, synth
    f = synth.make_frame(4000, dim=2, seed=83)
    grid = synth.lattice_grid(f.L, 48, 2)
    v_cl, _, max_rc = _gpu(ik, 2, f, grid, "clipped", 2.0)
    v_gl, _, _ = _gpu(ik, 2, f, grid, "fixedpoint", 2.0)
    v_ex, _, _ = _gpu(ik, 2, f, grid, "exact", 2.0)
    ov, _ = _exact_oracle(oracle, 2, f, grid, 2.0, max_rc)
    e_cl = _check(v_cl, ov, "clipped virial")
    _check(v_ex, ov, "exact virial")
    e_gl = rel_l2(uniq(v_gl), uniq(ov))
    # the fixed-point rule misses the jump at the edge of the support (~4e-4 here)
    assert np.all(e_gl > 30 * e_cl), (e_gl, e_cl)
    # the FP32 closed forms agree with each other beyond the rule's error
    assert np.all(rel_l2(uniq(v_cl), uniq(v_ex)) <= FP32_TOL)


def test_closed_form_modes_errors():
    from pyglasstools_gb300 import ikabi as ik, synth
    f = synth.make_frame(600, dim=2, seed=84)
    grid = synth.lattice_grid(f.L, 8, 2)
    with ik.IKContext() as c:
        c.set_box(2, [f.L, f.L, 1.0])
        c.set_poly12()
        with pytest.raises(ik.IKError):
            c.set_cgfunc("octic", 2.0, mode="clipped", order=5)   # Gaussian only
        c.set_cgfunc("octic", 2.0, mode="exact", order=5)
        c.set_grid(grid)
        c.set_frame(f.pos, f.diam, f.vel, f.mass)
        with pytest.raises(ik.IKError):
            c.compute("fp32")                                     # FP32 exact: Gaussian only
        c.compute("fp64")                                         # FP64 exact: any kernel
        c.set_cgfunc("gaussian", 6.0, mode="clipped", order=5, width=2.0)
        with pytest.raises(ik.IKError):
            c.compute("fp64")                                     # clipped: FP32 path only
        c.compute("fp32")
        c.upload_displacement(np.zeros_like(f.pos))
        with pytest.raises(ik.IKError):
            c.compute("fp32", ik.FIELD_VIRIAL | ik.FIELD_ELASTIC)  # elastic: the rule only
