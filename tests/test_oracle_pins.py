"""CPU tests pinning the FP64 oracle: against the reference's own kernel headers
(compiled by oracle/build_ref.sh, or their committed golden values), against
exactness properties of the quadrature rules and against closed forms."""
import numpy as np
import pytest

from conftest import rel_l2


def test_gl_rule_exact_on_polynomials(oracle):
    for n in (1, 2, 3, 5, 8, 15, 32, 64):
        x, w = oracle.gl_rule(n)
        assert np.all(np.diff(x) > 0)
        for k in range(2 * n):
            exact = 2.0 / (k + 1) if k % 2 == 0 else 0.0
            assert abs(np.sum(w * x ** k) - exact) < 5e-14 * max(1, n), (n, k)


def test_gk15_rule_degree_22(oracle):
    x, wk, wg = oracle.gk15_rule()
    xs = np.concatenate([-x[:0:-1], x])
    ws = np.concatenate([wk[:0:-1], wk])
    for k in range(23):
        exact = 2.0 / (k + 1) if k % 2 == 0 else 0.0
        assert abs(np.sum(ws * xs ** k) - exact) < 1e-14
    # the embedded Gauss-7 nodes are the 7-point Legendre roots
    gx, gw = oracle.gl_rule(7)
    np.testing.assert_allclose(x[[0, 2, 4, 6]], gx[3:], atol=1e-15)
    np.testing.assert_allclose(wg, gw[3:], atol=1e-15)


def test_force_matches_reference_header_golden(oracle, golden):
    """Polydisperse12 force/energy/stiffness: bit-identical to the reference's own
    Polydisperse12.h (values generated by compiling it; tests/golden/make_golden.py)."""
    g = golden("ref_kernels.npz")
    pot = oracle.make_poly12()
    f = np.array([oracle.force_divr(pot, a, b, c) for a, b, c in zip(g["rsq"], g["di"], g["dj"])])
    e = np.array([oracle.pair_energy(pot, a, b, c) for a, b, c in zip(g["rsq"], g["di"], g["dj"])])
    s = np.array([oracle.bond_stiffness(pot, a, b, c) for a, b, c in zip(g["rsq"], g["di"], g["dj"])])
    assert np.array_equal(f, g["force"])
    assert np.array_equal(e, g["energy"])
    assert np.array_equal(s, g["stiffness"])
    assert np.count_nonzero(f) > 100 and np.count_nonzero(f == 0) > 100  # both branches exercised


POT_KINDS = ["poly12", "lj", "fslj", "poly10", "poly106", "poly18", "polylj", "polyyukawa"]


@pytest.mark.parametrize("kind", POT_KINDS)
def test_pair_models_match_reference_headers_golden(oracle, golden, kind):
    """Force, energy and stiffness of each of the eight models: bit-identical to the reference's
    own header (potential/*.h compiled by oracle/build_ref.sh; tests/golden/make_golden.py),
    including pairs within a few ulp of the cut-off and strongly overlapping pairs."""
    g = golden("ref_potentials.npz")
    pot = oracle.make_potential(kind, float(g[f"{kind}_rc"]), g[f"{kind}_params"])
    rsq, di, dj = g[f"{kind}_rsq"], g[f"{kind}_di"], g[f"{kind}_dj"]
    f = np.array([oracle.force_divr(pot, a, b, c) for a, b, c in zip(rsq, di, dj)])
    e = np.array([oracle.pair_energy(pot, a, b, c) for a, b, c in zip(rsq, di, dj)])
    st = np.array([oracle.bond_stiffness(pot, a, b, c) for a, b, c in zip(rsq, di, dj)])
    assert np.array_equal(f, g[f"{kind}_force"])
    assert np.array_equal(e, g[f"{kind}_energy"])
    assert np.array_equal(st, g[f"{kind}_stiffness"])
    assert np.count_nonzero(f) > 100 and np.count_nonzero(f == 0) > 50


def test_pair_model_parameter_lists(oracle):
    """The constructors' coefficient formulas (potential/__init__.py:58-146) smooth each
    polynomial model to zero force at the cut-off (sigma = 1)."""
    for kind in ("poly12", "poly10", "poly106", "poly18", "polylj", "polyyukawa"):
        rc, prm = oracle.potential_params(kind)
        prm = list(prm)
        prm[2 if kind == "polyyukawa" else 1] = 0.0  # eps = 0: sigma = d
        pot = oracle.make_potential(kind, rc, prm)
        f = oracle.force_divr(pot, rc * rc * (1 - 1e-9), 1.0, 1.0)
        f_in = oracle.force_divr(pot, 1.0, 1.0, 1.0)
        assert abs(f) < 1e-6 * abs(f_in), kind


def test_cg_kernels_match_reference_headers_golden(oracle, golden):
    g = golden("ref_kernels.npz")
    rc = float(g["rc"])
    for kind in ("octic", "rect", "mollifier"):
        cg = oracle.make_cg(kind, rcut=rc)
        v = np.array([oracle.delta(cg, 2, x) for x in g["dr"]])
        assert np.array_equal(v, g[kind]), kind


def test_live_reference_build_if_present(oracle):
    """When the reference tree is on this machine, recompile its headers and compare live."""
    import ctypes as C
    R = oracle.ref_lib()
    if R is None:
        pytest.skip("oracle/_ref not built (no reference tree here)")
    rng = np.random.default_rng(7)
    pot = oracle.make_poly12(v0=1.3, eps=0.15, rcut=1.4)
    prm = (C.c_double * 5)(pot.v0, pot.eps, pot.c0, pot.c1, pot.c2)
    for _ in range(3000):
        rsq, di, dj = rng.uniform(0.05, 5.0), rng.uniform(0.6, 1.8), rng.uniform(0.6, 1.8)
        assert oracle.force_divr(pot, rsq, di, dj) == R.ref_poly12_force_divr(rsq, pot.scaled_rcut, prm, di, dj)
        assert oracle.pair_energy(pot, rsq, di, dj) == R.ref_poly12_energy(rsq, pot.scaled_rcut, prm, di, dj)
    for kind in POT_KINDS:  # every model, eps != 0 where it has one
        rc, q = oracle.potential_params(kind)
        q = list(q)
        q[2 if kind == "polyyukawa" else 1] = 0.12
        p = oracle.make_potential(kind, rc, q)
        arr = (C.c_double * len(q))(*q)
        K = oracle.POT_KIND[kind]
        for _ in range(400):
            di, dj = rng.uniform(0.6, 1.8), rng.uniform(0.6, 1.8)
            rsq = rng.uniform(0.02, 1.2) * (rc * 0.5 * (di + dj)) ** 2
            assert oracle.force_divr(p, rsq, di, dj) == R.ref_pot_force_divr(K, rsq, rc, arr, len(q), di, dj), kind
            assert oracle.pair_energy(p, rsq, di, dj) == R.ref_pot_energy(K, rsq, rc, arr, len(q), di, dj), kind
            assert oracle.bond_stiffness(p, rsq, di, dj) == R.ref_pot_stiffness(K, rsq, rc, arr, len(q), di, dj), kind


def test_octic_bond_closed_form(oracle):
    """Segment inside the support: the octic bond integral is a degree-8 polynomial in s;
    GL-5 integrates it exactly, and the exact mode agrees."""
    rng = np.random.default_rng(3)
    R = 2.0
    fixed = oracle.make_cg("octic", rcut=R, mode="fixedpoint", order=5)
    exact = oracle.make_cg("octic", rcut=R, mode="exact")
    for _ in range(200):
        ri = np.r_[rng.uniform(-0.6, 0.6, 2), 0.0]
        rij = np.r_[rng.uniform(-0.6, 0.6, 2), 0.0]
        x = np.zeros(3)
        # dense reference by Simpson on 20001 points
        s = np.linspace(0, 1, 20001)
        d = x[None, :] - (ri[None, :] + s[:, None] * rij[None, :])
        q = (d ** 2).sum(1) / R ** 2
        f = 15 / (8 * np.pi * R * R) * (1 - 2 * q ** 2 + q ** 4)
        h = s[1] - s[0]
        simpson = h / 3 * (f[0] + f[-1] + 4 * f[1:-1:2].sum() + 2 * f[2:-1:2].sum())
        a = oracle.bond(fixed, 2, x, ri, rij)
        b = oracle.bond(exact, 2, x, ri, rij)
        assert abs(a - simpson) < 1e-12 * abs(simpson)
        assert abs(b - simpson) < 1e-12 * abs(simpson)


def test_gaussian_exact_vs_clipped_adaptive(oracle):
    """Truncated Gaussian: erf closed form == adaptive GK15 on the clipped interval."""
    from scipy.integrate import quad
    rng = np.random.default_rng(5)
    w, R = 2.0, 6.0
    exact = oracle.make_cg("gaussian", rcut=R, mode="exact", width=w)
    norm = 1 / (2 * np.pi * w * w)
    for _ in range(300):
        ri = np.r_[rng.uniform(-6.5, 6.5, 2), 0.0]
        rij = np.r_[rng.uniform(-2, 2, 2), 0.0]
        x = np.zeros(3)
        f = lambda s: norm * np.exp(-np.sum((x - ri - s * rij) ** 2) / (2 * w * w)) \
            if np.sum((x - ri - s * rij) ** 2) < R * R else 0.0
        # split at the truncation crossings for the scipy reference
        u = x - ri
        bb, ub, uu = rij @ rij, u @ rij, u @ u
        disc = ub * ub - bb * (uu - R * R)
        pts = []
        if disc > 0:
            for r in ((ub - np.sqrt(disc)) / bb, (ub + np.sqrt(disc)) / bb):
                if 0 < r < 1:
                    pts.append(r)
        ref = quad(f, 0, 1, points=pts or None, epsabs=1e-15, epsrel=1e-13, limit=200)[0]
        assert abs(oracle.bond(exact, 2, x, ri, rij) - ref) < 1e-12 + 1e-10 * abs(ref)


def test_two_particle_hand_computed_field(oracle):
    """Two particles on the x axis, octic R = 2, one grid point: the virial field is
    0.5 * f(r) r^2 * [B(x; r1, r12) + B(x; r2, r21)] in xx only."""
    L = 20.0
    box = oracle.make_box(2, [L, L, 1.0])
    pos = np.array([[-0.5, 0.0, 0.0], [0.5, 0.0, 0.0]])
    diam = np.array([1.0, 1.0])
    pot = oracle.make_poly12()
    cg = oracle.make_cg("octic", rcut=2.0, mode="fixedpoint", order=5)
    grid = np.array([[0.3, 0.2, 0.0]])
    vir, kin = oracle.compute(box, pos, diam, pot, cg, grid)
    f = oracle.force_divr(pot, 1.0, 1.0, 1.0)
    x = grid[0]
    b12 = oracle.bond(cg, 2, x, pos[0], pos[1] - pos[0])
    b21 = oracle.bond(cg, 2, x, pos[1], pos[0] - pos[1])
    expect = 0.5 * f * 1.0 * (b12 + b21)
    assert abs(vir[0, 0, 0] - expect) < 1e-14 * abs(expect)
    assert vir[0, 1, 1] == 0.0 and vir[0, 0, 1] == 0.0
    assert np.all(kin == 0.0)


def test_selection_rule_half_weight(oracle):
    """A bond with only one end inside the support enters once (ordered pair (i,j) with
    i inside), a bond with both ends outside not at all (IrvingKirkwood.h:80-105)."""
    L = 30.0
    box = oracle.make_box(2, [L, L, 1.0])
    pot = oracle.make_poly12()
    cg = oracle.make_cg("octic", rcut=2.0, mode="fixedpoint", order=5)
    diam = np.array([1.0, 1.0])
    grid = np.array([[0.0, 0.0, 0.0]])
    pos = np.array([[1.5, 0.0, 0.0], [2.4, 0.0, 0.0]])  # i inside, j outside
    vir, _ = oracle.compute(box, pos, diam, pot, cg, grid)
    f = oracle.force_divr(pot, 0.81, 1.0, 1.0)
    b = oracle.bond(cg, 2, grid[0], pos[0], pos[1] - pos[0])
    assert abs(vir[0, 0, 0] - 0.5 * f * 0.81 * b) < 1e-15
    pos = np.array([[2.1, 0.5, 0.0], [2.1, -0.5, 0.0]])  # both outside, segment crosses support
    vir, _ = oracle.compute(box, pos, diam, pot, cg, grid)
    assert np.all(vir == 0.0)


def test_periodic_wrap_and_translation(oracle):
    """Translating the frame and the grid by a lattice vector, or wrapping particles
    into the box, leaves the field unchanged (min-image convention)."""
    from pyglasstools_gb300 import synth
    f = synth.make_frame(600, dim=2, seed=11)
    grid = synth.lattice_grid(f.L, 24, 2)
    box = oracle.make_box(2, [f.L, f.L, 1.0])
    pot = oracle.make_poly12()
    cg = oracle.make_cg("octic", rcut=2.0, mode="fixedpoint", order=5)
    v0, k0 = oracle.compute(box, f.pos, f.diam, pot, cg, grid, vel=f.vel, mass=f.mass)
    shifted = f.pos.copy()
    shifted[:, 0] += f.L  # an image of every particle
    v1, k1 = oracle.compute(box, shifted, f.diam, pot, cg, grid, vel=f.vel, mass=f.mass)
    assert np.max(np.abs(v1 - v0)) <= 1e-9 * np.max(np.abs(v0))
    assert np.max(np.abs(k1 - k0)) <= 1e-9 * np.max(np.abs(k0))


def test_xy_swap_symmetry(oracle):
    from pyglasstools_gb300 import synth
    f = synth.make_frame(500, dim=2, seed=12)
    n = 20
    grid = synth.lattice_grid(f.L, n, 2)
    box = oracle.make_box(2, [f.L, f.L, 1.0])
    pot = oracle.make_poly12()
    cg = oracle.make_cg("octic", rcut=2.0, mode="fixedpoint", order=5)
    v, _ = oracle.compute(box, f.pos, f.diam, pot, cg, grid)
    sw = f.pos[:, [1, 0, 2]]
    vs, _ = oracle.compute(box, sw, f.diam, pot, cg, grid)
    # grid point (i, j) of the swapped frame is (j, i) of the original
    v = v.reshape(n, n, 2, 2)
    vs = vs.reshape(n, n, 2, 2)
    np.testing.assert_allclose(vs[:, :, 0, 0], v.transpose(1, 0, 2, 3)[:, :, 1, 1], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(vs[:, :, 0, 1], v.transpose(1, 0, 2, 3)[:, :, 0, 1], rtol=1e-10, atol=1e-12)


def test_sum_rule_against_global_virial(oracle):
    """Integrating the IK virial field over the box recovers the global virial
    sum_{i<j} F_ij (x) r_ij (ThermoCalculator.h:68-90) up to the i-in-support
    selection rule, whose deficit shrinks as R grows relative to the bond length:
    the ratio approaches 1 from below, monotonically in R."""
    from pyglasstools_gb300 import synth
    f = synth.make_frame(400, dim=2, seed=4, jitter=0.02)
    n = 80
    grid = synth.lattice_grid(f.L, n + 1, 2)
    box = oracle.make_box(2, [f.L, f.L, 1.0])
    pot = oracle.make_poly12()
    glob = oracle.global_virial(box, f.pos, f.diam, pot)
    ratios = []
    for R in (2.0, 4.0, 6.0):
        cg = oracle.make_cg("octic", rcut=R, mode="fixedpoint", order=5)
        v, _ = oracle.compute(box, f.pos, f.diam, pot, cg, grid)
        v = v.reshape(n + 1, n + 1, 2, 2)[:n, :n]  # drop the periodic duplicate row/column
        integral = v.sum(axis=(0, 1)) * (f.L / n) ** 2
        ratios.append([integral[0, 0] / glob[0, 0], integral[1, 1] / glob[1, 1]])
    ratios = np.array(ratios)
    assert np.all(ratios < 1.0)
    assert np.all(np.diff(ratios, axis=0) > 0)
    assert np.all(ratios[-1] > 0.99)


def test_neighbors_definition(oracle):
    from pyglasstools_gb300 import synth
    f = synth.make_frame(300, dim=2, seed=9)
    box = oracle.make_box(2, [f.L, f.L, 1.0])
    offs, idx = oracle.neighbors(box, f.pos, 2.0)
    # brute force with the same FP64 min-image rule
    d = f.pos[None, :, :] - f.pos[:, None, :]
    d[..., :2] -= f.L * np.rint(d[..., :2] / f.L)
    r2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    for i in range(len(f.pos)):
        want = np.nonzero((r2[i] < 4.0) & (np.arange(len(f.pos)) != i))[0]
        assert np.array_equal(idx[offs[i]:offs[i + 1]], want)


def test_golden_fixture_field_regenerates(oracle, golden):
    """The committed oracle field on fixture frame 180 is what the oracle computes now."""
    fr = golden("fixture_frames.npz")
    gold = golden("oracle_fixture180.npz")
    pos = fr["pos180"].astype(np.float64)
    diam = fr["diam180"].astype(np.float64)
    L = float(fr["box180"][0])
    assert int(gold["nmax"]) == int(L / 0.25) == 127
    pts = np.linspace(-L / 2, L / 2, int(gold["nmax"]))
    gx, gy = np.meshgrid(pts, pts, indexing="ij")
    grid = np.stack([gx.ravel(), gy.ravel(), np.zeros(gx.size)], axis=1)
    sel = slice(0, None, 37)  # every 37th grid point keeps this test fast
    box = oracle.make_box(2, [L, L, 1.0])
    pot = oracle.make_poly12()
    cg = oracle.make_cg("octic", rcut=2.0, mode="fixedpoint", order=5)
    v, _ = oracle.compute(box, pos, diam, pot, cg, grid[sel], max_rc=float(gold["max_rcut"]))
    u = np.stack([v[:, 0, 0], v[:, 1, 1], v[:, 0, 1]], axis=1)
    assert np.max(rel_l2(u, gold["virial"][sel])) < 1e-13


@pytest.mark.parametrize("kind", ["octic", "mollifier"])
def test_adaptive_bond_integral_vs_scipy(oracle, kind):
    """The oracle's QAG-GK15 (the restatement of gsl_integration_qag key 1 that the GPU's
    adaptive mode is checked against) against scipy's QUADPACK with the support crossings
    given as break points: within its tolerance where the segment stays inside the support
    (a smooth integrand); where it crosses the edge, the kernel's kink there (the octic's
    curvature jumps, the mollifier's derivatives vanish) is invisible to QAG's K15 - G7
    estimate, as in GSL, and the answer is good to ~1e-7 relative."""
    from scipy.integrate import quad
    rng = np.random.default_rng(12)
    R = 2.0
    cg = oracle.make_cg(kind, rcut=R, mode="adaptive", width=R, epsabs=1e-13, epsrel=1e-11, limit=200)
    x = np.zeros(3)
    smooth = 0
    for _ in range(150):
        ri = np.r_[rng.uniform(-1.9, 1.9, 2), 0.0]
        rij = np.r_[rng.uniform(-1.5, 1.5, 2), 0.0]
        f = lambda s: oracle.delta(cg, 2, float(np.sum((x - ri - s * rij) ** 2)))
        u = x - ri
        bb, ub, uu = rij @ rij, u @ rij, u @ u
        disc = ub * ub - bb * (uu - R * R)
        pts = [r for r in ((ub - np.sqrt(disc)) / bb, (ub + np.sqrt(disc)) / bb) if 0 < r < 1] if disc > 0 else []
        ref = quad(f, 0, 1, points=pts or None, epsabs=1e-15, epsrel=1e-13, limit=200)[0]
        got = oracle.bond(cg, 2, x, ri, rij)
        tol = 1e-12 + 1e-6 * abs(ref) if pts else 1e-13 + 1e-10 * abs(ref)
        assert abs(got - ref) <= tol, (got, ref, pts)
        smooth += not pts
    assert smooth > 10


def _py_ik_field(pos, vel, mass, diam, L, grid, R=2.0, v0=1.0, eps=0.2, rc=1.25, order=5, dim=2):
    """An independent pure-Python restatement of IrvingKirkwood::compute for a handful of
    particles (irvingkirkwood/IrvingKirkwood.h:74-110): Polydisperse12 force
    (potential/Polydisperse12.h:38-55, coefficients potential/__init__.py:83-85), octic
    kernel (cgfunc/CGFuncOctic.h:16-29), GL-n bond integral on [0, 1] with numpy's
    Gauss-Legendre nodes, periodic min-image (x and y in 2D, x, y and z in 3D,
    SimBox.cc:15,37), the selection rule (ordered pairs, first particle inside the
    support) and the intended kinetic term.  The octic keeps its 2D normalisation in 3D,
    as the reference's does."""
    c1, c2 = 48.0 * v0 / rc ** 14, -21.0 * v0 / rc ** 16
    xi, wi = np.polynomial.legendre.leggauss(order)
    n = len(pos)
    max_rc = max(rc * diam.max(), diam.max())

    def mi(d):
        d = d.copy()
        d[:dim] -= L * np.round(d[:dim] / L)
        return d

    def force_divr(rsq, di, dj):
        sig = 0.5 * (di + dj) * (1.0 - eps * abs(di - dj))
        if rsq >= (rc * sig) ** 2:
            return 0.0
        s2 = sig * sig / rsq
        return (12.0 * v0 * s2 * s2 ** 6 - 2.0 * c1 - 4.0 * c2 * rsq / (sig * sig)) / (sig * sig)

    def delta(r2):
        if r2 >= R * R:
            return 0.0
        q2 = r2 / (R * R)
        return 15.0 / (8.0 * np.pi * R * R) * (1.0 - 2.0 * q2 * q2 + q2 ** 4)

    vir = np.zeros((len(grid), dim, dim))
    kin = np.zeros((len(grid), dim, dim))
    for g, x in enumerate(grid):
        for i in range(n):
            dx = mi(x - pos[i])
            if dx @ dx >= R * R:
                continue
            ri = x - dx
            w = delta(dx @ dx)
            kin[g] += mass[i] * np.outer(vel[i, :dim], vel[i, :dim]) * w
            for j in range(n):
                if j == i:
                    continue
                rij = mi(pos[j] - pos[i])
                if rij @ rij >= max_rc * max_rc:
                    continue
                b = 0.0
                for s_, w_ in zip(0.5 + 0.5 * xi, wi):
                    e = x - ri - s_ * rij
                    b += w_ * delta(e @ e)
                b *= 0.5
                f = force_divr(rij @ rij, diam[i], diam[j])
                vir[g] += 0.5 * b * f * np.outer(rij[:dim], rij[:dim])
    return vir, kin


def test_three_particle_independent_restatement(oracle):
    """Three particles straddling the periodic x boundary, 2D octic R = 2, GL-5: the
    oracle's virial and kinetic fields against the pure-Python restatement above."""
    L = 12.0
    base = np.array([[5.6, 0.0, 0.0], [6.5, 0.3, 0.0], [5.8, 1.0, 0.0]])
    pos = base.copy()
    pos[:, 0] = (pos[:, 0] + L / 2) % L - L / 2  # wrapped into [-L/2, L/2)
    vel = np.array([[0.3, -0.2, 0.0], [-0.1, 0.4, 0.0], [0.25, 0.15, 0.0]])
    mass = np.array([1.0, 1.3, 0.8])
    diam = np.array([1.0, 0.9, 1.1])
    gx = np.linspace(4.0, 7.5, 8)
    gx = (gx + L / 2) % L - L / 2
    gy = np.linspace(-1.5, 2.5, 7)
    grid = np.array([[a, b, 0.0] for a in gx for b in gy])
    box = oracle.make_box(2, [L, L, 1.0])
    pot = oracle.make_poly12()
    cg = oracle.make_cg("octic", rcut=2.0, mode="fixedpoint", order=5)
    vir, kin = oracle.compute(box, pos, diam, pot, cg, grid, vel=vel, mass=mass)
    pv, pk = _py_ik_field(pos, vel, mass, diam, L, grid)
    assert np.count_nonzero(np.abs(pv).sum(axis=(1, 2))) > 10  # bonds seen by many points
    assert np.max(np.abs(vir - pv)) <= 1e-12 * np.max(np.abs(pv))
    assert np.max(np.abs(kin - pk)) <= 1e-12 * np.max(np.abs(pk))


def test_four_particle_3d_independent_restatement(oracle):
    """3D: four particles around a box corner (wrapped in x, y and z), octic R = 2, GL-5,
    against the pure-Python restatement."""
    L = 10.0
    base = np.array([[4.7, 4.6, 4.8], [5.5, 4.9, 5.1], [4.9, 5.6, 4.6], [5.2, 5.1, 5.7]])
    pos = (base + L / 2) % L - L / 2
    rng = np.random.default_rng(7)
    vel = rng.normal(0.0, 0.4, (4, 3))
    mass = np.array([1.0, 0.7, 1.2, 0.9])
    diam = np.array([1.0, 0.85, 1.1, 0.95])
    ax = (np.linspace(3.5, 6.5, 5) + L / 2) % L - L / 2
    grid = np.array([[a, b, c] for a in ax for b in ax for c in ax])
    box = oracle.make_box(3, [L, L, L])
    pot = oracle.make_poly12()
    cg = oracle.make_cg("octic", rcut=2.0, mode="fixedpoint", order=5)
    vir, kin = oracle.compute(box, pos, diam, pot, cg, grid, vel=vel, mass=mass)
    pv, pk = _py_ik_field(pos, vel, mass, diam, L, grid, dim=3)
    assert np.count_nonzero(np.abs(pv).sum(axis=(1, 2))) > 20
    assert np.max(np.abs(vir - pv)) <= 1e-12 * np.max(np.abs(pv))
    assert np.max(np.abs(kin - pk)) <= 1e-12 * np.max(np.abs(pk))
