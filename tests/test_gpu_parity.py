"""GPU parity tests: the CUDA path (called through the C ABI, libik_gb300.so) against
the FP64 CPU oracle on the same seeded inputs and against the committed golden
fixtures.

Tolerances (stated per the path's contract):
  * neighbour lists: bit-exact (sets and order: j ascending);
  * plain FP64 path: relative L2 error per stress component <= 1e-12;
  * tuned FP32 path: relative L2 error per stress component <= 1e-5, and
    max |error| / max |T| <= 1e-4 (FP32 pair arithmetic, compensated sums).
"""
import numpy as np
import pytest

from conftest import rel_l2, uniq

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-5
FP32_MAX_TOL = 1e-4


@pytest.fixture(scope="module")
def ik():
    from pyglasstools_gb300 import ikabi
    return ikabi


def run_gpu(ik, dim, L, pos, diam, grid, cg, precision, vel=None, mass=None, max_rc=None, pot=(1.0, 0.2, 1.25),
            flags=0):
    with ik.IKContext() as c:
        c.set_flags(flags)
        c.set_box(dim, [L, L, L if dim == 3 else 1.0])
        c.set_poly12(*pot)
        c.set_cgfunc(**cg)
        if max_rc is not None:
            c.set_max_rcut(max_rc)
        c.set_grid(grid)
        c.set_frame(pos, diam, vel, mass)
        c.compute(precision)
        return c.get_field(ik.FIELD_VIRIAL), c.get_field(ik.FIELD_KINETIC), c.counters()


def run_oracle(oracle, dim, L, pos, diam, grid, cg, vel=None, mass=None, max_rc=None, pot=(1.0, 0.2, 1.25)):
    box = oracle.make_box(dim, [L, L, L if dim == 3 else 1.0])
    p = oracle.make_poly12(*pot)
    c = oracle.make_cg(cg["kind"], rcut=cg["rcut"], mode=cg.get("mode", "fixedpoint"), order=cg.get("order", 5),
                       width=cg.get("width", 0.0))
    return oracle.compute(box, pos, diam, p, c, grid, vel=vel, mass=mass, max_rc=max_rc)


def assert_fields(got, want, tol, maxtol=None, what=""):
    g, w = uniq(got), uniq(want)
    err = rel_l2(g, w)
    assert np.all(err <= tol), f"{what}: rel L2 per component {err} > {tol}"
    if maxtol is not None:
        m = np.max(np.abs(g - w), axis=0) / np.maximum(np.max(np.abs(w), axis=0), 1e-300)
        assert np.all(m <= maxtol), f"{what}: max-abs/max {m} > {maxtol}"


def fixture_case(golden, frame=180):
    fr = golden("fixture_frames.npz")
    pos = fr[f"pos{frame}"].astype(np.float64)
    diam = fr[f"diam{frame}"].astype(np.float64)
    L = float(fr[f"box{frame}"][0])
    nmax = int(L / 0.25)
    pts = np.linspace(-L / 2, L / 2, nmax)
    gx, gy = np.meshgrid(pts, pts, indexing="ij")
    grid = np.stack([gx.ravel(), gy.ravel(), np.zeros(gx.size)], axis=1)
    return pos, diam, L, grid


OCTIC = dict(kind="octic", rcut=2.0, mode="fixedpoint", order=5)


# --------------------------------------------------------------------------- neighbours
def test_neighbors_bitexact_fixture(ik, oracle, golden):
    pos, diam, L, _ = fixture_case(golden)
    box = oracle.make_box(2, [L, L, 1.0])
    rc = oracle.max_rcut(1.25, diam)
    with ik.IKContext() as c:
        c.set_box(2, [L, L, 1.0])
        c.set_poly12()
        c.set_frame(pos, diam)
        for radius in (rc, 2.0, 3.3):
            o_off, o_idx = oracle.neighbors(box, pos, radius)
            g_off, g_idx = c.neighbors(radius, n=len(pos))
            assert np.array_equal(o_off, g_off) and np.array_equal(o_idx, g_idx), radius


def test_neighbors_bitexact_3d_and_point_query(ik, oracle):
    from pyglasstools_gb300 import synth
    f = synth.make_frame(3000, dim=3, seed=21)
    box = oracle.make_box(3, [f.L] * 3)
    with ik.IKContext() as c:
        c.set_box(3, [f.L] * 3)
        c.set_poly12()
        c.set_frame(f.pos, f.diam)
        o_off, o_idx = oracle.neighbors(box, f.pos, 2.025)
        g_off, g_idx = c.neighbors(2.025, n=len(f.pos))
        assert np.array_equal(o_off, g_off) and np.array_equal(o_idx, g_idx)
        q = np.array([0.3, -1.1, 2.0])
        ids = c.neighbors_point(q, 2.5)
        d = q[None, :] - f.pos
        d -= f.L * np.rint(d / f.L)
        r2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        assert np.array_equal(ids, np.nonzero(r2 < 2.5 * 2.5)[0])


# --------------------------------------------------------------------------- fields
def test_fixture_frame_fp64_matches_golden(ik, golden):
    pos, diam, L, grid = fixture_case(golden)
    gold = golden("oracle_fixture180.npz")
    vir, kin, _ = run_gpu(ik, 2, L, pos, diam, grid, OCTIC, "fp64", max_rc=float(gold["max_rcut"]))
    err = rel_l2(uniq(vir), gold["virial"])
    assert np.all(err <= FP64_TOL), err
    assert np.all(kin == 0.0)  # the fixture has no velocities (GSD defaults)


def test_fixture_frame_fp32_matches_golden(ik, golden):
    pos, diam, L, grid = fixture_case(golden)
    gold = golden("oracle_fixture180.npz")
    vir, _, cnt = run_gpu(ik, 2, L, pos, diam, grid, OCTIC, "fp32", max_rc=float(gold["max_rcut"]))
    g = uniq(vir)
    err = rel_l2(g, gold["virial"])
    assert np.all(err <= FP32_TOL), err
    m = np.max(np.abs(g - gold["virial"]), axis=0) / np.max(np.abs(gold["virial"]), axis=0)
    assert np.all(m <= FP32_MAX_TOL), m
    assert cnt[0] > 0 and cnt[1] > 0 and cnt[2] > 0


def test_cfg0_virial_and_kinetic_both_precisions(ik, golden):
    from pyglasstools_gb300 import synth
    f = synth.make_frame(2000, dim=2, seed=0)
    gold = golden("oracle_cfg0.npz")
    assert f.pos.sum() == float(gold["pos_checksum"])
    grid = synth.lattice_grid(f.L, 64, 2)
    for prec, tol in (("fp64", FP64_TOL), ("fp32", FP32_TOL)):
        vir, kin, _ = run_gpu(ik, 2, f.L, f.pos, f.diam, grid, OCTIC, prec, vel=f.vel, mass=f.mass)
        ev = rel_l2(uniq(vir), gold["virial"])
        ek = rel_l2(uniq(kin), gold["kinetic"])
        assert np.all(ev <= tol), (prec, ev)
        assert np.all(ek <= tol), (prec, ek)


@pytest.mark.parametrize("seed", [1, 2])
def test_gaussian_2d_vs_oracle(ik, oracle, seed):
    from pyglasstools_gb300 import synth
    f = synth.make_frame(3000, dim=2, seed=seed)
    grid = synth.lattice_grid(f.L, 48, 2)
    cg = dict(kind="gaussian", rcut=6.0, mode="fixedpoint", order=5, width=2.0)
    ov, ok = run_oracle(oracle, 2, f.L, f.pos, f.diam, grid, cg, vel=f.vel, mass=f.mass)
    gv, gk, _ = run_gpu(ik, 2, f.L, f.pos, f.diam, grid, cg, "fp64", vel=f.vel, mass=f.mass)
    assert_fields(gv, ov, FP64_TOL, what="fp64 virial")
    assert_fields(gk, ok, FP64_TOL, what="fp64 kinetic")
    for flags in (0, 2):  # plain and Kahan-compensated per-lane sums
        gv, gk, _ = run_gpu(ik, 2, f.L, f.pos, f.diam, grid, cg, "fp32", vel=f.vel, mass=f.mass, flags=flags)
        assert_fields(gv, ov, FP32_TOL, FP32_MAX_TOL, what=f"fp32 virial flags={flags}")
        assert_fields(gk, ok, FP32_TOL, FP32_MAX_TOL, what=f"fp32 kinetic flags={flags}")


def test_3d_octic_vs_oracle(ik, oracle):
    from pyglasstools_gb300 import synth
    f = synth.make_frame(4000, dim=3, seed=3)
    grid = synth.lattice_grid(f.L, 14, 3)
    ov, ok = run_oracle(oracle, 3, f.L, f.pos, f.diam, grid, OCTIC, vel=f.vel, mass=f.mass)
    gv, gk, _ = run_gpu(ik, 3, f.L, f.pos, f.diam, grid, OCTIC, "fp64", vel=f.vel, mass=f.mass)
    assert_fields(gv, ov, FP64_TOL, what="3d fp64 virial")
    assert_fields(gk, ok, FP64_TOL, what="3d fp64 kinetic")
    gv, gk, _ = run_gpu(ik, 3, f.L, f.pos, f.diam, grid, OCTIC, "fp32", vel=f.vel, mass=f.mass)
    assert_fields(gv, ov, FP32_TOL, FP32_MAX_TOL, what="3d fp32 virial")
    assert_fields(gk, ok, FP32_TOL, FP32_MAX_TOL, what="3d fp32 kinetic")


@pytest.mark.parametrize("kind,order,rc", [("octic", 1, 2.0), ("octic", 3, 2.5), ("octic", 8, 2.0),
                                           ("mollifier", 5, 2.0), ("rect", 5, 2.0), ("gaussian", 7, 4.0)])
def test_kernels_and_orders_vs_oracle(ik, oracle, kind, order, rc):
    from pyglasstools_gb300 import synth
    f = synth.make_frame(1200, dim=2, seed=5)
    grid = synth.lattice_grid(f.L, 30, 2)
    cg = dict(kind=kind, rcut=rc, mode="fixedpoint", order=order, width=(rc / 3 if kind == "gaussian" else 0.0))
    if kind == "mollifier":
        cg["width"] = rc
    ov, ok = run_oracle(oracle, 2, f.L, f.pos, f.diam, grid, cg, vel=f.vel, mass=f.mass)
    gv, gk, _ = run_gpu(ik, 2, f.L, f.pos, f.diam, grid, cg, "fp64", vel=f.vel, mass=f.mass)
    assert_fields(gv, ov, FP64_TOL, what=f"{kind} fp64")
    assert_fields(gk, ok, FP64_TOL, what=f"{kind} fp64 kinetic")
    gv, gk, _ = run_gpu(ik, 2, f.L, f.pos, f.diam, grid, cg, "fp32", vel=f.vel, mass=f.mass)
    # the rect kernel is discontinuous at R: an FP32 node landing on the other side
    # of the cut changes that bond's integral by w_k/2, so its bound is looser
    tol = 2e-4 if kind == "rect" else FP32_TOL
    assert_fields(gv, ov, tol, what=f"{kind} fp32")


# --------------------------------------------------------------------------- edge cases
def test_empty_frame_and_single_particle(ik, oracle):
    L = 20.0
    grid = np.array([[0.0, 0.0, 0.0], [1.0, 0.5, 0.0], [9.0, -9.5, 0.0]])
    for prec in ("fp64", "fp32"):
        vir, kin, _ = run_gpu(ik, 2, L, np.zeros((0, 3)), np.zeros(0), grid, OCTIC, prec, max_rc=1.25)
        assert np.all(vir == 0) and np.all(kin == 0)
        pos = np.array([[0.5, 0.25, 0.0]])
        vel = np.array([[1.0, -2.0, 0.0]])
        vir, kin, _ = run_gpu(ik, 2, L, pos, np.ones(1), grid, OCTIC, prec, vel=vel, mass=np.array([2.0]))
        ov, ok = run_oracle(oracle, 2, L, pos, np.ones(1), grid, OCTIC, vel=vel, mass=np.array([2.0]))
        assert np.all(vir == 0)
        np.testing.assert_allclose(kin, ok, rtol=1e-6 if prec == "fp32" else 1e-14, atol=1e-300)


def test_grid_points_outside_box_and_periodic_duplicates(ik, oracle):
    from pyglasstools_gb300 import synth
    f = synth.make_frame(800, dim=2, seed=8)
    base = synth.lattice_grid(f.L, 12, 2)
    grid = np.concatenate([base, base + np.array([f.L, 0.0, 0.0]), base - np.array([0.0, 3 * f.L, 0.0])])
    ov, _ = run_oracle(oracle, 2, f.L, f.pos, f.diam, grid, OCTIC)
    for prec, tol in (("fp64", FP64_TOL), ("fp32", FP32_TOL)):
        gv, _, _ = run_gpu(ik, 2, f.L, f.pos, f.diam, grid, OCTIC, prec)
        assert_fields(gv, ov, tol, what=prec)
        n = len(base)
        np.testing.assert_allclose(gv[n:2 * n], gv[:n], rtol=1e-9 if prec == "fp64" else 1e-5, atol=1e-9)


def test_errors_are_reported_not_fatal(ik):
    from pyglasstools_gb300.ikabi import IKError
    with ik.IKContext() as c:
        c.set_box(2, [3.0, 3.0, 1.0])
        c.set_poly12()
        c.set_cgfunc("octic", 2.0)
        c.set_grid(np.zeros((1, 3)))
        c.set_frame(np.zeros((1, 3)), np.ones(1))
        with pytest.raises(IKError, match="IK_ERR_BOX"):
            c.compute("fp32")  # 2 * R_cg >= L
        with pytest.raises(IKError, match="IK_ERR_ARG"):
            c.set_frame(np.array([[np.nan, 0.0, 0.0]]), np.ones(1))
        with pytest.raises(IKError, match="IK_ERR_ARG"):
            c.set_frame(np.array([[0.0, 0.0, 0.5]]), np.ones(1))  # 2D frame with z != 0
        with pytest.raises(IKError, match="IK_ERR_ARG"):
            c.set_cgfunc("octic", 2.0, order=0)
        # the context stays usable after errors
        c.set_box(2, [30.0, 30.0, 1.0])
        c.set_frame(np.zeros((1, 3)), np.ones(1))
        c.compute("fp32")


def test_bond_capacity_growth_dense_cluster(ik, oracle):
    """A dense cluster gives particles more force-active bonds than the initial
    per-particle capacity (16 in 2D); the engine grows it and recomputes."""
    rng = np.random.default_rng(4)
    L = 30.0
    pos = np.zeros((60, 3))
    pos[:, :2] = rng.uniform(-0.6, 0.6, size=(60, 2))
    diam = np.full(60, 1.0)
    grid = np.array([[x, y, 0.0] for x in np.linspace(-2, 2, 9) for y in np.linspace(-2, 2, 9)])
    ov, _ = run_oracle(oracle, 2, L, pos, diam, grid, OCTIC)
    for prec, tol in (("fp64", FP64_TOL), ("fp32", FP32_TOL)):
        gv, _, _ = run_gpu(ik, 2, L, pos, diam, grid, OCTIC, prec)
        assert_fields(gv, ov, tol, what=prec)


def test_halo_chunking_and_cell_overflow_growth(ik, oracle):
    """One giant particle makes the cells wide (max_rcut = 1.25 * 10); small particles
    on a lattice of spacing 0.45 then put ~770 particles in a cell: the FP32 gather
    stages each halo in chunks and grows its per-warp buffer past 512."""
    L = 50.0
    a = 0.45
    k = np.arange(-L / 2 + a / 2, L / 2 - 1e-9, a)
    gx, gy = np.meshgrid(k, k, indexing="ij")
    lat = np.stack([gx.ravel(), gy.ravel(), np.zeros(gx.size)], axis=1)
    lat = lat[np.hypot(lat[:, 0], lat[:, 1]) > 6.6]  # keep the giant particle bond-free
    pos = np.concatenate([np.zeros((1, 3)), lat])
    diam = np.full(len(pos), 0.4)
    diam[0] = 10.0
    pot = (1.0, 0.0, 1.25)
    grid = np.array([[x, y, 0.0] for x in np.linspace(-20, 20, 11) for y in np.linspace(-20, 20, 11)])
    ov, _ = run_oracle(oracle, 2, L, pos, diam, grid, OCTIC, pot=pot)
    assert np.max(np.abs(ov)) > 0
    gv, _, _ = run_gpu(ik, 2, L, pos, diam, grid, OCTIC, "fp32", pot=pot)
    assert_fields(gv, ov, FP32_TOL, what="fp32 chunked halo")
    gv, _, _ = run_gpu(ik, 2, L, pos, diam, grid, OCTIC, "fp64", pot=pot)
    assert_fields(gv, ov, FP64_TOL, what="fp64")


def test_fp32_deterministic_and_order_independent(ik):
    from pyglasstools_gb300 import synth
    f = synth.make_frame(2500, dim=2, seed=13)
    grid = synth.lattice_grid(f.L, 40, 2)
    cg = dict(kind="gaussian", rcut=6.0, mode="fixedpoint", order=5, width=2.0)
    a, _, _ = run_gpu(ik, 2, f.L, f.pos, f.diam, grid, cg, "fp32")
    b, _, _ = run_gpu(ik, 2, f.L, f.pos, f.diam, grid, cg, "fp32")
    assert np.array_equal(a, b)  # no float atomics: bitwise reproducible
    # bond records compacted to CSR (the layout of very large frames): same records, same sums
    a_csr, _, cnt_csr = run_gpu(ik, 2, f.L, f.pos, f.diam, grid, cg, "fp32", flags=ik.FLAG_CSR_BONDS)
    _, _, cnt = run_gpu(ik, 2, f.L, f.pos, f.diam, grid, cg, "fp32")
    assert np.array_equal(a, a_csr) and cnt == cnt_csr
    perm = np.random.default_rng(0).permutation(len(f.pos))
    c, _, _ = run_gpu(ik, 2, f.L, f.pos[perm], f.diam[perm], grid, cg, "fp64")
    d, _, _ = run_gpu(ik, 2, f.L, f.pos, f.diam, grid, cg, "fp64")
    assert_fields(c, d, 1e-13, what="permuted input")


def test_counters_match_oracle_counts(ik, oracle):
    from pyglasstools_gb300 import synth
    f = synth.make_frame(900, dim=2, seed=17)
    grid = synth.lattice_grid(f.L, 20, 2)
    _, _, cnt = run_gpu(ik, 2, f.L, f.pos, f.diam, grid, OCTIC, "fp32")
    box = oracle.make_box(2, [f.L, f.L, 1.0])
    pot = oracle.make_poly12()
    offs, idx = oracle.neighbors(box, f.pos, oracle.max_rcut(1.25, f.diam))
    active = np.zeros(len(f.pos), np.int64)
    for i in range(len(f.pos)):
        for j in idx[offs[i]:offs[i + 1]]:
            d = f.pos[j] - f.pos[i]
            d[:2] -= f.L * np.rint(d[:2] / f.L)
            if oracle.force_divr(pot, float(d @ d), f.diam[i], f.diam[j]) != 0.0:
                active[i] += 1
    assert abs(cnt[0] - active.sum()) <= 2  # FP32 cut-off test may flip a bond at the cut
    d = grid[:, None, :2] - f.pos[None, :, :2]
    d -= f.L * np.rint(d / f.L)
    inside = (d ** 2).sum(-1) < 4.0
    assert cnt[1] == inside.sum()
    assert abs(cnt[2] - (inside * active[None, :]).sum()) <= 0.001 * cnt[2] + 4


def test_scalar_evaluations_match_oracle(ik, oracle):
    rng = np.random.default_rng(2)
    m = 500
    rij = np.zeros((m, 3))
    rij[:, :2] = rng.uniform(-1.6, 1.6, (m, 2))
    di, dj = rng.uniform(0.7, 1.6, m), rng.uniform(0.7, 1.6, m)
    pot = oracle.make_poly12()
    with ik.IKContext() as c:
        c.set_poly12()
        c.set_cgfunc("octic", 2.0, order=5)
        f, e = c.eval_pair(rij, di, dj)
        for k in range(m):
            r2 = float((rij[k, 0] * rij[k, 0] + rij[k, 1] * rij[k, 1]) + rij[k, 2] * rij[k, 2])
            assert f[k] == oracle.force_divr(pot, r2, di[k], dj[k])
            assert abs(e[k] - oracle.pair_energy(pot, r2, di[k], dj[k])) <= 1e-15 * max(1.0, abs(e[k]))
        x = np.zeros((m, 3))
        ri = np.zeros((m, 3))
        ri[:, :2] = rng.uniform(-2, 2, (m, 2))
        b, d = c.eval_bond(x, ri, rij)
        cg = oracle.make_cg("octic", rcut=2.0, order=5)
        for k in range(m):
            assert abs(b[k] - oracle.bond(cg, 2, x[k], ri[k], rij[k])) <= 1e-15
            assert abs(d[k] - oracle.delta(cg, 2, float(ri[k] @ ri[k]))) <= 1e-15


# --------------------------------------------------------------------------- reference-facing API
def test_python_api_end_to_end(tmp_path, golden, monkeypatch):
    """The reference's example script (test-irvingkirkwood-module.py) on two fixture
    frames through the mirrored Python API, written to <keyword>.xyz."""
    import pyglasstools_gb300 as pglass
    import pyglasstools_gb300.io as io
    import pyglasstools_gb300.irvingkirkwood as ikm
    import pyglasstools_gb300.irvingkirkwood.cgfunc as cgfunc
    import pyglasstools_gb300.potential as pot
    import pyglasstools_gb300.utils as utils

    class Fr:
        pass

    fx = golden("fixture_frames.npz")
    frames = []
    for f in (180, 199):
        fr = Fr()
        fr.pos = fx[f"pos{f}"].astype(np.float64)
        fr.diam = fx[f"diam{f}"].astype(np.float64)
        fr.L = float(fx[f"box{f}"][0])
        frames.append(fr)
    monkeypatch.chdir(tmp_path)
    pglass.reset()
    pot.polydisperse12(v0=1.0, eps=0.2, rcut=1.25)
    mycg = cgfunc.octic(rcut=2.0, mode="fixedpoint", order=5)
    utils.data_arrays(frames, ndim=2, checkpointfile="restart.log")
    calc = ikm.ikcalculator(cgfunc=mycg, dx=0.25, precision="fp64")
    io.fieldlogger(keyword="test-dump", names=['virialstress_00', 'virialstress_11', 'virialstress_01'],
                   solver=calc)
    pglass.analyze(frame_list=[0, 1], progress=False)
    pglass.reset()
    lines = open(tmp_path / "test-dump.xyz").read().splitlines()
    G = calc.gridsize
    assert lines[0] == f"{G} " and lines[1] == "#Frame 0  "
    assert len(lines) == 2 * (G + 2)
    gold = golden("oracle_fixture180.npz")["virial"]
    vals = np.array([[float(t) for t in ln.split()[3:6]] for ln in lines[2:2 + G]])
    xy = np.array([[float(t) for t in ln.split()[1:3]] for ln in lines[2:2 + G]])
    np.testing.assert_array_equal(xy, calc.gridpoints[:, :2])
    # values are printed with 6 significant digits
    np.testing.assert_allclose(vals, gold, rtol=6e-6, atol=1e-300)
    assert open(tmp_path / "restart.log").read() == "Frame 2"


@pytest.mark.parametrize("cg", [dict(kind="gaussian", rcut=6.0, mode="exact", order=5, width=2.0),
                                dict(kind="octic", rcut=2.0, mode="exact", order=5)])
def test_exact_bond_integral_fp64_vs_oracle(ik, oracle, cg):
    """Exact mode (segment clipped to the support; erf closed form for the Gaussian,
    GL-5 on the clipped interval for the octic) on the plain FP64 path."""
    from pyglasstools_gb300 import synth
    fr = synth.make_frame(2500, dim=2, seed=61)
    grid = synth.lattice_grid(fr.L, 40, 2)
    got_v, got_k, _ = run_gpu(ik, 2, fr.L, fr.pos, fr.diam, grid, cg, "fp64", vel=fr.vel, mass=fr.mass)
    want_v, want_k = run_oracle(oracle, 2, fr.L, fr.pos, fr.diam, grid, cg, vel=fr.vel, mass=fr.mass)
    assert_fields(got_v, want_v, FP64_TOL, what="exact virial")
    assert_fields(got_k, want_k, FP64_TOL, what="exact kinetic")
    if cg["kind"] != "gaussian":
        with pytest.raises(ik.IKError):
            run_gpu(ik, 2, fr.L, fr.pos, fr.diam, grid, cg, "fp32")  # FP32 exact mode: the Gaussian only


def test_radialcalculator_polar_output(tmp_path, golden, monkeypatch, ik):
    """radialcalculator (irvingkirkwood/__init__.py:80-166) + fieldlogger's polar lines
    (io.py:130-144) on a fixture frame: '1 id r theta T_00 T_11 T_01', the values those
    of the same computation on the same grid points through the C ABI."""
    import pyglasstools_gb300 as pglass
    import pyglasstools_gb300.io as io
    import pyglasstools_gb300.irvingkirkwood as ikm
    import pyglasstools_gb300.irvingkirkwood.cgfunc as cgfunc
    import pyglasstools_gb300.potential as pot
    import pyglasstools_gb300.utils as utils

    class Fr:
        pass

    fx = golden("fixture_frames.npz")
    fr = Fr()
    fr.pos = fx["pos180"].astype(np.float64)
    fr.diam = fx["diam180"].astype(np.float64)
    fr.L = float(fx["box180"][0])
    monkeypatch.chdir(tmp_path)
    pglass.reset()
    pot.polydisperse12(v0=1.0, eps=0.2, rcut=1.25)
    mycg = cgfunc.octic(rcut=2.0, mode="fixedpoint", order=5)
    utils.data_arrays([fr], ndim=2)
    calc = ikm.radialcalculator(cgfunc=mycg, center=np.array([1.0, -2.0, 0.0]), rmax=5, dr=0.5, precision="fp64")
    io.fieldlogger(keyword="polar", names=['virialstress_00', 'virialstress_11', 'virialstress_01'], solver=calc)
    pglass.analyze(frame_list=[0], progress=False)
    pglass.reset()
    lines = open(tmp_path / "polar.xyz").read().splitlines()
    G = calc.gridsize
    assert lines[0] == f"{G} " and len(lines) == G + 2
    rows = [ln.split() for ln in lines[2:]]
    assert [int(r[1]) for r in rows] == [int(v) for v in calc.gridid]
    np.testing.assert_array_equal(np.array([float(r[2]) for r in rows]), calc.globalr)
    np.testing.assert_array_equal(np.array([float(r[3]) for r in rows]), calc.globaltheta)
    vals = np.array([[float(t) for t in r[4:7]] for r in rows])
    with ik.IKContext() as c:
        c.set_box(2, [fr.L, fr.L, 1.0])
        c.set_poly12()
        c.set_cgfunc("octic", 2.0, order=5)
        c.set_grid(calc.gridpoints)
        c.set_frame(fr.pos, fr.diam)
        c.compute("fp64")
        v = c.get_field(ik.FIELD_VIRIAL)
    np.testing.assert_allclose(vals, uniq(v), rtol=6e-6, atol=1e-300)
