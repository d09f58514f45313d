"""GPU parity of the eight pair models (LJ, force-shifted LJ, Poly10/106/12/18,
PolyLJ, PolyYukawa): the device's FP64 force and energy against the oracle (itself
pinned bit for bit to the reference's headers), and the stress field of both paths
against the FP64 oracle.

Tolerances: force and energy bit-exact, except PolydisperseYukawa (CUDA's exp against
the host's: 1e-15 of the magnitude of the summed terms); FP64 field relative L2 per component <= 1e-12; FP32 field
<= 1e-5; the force-active bond set of the FP32 path equals the FP64 one exactly.
"""
import numpy as np
import pytest

from conftest import rel_l2, uniq

pytestmark = pytest.mark.gpu

KINDS = ["poly12", "lj", "fslj", "poly10", "poly106", "poly18", "polylj", "polyyukawa"]
OCTIC = dict(kind="octic", rcut=2.0, mode="fixedpoint", order=5)


@pytest.fixture(scope="module")
def ik():
    from pyglasstools_gb300 import ikabi
    return ikabi


def _params(oracle, kind):
    rc, prm = oracle.potential_params(kind)
    prm = list(prm)
    if kind in ("lj", "fslj"):
        prm[1] = 0.1          # vareps: the force-shifted force ignores it, its energy does not
    elif kind == "polyyukawa":
        prm[2] = 0.05
    elif kind == "poly18":
        prm[1] = 0.1
    return rc, prm


@pytest.mark.parametrize("kind", KINDS)
def test_pair_force_and_energy_match_oracle(ik, oracle, golden, kind):
    g = golden("ref_potentials.npz")
    rc, prm = float(g[f"{kind}_rc"]), g[f"{kind}_params"]
    x = np.sqrt(g[f"{kind}_rsq"])
    rij = np.stack([x, np.zeros_like(x), np.zeros_like(x)], axis=1)
    rsq = x * x  # the device forms |r_ij|^2 from r_ij
    di, dj = g[f"{kind}_di"], g[f"{kind}_dj"]
    with ik.IKContext() as c:
        c.set_potential(kind, rc, prm)
        f, e = c.eval_pair(rij, di, dj)
    pot = oracle.make_potential(kind, rc, prm)
    wf = np.array([oracle.force_divr(pot, a, b, d) for a, b, d in zip(rsq, di, dj)])
    we = np.array([oracle.pair_energy(pot, a, b, d) for a, b, d in zip(rsq, di, dj)])
    if kind == "polyyukawa":
        # CUDA's exp may differ from the host's by an ulp; near the cut-off the smoothing
        # terms cancel most of the Yukawa term, so the bound is on the terms' magnitude
        v0, kap, eps, c0, c1, c2 = prm
        sig = 0.5 * (di + dj) * (1 - eps * np.abs(di - dj))
        s2 = sig * sig
        r2inv, rs = s2 / rsq, rsq / s2
        ey = v0 * np.exp(-kap * np.sqrt(rs))
        fs = (np.abs(ey * (np.sqrt(r2inv) + kap) * r2inv) + abs(2 * c1) + np.abs(4 * c2 * rs)) / s2
        es = np.abs(ey * np.sqrt(r2inv)) + abs(c0) + np.abs(c1 * rs) + np.abs(c2 * rs * rs)
        assert np.all(np.abs(f - wf) <= 1e-15 * fs)
        assert np.all(np.abs(e - we) <= 1e-15 * es)
        assert np.array_equal(f == 0, wf == 0)
    else:
        np.testing.assert_array_equal(f, wf)
        np.testing.assert_array_equal(e, we)


def _run(ik, kind, rc, prm, fr, grid, prec, dim=2):
    with ik.IKContext() as c:
        c.set_box(dim, [fr.L, fr.L, fr.L if dim == 3 else 1.0])
        c.set_potential(kind, rc, prm)
        c.set_cgfunc(**OCTIC)
        c.set_grid(grid)
        c.set_frame(fr.pos, fr.diam, fr.vel, fr.mass)
        c.compute(prec)
        return c.get_field(ik.FIELD_VIRIAL), c.counters(), c.get_max_rcut()


@pytest.mark.parametrize("kind", KINDS)
def test_ik_field_both_precisions_vs_oracle(ik, oracle, kind):
    from pyglasstools_gb300 import synth
    fr = synth.make_frame(1500, dim=2, seed=60 + KINDS.index(kind))
    grid = synth.lattice_grid(fr.L, 24, 2)
    rc, prm = _params(oracle, kind)
    v64, c64, max_rc = _run(ik, kind, rc, prm, fr, grid, "fp64")
    v32, c32, _ = _run(ik, kind, rc, prm, fr, grid, "fp32")
    box = oracle.make_box(2, [fr.L, fr.L, 1.0])
    cg = oracle.make_cg("octic", rcut=2.0, mode="fixedpoint", order=5)
    want, _ = oracle.compute(box, fr.pos, fr.diam, oracle.make_potential(kind, rc, prm), cg, grid,
                             max_rc=max_rc)
    assert np.max(np.abs(want)) > 0
    assert np.all(rel_l2(uniq(v64), uniq(want)) <= 1e-12), kind
    assert np.all(rel_l2(uniq(v32), uniq(want)) <= 1e-5), kind
    assert c32[0] > 0 and (c64[0] == 0 or c32[0] == c64[0])


def test_lj_3d_vs_oracle(ik, oracle):
    from pyglasstools_gb300 import synth
    fr = synth.make_frame(1000, dim=3, seed=71)
    grid = synth.lattice_grid(fr.L, 6, 3)
    rc, prm = _params(oracle, "lj")
    box = oracle.make_box(3, [fr.L] * 3)
    cg = oracle.make_cg("octic", rcut=2.0, mode="fixedpoint", order=5)
    for prec, tol in (("fp64", 1e-12), ("fp32", 1e-5)):
        v, _, max_rc = _run(ik, "lj", rc, prm, fr, grid, prec, dim=3)
        want, _ = oracle.compute(box, fr.pos, fr.diam, oracle.make_potential("lj", rc, prm), cg, grid,
                                 max_rc=max_rc)
        assert np.all(rel_l2(uniq(v), uniq(want)) <= tol), prec


def test_fp32_bond_set_at_the_cut_off(ik, oracle):
    """Pairs placed within a few ulp of the truncated LJ cut-off (where its force jumps):
    the FP32 path keeps exactly the FP64 path's bonds."""
    rc, prm = 2.5, [1.0, 0.0]
    rng = np.random.default_rng(5)
    n = 144
    L = 96.0
    pos = np.zeros((2 * n, 3))
    diam = np.ones(2 * n)
    # pairs on a lattice of spacing 8 (no bond between pairs), partner at distance
    # rc * (1 + k ulp) along a random direction
    sites = np.stack(np.meshgrid(np.arange(12), np.arange(12), indexing="ij"), -1).reshape(-1, 2)
    base = -L / 2 + 4.0 + sites * 8.0
    ang = rng.uniform(0, 2 * np.pi, n)
    d = rc * (1.0 + rng.integers(-40, 41, n) * 2.0 ** -52)
    pos[:n, :2] = base
    pos[n:, 0] = base[:, 0] + d * np.cos(ang)
    pos[n:, 1] = base[:, 1] + d * np.sin(ang)
    grid = np.stack(np.meshgrid(np.linspace(-L / 2, L / 2, 40), np.linspace(-L / 2, L / 2, 40),
                                indexing="ij"), -1).reshape(-1, 2)
    grid = np.concatenate([grid, np.zeros((len(grid), 1))], axis=1)

    class F:
        pass

    fr = F()
    fr.L, fr.pos, fr.diam, fr.vel, fr.mass = L, pos, diam, None, None
    v64, c64, max_rc = _run(ik, "lj", rc, prm, fr, grid, "fp64")
    v32, c32, _ = _run(ik, "lj", rc, prm, fr, grid, "fp32")
    box = oracle.make_box(2, [L, L, 1.0])
    cg = oracle.make_cg("octic", rcut=2.0, mode="fixedpoint", order=5)
    want, _ = oracle.compute(box, pos, diam, oracle.make_potential("lj", rc, prm), cg, grid, max_rc=max_rc)
    inside = sum(1 for k in range(n) if oracle.force_divr(oracle.make_potential("lj", rc, prm),
                                                          float(np.sum((pos[n + k] - pos[k]) ** 2)), 1.0, 1.0) != 0)
    assert 0 < inside < n
    assert c32[0] == 2 * inside
    assert np.all(rel_l2(uniq(v64), uniq(want)) <= 1e-12)
    assert np.all(rel_l2(uniq(v32), uniq(want)) <= 1e-5)


def test_python_frontend_with_polydisperse_lj(tmp_path, golden, monkeypatch, oracle):
    """pyglasstools.potential.polydisperselj through ikcalculator, FP64, against the oracle."""
    import pyglasstools_gb300 as pglass
    import pyglasstools_gb300.irvingkirkwood as ikm
    import pyglasstools_gb300.irvingkirkwood.cgfunc as cgfunc
    import pyglasstools_gb300.io as io
    import pyglasstools_gb300.potential as pot
    import pyglasstools_gb300.utils as utils
    from pyglasstools_gb300 import synth

    fr = synth.make_frame(1200, dim=2, seed=81)
    monkeypatch.chdir(tmp_path)
    pglass.reset()
    p = pot.polydisperselj(v0=1.0, eps=0.1, rcut=2.5)
    mycg = cgfunc.octic(rcut=2.0, mode="fixedpoint", order=5)
    utils.data_arrays([fr], ndim=2)
    calc = ikm.ikcalculator(cgfunc=mycg, dx=1.0, precision="fp64")
    io.fieldlogger(keyword="plj", names=['virialstress_00', 'virialstress_11', 'virialstress_01'], solver=calc)
    pglass.analyze(frame_list=[0], progress=False)
    pglass.reset()
    lines = open(tmp_path / "plj.xyz").read().splitlines()
    G = calc.gridsize
    vals = np.array([[float(t) for t in ln.split()[3:6]] for ln in lines[2:2 + G]])
    box = oracle.make_box(2, [fr.L, fr.L, 1.0])
    cg = oracle.make_cg("octic", rcut=2.0, mode="fixedpoint", order=5)
    assert p.get_params()[0] == 1.0 and p.get_params()[1] == 0.1
    want, _ = oracle.compute(box, fr.pos, fr.diam, oracle.make_potential("polylj", 2.5, p.get_params()), cg,
                             np.ascontiguousarray(calc.gridpoints, dtype=np.float64))
    w = uniq(want)
    # values are printed with 6 significant digits
    np.testing.assert_allclose(vals, w, rtol=6e-6, atol=1e-9 * np.max(np.abs(w)))


def test_fp32_bond_record_range_is_reported(ik, oracle):
    """A 3D Lennard-Jones frame with ~4e7 force-active bond records: past what the FP32
    gather's (offset << 6 | count) staging word addresses.  The gather checks the CSR
    total before any work and reports IK_ERR_CAPACITY; the FP64 path computes the frame."""
    from pyglasstools_gb300 import synth
    fr = synth.make_frame(600000, dim=3, seed=91)
    grid = synth.lattice_grid(fr.L, 4, 3)
    rc, prm = 2.5, [1.0, 0.0]
    with ik.IKContext() as c:
        c.set_box(3, [fr.L] * 3)
        c.set_potential("lj", rc, prm)
        c.set_cgfunc("octic", 2.0, order=5)
        c.set_grid(grid)
        c.set_frame(fr.pos, fr.diam)
        with pytest.raises(ik.IKError) as e:
            c.compute("fp32", ik.FIELD_VIRIAL)
        assert "2^25" in str(e.value)
        c.compute("fp64", ik.FIELD_VIRIAL)
        v = c.get_field(ik.FIELD_VIRIAL)
        assert np.all(np.isfinite(v)) and np.max(np.abs(v)) > 0
