"""CPU tests: the C-ABI library loads and exports every declared entry point, the
pybind11 layer imports, host-side logic (grid, box, field formatting, checkpoint,
GSD reading) behaves like the reference's."""
import ctypes
import os
import re
import struct

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    hdrs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]
    names = set()
    for h in hdrs:
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(ik_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    from pyglasstools_gb300 import ikabi
    L = ctypes.CDLL(ikabi.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_last_error_and_version_without_gpu():
    from pyglasstools_gb300 import ikabi
    L = ikabi.lib()
    assert L.ik_version() >= 100
    h = ctypes.c_void_p()
    rc = L.ik_create(ctypes.byref(h), 0)
    if rc == 0:
        L.ik_destroy(h)
        pytest.skip("a GPU is present")
    assert rc == -2 and b"CUDA" in L.ik_last_error()
    assert L.ik_set_box(None, 2, None, None) == -1  # null context is an argument error


def test_pybind_modules_import_and_mirror_reference_names():
    import pyglasstools_gb300 as pg
    from pyglasstools_gb300 import _core
    for mod, names in {
        "_pyglasstools": ["SimBox", "ParticleSystem", "Communicator", "MPILogFile", "Manager"],
        "_potential": ["PairPotential", "PairPotentialLJ", "PairPotentialForceShiftedLJ", "PairPotentialPoly12",
                       "PairPotentialPoly18", "PairPotentialPoly10", "PairPotentialPoly106",
                       "PairPotentialPolyYukawa", "PairPotentialPolyLJ"],
        "_cgfunc": ["CoarseGrainFunction", "CGFuncOcticFixedPoint", "CGFuncOcticAdaptive", "CGFuncRectFixedPoint",
                    "CGFuncRectAdaptive", "CGFuncMollifierFixedPoint", "CGFuncMollifierAdaptive",
                    "CGFuncGaussianFixedPoint"],
        "_irvingkirkwood": ["IrvingKirkwood", "VirialStressField2D", "VirialStressField3D",
                            "KineticStressField2D", "KineticStressField3D"],
    }.items():
        m = getattr(_core, mod)
        for n in names:
            assert hasattr(m, n), (mod, n)
    assert pg.rank == 0 and pg.size == 1


def test_simbox_bounds_match_reference():
    from pyglasstools_gb300 import utils
    b = utils.simbox(Lx=10.0, Ly=12.0, Lz=3.0, ndim=2)
    assert list(b.boxsize) == [10.0, 12.0, 1.0]
    assert list(b.lowerbound) == [-5.0, -6.0, -0.5] and list(b.upperbound) == [5.0, 6.0, 0.5]
    assert list(b.periodic) == [1, 1, 0] and b.vol == 120.0


def test_lattice_grid_matches_reference_construction():
    from pyglasstools_gb300.irvingkirkwood import lattice_gridpoints
    L, dx = 31.84119, 0.25
    g = lattice_gridpoints(L, dx, 2)
    nmax = int(L / dx)
    pts = np.linspace(-L / 2, L / 2, nmax)
    want = np.array([[pts[i], pts[j], 0.0] for i in range(nmax) for j in range(nmax)])
    assert np.array_equal(g, want)


def test_field_formatting_like_cpp_ostream():
    from pyglasstools_gb300 import _core
    f = _core._irvingkirkwood.VirialStressField2D("virialstress", "2-TENSOR", False, 3)
    assert f.gettostring(0, 0) == "0 "
    with pytest.raises(IndexError):
        f.gettostring(4, 0)
    with pytest.raises(IndexError):
        f.gettostring(0, 3)


def test_particle_system_size_checks():
    from pyglasstools_gb300 import _core
    pg = _core._pyglasstools
    box = pg.SimBox(np.array([10.0, 10.0, 1.0]), np.zeros(3), 2)
    with pytest.raises(ValueError, match="mismatch"):
        pg.ParticleSystem(box, 3, [1.0, 1.0], [1.0, 1.0, 1.0], np.zeros((3, 3)), np.zeros((3, 3)))
    s = pg.ParticleSystem(box, 2, [1.0, 1.0], [1.0, 1.0], np.zeros((2, 3)), np.zeros((2, 3)))
    with pytest.raises(ValueError, match="mismatch"):
        s.setMass([1.0])


def _write_gsd(path, frames, version=(2, 0), corrupt=None):
    """Tiny GSD writer for tests (HOOMD schema, layout 1.0 or 2.0)."""
    names = ["configuration/box", "particles/N", "particles/diameter", "particles/position", "configuration/step"]
    chunks = []  # (frame, id, type, N, M, bytes)
    for f, fr in enumerate(frames):
        chunks.append((f, 0, 9, 6, 1, np.asarray(fr["box"], np.float32).tobytes()))
        chunks.append((f, 1, 3, 1, 1, np.uint32(fr["N"]).tobytes()))
        chunks.append((f, 2, 9, len(fr["diam"]), 1, np.asarray(fr["diam"], np.float32).tobytes()))
        chunks.append((f, 3, 9, len(fr["pos"]), 3, np.asarray(fr["pos"], np.float32).tobytes()))
        chunks.append((f, 4, 4, 1, 1, np.uint64(f).tobytes()))
    nl = b"".join(n.encode() + b"\0" for n in names).ljust(64 * len(names), b"\0") if version[0] == 2 else \
        b"".join(n.encode().ljust(64, b"\0") for n in names)
    body = bytearray()
    off = 256 + len(nl)
    index = []
    for (f, cid, typ, N, M, data) in chunks:
        index.append(struct.pack("<QQqIHBB", f, N, off + len(body), M, cid, typ, 0))
        body += data
    idx_loc = 256 + len(nl) + len(body)
    hdr = struct.pack("<QQQQQII", 0x65DF65DF65DF65DF, idx_loc, len(index), 256, len(names),
                      (1 << 16) | 4, (version[0] << 16) | version[1])
    hdr += b"gsd-test".ljust(64, b"\0") + b"hoomd".ljust(64, b"\0")
    hdr = hdr.ljust(256, b"\0")
    blob = bytes(hdr) + nl + bytes(body) + b"".join(index)
    if corrupt == "truncate":
        blob = blob[: len(blob) - 40]
    if corrupt == "magic":
        blob = b"\0" * 8 + blob[8:]
    open(path, "wb").write(blob)


def test_gsd_reader_roundtrip_and_defaults(tmp_path, golden):
    from pyglasstools_gb300 import gsd
    fx = golden("fixture_frames.npz")
    frames = [{"box": fx["box180"], "N": len(fx["diam180"]), "diam": fx["diam180"], "pos": fx["pos180"]},
              {"box": fx["box199"], "N": len(fx["diam199"]), "diam": fx["diam199"], "pos": fx["pos199"]}]
    for ver in ((1, 0), (2, 0)):
        p = tmp_path / f"t{ver[0]}.gsd"
        _write_gsd(p, frames, version=ver)
        t = gsd.open_trajectory(str(p))
        assert len(t) == 2
        f1 = t[1]
        assert np.array_equal(f1.position, fx["pos199"]) and np.array_equal(f1.diameter, fx["diam199"])
        assert np.all(f1.mass == 1.0) and np.all(f1.velocity == 0.0)  # HOOMD schema defaults
        assert f1.N == 1024 and abs(float(f1.box[0]) - 31.84119) < 1e-5


def test_gsd_reader_rejects_corrupt_files(tmp_path, golden):
    from pyglasstools_gb300 import gsd
    fx = golden("fixture_frames.npz")
    fr = [{"box": fx["box180"], "N": 1024, "diam": fx["diam180"], "pos": fx["pos180"]}]
    p = tmp_path / "bad.gsd"
    _write_gsd(p, fr, corrupt="truncate")
    with pytest.raises(gsd.GSDError):
        gsd.open_trajectory(str(p))
    _write_gsd(p, fr, corrupt="magic")
    with pytest.raises(gsd.GSDError, match="magic"):
        gsd.open_trajectory(str(p))
    fr[0]["N"] = 1000  # N chunk disagrees with the arrays
    _write_gsd(p, fr)
    with pytest.raises(gsd.GSDError, match="rows"):
        gsd.open_trajectory(str(p))[0]


def test_reference_fixture_decodes_if_present():
    path = os.path.join(os.environ.get("PYGLASSTOOLS_REF", "/root/reference"), "example_scripts",
                        "polydisperse12.gsd")
    if not os.path.exists(path):
        pytest.skip("reference fixture not on this machine")
    from pyglasstools_gb300 import gsd
    t = gsd.open_trajectory(path)
    assert len(t) == 201
    f = t[180]
    assert f.N == 1024 and np.all(f.mass == 1) and np.all(f.velocity == 0)


def test_checkpoint_resume_logic(tmp_path):
    from pyglasstools_gb300 import utils
    d = utils.data_gsd.__new__(utils.data_gsd)
    d.checkpointfile = str(tmp_path / "restart.log")
    assert d.setup_checkpoint(range(180, 200)) == list(range(180, 200))
    assert open(d.checkpointfile).read() == "Frame 180"
    open(d.checkpointfile, "w").write("Frame 190")
    assert d.setup_checkpoint(range(180, 200)) == list(range(190, 200))


def test_synthetic_generator_recipe():
    from pyglasstools_gb300 import synth
    f = synth.make_frame(2000, dim=2, seed=0)
    assert f.N == 2000 and abs(f.L - np.sqrt(2000)) < 1e-12
    assert f.diam.min() >= synth.SIGMA_MIN and f.diam.max() <= synth.SIGMA_MAX
    assert np.all(np.abs(f.pos[:, :2]) <= f.L / 2) and np.all(f.pos[:, 2] == 0)
    assert np.allclose(f.vel[:, :2].mean(0), 0, atol=1e-12)
    assert abs(np.mean(f.vel[:, :2] ** 2) - 0.3) < 0.03
    g = synth.make_frame(2000, dim=2, seed=0)
    assert np.array_equal(f.pos, g.pos)  # seeded, platform independent


def test_native_float_repr_matches_python_repr():
    """The bulk .xyz writer prints grid coordinates exactly like "{} ".format(x)."""
    from pyglasstools_gb300 import _core
    K = _core._irvingkirkwood
    rng = np.random.default_rng(0)
    vals = np.concatenate([rng.normal(0, 1, 3000) * 10.0 ** rng.integers(-14, 22, 3000),
                           [0.0, -0.0, 1.0, 2.0, 1e16, 1e15, 9999999999999998.0, 1e-4, 1e-5, 0.30000000000000004,
                            -2.5e-7, 100.0, 1234567.0, float("inf"), float("-inf")]])
    for v in vals:
        assert K.float_repr(float(v)) == repr(float(v)), v


def test_bulk_field_lines_match_per_point_formatting():
    """format_field_lines gives the text of the per-point gettostring loop
    (io.py:112-128 cartesian, :130-144 polar), here on zero-valued fields."""
    from pyglasstools_gb300 import _core
    K = _core._irvingkirkwood
    g = np.array([[-1.5, 0.25, 0.0], [3.0, 1e-7, 0.0], [2.0 / 3.0, -12.0, 0.0]])
    vir = K.VirialStressField2D("virialstress", "2-TENSOR", False, len(g))
    kin = K.KineticStressField2D("kineticstress", "2-TENSOR", True, len(g))
    comps = [(vir, 0), (vir, 3), (kin, 2)]
    want = "".join("1 {} {} ".format(p[0], p[1]) + vir.gettostring(0, i) + vir.gettostring(3, i)
                   + kin.gettostring(2, i) + "\n" for i, p in enumerate(g))
    assert K.format_field_lines(g[:, :2], comps) == want
    polar = np.array([[0, 0.0, 0.0], [1, 0.1, 0.5], [2, 0.2, 6.283185307179586]])
    want_p = "".join("1 {} {} {} ".format(int(p[0]), p[1], p[2]) + vir.gettostring(0, i) + "\n"
                     for i, p in enumerate(polar))
    assert K.format_field_lines(polar, [(vir, 0)], [0]) == want_p


def test_polar_grid_matches_reference_recipe():
    """radialcalculator's grid (irvingkirkwood/__init__.py:83-127): origin first, then
    rings with int(2 pi r / dr) points each."""
    from pyglasstools_gb300.irvingkirkwood import polar_gridpoints
    c = np.array([1.0, -2.0, 0.0])
    pts, gid, r, th = polar_gridpoints(c, "normal", rmax=2.0, dr=0.25)
    rr = np.linspace(0, 2.0, int(2.0 / 0.25))[1:]
    assert np.array_equal(pts[0], c) and gid[0] == 0 and r[0] == 0 and th[0] == 0
    counts = [int(2 * np.pi / (0.25 / x)) for x in rr]
    assert len(pts) == 1 + sum(counts)
    k = 1
    for i, (x, n) in enumerate(zip(rr, counts)):
        theta = np.linspace(0, 2 * np.pi, n)
        np.testing.assert_array_equal(th[k:k + n], theta)
        np.testing.assert_array_equal(gid[k:k + n], i + 1)
        np.testing.assert_allclose(pts[k:k + n, 0], x * np.cos(theta) + c[0], rtol=0, atol=0)
        k += n
    pl, _, rl, _ = polar_gridpoints((0, 0, 0), "log", rmax=4.0, rmin=0.5, dlnr=0.1)
    assert np.allclose(np.unique(rl[1:]), np.exp(np.linspace(np.log(0.5), np.log(4.0), int(np.log(8.0) / 0.1))))


def test_product_gk15_rule_exact_and_equal_to_oracle(oracle):
    """The adaptive mode's GK15 rule (computed by the library on the host): exact to
    degree 22, Gauss-7 embedded, equal to the oracle's independent construction."""
    from pyglasstools_gb300 import ikabi
    import ctypes as C
    x, wk, wg = np.zeros(8), np.zeros(8), np.zeros(4)
    dp = C.POINTER(C.c_double)
    assert ikabi.lib().ik_gk15_rule(x.ctypes.data_as(dp), wk.ctypes.data_as(dp), wg.ctypes.data_as(dp)) == 0
    xs = np.concatenate([-x[:0:-1], x])
    ws = np.concatenate([wk[:0:-1], wk])
    for k in range(23):
        exact = 2.0 / (k + 1) if k % 2 == 0 else 0.0
        assert abs(np.sum(ws * xs ** k) - exact) < 1e-14
    gx, gw = oracle.gl_rule(7)
    np.testing.assert_allclose(x[[0, 2, 4, 6]], gx[3:], atol=1e-15)
    np.testing.assert_allclose(wg, gw[3:], atol=1e-15)
    ox, owk, owg = oracle.gk15_rule()
    np.testing.assert_allclose(x, ox, rtol=0, atol=2e-16)
    np.testing.assert_allclose(wk, owk, rtol=0, atol=2e-16)


def test_batch_io_argument_checks():
    """IKContext.compute_batch_io checks its arrays before their pointers reach the device
    copies: one frame and one output triple per slot, C-contiguous float64, n x 3 / n."""
    from pyglasstools_gb300.ikabi import check_io_arrays
    n, G = 10, 7
    pos, diam = np.zeros((n, 3)), np.ones(n)
    vel, mass = np.zeros((n, 3)), np.ones(n)
    out = (np.zeros((G, 3)), np.zeros((G, 3)), None)
    check_io_arrays([0], [(pos, diam, vel, mass)], [out])
    check_io_arrays([0, 1], [(pos, diam, None, None)] * 2, [out, (None, None, None)])
    bad = [
        ([0, 1], [(pos, diam, vel, mass)], [out]),                        # count mismatch
        ([0], [(pos.astype(np.float32), diam, vel, mass)], [out]),        # float32
        ([0], [(np.zeros((3, n)).T, diam, vel, mass)], [out]),            # not C-contiguous
        ([0], [(np.zeros((n + 1, 3)), diam, vel, mass)], [out]),          # n mismatch
        ([0], [(pos, diam, np.zeros((n, 2)), mass)], [out]),              # vel shape
        ([0], [(pos, diam, vel, np.ones(n - 1))], [out]),                 # mass shape
        ([0], [(None, diam, vel, mass)], [out]),                          # positions required
        ([0], [(pos, diam.reshape(n, 1), vel, mass)], [out]),             # diam not 1-D
        ([0], [(pos, diam, vel, mass)], [(np.zeros((G, 3), np.float32), None, None)]),
        ([0], [(pos, diam, vel)], [out]),                                 # frame tuple
        ([], [], []),
    ]
    ro = np.zeros((G, 3))
    ro.flags.writeable = False
    bad.append(([0], [(pos, diam, vel, mass)], [(ro, None, None)]))     # read-only output
    for args in bad:
        with pytest.raises(ValueError):
            check_io_arrays(*args)
