"""GPU tests of ik_compute_fp64_noalloc, the entry point for callers that cannot call
cudaMalloc: a process whose device memory belongs to another framework's pool, a
service under a memory budget fixed at start-up, or code that must not enter the
allocator because it can wait for other streams' work.  The caller owns every input
and output buffer (allocated here with torch, as such a caller's framework would); the
entry point itself allocates nothing and keeps its scratch in a static device array.

Its output must equal the existing plain FP64 entry point's (ik_compute with
IK_PREC_FP64) within the FP64 tolerance of the parity tests (relative L2 <= 1e-12
per component), on two calls in a row with different frames -- the scratch array
keeps the first call's contents, so the second call checks that everything that must
start at zero is cleared.  Cases: 2D Gaussian, 3D octic, 2D mollifier, and a sparse
frame in a box large enough that the entry point widens its cells to stay within its
cell-list maximum.  Errors found on the device (a non-finite position, a particle
with more bonds than the scratch holds) come back as status codes.

This file is collected last on purpose; it passes alone in a fresh process and after
the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
IK_ERR_ARG, IK_ERR_CAPACITY = -1, -5
V0, EPS, RC = 1.0, 0.2, 1.25
PARAMS = np.array([V0, EPS, -28.0 * V0 / RC ** 12, 48.0 * V0 / RC ** 14, -21.0 * V0 / RC ** 16])


def _noalloc_fn():
    from pyglasstools_gb300 import ikabi
    L = ikabi.lib()
    f = L.ik_compute_fp64_noalloc
    dp, vp, i64, i32, d = C.POINTER(C.c_double), C.c_void_p, C.c_int64, C.c_int, C.c_double
    f.argtypes = [i32, dp, dp, d, dp, d, i32, i32, d, d, i64, vp, vp, vp, vp, i64, vp, vp, vp, vp]
    f.restype = i32
    return f


def _uniq(t):
    if t.shape[1] == 2:
        return np.stack([t[:, 0, 0], t[:, 1, 1], t[:, 0, 1]], axis=1)
    return np.stack([t[:, 0, 0], t[:, 1, 1], t[:, 2, 2], t[:, 0, 1], t[:, 0, 2], t[:, 1, 2]], axis=1)


def _reference_fields(dim, box, pos, diam, vel, mass, grid, cg):
    """The existing entry point: a context, ik_compute(IK_PREC_FP64)."""
    from pyglasstools_gb300 import ikabi
    with ikabi.IKContext() as c:
        c.set_box(dim, list(box))
        c.set_poly12(V0, EPS, RC)
        c.set_cgfunc(cg["kind"], cg["rcut"], order=cg["order"], width=cg["width"])
        c.set_grid(grid)
        c.set_frame(pos, diam, vel, mass)
        c.compute("fp64")
        max_rc = c.get_max_rcut()
        v = c.get_field(ikabi.FIELD_VIRIAL)
        k = c.get_field(ikabi.FIELD_KINETIC)
    return _uniq(v), _uniq(k), max_rc


def _rel_l2(a, b):
    return np.sqrt(((a - b) ** 2).sum(0)) / np.sqrt((b ** 2).sum(0))


def _call(fn, torch, dim, box, pos, diam, vel, mass, grid, cg, max_rc, nc):
    """One call of the no-allocation entry point on torch-owned device buffers; returns
    (status, virial, kinetic) with the outputs prefilled with NaN."""
    from pyglasstools_gb300 import ikabi
    dev = torch.device("cuda", 0)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)
    d_pos, d_diam, d_vel, d_mass, d_grid = t(pos), t(diam), t(vel), t(mass), t(grid)
    d_vir = torch.full((len(grid), nc), float("nan"), dtype=torch.float64, device=dev)
    d_kin = torch.full((len(grid), nc), float("nan"), dtype=torch.float64, device=dev)
    bx = np.asarray(box, dtype=np.float64)
    org = np.zeros(3)
    dptr = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev)
    rc_ = fn(dim, dptr(bx), dptr(org), RC, dptr(PARAMS), max_rc, ikabi.CG[cg["kind"]], cg["order"], cg["rcut"],
             cg["width"], len(pos), d_pos.data_ptr(), d_diam.data_ptr(), d_vel.data_ptr(), d_mass.data_ptr(),
             len(grid), d_grid.data_ptr(), d_vir.data_ptr(), d_kin.data_ptr(), stream.cuda_stream)
    return rc_, d_vir.cpu().numpy(), d_kin.cpu().numpy()


GAUSS = dict(kind="gaussian", rcut=6.0, order=5, width=2.0)
OCTIC = dict(kind="octic", rcut=2.0, order=5, width=0.0)
MOLLI = dict(kind="mollifier", rcut=2.0, order=5, width=0.0)


def _frames(case):
    """Two frames per case (a larger one first, then a smaller one): (dim, box, frame, grid)."""
    from pyglasstools_gb300 import synth
    out = []
    if case == "2d_gaussian":
        for n, seed, nmax in ((4000, 31, 40), (1500, 32, 24)):
            f = synth.make_frame(n, dim=2, seed=seed)
            out.append((2, [f.L, f.L, 1.0], f, synth.lattice_grid(f.L, nmax, 2), GAUSS))
    elif case == "3d_octic":
        for n, seed, nmax in ((4000, 41, 12), (2500, 42, 10)):
            f = synth.make_frame(n, dim=3, seed=seed)
            out.append((3, [f.L] * 3, f, synth.lattice_grid(f.L, nmax, 3), OCTIC))
    elif case == "2d_mollifier":
        for n, seed, nmax in ((3000, 51, 30), (2000, 52, 20)):
            f = synth.make_frame(n, dim=2, seed=seed)
            out.append((2, [f.L, f.L, 1.0], f, synth.lattice_grid(f.L, nmax, 2), MOLLI))
    elif case == "2d_wide_cells":
        # dense patches in a box of 300: floor(300 / max_rcut)^2 cells exceed the
        # entry point's cell-list maximum, so it widens its cells
        for n, seed, nmax in ((4000, 61, 120), (3000, 62, 100)):
            f = synth.make_frame(n, dim=2, seed=seed)
            out.append((2, [300.0, 300.0, 1.0], f, synth.lattice_grid(300.0, nmax, 2), OCTIC))
    return out


@pytest.mark.parametrize("case", ["2d_gaussian", "3d_octic", "2d_mollifier", "2d_wide_cells"])
def test_noalloc_matches_existing_entry_point_two_calls(case):
    torch = pytest.importorskip("torch")
    from pyglasstools_gb300 import ikabi
    fn = _noalloc_fn()
    # two calls in a row: the scratch keeps the first call's cell list and bonds
    for dim, box, f, grid, cg in _frames(case):
        nc = 3 if dim == 2 else 6
        want_v, want_k, max_rc = _reference_fields(dim, box, f.pos, f.diam, f.vel, f.mass, grid, cg)
        rc_, got_v, got_k = _call(fn, torch, dim, box, f.pos, f.diam, f.vel, f.mass, grid, cg, max_rc, nc)
        if rc_ != 0:
            raise AssertionError(ikabi.lib().ik_last_error().decode())
        assert np.all(np.isfinite(got_v)) and np.all(np.isfinite(got_k))
        assert np.any(want_v != 0.0)
        assert np.all(_rel_l2(got_v, want_v) <= FP64_TOL), (case, _rel_l2(got_v, want_v))
        assert np.all(_rel_l2(got_k, want_k) <= FP64_TOL), (case, _rel_l2(got_k, want_k))


def test_noalloc_reports_errors_found_on_the_device():
    torch = pytest.importorskip("torch")
    from pyglasstools_gb300 import ikabi, synth
    fn = _noalloc_fn()
    f = synth.make_frame(1000, dim=2, seed=71)
    grid = synth.lattice_grid(f.L, 16, 2)
    box = [f.L, f.L, 1.0]
    # a non-finite position
    pos = f.pos.copy()
    pos[17, 0] = np.nan
    rc_, _, _ = _call(fn, torch, 2, box, pos, f.diam, f.vel, f.mass, grid, GAUSS, 2.025, 3)
    assert rc_ == IK_ERR_ARG, rc_
    assert b"not finite" in ikabi.lib().ik_last_error()
    # forty particles within 0.3 of each other: 39 force-active bonds each, above the 32
    # that the scratch holds per particle
    rng = np.random.default_rng(72)
    cl = np.zeros((40, 3))
    cl[:, :2] = rng.uniform(-0.15, 0.15, size=(40, 2))
    d = np.ones(40)
    rc_, _, _ = _call(fn, torch, 2, [20.0, 20.0, 1.0], cl, d, np.zeros((40, 3)), d, synth.lattice_grid(20.0, 8, 2),
                      OCTIC, 1.25, 3)
    assert rc_ == IK_ERR_CAPACITY, rc_
    assert b"more than 32" in ikabi.lib().ik_last_error()
    # and the next call computes normally again
    want_v, want_k, max_rc = _reference_fields(2, box, f.pos, f.diam, f.vel, f.mass, grid, GAUSS)
    rc_, got_v, got_k = _call(fn, torch, 2, box, f.pos, f.diam, f.vel, f.mass, grid, GAUSS, max_rc, 3)
    assert rc_ == 0
    assert np.all(_rel_l2(got_v, want_v) <= FP64_TOL) and np.all(_rel_l2(got_k, want_k) <= FP64_TOL)


def test_noalloc_rejects_sizes_beyond_its_maximum():
    torch = pytest.importorskip("torch")
    from pyglasstools_gb300 import ikabi
    fn = _noalloc_fn()
    box = np.array([100.0, 100.0, 1.0])
    d = torch.zeros((5000, 3), dtype=torch.float64, device="cuda")
    rc_ = fn(2, box.ctypes.data_as(C.POINTER(C.c_double)), None, 1.25, PARAMS.ctypes.data_as(C.POINTER(C.c_double)),
             2.0, 0, 5, 2.0, 0.0, 5000, d.data_ptr(), d.data_ptr(), None, None, 1, d.data_ptr(), d.data_ptr(),
             None, None)
    assert rc_ == IK_ERR_CAPACITY
    assert b"exceeds the maximum of 4096" in ikabi.lib().ik_last_error()
