"""GPU test of ik_compute_fp64_noalloc, the entry point for callers that cannot call
cudaMalloc (code running where the allocator may not be entered, or whose device
memory belongs to another framework's pool).  The caller owns every input and output
buffer (allocated here with torch, as such a caller's framework would); the entry
point itself allocates nothing and keeps its scratch in a static device array.

Its output must equal the existing plain FP64 entry point's (ik_compute with
IK_PREC_FP64) within the FP64 tolerance of the parity tests (relative L2 <= 1e-12
per component), on two calls in a row with different frames -- the scratch array
keeps the first call's contents, so the second call checks that everything that must
start at zero is cleared.

This file is collected last on purpose; it passes alone in a fresh process and after
the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _noalloc_fn():
    from pyglasstools_gb300 import ikabi
    L = ikabi.lib()
    f = L.ik_compute_fp64_noalloc
    dp, vp, i64, i32, d = C.POINTER(C.c_double), C.c_void_p, C.c_int64, C.c_int, C.c_double
    f.argtypes = [i32, dp, dp, d, dp, d, i32, i32, d, d, i64, vp, vp, vp, vp, i64, vp, vp, vp, vp]
    f.restype = i32
    return f


def _reference_fields(frame, grid, cg):
    from pyglasstools_gb300 import ikabi
    with ikabi.IKContext() as c:
        c.set_box(2, [frame.L, frame.L, 1.0])
        c.set_poly12()
        c.set_cgfunc(cg["kind"], cg["rcut"], order=cg["order"], width=cg["width"])
        c.set_grid(grid)
        c.set_frame(frame.pos, frame.diam, frame.vel, frame.mass)
        c.compute("fp64")
        max_rc = c.get_max_rcut()
        v = c.get_field(ikabi.FIELD_VIRIAL)
        k = c.get_field(ikabi.FIELD_KINETIC)
    uniq = lambda t: np.stack([t[:, 0, 0], t[:, 1, 1], t[:, 0, 1]], axis=1)
    return uniq(v), uniq(k), max_rc


def _rel_l2(a, b):
    return np.sqrt(((a - b) ** 2).sum(0)) / np.sqrt((b ** 2).sum(0))


def test_noalloc_matches_existing_entry_point_two_calls():
    torch = pytest.importorskip("torch")
    from pyglasstools_gb300 import ikabi, synth
    fn = _noalloc_fn()
    cg = dict(kind="gaussian", rcut=6.0, order=5, width=2.0)
    v0, eps, rc = 1.0, 0.2, 1.25
    params = np.array([v0, eps, -28.0 * v0 / rc ** 12, 48.0 * v0 / rc ** 14, -21.0 * v0 / rc ** 16])
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    # two calls in a row: a larger frame first, then a smaller one (the scratch keeps
    # the first call's cell list and bonds)
    for n, seed, nmax in ((4000, 31, 40), (1500, 32, 24)):
        f = synth.make_frame(n, dim=2, seed=seed)
        grid = synth.lattice_grid(f.L, nmax, 2)
        want_v, want_k, max_rc = _reference_fields(f, grid, cg)
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)
        d_pos, d_diam, d_vel, d_mass, d_grid = t(f.pos), t(f.diam), t(f.vel), t(f.mass), t(grid)
        d_vir = torch.full((len(grid), 3), float("nan"), dtype=torch.float64, device=dev)
        d_kin = torch.full((len(grid), 3), float("nan"), dtype=torch.float64, device=dev)
        box = np.array([f.L, f.L, 1.0])
        org = np.zeros(3)
        torch.cuda.synchronize()
        rc_ = fn(2, box.ctypes.data_as(C.POINTER(C.c_double)), org.ctypes.data_as(C.POINTER(C.c_double)),
                 1.25, params.ctypes.data_as(C.POINTER(C.c_double)), max_rc, ikabi.CG[cg["kind"]], cg["order"],
                 cg["rcut"], cg["width"], n, d_pos.data_ptr(), d_diam.data_ptr(), d_vel.data_ptr(),
                 d_mass.data_ptr(), len(grid), d_grid.data_ptr(), d_vir.data_ptr(), d_kin.data_ptr(),
                 stream.cuda_stream)
        if rc_ != 0:
            raise AssertionError(ikabi.lib().ik_last_error().decode())
        got_v = d_vir.cpu().numpy()
        got_k = d_kin.cpu().numpy()
        assert np.all(np.isfinite(got_v)) and np.all(np.isfinite(got_k))
        assert np.all(_rel_l2(got_v, want_v) <= FP64_TOL), _rel_l2(got_v, want_v)
        assert np.all(_rel_l2(got_k, want_k) <= FP64_TOL), _rel_l2(got_k, want_k)


def test_noalloc_rejects_sizes_beyond_its_maximum():
    torch = pytest.importorskip("torch")
    from pyglasstools_gb300 import ikabi
    fn = _noalloc_fn()
    box = np.array([100.0, 100.0, 1.0])
    params = np.array([1.0, 0.2, -1.0, 1.0, -1.0])
    d = torch.zeros((5000, 3), dtype=torch.float64, device="cuda")
    rc_ = fn(2, box.ctypes.data_as(C.POINTER(C.c_double)), None, 1.25, params.ctypes.data_as(C.POINTER(C.c_double)),
             2.0, 0, 5, 2.0, 0.0, 5000, d.data_ptr(), d.data_ptr(), None, None, 1, d.data_ptr(), d.data_ptr(),
             None, None)
    assert rc_ == -5  # IK_ERR_CAPACITY
    assert b"exceeds the maximum of 4096" in ikabi.lib().ik_last_error()
