"""GPU parity at the full measured workloads: the CUDA path (through the C ABI) against
the FP64 CPU oracle on the same seeded frames, at the sizes the benchmark runs.

  * 2D, N = 64 000, a 256 x 256 lattice grid, Gaussian kernel of width 2 cut at 3
    widths, Gauss-Legendre-5: neighbour lists bit-exact; plain FP64 and tuned FP32
    (plain and Kahan-compensated per-lane sums) fields;
  * 3D, N = 32 000, a 64^3 grid, octic kernel R = 2: both precisions;
  * uneven batch: six frames of the uneven recipe (N from 1000 to 128 000, each with
    its own box and a grid of spacing ~1) computed as one batch (ik_compute_batch)
    on both paths.

Tolerances (the same as the small-size parity tests): neighbour lists bit-exact;
plain FP64 relative L2 per stress component <= 1e-12; tuned FP32 relative L2 per
component <= 1e-5 and max |error| / max |T| <= 1e-4.  The oracle restates
IrvingKirkwood::compute (irvingkirkwood/IrvingKirkwood.h:74-110) in FP64 and runs on
every host core (about a second per frame here).
"""
import numpy as np
import pytest

from conftest import rel_l2, uniq

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-5
FP32_MAX_TOL = 1e-4
GAUSS = dict(kind="gaussian", rcut=6.0, order=5, width=2.0)
OCTIC = dict(kind="octic", rcut=2.0, order=5, width=0.0)


def _check(got, want, tol, maxtol, what):
    g, w = uniq(got), uniq(want)
    err = rel_l2(g, w)
    assert np.all(err <= tol), f"{what}: rel L2 per component {err} > {tol}"
    if maxtol is not None:
        m = np.max(np.abs(g - w), axis=0) / np.maximum(np.max(np.abs(w), axis=0), 1e-300)
        assert np.all(m <= maxtol), f"{what}: max-abs/max {m} > {maxtol}"
    return float(err.max())


def _oracle(oracle, dim, L, f, grid, cg, max_rc=None):
    box = oracle.make_box(dim, [L, L, L if dim == 3 else 1.0])
    c = oracle.make_cg(cg["kind"], rcut=cg["rcut"], mode="fixedpoint", order=cg["order"], width=cg["width"])
    return oracle.compute(box, f.pos, f.diam, oracle.make_poly12(), c, grid, vel=f.vel, mass=f.mass, max_rc=max_rc)


def _context(ik, dim, L, grid, cg):
    c = ik.IKContext()
    c.set_box(dim, [L, L, L if dim == 3 else 1.0])
    c.set_poly12()
    c.set_cgfunc(cg["kind"], cg["rcut"], order=cg["order"], width=cg["width"])
    c.set_grid(grid)
    return c


@pytest.fixture(scope="module")
def frame2d():
    from pyglasstools_gb300 import synth
    f = synth.make_frame(64000, dim=2, seed=0)
    return f, synth.lattice_grid(f.L, 256, 2)


def test_headline_2d_n64k_neighbours_bitexact(frame2d, oracle):
    from pyglasstools_gb300 import ikabi as ik
    f, grid = frame2d
    box = oracle.make_box(2, [f.L, f.L, 1.0])
    with _context(ik, 2, f.L, grid, GAUSS) as c:
        c.set_frame(f.pos, f.diam, f.vel, f.mass)
        rc = c.get_max_rcut()
        assert rc == oracle.max_rcut(1.25, f.diam)
        for radius in (rc, 2.5):
            o_off, o_idx = oracle.neighbors(box, f.pos, radius)
            g_off, g_idx = c.neighbors(radius, n=len(f.pos))
            assert np.array_equal(o_off, g_off) and np.array_equal(o_idx, g_idx), radius


def test_headline_2d_n64k_g256_gauss_both_paths(frame2d, oracle):
    from pyglasstools_gb300 import ikabi as ik
    f, grid = frame2d
    ov, ok = _oracle(oracle, 2, f.L, f, grid, GAUSS)
    with _context(ik, 2, f.L, grid, GAUSS) as c:
        c.set_frame(f.pos, f.diam, f.vel, f.mass)
        c.compute("fp64")
        _check(c.get_field(ik.FIELD_VIRIAL), ov, FP64_TOL, None, "fp64 virial")
        _check(c.get_field(ik.FIELD_KINETIC), ok, FP64_TOL, None, "fp64 kinetic")
        for flags in (0, ik.FLAG_LANE_KAHAN):
            c.set_flags(flags)
            c.compute("fp32")
            _check(c.get_field(ik.FIELD_VIRIAL), ov, FP32_TOL, FP32_MAX_TOL, f"fp32 virial flags={flags}")
            _check(c.get_field(ik.FIELD_KINETIC), ok, FP32_TOL, FP32_MAX_TOL, f"fp32 kinetic flags={flags}")
            cnt = c.counters()
            # force-active (grid, i, j) triples of this workload: ~2.8e7 per frame
            assert 2.0e7 < cnt[2] < 3.6e7, cnt


def test_3d_n32k_g64_octic_both_paths(oracle):
    from pyglasstools_gb300 import ikabi as ik, synth
    f = synth.make_frame(32000, dim=3, seed=0)
    grid = synth.lattice_grid(f.L, 64, 3)
    ov, ok = _oracle(oracle, 3, f.L, f, grid, OCTIC)
    with _context(ik, 3, f.L, grid, OCTIC) as c:
        c.set_frame(f.pos, f.diam, f.vel, f.mass)
        c.compute("fp64")
        _check(c.get_field(ik.FIELD_VIRIAL), ov, FP64_TOL, None, "3d fp64 virial")
        _check(c.get_field(ik.FIELD_KINETIC), ok, FP64_TOL, None, "3d fp64 kinetic")
        for flags in (0, ik.FLAG_LANE_KAHAN):
            c.set_flags(flags)
            c.compute("fp32")
            _check(c.get_field(ik.FIELD_VIRIAL), ov, FP32_TOL, FP32_MAX_TOL, f"3d fp32 virial flags={flags}")
            _check(c.get_field(ik.FIELD_KINETIC), ok, FP32_TOL, FP32_MAX_TOL, f"3d fp32 kinetic flags={flags}")


def test_uneven_batch_six_frames_vs_oracle(oracle):
    """Frames of the uneven recipe (density 1, T = 0.3, own box, grid spacing ~1,
    Gaussian w = 2 cut at 6), N from ~1000 to ~128 000, as one batch on each path."""
    from pyglasstools_gb300 import ikabi as ik, synth
    Ns = [1000, 2900, 8500, 24000, 64000, 128000]
    frames = [synth.make_frame(n, dim=2, seed=7000 + k) for k, n in enumerate(Ns)]
    grids = [synth.lattice_grid(f.L, max(int(f.L), 2), 2) for f in frames]
    max_rc = 1.25 * 1.62  # the largest diameter the recipe draws, frozen for the batch
    c = ik.IKContext()
    try:
        c.set_poly12()
        c.set_cgfunc("gaussian", 6.0, order=5, width=2.0)
        c.reserve_slots(len(Ns))
        c.set_max_rcut(max_rc)
        for k, (f, g) in enumerate(zip(frames, grids)):
            c.set_slot_geometry(k, 2, [f.L, f.L, 1.0], g)
            c.upload_frame(k, f.pos, f.diam, f.vel, f.mass)
        slots = list(range(len(Ns)))[::-1]  # largest first, as a scheduler would
        want = [_oracle(oracle, 2, f.L, f, g, GAUSS, max_rc=max_rc) for f, g in zip(frames, grids)]
        for prec, tol, mtol in (("fp64", FP64_TOL, None), ("fp32", FP32_TOL, FP32_MAX_TOL)):
            for rep in range(2):  # first call (recording) and the graph replay
                c.compute_batch(slots, prec)
                c.synchronize()
                for k in range(len(Ns)):
                    ov, ok = want[k]
                    _check(c.get_field(ik.FIELD_VIRIAL, slot=k), ov, tol, mtol, f"{prec} virial N={Ns[k]} rep={rep}")
                    _check(c.get_field(ik.FIELD_KINETIC, slot=k), ok, tol, mtol, f"{prec} kinetic N={Ns[k]} rep={rep}")
    finally:
        c.close()
