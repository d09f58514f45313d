"""GPU tests of resident multi-frame work: frames kept in slots, computed one slot at a
time (ik_compute_slot) or as one batch (ik_compute_batch, replayed as a CUDA graph
after its first call).  The batch must give bit-identical fields to the per-slot
path -- the same kernels on the same inputs -- and must follow every change that
stales a recorded graph: new frame contents, a frame of another size, new
coarse-graining settings.  One slot is also checked against the FP64 oracle at the
FP32 tolerance.
"""
import numpy as np
import pytest

from conftest import rel_l2, uniq

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5
CG = dict(kind="gaussian", rcut=6.0, order=5, width=2.0)


def _frames(n, seeds):
    from pyglasstools_gb300 import synth
    return [synth.make_frame(n, dim=2, seed=s) for s in seeds]


def _context(ik, L, grid, nslots, cg=CG):
    c = ik.IKContext()
    c.set_box(2, [L, L, 1.0])
    c.set_poly12()
    c.set_cgfunc(cg["kind"], cg["rcut"], order=cg["order"], width=cg["width"])
    c.set_grid(grid)
    c.reserve_slots(nslots)
    return c


def _fields(ik, c, slots):
    return [(c.get_field(ik.FIELD_VIRIAL, slot=k), c.get_field(ik.FIELD_KINETIC, slot=k)) for k in slots]


def _upload(c, frames, slots=None):
    for k, f in zip(slots or range(len(frames)), frames):
        c.upload_frame(k, f.pos, f.diam, f.vel, f.mass)


def _per_slot(ik, c, slots, prec):
    for k in slots:
        c.compute_slot(k, prec)
    c.synchronize()
    return _fields(ik, c, slots)


def _batch(ik, c, slots, prec):
    c.compute_batch(slots, prec)
    c.synchronize()
    return _fields(ik, c, slots)


def _same(a, b):
    for (va, ka), (vb, kb) in zip(a, b):
        np.testing.assert_array_equal(va, vb)
        np.testing.assert_array_equal(ka, kb)


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_batch_replay_matches_per_slot(prec):
    from pyglasstools_gb300 import ikabi as ik, synth
    F, n = 6, 3000
    fr = _frames(n, range(100, 100 + F))
    L = fr[0].L
    grid = synth.lattice_grid(L, 40, 2)
    c = _context(ik, L, grid, F)
    _upload(c, fr)
    slots = list(range(F))
    want = _per_slot(ik, c, slots, prec)
    l0 = c.launch_count()
    got = _batch(ik, c, slots, prec)  # first call: plain launches + graph recording
    _same(got, want)
    assert c.launch_count() > l0
    got = _batch(ik, c, slots, prec)  # replay of the recorded graph
    _same(got, want)
    # new frame contents of the same size: the replay recomputes them
    fr2 = _frames(n, range(200, 200 + F))
    _upload(c, fr2)
    got = _batch(ik, c, slots, prec)
    want2 = _per_slot(ik, c, slots, prec)
    _same(got, want2)
    assert not np.array_equal(want2[0][0], want[0][0])
    c.close()


def test_batch_follows_size_and_setting_changes(oracle):
    from pyglasstools_gb300 import ikabi as ik, synth
    F, n = 4, 2500
    fr = _frames(n, range(300, 300 + F))
    L = fr[0].L
    grid = synth.lattice_grid(L, 32, 2)
    c = _context(ik, L, grid, F)
    _upload(c, fr)
    h = n // 2  # slot 1 starts with half of its frame's particles
    c.upload_frame(1, fr[1].pos[:h], fr[1].diam[:h], fr[1].vel[:h], fr[1].mass[:h])
    slots = [3, 1, 2, 0]  # any order of slots
    _batch(ik, c, slots, "fp32")
    _batch(ik, c, slots, "fp32")
    # a frame of another size in one slot (its buffers grow)
    big = fr[1]
    c.upload_frame(1, big.pos, big.diam, big.vel, big.mass)
    got = _batch(ik, c, slots, "fp32")
    want = _per_slot(ik, c, slots, "fp32")
    _same(got, want)
    # new coarse-graining width: the recorded graph holds the old one
    cg2 = dict(CG, width=1.5)
    c.set_cgfunc(cg2["kind"], cg2["rcut"], order=cg2["order"], width=cg2["width"])
    got = _batch(ik, c, slots, "fp32")
    want = _per_slot(ik, c, slots, "fp32")
    _same(got, want)
    # and the batch result of the resized slot against the FP64 oracle
    box = oracle.make_box(2, [L, L, 1.0])
    p = oracle.make_poly12(1.0, 0.2, 1.25)
    cgo = oracle.make_cg(cg2["kind"], rcut=cg2["rcut"], mode="fixedpoint", order=cg2["order"], width=cg2["width"])
    sub = grid[::7]
    ov, ok = oracle.compute(box, big.pos, big.diam, p, cgo, sub, vel=big.vel, mass=big.mass,
                            max_rc=c.get_max_rcut())
    gv, gk = got[slots.index(1)]
    assert np.all(rel_l2(uniq(gv[::7]), uniq(ov)) <= FP32_TOL)
    assert np.all(rel_l2(uniq(gk[::7]), uniq(ok)) <= FP32_TOL)
    c.close()


def test_batch_argument_errors():
    from pyglasstools_gb300 import ikabi as ik, synth
    fr = _frames(500, [7])
    L = fr[0].L
    c = _context(ik, L, synth.lattice_grid(L, 8, 2), 2)
    _upload(c, fr)
    with pytest.raises(ik.IKError):
        c.compute_batch([0, 5], "fp32")
    with pytest.raises(ik.IKError):
        c.compute_batch([], "fp32")
    c.compute_batch([0], "fp32")
    c.synchronize()
    c.close()


def test_autotuner_picks_a_candidate_and_keeps_results():
    """The autotuner times each candidate bin size x CTAs per SM on the batch and keeps
    the fastest; results under every tuning agree within the FP32 tolerance."""
    from pyglasstools_gb300 import ikabi as ik, synth
    F, n = 4, 6000
    fr = _frames(n, range(500, 500 + F))
    L = fr[0].L
    grid = synth.lattice_grid(L, 60, 2)
    c = _context(ik, L, grid, F)
    _upload(c, fr)
    slots = list(range(F))
    before = _batch(ik, c, slots, "fp32")
    best = c.autotune_batch(slots, "fp32", reps=2)
    assert best["bin_points"] in (12, 16, 20, 25, 36) and best["blocks_per_sm"] in (1, 2)
    assert best["ms_per_batch"] > 0
    assert c.get_tuning("bin_points") == best["bin_points"]
    after = _batch(ik, c, slots, "fp32")
    for (va, ka), (vb, kb) in zip(after, before):
        assert np.all(rel_l2(uniq(va), uniq(vb)) <= FP32_TOL)
        assert np.all(rel_l2(uniq(ka), uniq(kb)) <= FP32_TOL)
    c.close()


def test_uneven_batch_with_per_slot_geometry():
    """Frames of different sizes (their own boxes and grids of spacing 1) in one context,
    one CUDA-graph batch: each slot's fields equal those of a context set up for that
    frame alone, bit for bit (the same kernels on the same inputs)."""
    from pyglasstools_gb300 import ikabi as ik, synth
    sizes = [1000, 5200, 2300, 12000, 1700]
    fr = [synth.make_frame(n, dim=2, seed=700 + k) for k, n in enumerate(sizes)]
    grids = [synth.lattice_grid(f.L, int(f.L), 2) for f in fr]
    c = ik.IKContext()
    c.set_poly12()
    c.set_cgfunc("gaussian", 6.0, order=5, width=2.0)
    c.reserve_slots(len(fr))
    c.set_max_rcut(1.25 * 1.62)
    for k, (f, g) in enumerate(zip(fr, grids)):
        c.set_slot_geometry(k, 2, [f.L, f.L, 1.0], g)
        c.upload_frame(k, f.pos, f.diam, f.vel, f.mass)
    slots = list(range(len(fr)))
    for prec in ("fp32", "fp64"):
        got = _batch(ik, c, slots, prec)
        got2 = _batch(ik, c, slots, prec)  # graph replay
        for k, (f, g) in enumerate(zip(fr, grids)):
            with ik.IKContext() as one:
                one.set_box(2, [f.L, f.L, 1.0])
                one.set_poly12()
                one.set_cgfunc("gaussian", 6.0, order=5, width=2.0)
                one.set_max_rcut(1.25 * 1.62)
                one.set_grid(g)
                one.set_frame(f.pos, f.diam, f.vel, f.mass)
                one.compute(prec)
                want = (one.get_field(ik.FIELD_VIRIAL), one.get_field(ik.FIELD_KINETIC))
            assert got[k][0].shape == (len(g), 2, 2)
            np.testing.assert_array_equal(got[k][0], want[0])
            np.testing.assert_array_equal(got[k][1], want[1])
            np.testing.assert_array_equal(got2[k][0], want[0])
    c.close()


def test_float32_upload_equals_float64_upload():
    """ik_upload_frame_f32 (GSD float32 chunks widened on the GPU) gives the same device
    data -- and bit-identical fields -- as uploading the same values in FP64."""
    from pyglasstools_gb300 import ikabi as ik, synth
    f = synth.make_frame(3000, dim=2, seed=901)
    p32, d32 = f.pos.astype(np.float32), f.diam.astype(np.float32)
    v32, m32 = f.vel.astype(np.float32), f.mass.astype(np.float32)
    grid = synth.lattice_grid(f.L, 40, 2)
    c = _context(ik, f.L, grid, 2)
    c.upload_frame(0, p32.astype(np.float64), d32.astype(np.float64), v32.astype(np.float64), m32.astype(np.float64))
    c.upload_frame_f32(1, p32, d32, v32, m32)
    for prec in ("fp32", "fp64"):
        a, b = _per_slot(ik, c, [0, 1], prec)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
    c.close()


def test_async_download_is_not_overwritten_by_the_next_computation():
    """ik_download_field_async copies on its own stream; the slot's next computation
    waits for it, so a result being downloaded is never overwritten."""
    torch = pytest.importorskip("torch")
    from pyglasstools_gb300 import ikabi as ik, synth
    fr = _frames(6000, [911, 912])
    L = fr[0].L
    grid = synth.lattice_grid(L, 64, 2)
    c = _context(ik, L, grid, 1)
    want = []
    for f in fr:
        c.upload_frame(0, f.pos, f.diam, f.vel, f.mass)
        c.compute_slot(0, "fp32")
        c.synchronize()
        want.append(uniq(c.get_field(ik.FIELD_VIRIAL)))
    pinned = [torch.empty((len(grid), 3), dtype=torch.float64, pin_memory=True).numpy() for _ in fr]
    for k, f in enumerate(fr):  # no synchronisation between the frames
        c.upload_frame(0, f.pos, f.diam, f.vel, f.mass)
        c.compute_slot(0, "fp32")
        c.download_field_async(pinned[k], ik.FIELD_VIRIAL, 0)
    c.synchronize()
    for k in range(len(fr)):
        np.testing.assert_array_equal(pinned[k], want[k])
    c.close()


def test_batch_with_host_io_matches_per_slot():
    """ik_compute_batch_io: page-locked host frames in, host fields out, one graph; the
    first call (plain path) and the replays give the per-slot results bit for bit, and a
    replay reads the host inputs' new contents."""
    torch = pytest.importorskip("torch")
    from pyglasstools_gb300 import ikabi as ik, synth
    F, n = 5, 2500
    fr = _frames(n, range(600, 600 + F))
    L = fr[0].L
    grid = synth.lattice_grid(L, 36, 2)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    host = [(pin(f.pos), pin(f.diam), pin(f.vel), pin(f.mass)) for f in fr]
    outs = [(pin(np.zeros((len(grid), 3))), pin(np.zeros((len(grid), 3))), None) for _ in fr]
    c = _context(ik, L, grid, F)
    slots = list(range(F))

    def want_for(frames):
        ref = _context(ik, L, grid, F)
        _upload(ref, frames)
        res = [(uniq(v), uniq(k)) for v, k in _per_slot(ik, ref, slots, "fp32")]
        ref.close()
        return res

    want = want_for(fr)
    for rep in range(3):  # plain + recording, then replays
        c.compute_batch_io(slots, host, outs)
        c.synchronize()
        for k in slots:
            np.testing.assert_array_equal(outs[k][0], want[k][0])
            np.testing.assert_array_equal(outs[k][1], want[k][1])
    fr2 = _frames(n, range(700, 700 + F))
    for k, f in enumerate(fr2):  # same pointers, new contents
        host[k][0][:] = f.pos
        host[k][1][:] = f.diam
        host[k][2][:] = f.vel
        host[k][3][:] = f.mass
    c.compute_batch_io(slots, host, outs)
    c.synchronize()
    want2 = want_for(fr2)
    for k in slots:
        np.testing.assert_array_equal(outs[k][0], want2[k][0])
        np.testing.assert_array_equal(outs[k][1], want2[k][1])
    # pageable host memory is refused
    with pytest.raises(ik.IKError):
        c.compute_batch_io([0], [(fr[0].pos.copy(), fr[0].diam.copy(), None, None)], [(outs[0][0], None, None)])
    c.close()


def test_batch_with_host_io_fp64_and_partial_outputs():
    """The host-I/O batch on the FP64 path, frames without velocities, only the virial
    downloaded: equal to the per-slot results."""
    torch = pytest.importorskip("torch")
    from pyglasstools_gb300 import ikabi as ik, synth
    F, n = 3, 1500
    fr = _frames(n, range(800, 800 + F))
    L = fr[0].L
    grid = synth.lattice_grid(L, 24, 2)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    host = [(pin(f.pos), pin(f.diam), None, None) for f in fr]
    outs = [(pin(np.zeros((len(grid), 3))), None, None) for _ in fr]
    c = _context(ik, L, grid, F)
    slots = [2, 0, 1]
    for rep in range(2):
        c.compute_batch_io(slots, [host[k] for k in slots], [outs[k] for k in slots], precision="fp64",
                           fields=ik.FIELD_VIRIAL)
        c.synchronize()
    ref = _context(ik, L, grid, F)
    for k, f in enumerate(fr):
        ref.upload_frame(k, f.pos, f.diam)
    for k in range(F):
        ref.compute_slot(k, "fp64", ik.FIELD_VIRIAL)
    ref.synchronize()
    for k in range(F):
        np.testing.assert_array_equal(outs[k][0], uniq(ref.get_field(ik.FIELD_VIRIAL, slot=k)))
    ref.close()
    c.close()


def test_batch_with_host_io_refetches_fields_after_capacity_growth():
    """A replay whose new frame contents overflow the bond capacity: ik_synchronize re-runs
    the frame on the plain path with a larger capacity and copies its fields to the host
    again, so the host outputs equal the per-slot results."""
    torch = pytest.importorskip("torch")
    from pyglasstools_gb300 import ikabi as ik, synth
    F, n = 2, 2000
    fr = _frames(n, range(900, 900 + F))
    L = fr[0].L
    grid = synth.lattice_grid(L, 24, 2)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    host = [(pin(f.pos), pin(f.diam), pin(f.vel), pin(f.mass)) for f in fr]
    outs = [(pin(np.zeros((len(grid), 3))), pin(np.zeros((len(grid), 3))), None) for _ in fr]
    c = _context(ik, L, grid, F)
    c.set_max_rcut(1.25 * 1.62)
    slots = list(range(F))
    for _ in range(2):  # plain + recording, then a replay
        c.compute_batch_io(slots, host, outs)
        c.synchronize()
    # squeeze frame 1 towards the box centre: many more force-active bonds per particle
    dense = fr[1].pos.copy()
    dense[:, :2] *= 0.55
    host[1][0][:] = dense
    c.compute_batch_io(slots, host, outs)
    c.synchronize()
    ref = _context(ik, L, grid, F)
    ref.set_max_rcut(1.25 * 1.62)
    ref.upload_frame(0, fr[0].pos, fr[0].diam, fr[0].vel, fr[0].mass)
    ref.upload_frame(1, dense, fr[1].diam, fr[1].vel, fr[1].mass)
    want = [(uniq(v), uniq(k)) for v, k in _per_slot(ik, ref, slots, "fp32")]
    for k in slots:
        np.testing.assert_array_equal(outs[k][0], want[k][0])
        np.testing.assert_array_equal(outs[k][1], want[k][1])
    ref.close()
    c.close()
