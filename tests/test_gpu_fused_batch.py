"""GPU tests of fused batches: ik_compute_batch running every stage once over all frames
of a batch (bin, scan, scatter, sort + pack, bonds, one persistent gather over every
frame's work items, finish), recorded as one CUDA graph.

A fused batch must give the fields of the per-frame path bit for bit -- the same
arithmetic per particle, cell, bond and grid point -- for frames of different sizes with
their own boxes and grids, empty frames and frames without velocities, in 2D and 3D, with
plain or Kahan-compensated lane sums, for every coarse-graining kernel, and after a
replay whose new contents overflow the bond capacity (re-run on the per-frame path).
Its launch count per batch is at most ten kernels whatever the number of frames.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = (1, 2)  # virial, kinetic


def _ctx(ik, cg=("gaussian", 6.0, 2.0), max_rc=1.25 * 1.62):
    c = ik.IKContext()
    c.set_poly12()
    c.set_cgfunc(cg[0], cg[1], order=5, width=cg[2])
    c.set_max_rcut(max_rc)
    return c


def _alone(ik, dim, f, grid, cg=("gaussian", 6.0, 2.0), flags=0, max_rc=1.25 * 1.62):
    """The fields of one frame in a context of its own (per-frame path)."""
    with ik.IKContext() as one:
        one.set_flags(flags)
        one.set_box(dim, [f.L, f.L, f.L if dim == 3 else 1.0])
        one.set_poly12()
        one.set_cgfunc(cg[0], cg[1], order=5, width=cg[2])
        one.set_max_rcut(max_rc)
        one.set_grid(grid)
        one.set_frame(f.pos, f.diam, f.vel, f.mass)
        one.compute("fp32")
        return [one.get_field(fl) for fl in FIELDS], one.counters()


def _fields(ik, c, slots):
    return [[c.get_field(fl, slot=k) for fl in FIELDS] for k in slots]


def _uneven(dim, sizes, seed0):
    from pyglasstools_gb300 import synth
    fr = [synth.make_frame(n, dim=dim, seed=seed0 + k) for k, n in enumerate(sizes)]
    grids = [synth.lattice_grid(f.L, max(int(f.L) if dim == 2 else int(f.L / 2), 2), dim) for f in fr]
    return fr, grids


def _setup(ik, c, dim, fr, grids, no_vel=()):
    c.reserve_slots(len(fr))
    for k, (f, g) in enumerate(zip(fr, grids)):
        c.set_slot_geometry(k, dim, [f.L, f.L, f.L if dim == 3 else 1.0], g)
        if k in no_vel:
            c.upload_frame(k, f.pos, f.diam)
        else:
            c.upload_frame(k, f.pos, f.diam, f.vel, f.mass)


def test_fused_uneven_batch_equals_per_frame_and_lanes():
    from pyglasstools_gb300 import ikabi as ik, synth
    sizes = [3000, 800, 15000, 1200, 6100, 2000]
    fr, grids = _uneven(2, sizes, 1300)
    c = _ctx(ik)
    _setup(ik, c, 2, fr, grids, no_vel=(3,))
    slots = [4, 0, 2, 5, 1, 3]  # any order
    assert c.get_tuning("fused_batch") == 1
    c.compute_batch(slots, "fp32")  # plain launches + recording
    c.synchronize()
    l0 = c.launch_count()
    c.compute_batch(slots, "fp32")  # the fused graph
    c.synchronize()
    launches = c.launch_count() - l0
    assert launches <= 10, launches
    fused = _fields(ik, c, range(len(fr)))
    cnt_fused = [c.counters(k) for k in range(len(fr))]
    # the same batch on the lanes (one launch sequence per frame)
    c.set_tuning("fused_batch", 0)
    c.compute_batch(slots, "fp32")
    c.synchronize()
    l0 = c.launch_count()
    c.compute_batch(slots, "fp32")
    c.synchronize()
    assert c.launch_count() - l0 >= 6 * len(fr)
    lanes = _fields(ik, c, range(len(fr)))
    for k in range(len(fr)):
        for a, b in zip(fused[k], lanes[k]):
            np.testing.assert_array_equal(a, b)
        f = fr[k]
        if k == 3:  # uploaded without velocities: kinetic field zero
            f = synth.SynthFrame(2, f.L, f.pos, None, None, f.diam)
        want, cnt = _alone(ik, 2, f, grids[k])
        for a, b in zip(fused[k], want):
            np.testing.assert_array_equal(a, b)
        assert cnt_fused[k] == cnt, (k, cnt_fused[k], cnt)
    assert np.all(fused[3][1] == 0.0)
    c.close()


def test_fused_batch_with_an_empty_frame():
    from pyglasstools_gb300 import ikabi as ik
    fr, grids = _uneven(2, [2000, 1500, 2500], 1400)
    c = _ctx(ik)
    _setup(ik, c, 2, fr, grids)
    c.upload_frame(1, np.zeros((0, 3)), np.zeros(0))
    for _ in range(2):
        c.compute_batch([0, 1, 2], "fp32")
        c.synchronize()
    got = _fields(ik, c, range(3))
    assert np.all(got[1][0] == 0.0) and np.all(got[1][1] == 0.0)
    for k in (0, 2):
        want, _ = _alone(ik, 2, fr[k], grids[k])
        for a, b in zip(got[k], want):
            np.testing.assert_array_equal(a, b)
    c.close()


@pytest.mark.parametrize("flags", [0, 2])
def test_fused_batch_3d_octic_and_lane_sums(flags):
    from pyglasstools_gb300 import ikabi as ik
    fr, grids = _uneven(3, [4000, 1500, 6000], 1500)
    cg = ("octic", 2.0, 0.0)
    c = _ctx(ik, cg)
    c.set_flags(flags)
    _setup(ik, c, 3, fr, grids)
    slots = [0, 1, 2]
    for _ in range(2):
        c.compute_batch(slots, "fp32")
        c.synchronize()
    got = _fields(ik, c, slots)
    for k in slots:
        want, _ = _alone(ik, 3, fr[k], grids[k], cg, flags)
        for a, b in zip(got[k], want):
            np.testing.assert_array_equal(a, b)
    c.close()


@pytest.mark.parametrize("kind", ["octic", "rect", "mollifier", "gaussian"])
def test_fused_batch_every_kernel_2d_kahan(kind):
    from pyglasstools_gb300 import ikabi as ik
    fr, grids = _uneven(2, [2500, 4000], 1600 + len(kind))
    cg = (kind, 6.0, 2.0) if kind == "gaussian" else (kind, 2.0, 0.0)
    c = _ctx(ik, cg)
    c.set_flags(ik.FLAG_LANE_KAHAN)
    _setup(ik, c, 2, fr, grids)
    for _ in range(2):
        c.compute_batch([1, 0], "fp32")
        c.synchronize()
    for k in range(2):
        want, _ = _alone(ik, 2, fr[k], grids[k], cg, ik.FLAG_LANE_KAHAN)
        for a, b in zip(_fields(ik, c, [k])[0], want):
            np.testing.assert_array_equal(a, b)
    c.close()


def test_fused_replay_overflowing_bond_capacity_is_rerun():
    """New contents of one slot (same size) with more bonds per particle than the
    batch's capacity: the fused replay reports it, and ik_synchronize re-runs the batch's
    frames on the per-frame path with a larger capacity."""
    from pyglasstools_gb300 import ikabi as ik, synth
    fr, grids = _uneven(2, [3000, 2000], 1700)
    c = _ctx(ik)
    _setup(ik, c, 2, fr, grids)
    for _ in range(2):
        c.compute_batch([0, 1], "fp32")
        c.synchronize()
    dense = fr[1].pos.copy()
    dense[:, :2] *= 0.55
    c.upload_frame(1, dense, fr[1].diam, fr[1].vel, fr[1].mass)
    c.compute_batch([0, 1], "fp32")
    c.synchronize()
    got = _fields(ik, c, [0, 1])
    want0, _ = _alone(ik, 2, fr[0], grids[0])
    f1 = synth.SynthFrame(2, fr[1].L, dense, fr[1].vel, fr[1].mass, fr[1].diam)
    want1, _ = _alone(ik, 2, f1, grids[1])
    for a, b in zip(got[0], want0):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(got[1], want1):
        np.testing.assert_array_equal(a, b)
    c.close()


@pytest.mark.parametrize("io_batches,mapped", [(1, 0), (3, 0), (6, 0), (1, 1), (3, 1)])
def test_fused_host_io_sub_batches_equal_per_frame(io_batches, mapped):
    """ik_compute_batch_io of an eligible batch runs as fused sub-batches whose host copies
    overlap the other sub-batches' computation (copy engines), or with each sub-batch's
    copies as one kernel over the host arrays' device view (host-mapped).  Uneven frames
    with their own boxes and grids, one without velocities: the host fields equal the
    per-frame path bit for bit on the first call (plain path), on replays and after new
    contents, and a replay launches at most one validation per frame and eight kernels per
    sub-batch."""
    torch = pytest.importorskip("torch")
    from conftest import uniq
    from pyglasstools_gb300 import ikabi as ik, synth
    sizes = [3000, 800, 15000, 1200, 6100, 2000]
    fr, grids = _uneven(2, sizes, 1600)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    host = [(pin(f.pos), pin(f.diam), None if k == 3 else pin(f.vel), None if k == 3 else pin(f.mass))
            for k, f in enumerate(fr)]
    outs = [(pin(np.zeros((len(g), 3))), pin(np.zeros((len(g), 3))), None) for g in grids]
    c = _ctx(ik)
    _setup(ik, c, 2, fr, grids, no_vel=(3,))
    c.set_tuning("io_batches", io_batches)
    c.set_tuning("io_mapped", mapped)
    assert c.get_tuning("io_batches") == io_batches and c.get_tuning("io_mapped") == mapped
    slots = list(range(len(fr)))

    def want_for(frames):
        res = []
        for k, f in enumerate(frames):
            if k == 3:
                f = synth.SynthFrame(2, f.L, f.pos, None, None, f.diam)
            w, _ = _alone(ik, 2, f, grids[k])
            res.append([uniq(x) for x in w])
        return res

    def check(want):
        for k in slots:
            np.testing.assert_array_equal(outs[k][0], want[k][0])
            np.testing.assert_array_equal(outs[k][1], want[k][1])

    want = want_for(fr)
    for rep in range(3):  # plain path + recording, then replays
        l0 = c.launch_count()
        c.compute_batch_io(slots, host, outs)
        c.synchronize()
        if rep == 2:
            assert c.launch_count() - l0 <= len(fr) + 8 * io_batches
        check(want)
    fr2, _ = _uneven(2, sizes, 1700)  # same sizes and boxes, new contents
    for k, f in enumerate(fr2):
        host[k][0][:] = f.pos
        host[k][1][:] = f.diam
        if k != 3:
            host[k][2][:] = f.vel
            host[k][3][:] = f.mass
    c.compute_batch_io(slots, host, outs)
    c.synchronize()
    check(want_for(fr2))
    c.close()


def test_host_io_autotuner_keeps_a_candidate_and_the_fields():
    """ik_autotune_batch_io times the lanes and the fused sub-batches of a host-I/O batch,
    keeps one of them, and the host fields it leaves -- and those of the tuned replay --
    equal the per-frame path bit for bit."""
    torch = pytest.importorskip("torch")
    from conftest import uniq
    from pyglasstools_gb300 import ikabi as ik
    sizes = [2500, 900, 7000, 1800]
    fr, grids = _uneven(2, sizes, 1800)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    host = [(pin(f.pos), pin(f.diam), pin(f.vel), pin(f.mass)) for f in fr]
    outs = [(pin(np.zeros((len(g), 3))), pin(np.zeros((len(g), 3))), None) for g in grids]
    c = _ctx(ik)
    _setup(ik, c, 2, fr, grids)
    slots = list(range(len(fr)))
    best = c.autotune_batch_io(slots, host, outs, reps=1)
    assert best["io_batches"] in (0, 1, 2, 4) and best["io_mapped"] in (0, 1) and best["ms_per_batch"] > 0
    assert best["io_batches"] > 0 or best["io_mapped"] == 0
    assert c.get_tuning("io_batches") == best["io_batches"]
    want = [[uniq(x) for x in _alone(ik, 2, f, g)[0]] for f, g in zip(fr, grids)]
    for rep in range(2):
        if rep:
            c.compute_batch_io(slots, host, outs)
        c.synchronize()
        for k in slots:
            np.testing.assert_array_equal(outs[k][0], want[k][0])
            np.testing.assert_array_equal(outs[k][1], want[k][1])
    c.close()


@pytest.mark.parametrize("io_batches,mapped", [(0, 0), (1, 0), (1, 1)])
def test_host_io_sub_batches_validate_the_frames(io_batches, mapped):
    """Host-I/O batches check each frame without a launch of their own -- the binning checks
    the positions and the packing the diameters (lanes: per frame; fused sub-batches: over
    the batch), host-mapped copies also as they copy: a replay whose new contents hold a
    non-finite position, or a 2D position with z != 0, is reported as IK_ERR_ARG by
    synchronize; the context stays usable, and a replay of valid contents gives the
    per-frame fields."""
    torch = pytest.importorskip("torch")
    from conftest import uniq
    from pyglasstools_gb300 import ikabi as ik
    fr, grids = _uneven(2, [1500, 2600], 1900)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    host = [(pin(f.pos), pin(f.diam), pin(f.vel), pin(f.mass)) for f in fr]
    outs = [(pin(np.zeros((len(g), 3))), pin(np.zeros((len(g), 3))), None) for g in grids]
    c = _ctx(ik)
    _setup(ik, c, 2, fr, grids)
    c.set_tuning("io_batches", io_batches)
    c.set_tuning("io_mapped", mapped)
    slots = [0, 1]
    for _ in range(2):  # plain path + recording, then a replay
        c.compute_batch_io(slots, host, outs)
        c.synchronize()
    for k, bad in ((7, np.nan), (11, 0.25)):
        keep = host[1][0][k].copy()
        if np.isnan(bad):
            host[1][0][k, 0] = bad
        else:
            host[1][0][k, 2] = bad  # z of a 2D frame
        c.compute_batch_io(slots, host, outs)
        with pytest.raises(ik.IKError, match="IK_ERR_ARG"):
            c.synchronize()
        host[1][0][k] = keep
    c.compute_batch_io(slots, host, outs)
    c.synchronize()
    for k in slots:
        want = [uniq(x) for x in _alone(ik, 2, fr[k], grids[k])[0]]
        np.testing.assert_array_equal(outs[k][0], want[0])
        np.testing.assert_array_equal(outs[k][1], want[1])
    c.close()
