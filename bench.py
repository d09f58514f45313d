#!/usr/bin/env python
"""Irving-Kirkwood stress-field throughput on GB300 (frames/s).

Workload (default ``ik2d_n64k_g256_gauss``): 64 seeded 2D polydisperse12 frames,
N = 64,000 particles (L = 253), a 256 x 256 lattice grid, Gaussian coarse-graining
kernel of width 2 truncated at 3 widths, Gauss-Legendre-5 bond integrals, virial +
kinetic stress.  One step = one pass of the tuned FP32 path over the 64 frames.

  value        frames/s with the frames resident in HBM (cycled: 64 x 4 MB of
               inputs > L2), CUDA events on the engine's stream, max over ranks;
  e2e          frames/s through the C ABI with host buffers: pinned host->device
               upload of every frame and device->host read of both fields each step
               (ik_compute_batch_io: copies and kernels of a frame on its lane, one
               graph per step);
  plain_fp64   frames/s of the plain FP64 GPU kernels (same workload), and the
               tuned path's relative L2 error against them;
  roofline     the FP32 gather kernel: algorithmic FLOPs (66 per active (grid, i, j)
               triple, the GL-5-equivalent bond integral + 2D stress accumulation)
               per launch / its CUDA-event duration, against the FP32 FMA peak
               measured live on this GPU;
  cpu_baseline the FP64 oracle (restatement of IrvingKirkwood::compute) on all host
               cores over whole frames (about 10 s of work), with a single-core rate
               and the host's CPU count beside it.

``--impl reference`` times that CPU restatement of the reference's path alone.
``--gpus N`` under torchrun runs N independent replicas (the path is not sharded).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "IK stress frames/s, 2D N=64k 256² grid: tuned vs plain FP64 GPU @≤1e-5 rel"

WORKLOADS = {
    "ik2d_n64k_g256_gauss": dict(N=64000, dim=2, nmax=256, frames=64, cg=dict(kind="gaussian", rcut=6.0, width=2.0),
                                 desc="Gaussian w=2 cut at 3w (R=6), GL-5"),
    "ik2d_n2k_g64_octic": dict(N=2000, dim=2, nmax=64, frames=64, cg=dict(kind="octic", rcut=2.0, width=0.0),
                               desc="octic R=2, GL-5"),
    "ik3d_n32k_g64_octic": dict(N=32000, dim=3, nmax=64, frames=16, cg=dict(kind="octic", rcut=2.0, width=0.0),
                                desc="octic R=2, GL-5"),
}
FLOP_PER_TRIPLE = {2: 66, 3: 82}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ik2d_n64k_g256_gauss", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--lane-sums", default="kahan", choices=["kahan", "plain"],
                    help="per-lane sums of the FP32 gather in the headline: Kahan-compensated (default) or plain "
                         "FP32 (both merged across lanes and chunks with TwoSum); the other is timed beside it")
    ap.add_argument("--frames", type=int, default=0, help="override the frames per step (profiling)")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the learned-surrogate leg")
    ap.add_argument("--no-uneven", action="store_true", help="skip the uneven-batch leg")
    ap.add_argument("--no-graph", action="store_true",
                    help="enqueue every frame with its own launches instead of one CUDA-graph replay per step")
    ap.add_argument("--profile-mlp", action="store_true",
                    help="with --profile: run the surrogate mode (a small network trained first), "
                         "so that the tensor-core kernel appears in the launch list")
    ap.add_argument("--profile", action="store_true",
                    help="only warm-up + timed steps (for ncu launch lists); prints a short JSON line")
    ap.add_argument("--schedule", default="auto", choices=["auto", "fused", "lanes"],
                    help="batch schedule of the headline: chosen by the autotuner (default), or fixed: fused "
                         "(every stage once over the step's frames) or lanes (one launch sequence per frame)")
    ap.add_argument("--io-batches", type=int, default=-1,
                    help="schedule of the end-to-end step's copies: 0 per frame on the lanes, n fused sub-batches "
                         "(default: chosen by the host-I/O autotuner)")
    ap.add_argument("--profile-precision", default="fp32", choices=["fp32", "fp64"],
                    help="with --profile: the path the steps run (fp64 = the plain FP64 gather)")
    return ap.parse_args()


def synth_module():
    """The seeded frame generator (pyglasstools_gb300/synth.py, numpy only), loaded by
    path: importing it through the package would load the package's native extension,
    which the CPU-only reference arm must not map."""
    import importlib.util
    name = "ik_synth_frames"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, os.path.join(ROOT, "pyglasstools_gb300", "synth.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def make_frames(wl, rank):
    synth = synth_module()
    frames = [synth.make_frame(wl["N"], dim=wl["dim"], seed=10007 * rank + k) for k in range(wl["frames"])]
    grid = synth.lattice_grid(frames[0].L, wl["nmax"], wl["dim"])
    return frames, grid


def config_of(name, wl, world):
    return {"workload": name, "N": wl["N"], "dim": wl["dim"],
            "grid": "x".join([str(wl["nmax"])] * wl["dim"]), "cgfunc": wl["desc"],
            "potential": "polydisperse12 v0=1 eps=0.2 rcut=1.25", "frames_per_step": wl["frames"],
            "l2": "inputs larger than L2: %d resident frames cycled each step" % wl["frames"],
            "parallelism": "replicas x%d (no sharding)" % world}


# ---------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append((time.perf_counter(), parts))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0, t1):
        sel = [p for (t, p) in self.samples if t0 <= t <= t1] or [p for (_, p) in self.samples]
        if not sel:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(p[1]) for p in sel if num(p[1]) is not None]
        mx = [num(p[2]) for p in sel if num(p[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for p in sel for k in range(4) if p[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sel)}


# ---------------------------------------------------------------------------- dist helpers
def dist_setup(backend=None):
    """Replica setup from the torchrun environment: NCCL with one GPU per rank, or gloo
    (host-side tests).  The path is not sharded: ranks only meet at barriers and the
    max over ranks of the timed region."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = backend or "nccl"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------- CPU baseline
def cpu_sample(wl, frames, grid, g1, nthreads, k=0, fields=None):
    """Seconds the oracle takes for grid points [0, g1) of frame k on nthreads threads
    (its virial and kinetic fields appended to `fields` when a list is given)."""
    from oracle import oracle as O
    f = frames[k]
    box = O.make_box(wl["dim"], [f.L, f.L, f.L if wl["dim"] == 3 else 1.0])
    pot = O.make_poly12()
    cg = O.make_cg(wl["cg"]["kind"], rcut=wl["cg"]["rcut"], mode="fixedpoint", order=5, width=wl["cg"]["width"])
    t = time.perf_counter()
    out = O.compute(box, f.pos, f.diam, pot, cg, grid, vel=f.vel, mass=f.mass, g0=0, g1=g1, nthreads=nthreads)
    dt = time.perf_counter() - t
    if fields is not None:
        fields.append(out)
    return dt


def host_cpu_info():
    """CPUs this process may run on: the count the OS reports, the affinity mask and the
    cgroup v2 CPU quota (a quota below the affinity count time-slices the oracle's threads)."""
    info = {"nproc": os.cpu_count()}
    try:
        info["affinity"] = len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        info["affinity"] = None
    try:
        with open("/sys/fs/cgroup/cpu.max") as f:
            quota, period = f.read().split()[:2]
        info["cgroup_cpus"] = None if quota == "max" else float(quota) / float(period)
    except (OSError, ValueError):
        info["cgroup_cpus"] = None
    return info


def single_core_sample(wl, frames, grid):
    """The oracle on one thread over the whole of frame 0 (about ten seconds on one core):
    the per-core rate beside the all-threads baseline."""
    t = cpu_sample(wl, frames, grid, len(grid), 1)
    return {"value": 1.0 / t, "unit": "frames/s", "cores": 1,
            "sample": f"frame 0 whole ({len(grid)} grid points), one thread, {t:.2f} s"}


def reference_arm(args, wl, name):
    """The CPU restatement of the reference's path alone: one step = one whole frame
    (cell list, neighbour lists and every grid point), frames cycled over eight seeds."""
    world, rank, _ = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    nfr = min(wl["frames"], 8)
    frames, grid = make_frames(dict(wl, frames=nfr), 0)
    cores = O.threads(os.cpu_count() or 1)  # threads the oracle's loops actually run on
    G = len(grid)
    for k in range(args.warmup):
        cpu_sample(wl, frames, grid, G, cores, k=k % nfr)
    t = 0.0
    for k in range(args.steps):
        t += cpu_sample(wl, frames, grid, G, cores, k=k % nfr)
    value = args.steps / t
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_of(name, wl, world),
            "cpu_baseline": {"value": value, "unit": "frames/s", "cores": cores, "kind": "port",
                             "sample": f"one whole frame per step ({G} grid points; frames cycled over {nfr} "
                                       f"seeds), FP64 oracle restating IrvingKirkwood::compute, "
                                       f"OpenMP {cores} threads",
                             "host_cpus": host_cpu_info()},
            "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "native_libraries_mapped": repo_libraries_mapped()}
    print(json.dumps(line), flush=True)


def repo_libraries_mapped():
    """Shared objects of this repository mapped into the process (from /proc/self/maps;
    None where that file does not exist): the reference arm maps only the oracle's."""
    try:
        with open("/proc/self/maps") as f:
            paths = {ln.split()[-1] for ln in f if ln.rstrip().endswith(".so") or ".so." in ln}
    except OSError:
        return None
    return sorted(os.path.relpath(p, ROOT) for p in paths if p.startswith(ROOT + os.sep))


# ---------------------------------------------------------------------------- surrogate leg
MLP_TOL = 1e-6  # the surrogate stands in for the quadrature only in bins validated within this


def surrogate_leg(args, ctx, wl, F, stream, all_slots, v_plain):
    """The learned bond-integral surrogate on the same frames: train it on the GPU
    (2^22 samples), validate it, then time the FP32 path with the network standing in
    for the quadrature on bonds that cross the edge of the support, and state its error
    against the exact bond integral (FP64, erf closed form) next to the fixed-point rule's."""
    import torch
    from pyglasstools_gb300 import ikabi
    cg = wl["cg"]
    mlp = ikabi.MLP(torch.cuda.current_device())
    t0 = time.perf_counter()
    hist = mlp.train(nsamples=1 << 22, epochs=250, ctas=152, lr=2e-3, seed=5)
    train_s = time.perf_counter() - t0
    v_used = mlp.validate(n=1 << 22, seed=98, tol=MLP_TOL)
    ctx.set_mlp(mlp)

    def timed_mode(mode):
        """frames/s of the batch in a quadrature mode (graph replays, CUDA events), its
        kernel launches per step, and the virial field of slot 0."""
        ctx.set_cgfunc(cg["kind"], cg["rcut"], mode=mode, order=5, width=cg["width"])
        ctx.compute_batch(all_slots, "fp32")  # first call: plain launches, then the graph is recorded
        ctx.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        for _ in range(2):
            ctx.compute_batch(all_slots, "fp32")
        ctx.synchronize()
        launches0 = ctx.launch_count()
        e0.record(stream)
        for _ in range(args.steps):
            ctx.compute_batch(all_slots, "fp32")
        ctx.wait_all()
        e1.record(stream)
        ctx.synchronize()
        fps = F * args.steps / (e0.elapsed_time(e1) * 1e-3)
        return fps, (ctx.launch_count() - launches0) // args.steps, ctx.get_field(ikabi.FIELD_VIRIAL, slot=0)

    fps_net, launches, v_net = timed_mode("mlp")
    records = ctx.mlp_records(0)
    fallbacks = ctx.mlp_fallbacks(0)
    triples = ctx.counters(0)[2]
    # the closed forms as comparators: on the same crossing bonds, and on every bond
    fps_clip, _, v_clip = timed_mode("clipped")
    fps_exact32, _, v_exact32 = timed_mode("exact")
    # fixed-point FP32 and exact FP64 of frame 0
    ctx.set_cgfunc(cg["kind"], cg["rcut"], mode="fixedpoint", order=5, width=cg["width"])
    ctx.compute_slot(0, "fp32")
    ctx.synchronize()
    v_gl = ctx.get_field(ikabi.FIELD_VIRIAL, slot=0)
    ctx.set_cgfunc(cg["kind"], cg["rcut"], mode="exact", order=5, width=cg["width"])
    ctx.compute_slot(0, "fp64")
    ctx.synchronize()
    v_exact = ctx.get_field(ikabi.FIELD_VIRIAL, slot=0)
    ctx.set_cgfunc(cg["kind"], cg["rcut"], mode="fixedpoint", order=5, width=cg["width"])
    ctx.set_mlp(None)

    def rel(a, b):
        iu = [(0, 0), (1, 1), (0, 1)]
        return [float(np.linalg.norm(a[:, i, j] - b[:, i, j]) / np.linalg.norm(b[:, i, j])) for i, j in iu]

    out = {"value": fps_net, "unit": "frames/s", "gpu_launches_per_step": int(launches),
           "network": "4-64-64-64-1 SiLU, BF16 operands on tcgen05, FP32 accum; learns (B / GL-4 on the clipped segment - 1) * 1e4",
           "train": {"samples": 1 << 22, "steps": len(hist), "seconds": train_s, "final_loss": float(hist[-1])},
           "validation": {"rms_err": v_used["rms_err"], "max_err": v_used["max_err"],
                          "coverage_at_1e-6": v_used["coverage"], "tol": MLP_TOL,
                          "error": "|B_net - B_exact| per sample, B in units of the kernel's peak"},
           "rel_err_vs_exact_integral": {"surrogate_fp32": rel(v_net, v_exact), "fixed_point_gl5_fp32": rel(v_gl, v_exact),
                                         "plain_fp64_gl5": rel(v_plain, v_exact),
                                         "clipped_closed_form_fp32": rel(v_clip, v_exact),
                                         "exact_closed_form_fp32": rel(v_exact32, v_exact)},
           "comparators": {
               "clipped_closed_form_fp32": {
                   "frames_per_s": fps_clip,
                   "what": "erf closed form on the bonds the network stands in for, GL-5 elsewhere"},
               "exact_closed_form_fp32": {"frames_per_s": fps_exact32, "what": "erf closed form on every bond"},
               "network_over_clipped_closed_form": fps_net / fps_clip},
           "rel_diff_vs_plain_fp64_gl5": rel(v_net, v_plain),
           "records_slot0": records, "fallback_records_slot0": fallbacks, "triples_slot0": triples,
           "tensor_flop_per_eval": 2 * (4 * 64 * 3 + 128 * 64 * 2)}
    mlp.close()
    return out


# ---------------------------------------------------------------------------- uneven batch leg
def uneven_leg(args):
    """256 seeded 2D frames with N log-uniform on [1000, 128000] (density 1, each frame
    its own box and a grid of spacing ~1), Gaussian w = 2 cut at 6: the batch replayed
    as one CUDA graph with the autotuner's bin size and CTAs per SM, against the same
    frames launched one by one with the default tuning; and end to end from page-locked
    host frames to host fields, with the host-I/O autotuner's schedule of the copies and
    with the lanes."""
    import torch
    from pyglasstools_gb300 import ikabi, synth
    rng = np.random.default_rng(2024)
    F = 256
    Ns = np.exp(rng.uniform(np.log(1000.0), np.log(128000.0), F)).astype(int)
    c = ikabi.IKContext(torch.cuda.current_device())
    c.set_poly12()
    c.set_cgfunc("gaussian", 6.0, order=5, width=2.0)
    c.reserve_slots(F)
    c.set_max_rcut(1.25 * 1.62)
    G_total = 0
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    host, outs = [], []  # page-locked host frames and fields of the end-to-end batch
    for k, n in enumerate(Ns):
        f = synth.make_frame(int(n), dim=2, seed=5000 + k)
        grid = synth.lattice_grid(f.L, max(int(f.L), 2), 2)
        G_total += len(grid)
        c.set_slot_geometry(k, 2, [f.L, f.L, 1.0], grid)
        c.upload_frame(k, f.pos, f.diam, f.vel, f.mass)
        host.append((pin(f.pos), pin(f.diam), pin(f.vel), pin(f.mass)))
        outs.append((pin(np.zeros((len(grid), 3))), pin(np.zeros((len(grid), 3))), None))
    c.synchronize()
    slots = list(range(F))
    stream = torch.cuda.ExternalStream(c.stream())
    reps = max(3, min(args.steps, 10))

    def timed(fn):
        fn()
        c.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        c.wait_all()
        e1.record(stream)
        c.synchronize()
        return e0.elapsed_time(e1) / reps

    def per_frame():
        for k in slots:
            c.compute_slot(k, "fp32")

    def graph(fused):
        c.set_tuning("fused_batch", fused)
        c.compute_batch(slots, "fp32")  # first call: plain launches, then the graph is recorded
        c.synchronize()
        l0 = c.launch_count()
        ms = timed(lambda: c.compute_batch(slots, "fp32"))
        return ms, (c.launch_count() - l0) // (reps + 1)

    ms_plain = timed(per_frame)
    ms_fused, launches_fused = graph(1)
    ms_lanes, launches_lanes = graph(0)
    best = c.autotune_batch(slots, "fp32", reps=2)
    c.compute_batch(slots, "fp32")  # the tuned settings' first call records the graph again
    c.synchronize()
    l0 = c.launch_count()
    ms_graph = timed(lambda: c.compute_batch(slots, "fp32"))
    launches = (c.launch_count() - l0) // (reps + 1)
    # end to end (host frames in, host fields out), the copies' schedule autotuned, and the
    # lanes beside it: wall time per batch, synchronised
    io_best = c.autotune_batch_io(slots, host, outs, reps=3)

    def e2e():  # ms per batch: the median of three timed runs (the host link's rate varies run to run)
        for _ in range(3):
            c.compute_batch_io(slots, host, outs)
            c.synchronize()
        runs = []
        for _ in range(3):
            t0 = time.perf_counter()
            for _ in range(reps):
                c.compute_batch_io(slots, host, outs)
                c.synchronize()
            runs.append((time.perf_counter() - t0) / reps * 1e3)
        return float(np.median(runs))

    ms_e2e = e2e()
    c.set_tuning("io_batches", 0)
    c.set_tuning("blocks_per_sm", 0)
    ms_e2e_lanes = e2e()
    c.close()
    return {"workload": "256 frames, N log-uniform [1000, 128000], own box and grid (spacing ~1), Gaussian w=2 R=6",
            "particles": int(Ns.sum()), "grid_points": int(G_total),
            "per_frame_launches": {"frames_per_s": F / (ms_plain * 1e-3), "ms_per_batch": ms_plain},
            "fused_graph": {"frames_per_s": F / (ms_fused * 1e-3), "ms_per_batch": ms_fused,
                            "kernel_launches_per_batch": int(launches_fused),
                            "what": "every stage once over the batch: one persistent gather over all frames"},
            "lanes_graph": {"frames_per_s": F / (ms_lanes * 1e-3), "ms_per_batch": ms_lanes,
                            "kernel_launches_per_batch": int(launches_lanes),
                            "what": "one launch sequence per frame on eight streams, one graph"},
            "graph_autotuned": {"frames_per_s": F / (ms_graph * 1e-3), "ms_per_batch": ms_graph,
                                "tuning": best, "kernel_launches_per_batch": int(launches)},
            "e2e_autotuned": {"frames_per_s": F / (ms_e2e * 1e-3), "ms_per_batch": ms_e2e, "tuning": io_best,
                              "h2d_bytes_per_batch": int(Ns.sum()) * 64, "d2h_bytes_per_batch": int(G_total) * 48,
                              "what": "host frames in, host fields out, one graph per batch (ik_compute_batch_io)"},
            "e2e_lanes": {"frames_per_s": F / (ms_e2e_lanes * 1e-3), "ms_per_batch": ms_e2e_lanes,
                          "what": "the same with each frame's copies and kernels on one of eight lanes"},
            "speedup": ms_plain / ms_graph}


# ---------------------------------------------------------------------------- our arm
def ours(args, wl, name):
    import torch
    from pyglasstools_gb300 import ikabi

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    frames, grid = make_frames(wl, rank)
    F, D = wl["frames"], wl["dim"]
    NC = 3 if D == 2 else 6
    L = frames[0].L
    ctx = ikabi.IKContext(local)
    ctx.set_box(D, [L, L, L if D == 3 else 1.0])
    ctx.set_poly12()
    ctx.set_cgfunc(wl["cg"]["kind"], wl["cg"]["rcut"], order=5, width=wl["cg"]["width"])
    ctx.set_grid(grid)
    ctx.reserve_slots(F)
    for k, f in enumerate(frames):
        ctx.upload_frame(k, f.pos, f.diam, f.vel, f.mass)
        ctx.synchronize()
    stream = torch.cuda.ExternalStream(ctx.stream())
    # per-lane sums of the FP32 gather: Kahan-compensated in the headline by default
    lane_flags = ikabi.FLAG_LANE_KAHAN if args.lane_sums == "kahan" else 0
    ctx.set_flags(lane_flags)

    all_slots = list(range(F))
    tuning = None
    if args.schedule == "auto":  # the autotuner: schedule, bin size, CTAs per SM, halo per warp
        tuning = ctx.autotune_batch(all_slots, "fp32", reps=2)
    else:
        ctx.set_tuning("fused_batch", 1 if args.schedule == "fused" else 0)

    def step(prec="fp32", nfr=F):
        # one CUDA-graph replay per step for the whole batch of resident frames
        if nfr == F and not args.no_graph:
            ctx.compute_batch(all_slots, prec)
        else:
            for k in range(nfr):
                ctx.compute_slot(k, prec)

    if args.profile:
        if args.profile_mlp:  # surrogate mode: a small network, trained and validated first
            from pyglasstools_gb300 import ikabi
            mlp = ikabi.MLP(torch.cuda.current_device())
            mlp.train(nsamples=1 << 18, epochs=20, ctas=152, lr=2e-3, seed=5)
            mlp.validate(n=1 << 18, seed=98, tol=MLP_TOL)
            ctx.set_mlp(mlp)
            ctx.set_cgfunc(wl["cg"]["kind"], wl["cg"]["rcut"], mode="mlp", order=5, width=wl["cg"]["width"])
        for _ in range(args.warmup):
            step(args.profile_precision)
        ctx.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step(args.profile_precision)
        ctx.synchronize()
        dt = time.perf_counter() - t0
        print(json.dumps({"profile": name, "frames": F, "steps": args.steps, "host_s": dt,
                          "frames_per_s_host": F * args.steps / dt, "counters_slot0": ctx.counters(0)}))
        ctx.close()
        return

    clocks = ClockSampler(local)
    clocks.start()
    # ---- warm-up (also a soak so that the clock sampler sees the GPU under load)
    t_soak = time.perf_counter()
    for _ in range(max(args.warmup, 3)):
        step()
    ctx.synchronize()
    while time.perf_counter() - t_soak < 1.5:
        step()
        ctx.synchronize()
    # ---- timed region (device-resident inputs)
    barrier(world)
    torch.cuda.synchronize()
    ctx.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    launches0 = ctx.launch_count()
    t_host0 = time.perf_counter()
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    t_enq = time.perf_counter()
    ctx.wait_all()
    ev1.record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    t_host1 = time.perf_counter()
    launches = ctx.launch_count() - launches0
    ms = ev0.elapsed_time(ev1)
    barrier(world)
    ms_max = max_over_ranks(ms, world)
    value = world * F * args.steps / (ms_max * 1e-3)

    def timed_steps():
        for _ in range(3):
            step()
        ctx.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        l0 = ctx.launch_count()
        e0.record(stream)
        for _ in range(args.steps):
            step()
        ctx.wait_all()
        e1.record(stream)
        ctx.synchronize()
        return F * args.steps / (e0.elapsed_time(e1) * 1e-3), (ctx.launch_count() - l0) // args.steps

    # ---- the other per-lane summation beside the headline (same frames, same graph path)
    ctx.set_flags(ikabi.FLAG_LANE_KAHAN - lane_flags)
    other_value, _ = timed_steps()
    ctx.set_flags(lane_flags)
    # ---- and the other batch schedule: fused (the default) or one launch sequence per frame
    # (its CTAs per SM at their default: the tuned value belongs to the headline's schedule)
    fused0 = ctx.get_tuning("fused_batch")
    bps0 = ctx.get_tuning("blocks_per_sm")
    ctx.set_tuning("fused_batch", 1 - fused0)
    ctx.set_tuning("blocks_per_sm", 0)
    other_sched, other_launches = timed_steps()
    ctx.set_tuning("fused_batch", fused0)
    ctx.set_tuning("blocks_per_sm", bps0)
    schedules = {"headline": "fused" if fused0 else "lanes",
                 "fused_frames_per_s": value / world if fused0 else other_sched,
                 "lanes_frames_per_s": other_sched if fused0 else value / world,
                 "launches_per_step": {"headline": int(launches) // args.steps, "other": int(other_launches)}}
    lane_sums = {"headline": args.lane_sums,
                 "kahan_frames_per_s": value / world if lane_flags else other_value,
                 "plain_frames_per_s": other_value if lane_flags else value / world}

    # ---- end to end through the C ABI with host buffers
    pin = lambda shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    hpos = [pin((wl["N"], 3)) for _ in range(F)]
    hvel = [pin((wl["N"], 3)) for _ in range(F)]
    hmass = [pin((wl["N"],)) for _ in range(F)]
    hdiam = [pin((wl["N"],)) for _ in range(F)]
    for k, f in enumerate(frames):
        hpos[k][:] = f.pos
        hvel[k][:] = f.vel
        hmass[k][:] = f.mass
        hdiam[k][:] = f.diam
    hvir = [pin((len(grid), NC)) for _ in range(F)]
    hkin = [pin((len(grid), NC)) for _ in range(F)]

    # one graph per step (ik_compute_batch_io): each frame's upload, kernels and field
    # downloads on its lane, frames overlapping; the first call records it
    io_frames = [(hpos[k], hdiam[k], hvel[k], hmass[k]) for k in range(F)]
    io_outs = [(hvir[k], hkin[k], None) for k in range(F)]
    io_slots = list(range(F))

    def e2e_step():
        if args.no_graph:
            for k in range(F):
                ctx.upload_frame(k, hpos[k], hdiam[k], hvel[k], hmass[k])
                ctx.compute_slot(k, "fp32")
                ctx.download_field_async(hvir[k], ikabi.FIELD_VIRIAL, k)
                ctx.download_field_async(hkin[k], ikabi.FIELD_KINETIC, k)
        else:
            ctx.compute_batch_io(io_slots, io_frames, io_outs)
        ctx.synchronize()

    def e2e_run():
        for _ in range(1 + args.warmup):  # the first call runs the plain path and records the graph
            e2e_step()
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        t1 = time.perf_counter()
        return world * F * args.steps / max_over_ranks(t1 - t0, world)

    # the schedule of the copies: per frame on the lanes, or fused sub-batches whose copies
    # overlap the other sub-batches' computation -- chosen by the host-I/O autotuner (or
    # --io-batches); the other kind is timed beside it
    io_tuning = None
    if args.no_graph:
        pass
    elif args.io_batches >= 0:
        ctx.set_tuning("io_batches", args.io_batches)
    else:
        io_tuning = ctx.autotune_batch_io(io_slots, io_frames, io_outs, reps=4)
    nsub = ctx.get_tuning("io_batches") if not args.no_graph else 0
    io_mapped = ctx.get_tuning("io_mapped") if nsub else 0
    e2e_value = e2e_run()
    e2e_other, other_desc = None, None
    if not args.no_graph and ctx.get_tuning("fused_batch"):
        bps0 = ctx.get_tuning("blocks_per_sm")
        if nsub:
            ctx.set_tuning("io_batches", 0)
            ctx.set_tuning("blocks_per_sm", 0)
            other_desc = "lanes"
        else:
            ctx.set_tuning("io_batches", 8)
            ctx.set_tuning("io_mapped", 0)
            other_desc = "8 fused sub-batches"
        e2e_other = e2e_run()
        ctx.set_tuning("io_batches", nsub)
        ctx.set_tuning("io_mapped", io_mapped)
        ctx.set_tuning("blocks_per_sm", bps0)

    def io_desc(nb, mapped):
        if nb and mapped:
            return ("%d fused sub-batches of ~%d frames, each sub-batch's copies one kernel over the host arrays' "
                    "device view" % (min(nb, F), -(-F // min(nb, F))))
        if nb:
            return ("%d fused sub-batches of ~%d frames, copies overlapping the other sub-batches' computation"
                    % (min(nb, F), -(-F // min(nb, F))))
        return "lanes: each frame's copies and kernels on one of eight streams"
    e2e_schedule = io_desc(nsub, io_mapped)
    h2d = F * wl["N"] * (3 + 3 + 1 + 1) * 8
    d2h = F * len(grid) * NC * 2 * 8
    clocks.stop()

    # ---- plain FP64 GPU path on the same frames + error of the tuned path vs it
    nplain = min(F, 4)
    step("fp64", nplain)  # warm
    ctx.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    step("fp64", nplain)
    ctx.wait_all()
    e1.record(stream)
    ctx.synchronize()
    plain_value = nplain / (e0.elapsed_time(e1) * 1e-3)
    v64 = ctx.get_field(ikabi.FIELD_VIRIAL, slot=0)
    k64 = ctx.get_field(ikabi.FIELD_KINETIC, slot=0)
    ctx.compute_slot(0, "fp32")
    ctx.synchronize()
    v32 = ctx.get_field(ikabi.FIELD_VIRIAL, slot=0)
    k32 = ctx.get_field(ikabi.FIELD_KINETIC, slot=0)

    def relerr(a, b):
        iu = [(0, 0), (1, 1), (0, 1)] if D == 2 else [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
        return [float(np.linalg.norm(a[:, i, j] - b[:, i, j]) / np.linalg.norm(b[:, i, j])) for i, j in iu]

    err_v, err_k = relerr(v32, v64), relerr(k32, k64)

    # ---- roofline of the gather kernel (per-launch CUDA events around it)
    # one frame's gather timed alone (two CTAs per SM, the default for a frame alone; in the
    # lanes schedule the frames' gathers run side by side, one CTA per SM each)
    ctx.set_tuning("blocks_per_sm", 0)
    ctx.set_flags(ikabi.FLAG_TIMING | lane_flags)
    gms, trip, stages = [], [], []
    for k in range(F):
        ctx.compute_slot(k, "fp32")
        ctx.synchronize()
        t4 = ctx.timing()
        stages.append(t4)
        gms.append(t4[2])
        trip.append(ctx.counters(k)[2])
    ctx.set_flags(lane_flags)
    ctx.set_tuning("blocks_per_sm", bps0)
    stage_ms = np.mean(np.array(stages), axis=0)
    g_ms = float(np.mean(gms))
    A = float(np.mean(trip))
    flop = FLOP_PER_TRIPLE[D] * A
    achieved = flop / (g_ms * 1e-3) / 1e12
    per_frame_gather = {"kernel": "k_gather32<KAHAN=%d> (one frame per launch, timed alone)" % (1 if lane_flags else 0),
                        "achieved": achieved, "launch_ms": g_ms, "flop_per_launch": flop}
    roof_kernel = per_frame_gather["kernel"]
    # the fused gather: every frame of the step in one launch (CTAs per SM at the fused default)
    ctx.set_tuning("blocks_per_sm", 0)
    tf_ = [ctx.time_fused_batch(all_slots) for _ in range(4)][1:]
    ctx.set_tuning("blocks_per_sm", bps0)
    fg_ms = float(np.median([t["gather"] for t in tf_]))
    fA = float(sum(ctx.counters(k)[2] for k in range(F)))
    f_flop = FLOP_PER_TRIPLE[D] * fA
    fused_gather = {"kernel": "k_gather32<KAHAN=%d, BATCH> (fused: the %d frames of a step in one launch)" % (
                        1 if lane_flags else 0, F),
                    "achieved": f_flop / (fg_ms * 1e-3) / 1e12, "launch_ms": fg_ms, "flop_per_launch": f_flop}
    stage_ms_fused = {"prepare": float(np.median([t["prepare"] for t in tf_])), "gather": fg_ms,
                      "note": "ms per step of %d frames, CUDA events, no graph" % F}
    if fused0:  # the headline's gather
        g_ms, A, flop, achieved = fg_ms, fA, f_flop, fused_gather["achieved"]
        roof_kernel = fused_gather["kernel"]
    peak = ikabi.measure_fp32_peak(local)
    traffic = None
    traffic_batch_frame = None  # the fused gather's capture: DRAM bytes per frame
    tf = os.path.join(ROOT, "profiles", "traffic_per_launch.txt")
    if os.path.exists(tf):
        for ln in open(tf):
            parts = ln.split()
            if len(parts) >= 3 and parts[0] == "k_gather32" and parts[1] == name:
                traffic = float(parts[2])
            if len(parts) >= 4 and parts[0] == "k_gather32_batch" and parts[1] == name:
                traffic_batch_frame = float(parts[2]) / float(parts[3])

    surrogate = None
    if not args.no_surrogate and wl["cg"]["kind"] == "gaussian" and D == 2:
        surrogate = surrogate_leg(args, ctx, wl, F, stream, all_slots, v64)
    uneven = None
    if not args.no_uneven and name == "ik2d_n64k_g256_gauss":
        uneven = uneven_leg(args)

    out = {"metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator, shapes of the named config)",
           "config": config_of(name, wl, world),
           "e2e": {"value": e2e_value, "unit": "frames/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                   "schedule": e2e_schedule, "tuning": io_tuning,
                   "other_schedule": {"schedule": other_desc, "frames_per_s": e2e_other}},
           "gpu_launches": int(launches),
           "clocks": clocks.summary(t_soak, t_host1),
           "roofline": {"bound": "fp32",
                        "kernel": roof_kernel, "achieved": achieved, "peak": peak,
                        "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic,
                        "flop_per_launch": flop, "active_triples_per_launch": A, "launch_ms": g_ms,
                        "peak_source": "measured live: FFMA throughput probe (ik_measure_fp32_peak)"},
           "host_enqueue_ms_per_step": 1e3 * (t_enq - t_host0) / args.steps,
           "cuda_graph": not args.no_graph,
           "stage_ms_per_frame": {"cells": float(stage_ms[0]), "bonds": float(stage_ms[1]),
                                  "gather": float(stage_ms[2]), "total": float(stage_ms[3]),
                                  "note": "one frame at a time (no overlap), CUDA events"},
           "plain_fp64": {"value": plain_value, "unit": "frames/s", "frames_timed": nplain},
           "tuned_over_plain": value / plain_value,
           "rel_err_vs_fp64": {"virial": err_v, "kinetic": err_k},
           "lane_sums": lane_sums,
           "schedules": schedules,
           "tuning": tuning if tuning is not None else {"schedule": args.schedule},
           "per_frame_gather": per_frame_gather,
           "fused_gather": fused_gather,
           "stage_ms_fused": stage_ms_fused,
           "interactions_per_s": (A / F if fused0 else A) * value}
    if fused0:
        if traffic_batch_frame is not None:  # a smaller fused capture, scaled to the step's frames
            out["roofline"]["traffic"] = traffic_batch_frame * F
            out["roofline"]["traffic_note"] = ("ncu DRAM bytes of a fused gather over fewer frames, per frame "
                                               "x %d frames (the traffic grows in proportion to the frames)" % F)
        elif traffic is not None:  # the capture is of one frame's gather: scaled to the step's frames
            out["roofline"]["traffic"] = traffic * F
            out["roofline"]["traffic_note"] = "ncu DRAM bytes of one frame's gather x %d frames" % F
    if surrogate is not None:
        out["surrogate"] = surrogate
    if uneven is not None:
        out["uneven_batch"] = uneven
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as O
        cores = O.threads(os.cpu_count() or 1)  # threads the oracle's loops actually run on
        G = len(grid)
        t, nf = 0.0, 0  # whole frames, the step's frames cycled, until about 10 s of CPU work
        o0 = []  # the oracle's fields of frame 0: the error of both GPU paths against them
        while nf < 4096 and t < 10.0:
            t += cpu_sample(wl, frames, grid, G, cores, k=nf % len(frames), fields=o0 if nf == 0 else None)
            nf += 1
        out["rel_err_vs_oracle_frame0"] = {
            "tuned_fp32": {"virial": relerr(v32, o0[0][0]), "kinetic": relerr(k32, o0[0][1])},
            "plain_fp64": {"virial": relerr(v64, o0[0][0]), "kinetic": relerr(k64, o0[0][1])},
            "note": "relative L2 per stress component over the grid, FP64 CPU oracle (GL-5) of frame 0"}
        out["cpu_baseline"] = {"value": nf / t, "unit": "frames/s", "cores": cores, "kind": "port",
                               "sample": f"{nf} whole frame(s) of the workload (the step's {len(frames)} frames "
                                         f"cycled), FP64 oracle "
                                         f"restating IrvingKirkwood::compute, OpenMP {cores} threads, {t:.2f} s",
                               "host_cpus": host_cpu_info(),
                               "single_core": single_core_sample(wl, frames, grid)}
    ctx.close()
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    args = parse()
    wl = dict(WORKLOADS[args.workload])
    if args.frames > 0:
        wl["frames"] = args.frames
    if args.impl == "reference":
        reference_arm(args, wl, args.workload)
    else:
        ours(args, wl, args.workload)


if __name__ == "__main__":
    main()
