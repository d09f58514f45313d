"""ctypes binding of the C ABI in include/ik_gb300.h (libik_gb300.so).

This is the low-level route a host program takes without the pybind11 layer:
plain pointers and sizes, one status code per call, ``ik_last_error()`` text on
failure (raised here as ``IKError``).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libik_gb300.so")

IK_OK = 0
ERR = {-1: "IK_ERR_ARG", -2: "IK_ERR_CUDA", -3: "IK_ERR_STATE", -4: "IK_ERR_BOX",
       -5: "IK_ERR_CAPACITY", -6: "IK_ERR_TIMEOUT", -7: "IK_ERR_NOMEM", -8: "IK_ERR_UNSUPPORTED",
       -9: "IK_ERR_QUADRATURE"}
CG = {"octic": 0, "gaussian": 1, "rect": 2, "mollifier": 3}
QUAD = {"fixedpoint": 0, "adaptive": 1, "exact": 2, "mlp": 3, "clipped": 4}
PREC = {"fp64": 0, "fp32": 1}
FIELD_VIRIAL, FIELD_KINETIC, FIELD_ELASTIC = 1, 2, 4
FLAG_TIMING, FLAG_LANE_KAHAN, FLAG_CSR_BONDS = 1, 2, 4
TUNE = {"bin_points": 1, "blocks_per_sm": 2, "halo_cap": 3, "fused_batch": 4, "io_batches": 5, "io_mapped": 6}
POT = {"poly12": 0, "lj": 1, "fslj": 2, "poly10": 3, "poly106": 4, "poly18": 5, "polylj": 6,
       "polyyukawa": 7}

_lib = None


class IKError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERR.get(code, code)}: {msg}")
        self.code = code


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is not built (python -m pyglasstools_gb300._build)")
        L = C.CDLL(LIB_PATH)
        vp, dp, i64, i32 = C.c_void_p, C.POINTER(C.c_double), C.c_int64, C.c_int
        fp = C.POINTER(C.c_float)
        sig = {
            "ik_last_error": ([], C.c_char_p),
            "ik_version": ([], i32),
            "ik_create": ([C.POINTER(vp), i32], i32),
            "ik_destroy": ([vp], i32),
            "ik_set_box": ([vp, i32, dp, dp], i32),
            "ik_set_potential_poly12": ([vp, C.c_double, dp], i32),
            "ik_set_potential": ([vp, i32, C.c_double, dp, i32], i32),
            "ik_potential_nparams": ([i32], i32),
            "ik_compute_thermo": ([vp, i32, dp, i64], i32),
            "ik_compute_batch_io": ([vp, C.POINTER(i32), i32, i32, i32, C.POINTER(i64), C.POINTER(dp), C.POINTER(dp),
                                     C.POINTER(dp), C.POINTER(dp), C.POINTER(dp)], i32),
            "ik_autotune_batch_io": ([vp, C.POINTER(i32), i32, i32, i32, C.POINTER(i64), C.POINTER(dp),
                                      C.POINTER(dp), C.POINTER(dp), C.POINTER(dp), C.POINTER(dp), i32,
                                      C.POINTER(i32), C.POINTER(C.c_float)], i32),
            "ik_gk15_rule": ([dp, dp, dp], i32),
            "ik_set_cgfunc": ([vp, i32, i32, i32, C.c_double, C.c_double], i32),
            "ik_set_adaptive": ([vp, i32, C.c_double, C.c_double], i32),
            "ik_set_max_rcut": ([vp, C.c_double], i32),
            "ik_get_max_rcut": ([vp, dp], i32),
            "ik_set_grid": ([vp, i64, dp], i32),
            "ik_reserve_slots": ([vp, i32], i32),
            "ik_set_slot_geometry": ([vp, i32, i32, dp, dp, i64, dp], i32),
            "ik_upload_displacement": ([vp, i32, i64, dp], i32),
            "ik_upload_frame_f32": ([vp, i32, i64, fp, fp, fp, fp], i32),
            "ik_upload_frame": ([vp, i32, i64, dp, dp, dp, dp], i32),
            "ik_set_frame": ([vp, i64, dp, dp, dp, dp], i32),
            "ik_compute_slot": ([vp, i32, i32, i32], i32),
            "ik_synchronize": ([vp], i32),
            "ik_compute": ([vp, i32, i32], i32),
            "ik_get_field": ([vp, i32, i32, dp, i64], i32),
            "ik_get_neighbors": ([vp, i32, C.c_double, C.POINTER(C.c_int64), C.POINTER(C.c_int32), i64,
                                  C.POINTER(C.c_int64)], i32),
            "ik_get_neighbors_point": ([vp, i32, dp, C.c_double, C.POINTER(C.c_int32), i64,
                                        C.POINTER(C.c_int64)], i32),
            "ik_eval_pair": ([vp, i64, dp, dp, dp, dp, dp], i32),
            "ik_eval_bond": ([vp, i64, dp, dp, dp, dp, dp], i32),
            "ik_set_flags": ([vp, i32], i32),
            "ik_get_timing": ([vp, C.POINTER(C.c_float)], i32),
            "ik_get_counters": ([vp, i32, C.POINTER(C.c_int64)], i32),
            "ik_get_stream": ([vp, C.POINTER(vp)], i32),
            "ik_download_field_async": ([vp, i32, i32, dp, i64], i32),
            "ik_measure_fp32_peak": ([i32, dp], i32),
            "ik_get_launch_count": ([vp, C.POINTER(C.c_int64)], i32),
            "ik_wait_all": ([vp], i32),
            "ik_compute_batch": ([vp, C.POINTER(C.c_int), i32, i32, i32], i32),
            "ik_set_mlp": ([vp, vp], i32),
            "ik_set_tuning": ([vp, i32, i32], i32),
            "ik_time_fused_batch": ([vp, C.POINTER(C.c_int), i32, i32, C.POINTER(C.c_float)], i32),
            "ik_get_tuning": ([vp, i32, C.POINTER(C.c_int)], i32),
            "ik_autotune_batch": ([vp, C.POINTER(C.c_int), i32, i32, i32, i32, C.POINTER(C.c_int),
                                   C.POINTER(C.c_int), C.POINTER(C.c_float)], i32),
            "ik_get_mlp_records": ([vp, i32, C.POINTER(C.c_int64)], i32),
            "ik_get_mlp_fallbacks": ([vp, i32, C.POINTER(C.c_int64)], i32),
            "ik_mlp_create": ([C.POINTER(vp), i32], i32),
            "ik_mlp_destroy": ([vp], i32),
            "ik_mlp_num_params": ([], i32),
            "ik_mlp_init": ([vp, C.c_uint64], i32),
            "ik_mlp_set_params": ([vp, fp, i64], i32),
            "ik_mlp_get_params": ([vp, fp, i64], i32),
            "ik_mlp_samples": ([vp, i64, C.c_uint64, fp, dp], i32),
            "ik_mlp_grad": ([vp, i64, fp, fp, fp, dp], i32),
            "ik_mlp_train": ([vp, i64, i32, i32, C.c_double, C.c_uint64, dp, i64], i32),
            "ik_mlp_eval": ([vp, i64, fp, fp, i32], i32),
            "ik_mlp_test_stall": ([vp, i32], i32),
            "ik_mlp_validate": ([vp, i64, C.c_uint64, C.c_double, dp, dp, dp, dp, i64], i32),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _fp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def _c64(a, shape=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


def check_io_arrays(slots, frames, outs):
    """Arguments of IKContext.compute_batch_io, checked before their raw pointers go to the
    device copies: one (pos, diam, vel, mass) frame and one (virial, kinetic, elastic)
    output triple per slot; every array C-contiguous float64 (outputs also writeable);
    pos and vel n x 3, diam and mass n (n = len(diam)); vel, mass and outputs may be None.
    Raises ValueError."""
    if not (len(slots) == len(frames) == len(outs)) or len(slots) == 0:
        raise ValueError("compute_batch_io: one frame and one output triple per slot")

    def ok(a, what, shape, out=False):
        if a is None:
            return
        if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
            raise ValueError(f"compute_batch_io: {what} must be a C-contiguous float64 array")
        if out and not a.flags.writeable:
            raise ValueError(f"compute_batch_io: {what} must be writeable")
        if shape is not None and a.shape != shape:
            raise ValueError(f"compute_batch_io: {what} has shape {a.shape}, expected {shape}")

    for k, (f, o) in enumerate(zip(frames, outs)):
        if len(f) != 4 or len(o) != 3:
            raise ValueError(f"compute_batch_io: frame {k} needs (pos, diam, vel, mass) and (virial, kinetic, elastic)")
        pos, diam, vel, mass = f
        if pos is None or diam is None:
            raise ValueError(f"compute_batch_io: frame {k} needs positions and diameters")
        ok(diam, f"frame {k} diam", None)
        if diam.ndim != 1:
            raise ValueError(f"compute_batch_io: frame {k} diam must be one-dimensional")
        n = len(diam)
        ok(pos, f"frame {k} pos", (n, 3))
        ok(vel, f"frame {k} vel", (n, 3))
        ok(mass, f"frame {k} mass", (n,))
        for q, name in enumerate(("virial", "kinetic", "elastic")):
            ok(o[q], f"frame {k} {name} output", None, out=True)


def check(rc):
    if rc != IK_OK:
        raise IKError(rc, lib().ik_last_error().decode(errors="replace"))


class IKContext:
    """One engine context (one CUDA stream) -- see include/ik_gb300.h."""

    def __init__(self, device=0):
        self._h = C.c_void_p()
        check(lib().ik_create(C.byref(self._h), device))
        self.dim = None
        self.G = 0

    def close(self):
        if self._h:
            lib().ik_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # configuration ---------------------------------------------------------
    def set_box(self, dim, boxsize, origin=(0.0, 0.0, 0.0)):
        b = np.broadcast_to(np.asarray(boxsize, np.float64), (3,)).copy()
        o = np.asarray(origin, np.float64).copy()
        check(lib().ik_set_box(self._h, dim, _dp(b), _dp(o)))
        self.dim = dim

    def set_poly12(self, v0=1.0, eps=0.2, rcut=1.25):
        p = np.array([v0, eps, -28.0 * v0 / rcut ** 12, 48.0 * v0 / rcut ** 14, -21.0 * v0 / rcut ** 16])
        check(lib().ik_set_potential_poly12(self._h, rcut, _dp(p)))

    def set_potential(self, kind, rcut, params):
        """Any of the eight pair models (POT), params in the reference's order."""
        p = np.ascontiguousarray(params, dtype=np.float64)
        check(lib().ik_set_potential(self._h, POT[kind] if isinstance(kind, str) else int(kind), rcut,
                                     _dp(p), len(p)))

    def set_cgfunc(self, kind, rcut, mode="fixedpoint", order=5, width=0.0):
        check(lib().ik_set_cgfunc(self._h, CG[kind], QUAD[mode], order, rcut, width))

    def set_adaptive(self, neval, relerr, abserr):
        """Tolerances of the adaptive bond integral (AdaptiveCGFunc(neval, relerr, abserr, rcut))."""
        check(lib().ik_set_adaptive(self._h, int(neval), float(relerr), float(abserr)))

    def set_max_rcut(self, r):
        check(lib().ik_set_max_rcut(self._h, r))

    def get_max_rcut(self):
        v = C.c_double()
        check(lib().ik_get_max_rcut(self._h, C.byref(v)))
        return v.value

    def set_grid(self, grid):
        g = _c64(grid, (-1, 3))
        check(lib().ik_set_grid(self._h, len(g), _dp(g)))
        self.G = len(g)

    def set_flags(self, flags):
        check(lib().ik_set_flags(self._h, flags))

    # frames ----------------------------------------------------------------
    def reserve_slots(self, n):
        check(lib().ik_reserve_slots(self._h, n))

    def upload_frame_f32(self, slot, pos, diam, vel=None, mass=None):
        """Upload float32 arrays (e.g. GSD chunks) into a slot; widened to FP64 on the GPU."""
        f = lambda a, shape=None: None if a is None else np.ascontiguousarray(a, dtype=np.float32).reshape(
            shape if shape else -1)
        p, d, v, m = f(pos, (-1, 3)), f(diam), f(vel, (-1, 3)), f(mass)
        self._keep = (p, d, v, m)  # the copies may be asynchronous (pinned memory)
        check(lib().ik_upload_frame_f32(self._h, slot, len(p), _fp(p), _fp(v), _fp(m), _fp(d)))

    def upload_displacement(self, disp, slot=0):
        """Per-particle displacements (n x 3) for the elastic virial field."""
        d = _c64(disp, (-1, 3))
        check(lib().ik_upload_displacement(self._h, slot, len(d), _dp(d)))

    def set_slot_geometry(self, slot, dim, box, grid, origin=(0.0, 0.0, 0.0)):
        """Give `slot` a box and grid of its own (uneven batches)."""
        b = _c64(box)
        o = _c64(origin)
        g = _c64(grid, (-1, 3))
        check(lib().ik_set_slot_geometry(self._h, slot, dim, _dp(b), _dp(o), len(g), _dp(g)))
        self.slot_G = getattr(self, "slot_G", {})
        self.slot_G[slot] = len(g)
        if self.dim is None:
            self.dim = dim

    def upload_frame(self, slot, pos, diam, vel=None, mass=None):
        pos = _c64(pos, (-1, 3))
        diam = _c64(diam)
        vel = _c64(vel, (-1, 3))
        mass = _c64(mass)
        self._keep = (pos, diam, vel, mass)  # alive until the async copy completes
        check(lib().ik_upload_frame(self._h, slot, len(diam), _dp(pos), _dp(vel), _dp(mass), _dp(diam)))

    def set_frame(self, pos, diam, vel=None, mass=None):
        self.upload_frame(0, pos, diam, vel, mass)
        self.synchronize()

    def compute_slot(self, slot, precision="fp32", fields=FIELD_VIRIAL | FIELD_KINETIC):
        check(lib().ik_compute_slot(self._h, slot, PREC[precision], fields))

    def set_tuning(self, param, value):
        check(lib().ik_set_tuning(self._h, TUNE[param], int(value)))

    def get_tuning(self, param):
        v = C.c_int()
        check(lib().ik_get_tuning(self._h, TUNE[param], C.byref(v)))
        return v.value

    def autotune_batch(self, slots, precision="fp32", fields=FIELD_VIRIAL | FIELD_KINETIC, reps=3):
        """Time the batch under each candidate tuning, keep the fastest; returns it."""
        arr = (C.c_int * len(slots))(*slots)
        bp, bk, ms = C.c_int(), C.c_int(), C.c_float()
        check(lib().ik_autotune_batch(self._h, arr, len(slots), PREC[precision], fields, reps, C.byref(bp),
                                      C.byref(bk), C.byref(ms)))
        return {"bin_points": bp.value, "blocks_per_sm": bk.value, "halo_cap": self.get_tuning("halo_cap"),
                "fused_batch": self.get_tuning("fused_batch"), "ms_per_batch": ms.value}

    def time_fused_batch(self, slots, fields=FIELD_VIRIAL | FIELD_KINETIC):
        """Run the batch once fused (no graph) with CUDA events around its stages:
        {"prepare", "gather", "total"} in ms."""
        arr = (C.c_int * len(slots))(*slots)
        ms = (C.c_float * 4)()
        check(lib().ik_time_fused_batch(self._h, arr, len(slots), fields, ms))
        return {"prepare": ms[0], "gather": ms[2], "total": ms[3]}

    def set_mlp(self, mlp):
        """Attach a validated surrogate (MLP) used by cgfunc mode "mlp" on the FP32 path."""
        check(lib().ik_set_mlp(self._h, None if mlp is None else mlp._h))
        self._mlp = mlp

    def compute_batch(self, slots, precision="fp32", fields=FIELD_VIRIAL | FIELD_KINETIC):
        """Compute several slots as one batch (replayed as a CUDA graph after the first call)."""
        arr = (C.c_int * len(slots))(*slots)
        check(lib().ik_compute_batch(self._h, arr, len(slots), PREC[precision], fields))

    def synchronize(self):
        check(lib().ik_synchronize(self._h))

    def wait_all(self):
        """Main stream waits (on the device) for all enqueued work."""
        check(lib().ik_wait_all(self._h))

    def compute(self, precision="fp32", fields=FIELD_VIRIAL | FIELD_KINETIC):
        check(lib().ik_compute(self._h, PREC[precision], fields))

    def get_field(self, field=FIELD_VIRIAL, slot=0):
        D = self.dim
        G = getattr(self, "slot_G", {}).get(slot, self.G)
        out = np.zeros((G, D, D))
        check(lib().ik_get_field(self._h, slot, field, _dp(out), out.size))
        # column-major per grid point -> [g, a, b] = T_ab (symmetric)
        return out.transpose(0, 2, 1).copy()

    # queries ---------------------------------------------------------------
    def neighbors(self, radius, slot=0, n=None):
        if n is None:
            raise ValueError("pass n = number of particles of the slot")
        offs = np.zeros(n + 1, np.int64)
        nnz = C.c_int64()
        check(lib().ik_get_neighbors(self._h, slot, radius, offs.ctypes.data_as(C.POINTER(C.c_int64)), None, 0,
                                     C.byref(nnz)))
        idx = np.zeros(max(nnz.value, 1), np.int32)
        check(lib().ik_get_neighbors(self._h, slot, radius, offs.ctypes.data_as(C.POINTER(C.c_int64)),
                                     idx.ctypes.data_as(C.POINTER(C.c_int32)), nnz.value, C.byref(nnz)))
        return offs, idx[:nnz.value]

    def neighbors_point(self, point, radius, slot=0):
        p = np.asarray(point, np.float64).copy()
        cnt = C.c_int64()
        check(lib().ik_get_neighbors_point(self._h, slot, _dp(p), radius, None, 0, C.byref(cnt)))
        ids = np.zeros(max(cnt.value, 1), np.int32)
        check(lib().ik_get_neighbors_point(self._h, slot, _dp(p), radius, ids.ctypes.data_as(C.POINTER(C.c_int32)),
                                           cnt.value, C.byref(cnt)))
        return ids[:cnt.value]

    def eval_pair(self, rij, di, dj):
        rij = _c64(rij, (-1, 3))
        di = _c64(di)
        dj = _c64(dj)
        f = np.zeros(len(di))
        e = np.zeros(len(di))
        check(lib().ik_eval_pair(self._h, len(di), _dp(rij), _dp(di), _dp(dj), _dp(f), _dp(e)))
        return f, e

    def eval_bond(self, x, ri, rij):
        x = _c64(x, (-1, 3))
        ri = _c64(ri, (-1, 3))
        rij = _c64(rij, (-1, 3))
        b = np.zeros(len(x))
        d = np.zeros(len(x))
        check(lib().ik_eval_bond(self._h, len(x), _dp(x), _dp(ri), _dp(rij), _dp(b), _dp(d)))
        return b, d

    def timing(self):
        t = (C.c_float * 4)()
        check(lib().ik_get_timing(self._h, t))
        return list(t)

    def stream(self):
        v = C.c_void_p()
        check(lib().ik_get_stream(self._h, C.byref(v)))
        return v.value

    def download_field_async(self, out, field=FIELD_VIRIAL, slot=0):
        """out: C-contiguous float64 (G, NC) host array (pinned for overlap)."""
        if not (isinstance(out, np.ndarray) and out.dtype == np.float64 and out.flags.c_contiguous
                and out.flags.writeable):
            raise ValueError("download_field_async: out must be a writeable C-contiguous float64 array")
        check(lib().ik_download_field_async(self._h, slot, field, _dp(out), out.size))

    def launch_count(self):
        v = C.c_int64()
        check(lib().ik_get_launch_count(self._h, C.byref(v)))
        return v.value

    def compute_batch_io(self, slots, frames, outs, precision="fp32", fields=FIELD_VIRIAL | FIELD_KINETIC):
        """One CUDA-graph batch with host I/O (ik_compute_batch_io).  frames[k] =
        (pos, diam, vel, mass) page-locked float64 arrays (vel / mass may be None);
        outs[k] = (virial, kinetic, elastic) page-locked float64 (g, NC) arrays or None.
        Complete after synchronize()."""
        sl, cnt, nn, pos, vel, mass, diam, out = self._io_call_args(slots, frames, outs)
        check(lib().ik_compute_batch_io(self._h, sl, cnt, PREC[precision], fields, nn, pos, vel, mass, diam, out))

    def _io_call_args(self, slots, frames, outs):
        """The ctypes arguments of a host-I/O batch, kept while the same arrays come back
        (the arrays held, so their ids stay theirs)."""
        arrays = tuple(a for f in frames for a in f) + tuple(o for os_ in outs for o in os_)
        ids = tuple(map(id, arrays))
        cached = getattr(self, "_io_args", None)
        if cached is None or cached[0] != ids or cached[2] != list(slots):
            check_io_arrays(slots, frames, outs)
            cnt = len(slots)
            P = C.POINTER(C.c_double)
            ptr = lambda a: a.ctypes.data_as(P) if a is not None else None
            args = ((C.c_int * cnt)(*slots), cnt, (C.c_int64 * cnt)(*[len(f[1]) for f in frames]),
                    (P * cnt)(*[ptr(f[0]) for f in frames]), (P * cnt)(*[ptr(f[2]) for f in frames]),
                    (P * cnt)(*[ptr(f[3]) for f in frames]), (P * cnt)(*[ptr(f[1]) for f in frames]),
                    (P * (3 * cnt))(*[ptr(o) for os_ in outs for o in os_]))
            self._io_args = cached = (ids, arrays, list(slots), args)
        return cached[3]

    def autotune_batch_io(self, slots, frames, outs, precision="fp32", fields=FIELD_VIRIAL | FIELD_KINETIC, reps=3):
        """Time compute_batch_io (arguments as there) under each schedule of its copies --
        per frame on the lanes, or fused sub-batches -- keep the fastest; returns
        {"io_batches", "io_mapped", "blocks_per_sm", "ms_per_batch"} (io_batches 0: the lanes)."""
        sl, cnt, nn, pos, vel, mass, diam, out = self._io_call_args(slots, frames, outs)
        nb, ms = C.c_int(), C.c_float()
        check(lib().ik_autotune_batch_io(self._h, sl, cnt, PREC[precision], fields, nn, pos, vel, mass, diam, out,
                                         reps, C.byref(nb), C.byref(ms)))
        return {"io_batches": nb.value, "io_mapped": self.get_tuning("io_mapped"),
                "blocks_per_sm": self.get_tuning("blocks_per_sm"), "ms_per_batch": ms.value}

    def compute_thermo(self, slot=0):
        """Global observables of a slot's frame: dict of potentialenergy (float),
        virialstress, elasticvirialstress, kineticstress ([a, b]) and borntensor
        ([i, j, k, l]), each per unit volume."""
        D = self.dim
        out = np.zeros(1 + 3 * D * D + D ** 4)
        check(lib().ik_compute_thermo(self._h, slot, _dp(out), len(out)))
        D2 = D * D
        t = lambda k: out[1 + k * D2:1 + (k + 1) * D2].reshape(D, D).T.copy()
        return {"potentialenergy": float(out[0]), "virialstress": t(0), "elasticvirialstress": t(1),
                "kineticstress": t(2), "borntensor": out[1 + 3 * D2:].reshape(D, D, D, D).transpose(3, 2, 1, 0).copy()}

    def counters(self, slot=0):
        c = (C.c_int64 * 3)()
        check(lib().ik_get_counters(self._h, slot, c))
        return list(c)

    def mlp_records(self, slot=0):
        v = C.c_int64()
        check(lib().ik_get_mlp_records(self._h, slot, C.byref(v)))
        return v.value

    def mlp_fallbacks(self, slot=0):
        """Surrogate records of the last computation that kept their fixed-point value."""
        v = C.c_int64()
        check(lib().ik_get_mlp_fallbacks(self._h, slot, C.byref(v)))
        return v.value


def measure_fp32_peak(device=0):
    v = C.c_double()
    check(lib().ik_measure_fp32_peak(device, C.byref(v)))
    return v.value


MLP_BINS = 2 * 12 * 24 * 16   # (w, d, a, b) bins of the surrogate's use table


class MLP:
    """Learned bond-integral surrogate (ik_mlp_* in include/ik_gb300.h)."""

    def __init__(self, device=0):
        self._h = C.c_void_p()
        check(lib().ik_mlp_create(C.byref(self._h), device))
        self.nparams = lib().ik_mlp_num_params()

    def close(self):
        if self._h:
            lib().ik_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init(self, seed=0):
        check(lib().ik_mlp_init(self._h, seed))

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(lib().ik_mlp_set_params(self._h, _fp(p), p.size))

    def get_params(self):
        p = np.empty(self.nparams, dtype=np.float32)
        check(lib().ik_mlp_get_params(self._h, _fp(p), p.size))
        return p

    def samples(self, n, seed=0):
        """n seeded samples {d, a, b, w} (float32) and their labels B (float64)."""
        f = np.empty((n, 4), dtype=np.float32)
        lab = np.empty(n, dtype=np.float64)
        check(lib().ik_mlp_samples(self._h, n, seed, _fp(f), _dp(lab)))
        return f, lab

    def grad(self, feats, targets):
        f = np.ascontiguousarray(feats, dtype=np.float32)
        y = np.ascontiguousarray(targets, dtype=np.float32)
        g = np.empty(self.nparams, dtype=np.float32)
        loss = C.c_double()
        check(lib().ik_mlp_grad(self._h, len(f), _fp(f), _fp(y), _fp(g), C.byref(loss)))
        return g, loss.value

    def train(self, nsamples=1 << 22, epochs=10, ctas=152, lr=2e-3, seed=1):
        batch = ctas * 128
        steps = ((nsamples + batch - 1) // batch) * epochs
        hist = np.zeros(steps, dtype=np.float64)
        check(lib().ik_mlp_train(self._h, nsamples, epochs, ctas, lr, seed, _dp(hist), steps))
        return hist

    def test_stall(self, on=True):
        """Failure-detection test hook: the tensor-core kernels issue no MMA and their
        bounded completion wait runs out (IK_ERR_TIMEOUT) until turned off again."""
        check(lib().ik_mlp_test_stall(self._h, 1 if on else 0))

    def eval(self, feats, kernel=0, raw=False):
        """kernel 0: tensor cores (BF16); 1: CUDA cores, BF16 arithmetic; 2: CUDA cores, FP32.
        raw: the network's output y = (B / base - 1) * 1e4 instead of B."""
        f = np.ascontiguousarray(feats, dtype=np.float32)
        out = np.empty(len(f), dtype=np.float32)
        check(lib().ik_mlp_eval(self._h, len(f), _fp(f), _fp(out), kernel | (4 if raw else 0)))
        return out

    def validate(self, n=1 << 20, seed=7, tol=1e-6):
        cov, mx, rms = C.c_double(), C.c_double(), C.c_double()
        bins = np.zeros(MLP_BINS, dtype=np.float64)
        check(lib().ik_mlp_validate(self._h, n, seed, tol, C.byref(cov), C.byref(mx), C.byref(rms), _dp(bins),
                                    MLP_BINS))
        return {"coverage": cov.value, "max_err": mx.value, "rms_err": rms.value, "bin_max_err": bins}
