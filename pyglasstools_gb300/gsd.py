"""Minimal GSD trajectory reader (file layout versions 1.x and 2.x), written from the
public GSD file-format description.  It replaces the ``gsd.hoomd`` Python module
that the reference's ``utils.read_gsd`` uses (pyglasstools/utils.py:5,41-43).

Frame semantics follow the HOOMD schema: a chunk missing from frame ``f`` is taken
from frame 0 when frame 0 has it, else the schema default (mass 1, velocity 0,
diameter 1, box [1,1,1,0,0,0]).
"""
from __future__ import annotations

import os
import struct

import numpy as np

_MAGIC = 0x65DF65DF65DF65DF
_DTYPES = {1: np.uint8, 2: np.uint16, 3: np.uint32, 4: np.uint64, 5: np.int8, 6: np.int16,
           7: np.int32, 8: np.int64, 9: np.float32, 10: np.float64, 11: np.uint8}


class GSDError(ValueError):
    pass


class GSDFile:
    """Read-only random access to the chunks of a GSD file."""

    def __init__(self, path: str):
        self.path = path
        with open(path, "rb") as f:
            self._buf = f.read()
        b = self._buf
        if len(b) < 256:
            raise GSDError(f"{path}: truncated GSD header ({len(b)} bytes)")
        magic, idx_loc, idx_n, nl_loc, nl_n = struct.unpack_from("<QQQQQ", b, 0)
        if magic != _MAGIC:
            raise GSDError(f"{path}: not a GSD file (bad magic)")
        self.schema_version, self.gsd_version = struct.unpack_from("<II", b, 40)
        self.application = b[48:112].split(b"\0", 1)[0].decode(errors="replace")
        self.schema = b[112:176].split(b"\0", 1)[0].decode(errors="replace")
        major = self.gsd_version >> 16
        if major not in (1, 2):
            raise GSDError(f"{path}: unsupported GSD version {major}")
        # name list
        if nl_loc + 64 * nl_n > len(b) or nl_loc >= len(b):
            raise GSDError(f"{path}: truncated name list")
        names = []
        if major == 1:
            for k in range(nl_n):
                raw = b[nl_loc + 64 * k: nl_loc + 64 * (k + 1)].split(b"\0", 1)[0]
                if not raw:
                    break
                names.append(raw.decode())
        else:
            # layout 2.x: a block of namelist_allocated_entries * 64 bytes holding
            # null-terminated names, ended by an empty name
            pos = nl_loc
            end = min(len(b), nl_loc + 64 * nl_n)
            while pos < end:
                stop = b.find(b"\0", pos, end)
                if stop <= pos:
                    break
                names.append(b[pos:stop].decode())
                pos = stop + 1
        self.names = names
        # index
        if idx_loc + 32 * idx_n > len(b):
            raise GSDError(f"{path}: truncated index")
        self._index = {}
        nframes = 0
        for k in range(idx_n):
            frame, N, loc, M, cid, typ, _flags = struct.unpack_from("<QQqIHBB", b, idx_loc + 32 * k)
            if loc == 0:
                continue
            if cid >= len(names):
                raise GSDError(f"{path}: index entry {k} names unknown chunk id {cid}")
            if typ not in _DTYPES:
                raise GSDError(f"{path}: index entry {k} has unknown type {typ}")
            nbytes = N * M * np.dtype(_DTYPES[typ]).itemsize
            if loc < 0 or loc + nbytes > len(b):
                raise GSDError(f"{path}: chunk {names[cid]} of frame {frame} runs past end of file")
            self._index[(frame, names[cid])] = (N, M, loc, typ)
            nframes = max(nframes, frame + 1)
        self.nframes = nframes

    def __len__(self):
        return self.nframes

    def chunk_exists(self, frame: int, name: str) -> bool:
        return (frame, name) in self._index

    def read_chunk(self, frame: int, name: str) -> np.ndarray:
        try:
            N, M, loc, typ = self._index[(frame, name)]
        except KeyError:
            raise GSDError(f"{self.path}: frame {frame} has no chunk {name}") from None
        dt = np.dtype(_DTYPES[typ]).newbyteorder("<")
        a = np.frombuffer(self._buf, dtype=dt, count=N * M, offset=loc)
        return a.reshape(N, M) if M > 1 else a.copy()


class Frame:
    """One HOOMD-schema frame: box, N, position, velocity, mass, diameter (float32
    as stored; callers convert to float64 as the reference's ParticleSystem does)."""

    def __init__(self, box, N, position, velocity, mass, diameter, step):
        self.box = box
        self.N = N
        self.position = position
        self.velocity = velocity
        self.mass = mass
        self.diameter = diameter
        self.step = step


class HOOMDTrajectory:
    """Sequence access to HOOMD-schema frames with frame-0 fallback and defaults."""

    def __init__(self, path: str):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.file = GSDFile(path)
        if self.file.schema != "hoomd":
            raise GSDError(f"{path}: schema '{self.file.schema}' is not 'hoomd'")

    def __len__(self):
        return len(self.file)

    def _get(self, f, name, default):
        if self.file.chunk_exists(f, name):
            return self.file.read_chunk(f, name)
        if self.file.chunk_exists(0, name):
            return self.file.read_chunk(0, name)
        return default

    def __getitem__(self, f: int) -> Frame:
        if f < 0:
            f += len(self)
        if not 0 <= f < len(self):
            raise IndexError(f"frame {f} out of range (0..{len(self) - 1})")
        box = np.asarray(self._get(f, "configuration/box", np.array([1, 1, 1, 0, 0, 0], np.float32)),
                         dtype=np.float32).reshape(-1)
        Narr = self._get(f, "particles/N", np.array([0], np.uint32))
        N = int(np.asarray(Narr).reshape(-1)[0])
        pos = self._get(f, "particles/position", None)
        pos = np.zeros((N, 3), np.float32) if pos is None else np.asarray(pos, np.float32).reshape(-1, 3)
        vel = self._get(f, "particles/velocity", None)
        vel = np.zeros((N, 3), np.float32) if vel is None else np.asarray(vel, np.float32).reshape(-1, 3)
        mass = self._get(f, "particles/mass", None)
        mass = np.ones(N, np.float32) if mass is None else np.asarray(mass, np.float32).reshape(-1)
        diam = self._get(f, "particles/diameter", None)
        diam = np.ones(N, np.float32) if diam is None else np.asarray(diam, np.float32).reshape(-1)
        for nm, a in (("position", pos), ("velocity", vel), ("mass", mass), ("diameter", diam)):
            if len(a) != N:
                raise GSDError(f"{self.file.path}: frame {f} particles/{nm} has {len(a)} rows, N = {N}")
        step = self._get(f, "configuration/step", np.array([0], np.uint64))
        return Frame(box, N, pos, vel, mass, diam, int(np.asarray(step).reshape(-1)[0]))


def open_trajectory(path: str) -> HOOMDTrajectory:
    return HOOMDTrajectory(path)


def upload_frames(ctx, traj, frames, slots=None):
    """Stream GSD frames into resident slots of an engine context (ikabi.IKContext):
    the float32 chunks go to the GPU as stored (half the bytes of FP64) and are
    widened there, with no per-particle Python conversion -- the work the reference's
    data_gsd.update (utils.py:85-101) does with Python lists on every frame."""
    slots = list(range(len(frames))) if slots is None else list(slots)
    for f, s in zip(frames, slots):
        fr = traj[f]
        ctx.upload_frame_f32(s, fr.position, fr.diameter, fr.velocity, fr.mass)
    return slots
