"""Frame input: ``read_gsd`` / ``data_gsd`` / ``simbox`` (pyglasstools/utils.py) on
top of the package's own GSD reader (pyglasstools_gb300.gsd)."""
import os

import numpy as np

import pyglasstools_gb300
from pyglasstools_gb300 import _core, rank
from pyglasstools_gb300 import gsd as _gsd

_pyglasstools = _core._pyglasstools


class simbox(object):
    R"""Simulation box (utils.py:7-39): [-L/2 - origin, L/2 - origin]."""

    def __init__(self, Lx=1.0, Ly=1.0, Lz=1.0, origin=np.zeros(3), ndim=3, L=None, volume=None):
        if ndim == 2:
            Lz = 1.0
        if L is not None:
            self.cppsimbox = _pyglasstools.SimBox(float(L), np.asarray(origin, np.float64), ndim)
        else:
            boxsize = np.array([Lx, Ly, Lz]).astype('float64')
            self.cppsimbox = _pyglasstools.SimBox(boxsize, np.asarray(origin, np.float64), ndim)

    def __getattr__(self, attr):
        return getattr(self.cppsimbox, attr)


def read_gsd(filename, checkpointfile=None, frame_num=0, ndim=2):
    traj = _gsd.open_trajectory(filename)
    return data_gsd(traj, checkpointfile, frame_num, ndim)


def _as64(a, shape=None):
    a = np.asarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


class data_gsd(object):
    R"""Particle data of one GSD frame (utils.py:45-141).  ``update(f)`` builds the
    frame's ParticleSystem; the box of each frame is used (the reference keeps
    the frame-0 box because update() assigns ``self.simbox`` but rebuilds from
    ``self.pysimbox``; the two agree whenever the box is constant)."""

    def __init__(self, traj_gsd, checkpointfile, frame_num, ndim=2):
        self.frame_num = frame_num
        self.checkpointfile = checkpointfile
        self.traj = traj_gsd
        self.ndim = ndim
        self._load(frame_num)
        pyglasstools_gb300.set_sysdata(self)

    def _load(self, frame_num):
        fr = self.traj[frame_num]
        self.pysimbox = simbox(Lx=float(fr.box[0]), Ly=float(fr.box[1]), Lz=float(fr.box[2]), ndim=self.ndim)
        self.cppparticledata = _pyglasstools.ParticleSystem(
            self.pysimbox.cppsimbox, int(fr.N), _as64(fr.diameter), _as64(fr.mass),
            _as64(fr.position, (-1, 3)), _as64(fr.velocity, (-1, 3)))

    def setup_checkpoint(self, frame_list):
        frame_list = list(frame_list)
        if self.checkpointfile is not None and not os.path.exists(self.checkpointfile):
            if rank == 0:
                with open(self.checkpointfile, "w") as f:
                    f.write("Frame {}".format(frame_list[0]))
        elif self.checkpointfile is not None and os.path.exists(self.checkpointfile):
            with open(self.checkpointfile, "r") as f:
                frame_num = int(f.readline().split(' ')[1])
            frame_list = [i for i in range(frame_num, frame_list[-1] + 1)]
        return frame_list

    def update(self, frame_num):
        if frame_num != self.frame_num:
            self._load(frame_num)
            self.frame_num = frame_num

    def move_particles(self, displacement=None):
        if displacement is None:
            self.cppparticledata.moveParticles()
        else:
            self.cppparticledata.moveParticles(displacement)

    def set_displacement(self, displacement):
        self.cppparticledata.setDisplacement(displacement)

    def get_displacement(self):
        return self.cppparticledata.getDisplacement()

    def set_diameters(self, diameter):
        self.cppparticledata.setDiameter(np.asarray(diameter, np.float64))

    def get_diameters(self):
        return self.cppparticledata.getDiameter()

    def set_mass(self, mass):
        self.cppparticledata.setMass(np.asarray(mass, np.float64))

    def get_mass(self):
        return self.cppparticledata.getMass()

    def set_position(self, position):
        self.cppparticledata.setAtomPosition(np.asarray(position, np.float64))

    def get_position(self):
        return self.cppparticledata.getAtomPosition()

    def set_velocity(self, velocity):
        self.cppparticledata.setAtomVelocity(np.asarray(velocity, np.float64))

    def get_velocity(self):
        return self.cppparticledata.getAtomVelocity()

    def get_neighbors(self, point, radius):
        return self.cppparticledata.getNeighbors(point, radius)

    def get_neighborsdistance(self, tag, radius):
        return self.cppparticledata.getNeighborsDistance(tag, radius)


class data_arrays(data_gsd):
    R"""In-memory frames (no GSD file): ``frames`` is a list of objects with
    ``pos`` (n,3), ``diam`` (n,), optional ``vel`` (n,3), ``mass`` (n,) and ``L``."""

    def __init__(self, frames, ndim=2, checkpointfile=None, frame_num=0):
        self.frames = frames
        self.traj = None
        self.ndim = ndim
        self.checkpointfile = checkpointfile
        self.frame_num = frame_num
        self._load(frame_num)
        pyglasstools_gb300.set_sysdata(self)

    def _load(self, frame_num):
        fr = self.frames[frame_num]
        L = np.broadcast_to(np.asarray(fr.L, np.float64), (3,))
        self.pysimbox = simbox(Lx=L[0], Ly=L[1], Lz=L[2], ndim=self.ndim)
        n = len(fr.pos)
        vel = getattr(fr, "vel", None)
        mass = getattr(fr, "mass", None)
        self.cppparticledata = _pyglasstools.ParticleSystem(
            self.pysimbox.cppsimbox, n, _as64(fr.diam), _as64(np.ones(n) if mass is None else mass),
            _as64(fr.pos, (-1, 3)), _as64(np.zeros((n, 3)) if vel is None else vel, (-1, 3)))
