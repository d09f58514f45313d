"""Output (pyglasstools/io.py): ``logfile(filename, names, solver)`` for the global
observables of ``thermo.calculator``, and ``fieldlogger(keyword, names, solver)``
writes ``<keyword>.xyz`` -- per frame a ``gridsize`` line, a ``#Frame n`` line, then
one line per grid point ``1 x y [z] T_ab ...`` with the values formatted like a
default C++ ostream (6 significant digits)."""
import os

import numpy as np

import pyglasstools_gb300
from pyglasstools_gb300 import _core, comm, loggers_list, rank, size
from pyglasstools_gb300 import irvingkirkwood

_pyglasstools = _core._pyglasstools
_irvingkirkwood = _core._irvingkirkwood


class logfile(object):
    R"""Global observables, one line per frame (pyglasstools/io.py:9-80): a header
    ``Frame name ...`` (unless resuming from a non-empty checkpoint), then per frame
    ``frame v v ...`` with each value as std::to_string writes it (six decimals).
    Names: ``potentialenergy``, ``virialstress_ab``, ``elasticvirialstress_ab``,
    ``kineticstress_ab``, ``borntensor_ijkl``.  (The reference looks elastic names up
    under 'virialstress', which it never creates for them; here they read the elastic
    observable.)"""

    def __init__(self, filename, names, solver):
        self.filename = filename
        self.__obs_names = names
        if solver is None:
            raise ValueError("[ERROR] User must specify solver object!")
        if names is None:
            raise ValueError("[ERROR] User must specify list of observables to save!")
        if filename is None:
            raise ValueError("[ERROR] User must specify a filename for the logfile!")
        from pyglasstools_gb300 import thermo
        self.solver = solver
        loggers_list.append(self)
        self.file = _pyglasstools.MPILogFile(comm, self.filename)
        sysdata = pyglasstools_gb300.get_sysdata()
        self.global_obs = thermo.initialize_global(self.__obs_names, sysdata.pysimbox.dim)
        self.solver.add_observables(self.global_obs)
        ck = sysdata.checkpointfile
        if rank == 0 and (ck is None or not os.path.exists(ck) or os.path.getsize(ck) == 0):
            self.file.write_shared("{} ".format("Frame"))
            for name in self.__obs_names:
                self.file.write_shared("{} ".format(name))
            self.file.write_shared("\n")
            self.file.flush()

    def save(self, frame_num):
        if rank == 0:
            Dim = pyglasstools_gb300.get_sysdata().pysimbox.dim
            self.file.write_shared("{} ".format(frame_num))
            for name in self.__obs_names:
                if "potentialenergy" in name:
                    self.global_obs['potentialenergy'].save(self.file, 0)
                    self.file.write_shared(" ")
                if "virialstress" in name:
                    i, j = int(name[-2]), int(name[-1])
                    key = 'elasticvirialstress' if "elastic" in name else 'virialstress'
                    self.global_obs[key].save(self.file, i + Dim * j)
                    self.file.write_shared(" ")
                elif "kineticstress" in name:
                    i, j = int(name[-2]), int(name[-1])
                    self.global_obs['kineticstress'].save(self.file, i + Dim * j)
                    self.file.write_shared(" ")
                elif "borntensor" in name:
                    i, j, k, l = (int(c) for c in name[-4:])
                    self.global_obs['borntensor'].save(self.file, l + Dim * (k + Dim * (j + Dim * i)))
                    self.file.write_shared(" ")
            self.file.write_shared("\n")
            self.file.flush()


class fieldlogger(object):
    def __init__(self, keyword, names, solver):
        self.__obs_names = names
        if solver is None:
            raise ValueError("[ERROR] User must specify solver object!")
        if names is None:
            raise ValueError("[ERROR] User must specify list of observables to save!")
        self.solver = solver
        loggers_list.append(self)
        self.field_obs = irvingkirkwood.initialize_field(
            self.__obs_names, pyglasstools_gb300.get_sysdata().pysimbox.dim, self.solver.gridpoints)
        self.solver.add_observables(self.field_obs)
        self.file = _pyglasstools.MPILogFile(comm, "{}".format(keyword) + ".xyz")

    def _components(self, Dim):
        return [(self.field_obs[name[:-3]], int(name[-2]) + Dim * int(name[-1])) for name in self.__obs_names]

    def save_perrank(self, frame_num):
        """``1 x y [z] T...`` per grid point (io.py:112-128), formatted natively in one
        pass (the same text as the per-point gettostring loop)."""
        Dim = pyglasstools_gb300.get_sysdata().pysimbox.dim
        gp = np.asarray(self.solver.gridpoints, dtype=np.float64)
        cols = gp[:, :3] if Dim == 3 else gp[:, :2]
        self.file.write_shared(_irvingkirkwood.format_field_lines(cols, self._components(Dim)))

    def save_perrank_polar(self, frame_num):
        """``1 id r theta T...`` per grid point of a radialcalculator (io.py:130-144)."""
        Dim = pyglasstools_gb300.get_sysdata().pysimbox.dim
        cols = np.stack([np.asarray(self.solver.gridid, dtype=np.float64),
                         np.asarray(self.solver.globalr, dtype=np.float64),
                         np.asarray(self.solver.globaltheta, dtype=np.float64)], axis=1)
        self.file.write_shared(_irvingkirkwood.format_field_lines(cols, self._components(Dim), [0]))

    def save(self, frame_num):
        if rank == 0:
            self.file.write_shared("{:d} \n".format(self.solver.gridsize))
            self.file.write_shared("#Frame {:d}  \n".format(frame_num))
        comm.barrier()
        if self.solver.coordmode == "cartesian":
            self.save_perrank(frame_num)
        elif self.solver.coordmode == "polar":
            self.save_perrank_polar(frame_num)
        self.file.flush()
