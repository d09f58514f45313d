"""Field output (pyglasstools/io.py:82-169): ``fieldlogger(keyword, names, solver)``
writes ``<keyword>.xyz`` -- per frame a ``gridsize`` line, a ``#Frame n`` line, then
one line per grid point ``1 x y [z] T_ab ...`` with the values formatted like a
default C++ ostream (6 significant digits)."""
import numpy as np

import pyglasstools_gb300
from pyglasstools_gb300 import _core, comm, loggers_list, rank, size
from pyglasstools_gb300 import irvingkirkwood

_pyglasstools = _core._pyglasstools
_irvingkirkwood = _core._irvingkirkwood


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
