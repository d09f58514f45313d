"""Field output (pyglasstools/io.py:82-169): ``fieldlogger(keyword, names, solver)``
writes ``<keyword>.xyz`` -- per frame a ``gridsize`` line, a ``#Frame n`` line, then
one line per grid point ``1 x y [z] T_ab ...`` with the values formatted like a
default C++ ostream (6 significant digits)."""
import pyglasstools_gb300
from pyglasstools_gb300 import _core, comm, loggers_list, rank, size
from pyglasstools_gb300 import irvingkirkwood

_pyglasstools = _core._pyglasstools


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

    def save_perrank(self, frame_num):
        Dim = pyglasstools_gb300.get_sysdata().pysimbox.dim
        gp = self.solver.gridpoints
        lines = []
        for index in range(len(gp)):
            outline = "{} ".format(1)
            outline += "{} ".format(gp[index][0])
            outline += "{} ".format(gp[index][1])
            if Dim == 3:
                outline += "{} ".format(gp[index][2])
            for name in self.__obs_names:
                i = int(name[-2])
                j = int(name[-1])
                outline += self.field_obs[name[:-3]].gettostring(i + Dim * j, index)
            lines.append(outline + "\n")
        self.file.write_shared("".join(lines))

    def save(self, frame_num):
        if rank == 0:
            self.file.write_shared("{:d} \n".format(self.solver.gridsize))
            self.file.write_shared("#Frame {:d}  \n".format(frame_num))
        comm.barrier()
        if self.solver.coordmode == "cartesian":
            self.save_perrank(frame_num)
        self.file.flush()
