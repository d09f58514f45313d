"""pyglasstools_gb300 -- GB300 (sm_103a) implementation of pyglasstools' Irving-Kirkwood
stress-field path behind the reference's Python API.

Same entry points as the reference package (pyglasstools/__init__.py):
``comm``, ``rank``, ``size``, ``analyze(frame_list)``, ``set_sysdata`` /
``get_sysdata`` / ``set_potential`` / ``get_potential``, ``loggers_list``,
``solvers_list``, ``reset``.  Submodules: ``potential``, ``irvingkirkwood``
(+ ``irvingkirkwood.cgfunc``), ``utils``, ``io``.

Every computation runs in the CUDA library ``libik_gb300.so`` through the
pybind11 module ``_core``; importing fails loudly when they have not been built
(``python -m pyglasstools_gb300._build``).
"""
import os
import signal
import sys

try:
    from pyglasstools_gb300 import _core
except ImportError as e:  # pragma: no cover - exercised only without a build
    raise ImportError(
        "pyglasstools_gb300: the native extension is not built or cannot load "
        f"({e}); run `python -m pyglasstools_gb300._build` on a machine with nvcc") from e

_pyglasstools = _core._pyglasstools

# Single-process communicator (rank 0 of 1): one GPU per process, no MPI.
comm = _pyglasstools.Communicator()
rank = comm.getRank()
size = comm.getSizeGlobal()

savemode = "unordered"


def set_savemode(name):
    global savemode
    savemode = name


loggers_list = []
solvers_list = []
globalsysdata = None
globalpotential = None


def set_sysdata(sysdata):
    global globalsysdata
    globalsysdata = sysdata


def update_sysdata(frame_num):
    globalsysdata.update(frame_num)


def get_sysdata():
    return globalsysdata


def set_potential(potential):
    global globalpotential
    globalpotential = potential


def get_potential():
    return globalpotential


def reset():
    loggers_list.clear()
    solvers_list.clear()


import atexit  # noqa: E402

atexit.register(reset)


class DelayedInterrupt(object):
    """Defers SIGINT/SIGTERM while a frame's output is written (pyglasstools/__init__.py:88-102)."""

    def __enter__(self):
        self.signal_received = False
        self.old_handler = {}
        for sig in (signal.SIGINT, signal.SIGTERM):
            self.old_handler[sig] = signal.signal(sig, self.handler)

    def handler(self, sig, frame):
        self.signal_received = (sig, frame)
        print(f"Signal {sig} received by Process [{rank}]. Delaying KeyboardInterrupt.")

    def __exit__(self, type, value, traceback):
        for sig in (signal.SIGINT, signal.SIGTERM):
            signal.signal(sig, self.old_handler[sig])
        if self.signal_received:
            sig, frame = self.signal_received
            handler = self.old_handler[sig]
            if callable(handler):
                handler(sig, frame)


def analyze(frame_list, progress=True):
    """Per frame: update and run every solver, save every logger, checkpoint
    (pyglasstools/__init__.py:107-138)."""
    frame_list = list(frame_list)
    totallength = len(frame_list)
    frame_list = globalsysdata.setup_checkpoint(frame_list)
    if not frame_list:
        if rank == 0:
            print("No more frames to analyze. Check your logfiles/output")
        return
    bar = None
    if progress and rank == 0:
        try:
            from tqdm import tqdm
            bar = tqdm(total=totallength, file=sys.stdout, leave=False, initial=frame_list[0])
        except ImportError:
            bar = None
    for frame_num in frame_list:
        for solver in solvers_list:
            solver.update(frame_num)
            solver.run()
        with DelayedInterrupt():
            for logger in loggers_list:
                logger.save(frame_num)
            if rank == 0 and globalsysdata.checkpointfile is not None:
                with open(globalsysdata.checkpointfile, "w") as f:
                    f.write("Frame {}".format(frame_num + 1))
            if bar is not None:
                bar.update(1)
            comm.barrier()
    if bar is not None:
        bar.close()


from pyglasstools_gb300 import utils  # noqa: E402,F401
