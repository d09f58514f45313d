"""In-tree build of the native parts: libik_gb300.so (CUDA, sm_103a) and the
pybind11 extension _core (C++).  Called by __graft_entry__.build() and by
``python -m pyglasstools_gb300._build``."""
from __future__ import annotations

import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libik_gb300.so")
# longest first: the build runs them in parallel
CU_SOURCES = ["ik_gather32.cu", "ik_gather32_aux.cu", "ik_gather32_batch.cu", "ik_gather32_exact.cu", "ik_mlp.cu", "ik_api.cu", "ik_cells.cu", "ik_gather64.cu",
              "ik_noalloc.cu", "ik_bonds.cu", "ik_batch.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "ik_gb300.h"))
    return hs


def build_cuda(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                         "-Xptxas", "-v", "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        logs = list(ex.map(lambda c: _run(c, verbose), jobs))
    with open(os.path.join(BUILD, "ptxas.log"), "a") as f:
        for r in logs:
            f.write(r.stderr)
    if _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs], verbose)
    return LIB


def _pybind_include():
    # Prefer the pybind11 headers bundled with torch (present on every machine this
    # builds on), else a standalone pybind11.
    import importlib.util
    spec = importlib.util.find_spec("torch")
    if spec and spec.origin:
        inc = os.path.join(os.path.dirname(spec.origin), "include")
        if os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
            return inc
    try:
        import pybind11
        return pybind11.get_include()
    except ImportError:
        pass
    raise RuntimeError("pybind11 headers not found (neither torch nor pybind11 is importable)")


def build_bindings(verbose=False):
    ext = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    target = os.path.join(HERE, "_core" + ext)
    src = os.path.join(CSRC, "bindings.cpp")
    if not _stale(target, [src, LIB] + _headers()):
        return target
    inc = [sysconfig.get_paths()["include"], _pybind_include(), os.path.join(ROOT, "include")]
    # no FMA contraction in host arithmetic (getRcut, max_rcut) on hosts that have FMA
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-shared", "-fPIC", "-std=c++17", "-fvisibility=hidden",
           "-ffp-contract=off"]
    for i in inc:
        cmd += ["-I", i]
    cmd += [src, "-o", target, "-L" + HERE, "-lik_gb300", "-Wl,-rpath,$ORIGIN"]
    _run(cmd, verbose)
    return target


def build(verbose=False):
    build_cuda(verbose)
    build_bindings(verbose)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
