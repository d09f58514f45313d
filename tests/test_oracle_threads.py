"""The oracle builds its quadrature rules (Gauss-Legendre per order, GK15) once per process,
on first use, possibly from inside its OpenMP loop.  A fresh process that first meets the
rules with many threads gives the same bits as one that runs single-threaded."""
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys
import numpy as np
sys.path.insert(0, {root!r})
from oracle import oracle as O
rng = np.random.default_rng(3)
n, L = 300, 18.0
pos = np.zeros((n, 3)); pos[:, :2] = rng.uniform(-L / 2, L / 2, (n, 2))
diam = rng.uniform(0.8, 1.2, n)
vel = np.zeros((n, 3)); vel[:, :2] = rng.normal(0, 0.5, (n, 2))
mass = np.ones(n)
box = O.make_box(2, [L, L, 1.0])
pot = O.make_poly12()
g = np.linspace(-L / 2, L / 2, 24)
grid = np.zeros((24 * 24, 3)); grid[:, 0] = np.repeat(g, 24); grid[:, 1] = np.tile(g, 24)
outs = []
for cg in (O.make_cg("octic", rcut=2.0, mode="fixedpoint", order=7),
           O.make_cg("octic", rcut=2.0, mode="fixedpoint", order=11),
           O.make_cg("gaussian", rcut=3.0, mode="adaptive", width=1.0, epsrel=1e-8, epsabs=1e-12, limit=100)):
    vir, kin = O.compute(box, pos, diam, pot, cg, grid, vel=vel, mass=mass, nthreads={threads})
    outs += [vir, kin]
np.save({out!r}, np.stack([np.asarray(o).ravel() for o in outs]))
"""


def _run(tmp_path, threads):
    out = str(tmp_path / f"t{threads}.npy")
    code = SCRIPT.format(root=ROOT, threads=threads, out=out)
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    return np.load(out)


def test_rules_built_once_are_thread_safe(tmp_path):
    a = _run(tmp_path, 1)
    b = _run(tmp_path, 8)
    assert np.array_equal(a, b)
    assert np.abs(a).max() > 0
