"""Generates the committed golden fixtures under tests/golden/.

Run in a checkout that has the reference tree next to it (default
/root/reference, override with PYGLASSTOOLS_REF):

    python tests/golden/make_golden.py

Outputs
  fixture_frames.npz   frames 180 and 199 of example_scripts/polydisperse12.gsd
                       (float32 positions/diameters as stored, box), decoded by
                       pyglasstools_gb300.gsd -- the frames the reference's
                       example script test-irvingkirkwood-module.py analyses.
  ref_kernels.npz      Polydisperse12 force/energy/stiffness and Octic/Rect/Mollifier
                       values produced by the REFERENCE'S OWN headers compiled by
                       oracle/build_ref.sh, on seeded random inputs.
  ref_potentials.npz   force, energy and stiffness of all eight pair models (LJ, force-shifted LJ,
                       Poly10/106/12/18, PolyLJ, PolyYukawa) from the reference's own
                       headers, on seeded inputs that include overlaps and pairs
                       within 1e-12 of the cut-off.
  oracle_fixture180.npz  the oracle's virial field (xx, yy, xy per grid point) on frame 180 with the example
                       script's settings (octic R = 2, Gauss-Legendre 5, dx = 0.25).
  oracle_cfg0.npz      the oracle's virial + kinetic fields on a seeded synthetic
                       2D frame (N = 2000, 64 x 64 grid, octic R = 2, GL-5).
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from pyglasstools_gb300 import gsd as G  # noqa: E402
from pyglasstools_gb300 import synth  # noqa: E402

REF = os.environ.get("PYGLASSTOOLS_REF", "/root/reference")


def frames():
    traj = G.open_trajectory(os.path.join(REF, "example_scripts", "polydisperse12.gsd"))
    out = {}
    for f in (180, 199):
        fr = traj[f]
        out[f"pos{f}"] = fr.position.astype(np.float32)
        out[f"diam{f}"] = fr.diameter.astype(np.float32)
        out[f"box{f}"] = fr.box.astype(np.float32)
    out["nframes"] = np.int64(len(traj))
    np.savez_compressed(os.path.join(HERE, "fixture_frames.npz"), **out)
    return out


def ref_kernels():
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    R = O.ref_lib()
    assert R is not None, "oracle/_ref/libref_kernels.so was not built"
    rng = np.random.default_rng(1234)
    m = 1500
    rsq = rng.uniform(0.05, 4.5, m)
    di = rng.uniform(0.7, 1.7, m)
    dj = rng.uniform(0.7, 1.7, m)
    pot = O.make_poly12()
    prm = (C.c_double * 5)(pot.v0, pot.eps, pot.c0, pot.c1, pot.c2)
    f = np.array([R.ref_poly12_force_divr(a, pot.scaled_rcut, prm, b, c) for a, b, c in zip(rsq, di, dj)])
    e = np.array([R.ref_poly12_energy(a, pot.scaled_rcut, prm, b, c) for a, b, c in zip(rsq, di, dj)])
    s = np.array([R.ref_poly12_stiffness(a, pot.scaled_rcut, prm, b, c) for a, b, c in zip(rsq, di, dj)])
    rc = 2.0
    dr = rng.uniform(0.0, 1.2 * rc * rc, m)
    octic = np.array([R.ref_octic(rc, x) for x in dr])
    rect = np.array([R.ref_rect(rc, x) for x in dr])
    moll = np.array([R.ref_mollifier(rc, x) for x in dr])
    np.savez_compressed(os.path.join(HERE, "ref_kernels.npz"), rsq=rsq, di=di, dj=dj, force=f, energy=e,
                        stiffness=s, rc=rc, dr=dr, octic=octic, rect=rect, mollifier=moll)


# models and constructor keywords of the pinned cases (non-default non-additivity)
POT_CASES = [("poly12", {}), ("lj", {"eps": 1.0, "vareps": 0.1, "rcut": 2.5}),
             ("fslj", {"eps": 1.0, "vareps": 0.1, "rcut": 2.5}), ("poly10", {}), ("poly106", {}),
             ("poly18", {"eps": 0.1}), ("polylj", {}), ("polyyukawa", {"eps": 0.05, "kappa": 1.5})]


def ref_potentials():
    R = O.ref_lib()
    assert R is not None, "oracle/_ref/libref_kernels.so was not built"
    rng = np.random.default_rng(4321)
    out = {}
    m = 600
    for kind, kw in POT_CASES:
        rc, prm = O.potential_params(kind, **kw)
        di = rng.uniform(0.7, 1.7, m)
        dj = rng.uniform(0.7, 1.7, m)
        eps = prm[2] if kind == "polyyukawa" else prm[1]
        sig = 0.5 * (di + dj) * (1 - eps * np.abs(di - dj))
        cut = rc * rc * sig * sig
        u = rng.uniform(0.02, 1.3, m)
        rsq = u * cut
        k = m // 10  # pairs at the cut-off: exact, and within a few ulp either side
        rsq[:k] = cut[:k] * (1.0 + rng.integers(-3, 4, k) * 2.0 ** -52)
        arr = (C.c_double * len(prm))(*prm)
        K = O.POT_KIND[kind]
        out[f"{kind}_rc"] = np.float64(rc)
        out[f"{kind}_params"] = np.asarray(prm, np.float64)
        out[f"{kind}_rsq"], out[f"{kind}_di"], out[f"{kind}_dj"] = rsq, di, dj
        out[f"{kind}_force"] = np.array([R.ref_pot_force_divr(K, a, rc, arr, len(prm), b, c)
                                         for a, b, c in zip(rsq, di, dj)])
        out[f"{kind}_energy"] = np.array([R.ref_pot_energy(K, a, rc, arr, len(prm), b, c)
                                          for a, b, c in zip(rsq, di, dj)])
        out[f"{kind}_stiffness"] = np.array([R.ref_pot_stiffness(K, a, rc, arr, len(prm), b, c)
                                             for a, b, c in zip(rsq, di, dj)])
    np.savez_compressed(os.path.join(HERE, "ref_potentials.npz"), **out)


def oracle_fixture(fr):
    pos = fr["pos180"].astype(np.float64)
    diam = fr["diam180"].astype(np.float64)
    L = float(fr["box180"][0])
    box = O.make_box(2, [L, L, 1.0])
    nmax = int(L / 0.25)
    pts = np.linspace(-L / 2.0, L / 2.0, nmax)
    gx, gy = np.meshgrid(pts, pts, indexing="ij")
    grid = np.stack([gx.ravel(), gy.ravel(), np.zeros(gx.size)], axis=1)
    pot = O.make_poly12()
    cg = O.make_cg("octic", rcut=2.0, mode="fixedpoint", order=5)
    vir, _ = O.compute(box, pos, diam, pot, cg, grid)
    uniq = np.stack([vir[:, 0, 0], vir[:, 1, 1], vir[:, 0, 1]], axis=1)  # xx, yy, xy
    np.savez_compressed(os.path.join(HERE, "oracle_fixture180.npz"), virial=uniq, nmax=nmax,
                        max_rcut=O.max_rcut(pot.scaled_rcut, diam))


def oracle_cfg0():
    f = synth.make_frame(2000, dim=2, seed=0)
    grid = synth.lattice_grid(f.L, 64, 2)
    box = O.make_box(2, [f.L, f.L, 1.0])
    pot = O.make_poly12()
    cg = O.make_cg("octic", rcut=2.0, mode="fixedpoint", order=5)
    vir, kin = O.compute(box, f.pos, f.diam, pot, cg, grid, vel=f.vel, mass=f.mass)
    u = lambda t: np.stack([t[:, 0, 0], t[:, 1, 1], t[:, 0, 1]], axis=1)  # xx, yy, xy
    np.savez_compressed(os.path.join(HERE, "oracle_cfg0.npz"), virial=u(vir), kinetic=u(kin),
                        pos_checksum=np.float64(f.pos.sum()), diam_checksum=np.float64(f.diam.sum()))


if __name__ == "__main__":
    O.build()
    fr = frames()
    ref_kernels()
    ref_potentials()
    oracle_fixture(fr)
    oracle_cfg0()
    for fn in sorted(os.listdir(HERE)):
        if fn.endswith(".npz"):
            print(fn, os.path.getsize(os.path.join(HERE, fn)))
