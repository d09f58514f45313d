"""GPU tests of the global thermodynamic observables (ik_compute_thermo; the reference's
ThermoCalculator with every Global* observable, thermo/module-thermo.cpp:7-20) against the
FP64 oracle: relative error <= 1e-12 per observable (FP64 sums in another order), bit
identical across calls; and the Python front-end (thermo.calculator + io.logfile)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _close(got, want, what):
    for k, v in want.items():
        v = np.asarray(v, np.float64)
        g = np.asarray(got[k], np.float64)
        scale = max(np.max(np.abs(v)), 1e-300)
        assert np.max(np.abs(g - v)) <= TOL * scale, (what, k, np.max(np.abs(g - v)) / scale)


@pytest.mark.parametrize("kind,dim,n", [("poly12", 2, 3000), ("lj", 2, 3000), ("polyyukawa", 2, 2500),
                                        ("fslj", 3, 2000), ("poly18", 3, 2000), ("polylj", 2, 2500)])
def test_thermo_matches_oracle(oracle, kind, dim, n):
    from pyglasstools_gb300 import ikabi as ik, synth
    fr = synth.make_frame(n, dim=dim, seed=17)
    rc, prm = oracle.potential_params(kind)
    prm = list(prm)
    if kind in ("lj", "fslj"):
        prm[1] = 0.1
    rng = np.random.default_rng(9)
    disp = np.zeros((n, 3))
    disp[:, :dim] = rng.normal(0, 0.03, (n, dim))
    box = [fr.L, fr.L, fr.L if dim == 3 else 1.0]
    with ik.IKContext() as c:
        c.set_box(dim, box)
        c.set_potential(kind, rc, prm)
        c.set_frame(fr.pos, fr.diam, fr.vel, fr.mass)
        c.upload_displacement(disp)
        got = c.compute_thermo()
        again = c.compute_thermo()
        max_rc = c.get_max_rcut()
    want = oracle.global_thermo(oracle.make_box(dim, box), fr.pos, fr.diam, oracle.make_potential(kind, rc, prm),
                                vel=fr.vel, mass=fr.mass, disp=disp, max_rc=max_rc)
    _close(got, want, kind)
    for k in got:
        np.testing.assert_array_equal(np.asarray(got[k]), np.asarray(again[k]))


def test_thermo_without_displacement_or_velocities(oracle):
    from pyglasstools_gb300 import ikabi as ik, synth
    fr = synth.make_frame(2000, dim=2, seed=18)
    with ik.IKContext() as c:
        c.set_box(2, [fr.L, fr.L, 1.0])
        c.set_poly12()
        c.set_frame(fr.pos, fr.diam)
        got = c.compute_thermo()
        max_rc = c.get_max_rcut()
    assert np.all(got["elasticvirialstress"] == 0) and np.all(got["kineticstress"] == 0)
    want = oracle.global_thermo(oracle.make_box(2, [fr.L, fr.L, 1.0]), fr.pos, fr.diam, oracle.make_poly12(),
                                max_rc=max_rc)
    _close(got, want, "no velocities")


def test_thermo_errors():
    from pyglasstools_gb300 import ikabi as ik
    with ik.IKContext() as c:
        with pytest.raises(ik.IKError):
            c.dim = 2
            c.compute_thermo()                      # no box, potential or frame


def test_thermo_frontend_logfile(tmp_path, golden, monkeypatch, oracle):
    """The reference's thermo example (example_scripts/thermo/test-thermo-module.py):
    Born tensor and virial stress of the fixture frames through thermo.calculator and
    io.logfile, against the oracle (values written with six decimals)."""
    import pyglasstools_gb300 as pglass
    import pyglasstools_gb300.io as io
    import pyglasstools_gb300.potential as pot
    import pyglasstools_gb300.thermo as thermo
    import pyglasstools_gb300.utils as utils

    class Fr:
        pass

    fx = golden("fixture_frames.npz")
    frames = []
    for f in (180, 199):
        fr = Fr()
        fr.pos = fx[f"pos{f}"].astype(np.float64)
        fr.diam = fx[f"diam{f}"].astype(np.float64)
        fr.L = float(fx[f"box{f}"][0])
        frames.append(fr)
    monkeypatch.chdir(tmp_path)
    pglass.reset()
    pot.polydisperse12(v0=1.0, eps=0.2, rcut=1.25)
    utils.data_arrays(frames, ndim=2, checkpointfile="restart.log")
    calc = thermo.calculator()
    bnames = ['borntensor_0000', 'borntensor_0011', 'borntensor_0001', 'borntensor_1111', 'borntensor_1101',
              'borntensor_0101']
    io.logfile(filename="borntensor.log", names=bnames, solver=calc)
    vnames = ['virialstress_00', 'virialstress_11', 'virialstress_01', 'potentialenergy']
    io.logfile(filename="virialstress.log", names=vnames, solver=calc)
    pglass.analyze(frame_list=[0, 1], progress=False)
    pglass.reset()
    bl = open(tmp_path / "borntensor.log").read().splitlines()
    vl = open(tmp_path / "virialstress.log").read().splitlines()
    assert bl[0] == "Frame " + " ".join(bnames) + " " and len(bl) == 3
    assert vl[0] == "Frame " + " ".join(vnames) + " " and len(vl) == 3
    for k, fr in enumerate(frames):
        box = oracle.make_box(2, [fr.L, fr.L, 1.0])
        max_rc = oracle.max_rcut(1.25, frames[0].diam)  # frozen at construction
        w = oracle.global_thermo(box, fr.pos, fr.diam, oracle.make_poly12(), max_rc=max_rc)
        brow = bl[1 + k].split()
        vrow = vl[1 + k].split()
        assert brow[0] == str(k) and vrow[0] == str(k)
        B = w["borntensor"]
        want_b = [B[0, 0, 0, 0], B[0, 0, 1, 1], B[0, 0, 0, 1], B[1, 1, 1, 1], B[1, 1, 0, 1], B[0, 1, 0, 1]]
        want_v = [w["virialstress"][0, 0], w["virialstress"][1, 1], w["virialstress"][0, 1], w["potentialenergy"]]
        for txt, v in zip(brow[1:], want_b):
            assert txt == "{:.6f}".format(v) or abs(float(txt) - v) <= 1.5e-6, (txt, v)
        for txt, v in zip(vrow[1:], want_v):
            assert txt == "{:.6f}".format(v) or abs(float(txt) - v) <= 1.5e-6, (txt, v)
