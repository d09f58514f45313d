"""Host-side tests of the thermo front-end (no GPU): observable selection
(thermo/__init__.py:8-37), the logfile header and line layout (io.py:9-80) with values
as std::to_string writes them."""
import numpy as np
import pytest


def test_initialize_global_selects_observables():
    from pyglasstools_gb300 import thermo
    obs = thermo.initialize_global(["potentialenergy", "virialstress_01", "kineticstress_00", "borntensor_0101"], 2)
    assert set(obs) == {"potentialenergy", "virialstress", "kineticstress", "borntensor"}
    assert type(obs["borntensor"]).__name__ == "GlobalBornTensor2D"
    assert len(obs["borntensor"].val) == 16 and len(obs["virialstress"].val) == 4
    obs = thermo.initialize_global(["elasticvirialstress_00"], 3)
    assert set(obs) == {"elasticvirialstress"}
    assert type(obs["elasticvirialstress"]).__name__ == "GlobalElasticVirialStress3D"
    assert obs["elasticvirialstress"].islocal is False
    assert thermo.initialize_global(["kineticstress_00"], 3)["kineticstress"].islocal is True
    with pytest.raises(ValueError):
        thermo.initialize_global(["virialstress_00"], 4)


def test_logfile_header_and_rows(tmp_path, monkeypatch):
    import pyglasstools_gb300 as pglass
    import pyglasstools_gb300.io as io
    import pyglasstools_gb300.utils as utils

    class Fr:
        pass

    fr = Fr()
    fr.pos = np.zeros((4, 3))
    fr.pos[:, 0] = [-1.5, -0.5, 0.5, 1.5]
    fr.diam = np.ones(4)
    fr.L = 8.0

    class Solver:
        def __init__(self):
            self.obs = {}

        def add_observables(self, o):
            self.obs.update(o)

    monkeypatch.chdir(tmp_path)
    pglass.reset()
    utils.data_arrays([fr], ndim=2)
    s = Solver()
    names = ["potentialenergy", "virialstress_01", "borntensor_0011"]
    log = io.logfile(filename="t.log", names=names, solver=s)
    assert set(s.obs) == {"potentialenergy", "virialstress", "borntensor"}
    log.save(7)
    log.file.close()
    pglass.reset()
    lines = open(tmp_path / "t.log").read().splitlines()
    assert lines == ["Frame potentialenergy virialstress_01 borntensor_0011 ",
                     "7 0.000000 0.000000 0.000000 "]
