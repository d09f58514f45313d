R"""Global thermodynamic observables (pyglasstools/thermo/__init__.py): the potential
energy, virial, elastic virial, kinetic stress and Born stiffness tensor of a frame, per
unit volume, computed on the GPU over the same cell list as the stress fields
(ik_compute_thermo in include/ik_gb300.h)."""
import pyglasstools_gb300
from pyglasstools_gb300 import _core, solvers_list

_thermo = _core._thermo
_pyglasstools = _core._pyglasstools


def initialize_global(names, dim):
    """The observables a list of names asks for (thermo/__init__.py:8-37)."""
    if dim not in (2, 3):
        raise ValueError("[ERROR]: dim must be 2 or 3")
    D = "{}D".format(dim)
    list_obs = {}
    if any("potentialenergy" in s for s in names):
        list_obs['potentialenergy'] = getattr(_thermo, "GlobalPotentialEnergy" + D)("potentialenergy", "SCALAR", False)
    if any("virialstress" in s for s in names):
        if any("elastic" in s for s in names):
            list_obs['elasticvirialstress'] = getattr(_thermo, "GlobalElasticVirialStress" + D)(
                "elasticvirialstress", "2-TENSOR", False)
        else:
            list_obs['virialstress'] = getattr(_thermo, "GlobalVirialStress" + D)("virialstress", "2-TENSOR", False)
    if any("kineticstress" in s for s in names):
        list_obs['kineticstress'] = getattr(_thermo, "GlobalKineticStress" + D)("kineticstress", "2-TENSOR", True)
    if any("borntensor" in s for s in names):
        list_obs['borntensor'] = getattr(_thermo, "GlobalBornTensor" + D)("borntensor", "4-TENSOR", False)
    return list_obs


class calculator(object):
    R"""thermo.calculator() (thermo/__init__.py:39-58): a ThermoCalculator on the current
    system and pair potential, registered as a solver of ``pyglasstools_gb300.analyze``."""

    def __init__(self):
        self.manager = _pyglasstools.Manager()
        self.thermocalculator = _thermo.ThermoCalculator(pyglasstools_gb300.get_sysdata().cppparticledata,
                                                         pyglasstools_gb300.get_potential().cpppairpotential)
        solvers_list.append(self)

    def add_observables(self, observables):
        for name in observables:
            self.thermocalculator.addObservable(observables[name])

    def run(self):
        self.thermocalculator.compute()

    def update(self, frame_num):
        pyglasstools_gb300.update_sysdata(frame_num)
        self.thermocalculator.setSystemData(pyglasstools_gb300.get_sysdata().cppparticledata)
