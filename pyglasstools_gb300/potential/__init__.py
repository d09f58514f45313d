R"""Pair potentials (pyglasstools/potential/__init__.py)."""
import numpy as np

import pyglasstools_gb300
from pyglasstools_gb300 import _core

_potential = _core._potential


class pairpotential(object):
    R"""Common methods of a pair potential (potential/__init__.py:9-55)."""

    def __init__(self):
        self.cpppairpotential = None
        self.name = None
        self.dict_params = None

    def get_potentialname(self):
        return self.name

    def set_scaledrcut(self, rcut):
        self.cpppairpotential.scaled_rcut = rcut

    def get_scaledrcut(self):
        return self.cpppairpotential.scaled_rcut

    def set_params(self, val, num):
        if isinstance(num, str):
            self.cpppairpotential.setParams(val, self.dict_params[num])
        elif isinstance(num, int):
            self.cpppairpotential.setParams(val, num)

    def get_params(self, num=None):
        if num is None:
            return self.cpppairpotential.getParams()
        if isinstance(num, str):
            return self.cpppairpotential.getParams()[self.dict_params[num]]
        return self.cpppairpotential.getParams()[num]

    def print_params(self):
        params = self.cpppairpotential.getParams()
        for key in self.dict_params:
            print("{}: {} ".format(key, params[self.dict_params[key]]))

    def get_pairforce(self, rij, di, dj):
        rij = np.asarray(rij, dtype=np.float64)
        if len(rij) == 2:
            rij = np.append(rij, 0.0)
        return self.cpppairpotential.getPairForceDivR(rij, di, dj) * np.linalg.norm(rij)

    def get_pairenergy(self, rij, di, dj):
        rij = np.asarray(rij, dtype=np.float64)
        if len(rij) == 2:
            rij = np.append(rij, 0.0)
        return self.cpppairpotential.getPairEnergy(rij, di, dj)


class polydisperse12(pairpotential):
    R"""Poly12 pair potential with smoothing coefficients c0, c1, c2
    (potential/__init__.py:78-88)."""

    def __init__(self, v0=1.0, eps=0.2, rcut=1.25):
        self.name = "polydisperse-12"
        c0 = -28.0 * v0 / rcut ** 12
        c1 = 48.0 * v0 / rcut ** 14
        c2 = -21.0 * v0 / rcut ** 16
        self.cpppairpotential = _potential.PairPotentialPoly12(rcut, [v0, eps, c0, c1, c2])
        self.dict_params = {'v0': 0, 'eps': 1, 'c0': 2, 'c1': 3, 'c2': 4}
        pyglasstools_gb300.set_potential(self)
