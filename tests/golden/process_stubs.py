"""Process objects with fixed rates and the attributes that
pymulskips.setuprun.run_mulskips reads from its process classes (it
dispatches on the class name: CVD, PVD, PhaseChange).  make_fixtures.py
writes start.dat with the reference's writer for them, and the tests write it
with mulskips_gb300.setuprun for the same objects."""
import itertools

import numpy as np

SF = 5.43 / 12


def _indices(n):
    return [t for t in itertools.product(range(4), repeat=n) if 1 <= sum(t) <= 3]


class CVD:
    """Si with one coverage species (H)."""
    listcry, listcryZ, listcov, listcovZ = ["Si"], [14], ["H"], [1]
    KMC_sf = SF
    calibration_params = {"note": "fixed rates"}

    def indices(self):
        return _indices(2)

    def get_PtransE(self):
        E = np.zeros((1, 4, 4))
        for i, j in self.indices():
            E[0, i, j] = 1.0e3 * 10.0 ** (-(i + 0.5 * j))
        return E

    def get_PtransD(self):
        return np.array([[85.0, 85.0, 85.0]])

    def get_PtransAbs(self):
        return np.array([[287.0, 287.0, 287.0]])

    def get_PtransDes(self):
        return np.array([[40.0, 40.0, 40.0]])


class PVD:
    """SiGe with a substrate Ge fraction of 0.3."""
    listcry, listcryZ, listcov, listcovZ = ["Si", "Ge"], [14, 32], [], []
    KMC_sf = SF
    calibration_params = {"X0": [0.0, 0.3]}

    def indices(self):
        return _indices(2)

    def get_PtransE(self):
        E = np.zeros((2, 4, 4))
        for s in range(2):
            for i, j in self.indices():
                E[s, i, j] = 1.0e7 * 10.0 ** (-(2 * i + j + s))
        return E

    def get_PtransD(self):
        return np.array([[0.5, 0.5, 0.5], [0.2, 0.2, 0.2]])


class PhaseChange:
    """Si melting and solidification (the LA law): energetics in eV."""
    listcry, listcryZ, listcov, listcovZ = ["Si"], [14], [], []
    KMC_sf = SF
    Tm = [1688.0]
    calibration_params = {"P0": [1.33e17], "A": [175.0], "Tflex": [1200.0]}

    def indices(self):
        return _indices(1)

    def get_energetics_evap(self):
        return np.array([[0.0, 4.5, 5.0, 5.5]])

    def get_energetics_depo(self):
        return np.array([[5.0, 5.0, 5.0]])
