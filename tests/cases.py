"""Seeded test cases shared by the CPU and GPU tests: the benchmark geometries
at reduced resolution, with the oracle's coefficients and right-hand side."""
import numpy as np

from fortrancfd_gb300 import inputs
from oracle import oracle as orc


class Built:
    def __init__(self, case):
        self.case = case
        self.phi = inputs.level_set(case)
        self.rho = orc.rho_from_phi(self.phi, case.eps, case.rho_pos, case.rho_neg)
        self.coef = orc.face_coef(self.rho, case.spacing)
        self.u, self.v, self.w = inputs.velocity(case)
        self.b = orc.divergence(self.u, self.v, self.w, case.dt, case.spacing)

    @property
    def shape(self):
        return self.case.shape

    @property
    def spacing(self):
        return self.case.spacing


_cache = {}


def config(index, scale=1):
    key = (index, scale)
    if key not in _cache:
        _cache[key] = Built(inputs.config(index, scale))
    return _cache[key]


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
