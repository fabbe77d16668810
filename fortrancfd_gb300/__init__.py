"""GB300-native pressure-Poisson multigrid for the two-phase solvers of
ntu-d09525007/FortranCFD.

The product is libgbmg.so (CUDA kernels for sm_103a + the C ABI of
include/gbmg.h).  This package holds its sources (csrc/), the in-tree build
recipe (build.py), the ctypes binding (_lib.py), the host-side mirror of the
reference's pressure routine (ppe.py), the differentiable solve (autograd.py),
the registered operator torch.ops.gbmg.solve (ops.py), the level-set
advection of the interface solver (levelset.py), the Adams-Bashforth momentum
step around the projection with the CCD curvature (momentum.py), the whole
two-phase time step over those (timestep.py) and the seeded synthetic inputs
(inputs.py).
"""
from .ppe import ConvergenceError, GBMGError, PressurePoisson  # noqa: F401
from .levelset import LevelSet, node_velocity  # noqa: F401
from .momentum import (NSParams, bc, curv, ls_mv, mass_preserving_level_set,  # noqa: F401
                       ns_ab_predictor, ns_ab_solver, rho_mu, velbc, vof_wlic_solver, ibm_bc)
from .timestep import InterfaceParams, TwoPhaseStep  # noqa: F401

try:  # torch.ops.gbmg.solve (torch is optional for host-memory use)
    from . import ops  # noqa: F401
except ImportError:  # pragma: no cover
    pass

__all__ = ["PressurePoisson", "LevelSet", "node_velocity", "NSParams", "ns_ab_solver",
           "ns_ab_predictor", "velbc", "curv", "rho_mu", "bc", "mass_preserving_level_set", "ls_mv",
           "vof_wlic_solver", "ibm_bc",
           "TwoPhaseStep", "InterfaceParams",
           "ConvergenceError", "GBMGError"]
