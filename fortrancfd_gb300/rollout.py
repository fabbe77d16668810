"""Differentiable multi-step projection rollout (no reference counterpart).

The bubbles' level set is phi = min_b (|x - c_b| - r_b) written in torch, so
it is differentiable with respect to the centres c_b and radii r_b; each step
translates the bubbles rigidly, builds b_k = div(u*_k)/dt from a fresh seeded
u*_k on the GPU, and solves p_k = PressureSolve(phi_k, b_k).  The loss is
J = sum_k |p_k|^2 / 2.  Memory per step: PressureSolve keeps phi_k and p_k
only (the operator is rebuilt and the adjoint solved in backward), and the
level-set construction is checkpointed (recomputed in backward).
"""
import numpy as np
import torch
from torch.utils.checkpoint import checkpoint

from . import inputs
from .autograd import pressure_solve
from .ppe import PressurePoisson


def level_set(centers, radii, shape, extent):
    """phi (nz, ny, nx) = min over bubbles of distance to centre minus radius;
    centers (nb, 3) and radii (nb,) are float64 tensors on the target device."""
    nz, ny, nx = shape
    Lx, Ly, Lz = extent
    dev, dt = centers.device, centers.dtype
    x = (torch.arange(nx, device=dev, dtype=dt) + 0.5) * (Lx / nx)
    y = (torch.arange(ny, device=dev, dtype=dt) + 0.5) * (Ly / ny)
    z = (torch.arange(nz, device=dev, dtype=dt) + 0.5) * (Lz / nz)
    phi = None
    for bi in range(centers.shape[0]):
        c = centers[bi]
        d2 = (x[None, None, :] - c[0]) ** 2 + (y[None, :, None] - c[1]) ** 2
        if nz > 1:
            d2 = d2 + (z[:, None, None] - c[2]) ** 2
        d = torch.sqrt(d2) - radii[bi]
        phi = d if phi is None else torch.minimum(phi, d)
    return phi


def step_rhs(case, solver: PressurePoisson, k, device):
    """b_k = div(u*_k)/dt on the GPU, u*_k ~ N(0,1) from seed (case.seed, k)."""
    u, v, w = inputs.velocity(case, seed=[case.seed, 1000 + k])
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(device) for a in (u, v, w)]
    return solver.divergence(t[0], t[1], t[2], case.dt)


def rollout_loss(centers, radii, case, solver: PressurePoisson, steps=None, tol=1e-10,
                 adjoint_tol=None):
    """J = sum_k |p_k|^2/2 over the rollout; differentiable in centers, radii."""
    steps = case.extra.get("steps", 20) if steps is None else steps
    shift = torch.tensor(case.extra.get("shift", (0.0, 0.0, 0.5)), dtype=centers.dtype,
                         device=centers.device)
    J = torch.zeros((), dtype=centers.dtype, device=centers.device)
    for k in range(steps):
        ck = centers + shift * (k * case.dt)
        phi = checkpoint(level_set, ck, radii, case.shape, case.extent, use_reentrant=False)
        b = step_rhs(case, solver, k, centers.device)
        p = pressure_solve(phi, b, solver, case.eps, case.rho_pos, case.rho_neg, tol, adjoint_tol)
        J = J + 0.5 * (p * p).sum()
    return J
