"""Differentiable multi-step projection rollout (no reference counterpart).

The bubbles' level set is phi = min_b (|x - c_b| - r_b) written in torch, so
it is differentiable with respect to the centres c_b and radii r_b; each step
translates the bubbles rigidly, builds b_k = div(u*_k)/dt from a fresh seeded
u*_k drawn on the GPU, and solves p_k = PressureSolve(phi_k, b_k).  The loss is
J = sum_k |p_k|^2 / 2.  Memory per step: PressureSolve keeps phi_k and p_k
only (the operator is rebuilt and the adjoint solved in backward), and the
level-set construction is checkpointed (recomputed in backward).
"""
import torch
from torch.utils.checkpoint import checkpoint

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


def step_velocity(case, k, device):
    """u*_k, v*_k, w*_k ~ N(0,1) on interior faces, 0 on walls, drawn on the
    device from a generator seeded with (case.seed, k)."""
    g = torch.Generator(device=device)
    g.manual_seed(int(case.seed) * 100003 + 1000 + int(k))
    nz, ny, nx = case.shape
    f64 = torch.float64
    u = torch.randn((nz, ny, nx + 1), generator=g, device=device, dtype=f64)
    v = torch.randn((nz, ny + 1, nx), generator=g, device=device, dtype=f64)
    w = torch.randn((nz + 1, ny, nx), generator=g, device=device, dtype=f64)
    u[..., 0] = 0.0
    u[..., -1] = 0.0
    v[:, 0, :] = 0.0
    v[:, -1, :] = 0.0
    w[0] = 0.0
    w[-1] = 0.0
    return u, v, w


def step_rhs(case, solver: PressurePoisson, k, device):
    """b_k = div(u*_k)/dt on the GPU from step_velocity."""
    u, v, w = step_velocity(case, k, device)
    return solver.divergence(u, v, w, case.dt)


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
