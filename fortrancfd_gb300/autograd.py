"""Differentiable pressure solve: torch.autograd.Function with a hand-written
adjoint that reuses the same multigrid (no reference counterpart; the
reference's solvers are not differentiable).

Forward: rho = rho_pos H(phi) + rho_neg (1 - H), face coefficients
2/(rho_i + rho_nb)/h^2, p = A^+ (b - mean b) (mean-free), on the GPU.
Backward, for the incoming g = dJ/dp: A is symmetric, so the adjoint is one
more solve with the same operator, lam = A^+ (g - mean g); then
    dJ/db   = lam
    dJ/dphi = sum over faces (lam_nb - lam_i)(p_nb - p_i) dcoe/drho * drho/dphi
computed by the gbmg_adjoint kernel.  Only phi (or rho) and p are saved; the
operator is rebuilt from them in backward, so a rollout keeps one level set
and one pressure per step.

The adjoint solve runs to adjoint_tol (default: the forward tol).  Its
right-hand side g is typically smooth, so A^+ g is large and the attainable
FP64 relative residual of the adjoint is higher than the forward's: a forward
solved to 1e-13 for finite-difference checks pairs with an adjoint to 1e-10.
"""
import torch

from .ppe import PressurePoisson


class PressureSolve(torch.autograd.Function):
    """p = PressureSolve.apply(phi, b, solver, eps, rho_pos, rho_neg, tol, adjoint_tol)."""

    @staticmethod
    def forward(ctx, phi, b, solver: PressurePoisson, eps, rho_pos, rho_neg, tol,
                adjoint_tol=None):
        solver.rho_mu(phi.detach(), eps, rho_pos, rho_neg)
        p = torch.zeros_like(b)
        solver.solve(b.detach(), p, tol=tol)
        ctx.solver = solver
        ctx.args = (eps, rho_pos, rho_neg, tol if adjoint_tol is None else adjoint_tol)
        ctx.save_for_backward(phi, p)
        return p

    @staticmethod
    def backward(ctx, grad_p):
        phi, p = ctx.saved_tensors
        eps, rho_pos, rho_neg, tol = ctx.args
        s = ctx.solver
        s.ensure_rho_mu(phi.detach(), eps, rho_pos, rho_neg)  # rebuilt if the solver moved on
        lam = torch.zeros_like(p)
        s.solve(grad_p.contiguous(), lam, tol=tol)
        grad_phi = None
        if ctx.needs_input_grad[0]:
            _, grad_phi = s.adjoint(p, lam, phi.detach(), eps, rho_pos, rho_neg)
        grad_b = lam if ctx.needs_input_grad[1] else None
        return grad_phi, grad_b, None, None, None, None, None, None


class PressureSolveRho(torch.autograd.Function):
    """p = PressureSolveRho.apply(rho, b, solver, tol, adjoint_tol): the same with
    the cell density as the input."""

    @staticmethod
    def forward(ctx, rho, b, solver: PressurePoisson, tol, adjoint_tol=None):
        solver.ppe_init(rho.detach())
        p = torch.zeros_like(b)
        solver.solve(b.detach(), p, tol=tol)
        ctx.solver, ctx.tol = solver, tol if adjoint_tol is None else adjoint_tol
        ctx.save_for_backward(rho, p)
        return p

    @staticmethod
    def backward(ctx, grad_p):
        rho, p = ctx.saved_tensors
        s = ctx.solver
        s.ensure_ppe_init(rho.detach())
        lam = torch.zeros_like(p)
        s.solve(grad_p.contiguous(), lam, tol=ctx.tol)
        grad_rho = s.adjoint(p, lam)[0] if ctx.needs_input_grad[0] else None
        grad_b = lam if ctx.needs_input_grad[1] else None
        return grad_rho, grad_b, None, None, None


def pressure_solve(phi, b, solver, eps, rho_pos=1000.0, rho_neg=1.0, tol=1e-10, adjoint_tol=None):
    """Differentiable p(phi, b); phi and b are float64 CUDA tensors."""
    return PressureSolve.apply(phi, b, solver, eps, rho_pos, rho_neg, tol, adjoint_tol)
