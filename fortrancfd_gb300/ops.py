"""torch.ops.gbmg.solve: the pressure solve as a registered torch operator.

    p = torch.ops.gbmg.solve(rho, b, dx, dy, dz, tol, adjoint_tol, precision)

rho (cell density) and b (right-hand side) are float64 CUDA tensors of shape
(nz, ny, nx) (nz = 1 for 2D); p is the mean-free solution of A p = b with the
operator of ppe_sor_init (face coefficients 2/(rho_i + rho_nb)/h^2), solved
from zero to the relative residual tol by libgbmg on the tensors' device.
The operator is differentiable in rho and b: backward solves the adjoint
A lam = dJ/dp to adjoint_tol and applies gbmg_adjoint (no reference
counterpart; the reference's solvers are Fortran subroutines with no tensor
interface).  precision: "fp64" or "mixed".

Handles (the multigrid hierarchy on the device) are cached per shape,
spacing, precision and device, so repeated calls allocate nothing new.  A
handle is not re-entrant, so every call holds its handle's lock from setting
the operator to the end of the solve (and of the adjoint in backward): calls
from several host threads on the same shape take turns.
"""
import threading

import torch

from .ppe import PressurePoisson

_handles = {}
_lock = threading.Lock()


def _handle(shape, spacing, precision, device):
    """(handle, its lock) for this shape, spacing, precision and device."""
    key = (tuple(shape), tuple(spacing), precision, device.index)
    with _lock:
        entry = _handles.get(key)
        if entry is None:
            s = PressurePoisson(shape, spacing, precision=precision, krylov=True,
                                max_cycles=400, device=device.index)
            entry = (s, threading.Lock())
            _handles[key] = entry
        return entry


def clear_cache():
    """Destroy the cached handles (frees their device memory)."""
    with _lock:
        for s, lock in _handles.values():
            with lock:
                s.close()
        _handles.clear()


def _check(rho, b):
    if rho.shape != b.shape or rho.dim() != 3:
        raise ValueError("rho and b must have the same (nz, ny, nx) shape")
    if rho.dtype != torch.float64 or b.dtype != torch.float64 or not b.is_cuda:
        raise TypeError("rho and b must be float64 CUDA tensors")


@torch.library.custom_op("gbmg::solve", mutates_args=())
def solve(rho: torch.Tensor, b: torch.Tensor, dx: float, dy: float, dz: float, tol: float,
          adjoint_tol: float, precision: str) -> torch.Tensor:
    _check(rho, b)
    s, lock = _handle(b.shape, (dx, dy, dz), precision, b.device)
    p = torch.zeros_like(b, memory_format=torch.contiguous_format)
    with lock:
        s.ppe_init(rho.contiguous())
        s.solve(b.contiguous(), p, tol=tol)
    return p


@solve.register_fake
def _(rho, b, dx, dy, dz, tol, adjoint_tol, precision):
    return torch.empty_like(b, memory_format=torch.contiguous_format)


def _setup_context(ctx, inputs, output):
    rho, b, dx, dy, dz, tol, adjoint_tol, precision = inputs
    ctx.save_for_backward(rho, output)
    ctx.cfg = (dx, dy, dz, adjoint_tol, precision)


def _backward(ctx, grad_p):
    rho, p = ctx.saved_tensors
    dx, dy, dz, adjoint_tol, precision = ctx.cfg
    s, lock = _handle(p.shape, (dx, dy, dz), precision, p.device)
    lam = torch.zeros_like(p)
    with lock:
        s.ppe_init(rho.contiguous())
        s.solve(grad_p.contiguous(), lam, tol=adjoint_tol)
        grad_rho = s.adjoint(p, lam)[0] if ctx.needs_input_grad[0] else None
    grad_b = lam if ctx.needs_input_grad[1] else None
    return grad_rho, grad_b, None, None, None, None, None, None


solve.register_autograd(_backward, setup_context=_setup_context)
