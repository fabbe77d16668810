"""Central differences of the pressure solve without cancellation, for checking
gradients (no reference counterpart: the reference's solvers are not
differentiable).

For J(phi) = 1/2 |p(phi) - p_t|^2 with A(phi) p = b, the plain central
difference (J(phi + h v) - J(phi - h v)) / 2h subtracts two nearly equal
losses: each carries the error of its solve relative to |b|, while their
difference is of order h.  With h = 1e-6 that noise, not the gradient, sets
the agreement (a few 1e-6 on the 1024^2 eight-bubble case).  The same
difference is computed here from its parts:
    A+ p+ = b,  A- p- = b  =>  A+ (p+ - p-) = (A- - A+) p-,
so d = p+ - p- solves one system whose right-hand side is already of order h,
and
    J(phi + h v) - J(phi - h v) = sum d (p- - p_t) + 1/2 sum d^2
holds exactly.  The face coefficients of A- and A+ differ by far less than a
factor 2, so their difference is exact in FP64 (Sterbenz's lemma), and the
solve for d has a relative tolerance of its own size.
"""
import torch

from .ppe import PressurePoisson


def operator_apply(coef, p):
    """(A p)_i = sum over faces of c_f (p_nb - p_i) for cell-shaped low-face
    coefficient arrays (cx couples cells i-1 and i along x; walls are 0)."""
    out = torch.zeros_like(p)
    for axis, c in zip((2, 1, 0), coef):
        if p.shape[axis] < 2:
            continue
        hi = [slice(None)] * 3
        lo = [slice(None)] * 3
        hi[axis] = slice(1, None)
        lo[axis] = slice(None, -1)
        hi, lo = tuple(hi), tuple(lo)
        f = c[hi] * (p[hi] - p[lo])
        out[lo] += f
        out[hi] -= f
    return out


def central_difference(solver: PressurePoisson, phi, b, p_t, v, h, eps, rho_pos, rho_neg,
                       tol=1e-12, diff_tol=1e-10):
    """(J(phi + h v) - J(phi - h v)) / (2 h) for J = 1/2 |p(phi, b) - p_t|^2,
    from p- = p(phi - h v) and d = p(phi + h v) - p(phi - h v) (one solve of
    (A-) p- = b to tol and one of (A+) d = (A- - A+) p- to diff_tol).  solver
    should be an FP64 handle; phi, b, p_t, v are float64 CUDA tensors of the
    grid's shape.  Leaves the solver's operator at phi + h v."""
    dev = b.device
    solver.rho_mu(phi - h * v, eps, rho_pos, rho_neg)
    c_minus = [torch.from_numpy(a).to(dev) for a in solver.level_coef(0)]
    p_minus = torch.zeros_like(b)
    solver.solve(b, p_minus, tol=tol)
    solver.rho_mu(phi + h * v, eps, rho_pos, rho_neg)
    c_plus = [torch.from_numpy(a).to(dev) for a in solver.level_coef(0)]
    dc = [a - c for a, c in zip(c_minus, c_plus)]
    r = operator_apply(dc, p_minus)
    d = torch.zeros_like(b)
    solver.solve(r, d, tol=diff_tol)
    dj = (d * (p_minus - p_t)).sum() + 0.5 * (d * d).sum()
    return float(dj / (2.0 * h))
