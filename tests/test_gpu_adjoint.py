"""GPU tests of the differentiable solve: the adjoint kernel against the FP64
oracle adjoint, and autograd gradients (with respect to b and to the level set
phi, through H_eps and beta) against central finite differences.

Tolerances: the adjoint kernel does the oracle's arithmetic (1e-12 relative);
gradients from FP64 forward solves to a relative residual of 1e-13 (a few
times the FP64 floor of these density-ratio-1000 cases) and adjoint solves to
1e-10 (the adjoint's right-hand side p - p_t is smooth, which raises its
floor) match central differences with step 1e-6 to 1e-6 relative along random
unit directions; the mixed-precision forward and
backward match the FP64 oracle adjoint to 1e-6 relative L2.
"""
import numpy as np
import pytest
import torch

from fortrancfd_gb300 import PressurePoisson, inputs
from fortrancfd_gb300.autograd import PressureSolveRho, pressure_solve
from oracle import oracle as orc
from tests.cases import rel_l2

pytestmark = pytest.mark.gpu


def small_case():
    # the adjoint benchmark geometry (8 circles in 2D) at 128^2
    return inputs.config(3, 8)


def test_adjoint_kernel_matches_oracle(cuda):
    case = small_case()
    rng = np.random.default_rng(11)
    phi = inputs.level_set(case)
    rho = orc.rho_from_phi(phi, case.eps, case.rho_pos, case.rho_neg)
    p = rng.standard_normal(case.shape)
    lam = rng.standard_normal(case.shape)
    want_rho, want_phi = orc.adjoint(rho, p, lam, case.spacing, phi, case.eps, case.rho_pos,
                                     case.rho_neg)
    with PressurePoisson(case.shape, case.spacing) as s:
        s.ppe_init(rho)
        g_rho, g_phi = s.adjoint(p, lam, phi, case.eps, case.rho_pos, case.rho_neg)
    np.testing.assert_allclose(g_rho, want_rho, rtol=1e-12, atol=1e-12 * np.abs(want_rho).max())
    np.testing.assert_allclose(g_phi, want_phi, rtol=1e-12, atol=1e-12 * np.abs(want_phi).max())


def _loss_setup(cuda):
    case = small_case()
    phi = torch.from_numpy(inputs.level_set(case)).to(cuda)
    b = torch.from_numpy(orc.divergence(*inputs.velocity(case), case.dt, case.spacing)).to(cuda)
    bt = torch.from_numpy(
        orc.divergence(*inputs.velocity(case, seed=case.extra["target_seed"]), case.dt,
                       case.spacing)).to(cuda)
    return case, phi, b, bt


@pytest.mark.parametrize("wrt", ["phi", "b"])
def test_gradients_match_central_differences(cuda, wrt):
    case, phi, b, bt = _loss_setup(cuda)
    kw = dict(eps=case.eps, rho_pos=case.rho_pos, rho_neg=case.rho_neg)
    with PressurePoisson(case.shape, case.spacing, krylov=True, max_cycles=600) as s, \
            PressurePoisson(case.shape, case.spacing, krylov=True, max_cycles=600) as st:
        p_t = pressure_solve(phi, bt, st, tol=1e-13, **kw).detach()

        def J(ph, bb):
            p = pressure_solve(ph, bb, s, tol=1e-13, adjoint_tol=1e-10, **kw)
            return 0.5 * ((p - p_t) ** 2).sum()

        x = (phi if wrt == "phi" else b).clone().requires_grad_(True)
        loss = J(x, b) if wrt == "phi" else J(phi, x)
        loss.backward()
        g = x.grad
        rng = np.random.default_rng(21)
        h = 1e-6 if wrt == "phi" else 1e-6 * float(b.abs().max())
        for _ in range(16):
            v = torch.from_numpy(rng.standard_normal(case.shape)).to(cuda)
            v /= v.norm()
            with torch.no_grad():
                if wrt == "phi":
                    jp, jm = J(phi + h * v, b), J(phi - h * v, b)
                else:
                    jp, jm = J(phi, b + h * v), J(phi, b - h * v)
            fd = float((jp - jm) / (2 * h))
            ad = float((g * v).sum())
            assert abs(fd - ad) <= 1e-6 * max(abs(fd), 1e-30) + 1e-9 * float(g.norm()), (fd, ad)


def test_mixed_gradient_matches_fp64_oracle_adjoint(cuda):
    case, phi, b, bt = _loss_setup(cuda)
    phin, bn, btn = phi.cpu().numpy(), b.cpu().numpy(), bt.cpu().numpy()
    # FP64 oracle: forward, target, adjoint
    rho = orc.rho_from_phi(phin, case.eps, case.rho_pos, case.rho_neg)
    coef = orc.face_coef(rho, case.spacing)
    p_o, _ = orc.mg_solve(coef, bn, tol=1e-13, max_cycles=400, krylov=1)
    pt_o, _ = orc.mg_solve(coef, btn, tol=1e-13, max_cycles=400, krylov=1)
    lam_o, _ = orc.mg_solve(coef, (p_o - pt_o).copy(), tol=1e-13, max_cycles=400, krylov=1)
    _, gphi_o = orc.adjoint(rho, p_o, lam_o, case.spacing, phin, case.eps, case.rho_pos,
                            case.rho_neg)
    kw = dict(eps=case.eps, rho_pos=case.rho_pos, rho_neg=case.rho_neg)
    with PressurePoisson(case.shape, case.spacing, precision="mixed", krylov=True,
                         max_cycles=400) as s:
        p_t = pressure_solve(phi, bt, s, tol=1e-12, **kw).detach()
        x = phi.clone().requires_grad_(True)
        bb = b.clone().requires_grad_(True)
        loss = 0.5 * ((pressure_solve(x, bb, s, tol=1e-12, adjoint_tol=1e-10, **kw) - p_t)
                      ** 2).sum()
        loss.backward()
    assert rel_l2(x.grad.cpu().numpy(), gphi_o) <= 1e-6
    assert rel_l2(bb.grad.cpu().numpy(), lam_o - lam_o.mean()) <= 1e-6


def test_rho_input_function(cuda):
    case, phi, b, bt = _loss_setup(cuda)
    rho = torch.from_numpy(orc.rho_from_phi(phi.cpu().numpy(), case.eps, case.rho_pos,
                                            case.rho_neg)).to(cuda).requires_grad_(True)
    with PressurePoisson(case.shape, case.spacing, krylov=True, max_cycles=400) as s:
        p = PressureSolveRho.apply(rho, b, s, 1e-13, 1e-10)
        (0.5 * (p ** 2).sum()).backward()
        g = rho.grad
        v = torch.from_numpy(np.random.default_rng(3).standard_normal(case.shape)).to(cuda)
        v /= v.norm()
        h = 1e-6 * float(rho.detach().abs().max())
        with torch.no_grad():
            jp = 0.5 * (PressureSolveRho.apply(rho.detach() + h * v, b, s, 1e-13) ** 2).sum()
            jm = 0.5 * (PressureSolveRho.apply(rho.detach() - h * v, b, s, 1e-13) ** 2).sum()
    fd = float((jp - jm) / (2 * h))
    # the density enters every coefficient directly, so this gradient feels the
    # adjoint's FP64 floor (~1e-10 relative residual here) more: 2e-6
    assert abs(fd - float((g * v).sum())) <= 2e-6 * abs(fd)


def test_rollout_gradient_matches_central_differences(cuda):
    """Config-4 geometry at 1/8 resolution (16 x 16 x 32), 3 steps: dJ/dcentres
    and dJ/dradii through the checkpointed level set and the adjoint solves."""
    from fortrancfd_gb300.rollout import rollout_loss

    case = inputs.config(4, 8)
    c0 = torch.from_numpy(case.centers.copy()).to(cuda)
    r0 = torch.from_numpy(case.radii.copy()).to(cuda)
    with PressurePoisson(case.shape, case.spacing, krylov=True, max_cycles=400) as s:
        c = c0.clone().requires_grad_(True)
        r = r0.clone().requires_grad_(True)
        J = rollout_loss(c, r, case, s, steps=3, tol=1e-13, adjoint_tol=1e-10)
        J.backward()
        h = 1e-6
        checks = [("c", 0, 2), ("c", 1, 0), ("c", 3, 1), ("r", 2, None), ("r", 0, None)]
        for kind, i, a in checks:
            d = torch.zeros_like(c0 if kind == "c" else r0)
            if kind == "c":
                d[i, a] = h
            else:
                d[i] = h
            with torch.no_grad():
                if kind == "c":
                    jp = rollout_loss(c0 + d, r0, case, s, steps=3, tol=1e-13)
                    jm = rollout_loss(c0 - d, r0, case, s, steps=3, tol=1e-13)
                    ad = float(c.grad[i, a])
                else:
                    jp = rollout_loss(c0, r0 + d, case, s, steps=3, tol=1e-13)
                    jm = rollout_loss(c0, r0 - d, case, s, steps=3, tol=1e-13)
                    ad = float(r.grad[i])
            fd = float((jp - jm) / (2 * h))
            assert abs(fd - ad) <= 1e-5 * abs(fd) + 1e-9 * abs(float(J.detach())), (kind, i, a, fd, ad)


def test_gradient_matches_cancellation_free_central_differences(cuda):
    """The mixed-precision gradient with respect to phi against central
    differences with step 1e-6 along 16 random unit directions, each formed
    from p(phi - h v) and one solve for p(phi + h v) - p(phi - h v)
    (gradcheck.central_difference), so that the two losses are never
    subtracted: agreement to 1e-6 relative in every direction."""
    from fortrancfd_gb300.gradcheck import central_difference
    case, phi, b, bt = _loss_setup(cuda)
    kw = dict(eps=case.eps, rho_pos=case.rho_pos, rho_neg=case.rho_neg)
    with PressurePoisson(case.shape, case.spacing, precision="mixed", krylov="fgmres",
                         max_cycles=400) as s, \
            PressurePoisson(case.shape, case.spacing, krylov=True, max_cycles=600) as s64:
        p_t = pressure_solve(phi, bt, s, tol=1e-10, **kw).detach()
        x = phi.clone().requires_grad_(True)
        p = pressure_solve(x, b, s, tol=1e-10, adjoint_tol=1e-8, **kw)
        (0.5 * ((p - p_t) ** 2).sum()).backward()
        g = x.grad
        rng = np.random.default_rng(31)
        errs = []
        with torch.no_grad():
            for _ in range(16):
                v = torch.from_numpy(rng.standard_normal(case.shape)).to(cuda)
                v /= v.norm()
                fd = central_difference(s64, phi, b, p_t, v, 1e-6, **kw)
                errs.append(abs(fd - float((g * v).sum())) / abs(fd))
    assert max(errs) <= 1e-6, errs
