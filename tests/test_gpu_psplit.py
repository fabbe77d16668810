"""GPU tests of the pressure-split projection (gbmg_set_split /
gbmg_project_split, the form of the DomainDecomposition solver).

The velocity correction is compared bit for bit with the oracle's applied to
the pressure the GPU returned; the pressure is the oracle's solution of the
Laplacian with the oracle's split source to 1e-8 relative (solves to 1e-12);
the corrected velocity is divergence-free to the solve tolerance."""
import numpy as np
import pytest
import torch

from fortrancfd_gb300 import GBMGError, PressurePoisson, inputs
from oracle import oracle as orc
from tests.cases import rel_l2

pytestmark = pytest.mark.gpu


def _case(shape):
    case = inputs.custom(shape, centers=((0.45, 0.55, 0.4),), radii=(0.25,), seed=4)
    phi = inputs.level_set(case)
    rho = orc.rho_from_phi(phi, case.eps, 1.0, 1e-3)  # heavy 1, light rho_12
    u, v, w = inputs.velocity(case)
    p_hat = np.random.default_rng(6).standard_normal(case.shape) * 10.0
    return case, rho, (u, v, w), p_hat


@pytest.mark.parametrize("shape,precision", [((32, 32, 32), "fp64"), ((32, 32, 32), "mixed"),
                                             ((1, 64, 64), "fp64"), ((16, 24, 32), "mixed")])
def test_split_projection_matches_oracle(cuda, shape, precision):
    case, rho, (u, v, w), p_hat = _case(shape)
    rho12 = 1e-3
    with PressurePoisson(case.shape, case.spacing, precision=precision, max_cycles=200) as s:
        s.ppe_mg_solver_init(rho, rho12)
        uo, vo, wo = u.copy(), v.copy(), w.copy()
        p, st = s.ppe_mg_solver(uo, vo, wo, case.dt, p_hat, tol=1e-12)
    assert st["status"] == 0 and st["rel_residual"] < 1e-12
    # correction: bitwise the oracle's with the same pressure
    want = orc.split_correct(rho, p, p_hat, rho12, case.dt, u, v, w, case.spacing)
    for a, b in zip((uo, vo, wo), want):
        np.testing.assert_array_equal(a, b)
    # pressure: the oracle's Laplacian solve of the oracle's split source
    src = orc.split_rhs(rho, u, v, w, p_hat, rho12, case.dt, case.spacing)
    lap = orc.face_coef(np.ones_like(rho), case.spacing)
    p_or, st_or = orc.mg_solve(lap, src - src.mean(), tol=1e-13, max_cycles=200)
    assert rel_l2(p, p_or) <= 1e-8
    mx0, _ = orc.div_stats(u, v, w, case.spacing)
    mx, _ = orc.div_stats(uo, vo, wo, case.spacing)
    assert mx < 1e-8 * mx0


def test_split_projection_device_tensors_and_state(cuda):
    case, rho, (u, v, w), p_hat = _case((16, 16, 16))
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)  # noqa: E731
    with PressurePoisson(case.shape, case.spacing) as s:
        with pytest.raises(GBMGError):  # no split operator yet
            s.ppe_mg_solver(t(u), t(v), t(w), case.dt, t(p_hat))
        s.ppe_mg_solver_init(t(rho), 1e-3)
        ud, vd, wd = t(u), t(v), t(w)
        p, st = s.ppe_mg_solver(ud, vd, wd, case.dt, t(p_hat), tol=1e-11)
        uh, vh, wh = u.copy(), v.copy(), w.copy()
        ph, _ = s.ppe_mg_solver(uh, vh, wh, case.dt, p_hat, tol=1e-11)
        np.testing.assert_array_equal(p.cpu().numpy(), ph)
        np.testing.assert_array_equal(ud.cpu().numpy(), uh)
        # the plain projection needs the density form back
        with pytest.raises(GBMGError):
            s.ppe_solver(u.copy(), v.copy(), w.copy(), case.dt)
        s.ppe_init(rho)
        s.ppe_solver(u.copy(), v.copy(), w.copy(), case.dt)
