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


def _driver_oracle(rho, u, v, w, p_hat, rho12, dt, spacing, tol_rms, restarts, max_cycles):
    """The DomainDecomposition driver's loop ("DomainDecomposition/3D/src/
    ns_solver/ns_ppe_mg_solver.f90:17-50") on the oracle: V(2,2) cycles on the
    Laplacian from p^; a cycle that cuts the relative residual by under 1% (or
    raises it) restarts from p^ = 1.5 p - 0.5 p^ with the source rebuilt, at most
    `restarts` times; after that such a cycle stops once the residual is under
    1000 tol; otherwise the loop stops under tol (the RMS threshold as a
    relative one).  Returns (p, p^, restarts made, cycles)."""
    lap = orc.face_coef(np.ones_like(rho), spacing)
    ph = p_hat.copy()
    cycles = 0
    for restart in range(restarts + 1):
        src = orc.split_rhs(rho, u, v, w, ph, rho12, dt, spacing)
        b = src - src.mean()
        bn = np.linalg.norm(b)
        tol = tol_rms * np.sqrt(b.size) / bn
        _, s0 = orc.residual(lap, ph, b)
        prev = np.sqrt(s0) / bn
        _, st = orc.mg_solve(lap, b, p0=ph, tol=0.0, max_cycles=max_cycles)
        stop, stagnated = len(st["history"]), False
        for k, rel in enumerate(st["history"], 1):
            grow = rel / prev
            if grow > 1.0 or abs(grow - 1.0) < 0.01:
                if restart < restarts:
                    stop, stagnated = k, True
                    break
                if rel < 1000.0 * tol:
                    stop = k
                    break
            elif rel < tol:
                stop = k
                break
            prev = rel
        p, _ = orc.mg_solve(lap, b, p0=ph, tol=0.0, max_cycles=stop)
        cycles += stop
        if not stagnated:
            return p, ph, restart, cycles
        ph = 1.5 * p + (1.0 - 1.5) * ph
    raise AssertionError("unreachable")


def test_split_restarts_match_the_driver(cuda):
    """gbmg_params.split_restarts: a tolerance below the FP64 floor makes every
    solve stagnate, so the driver restarts five times and then runs to the
    cycle limit; pressure and corrected velocity against the driver's loop
    restated on the oracle (the stagnating cycle can differ by one between
    the two at the rounding floor, which moves p at the rounding level)."""
    case, rho, (u, v, w), p_hat = _case((32, 32, 32))
    rho12, tol_rms, maxc = 1e-3, 1e-30, 60
    want_p, want_ph, want_r, want_c = _driver_oracle(rho, u, v, w, p_hat, rho12, case.dt,
                                                     case.spacing, tol_rms, 5, maxc)
    assert want_r == 5
    with PressurePoisson(case.shape, case.spacing, split_restarts=5, stop_rule="rms",
                         max_cycles=maxc) as s:
        s.ppe_mg_solver_init(rho, rho12)
        uo, vo, wo = u.copy(), v.copy(), w.copy()
        p, st = s.ppe_mg_solver(uo, vo, wo, case.dt, p_hat, tol=tol_rms, check=False)
    assert st["restarts"] == 5 and st["status"] != 0
    assert abs(st["cycles"] - want_c) <= 6, (st["cycles"], want_c)
    assert rel_l2(p, want_p) <= 1e-9
    want_u = orc.split_correct(rho, want_p, want_ph, rho12, case.dt, u, v, w, case.spacing)
    for a, b in zip((uo, vo, wo), want_u):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-9 * np.abs(b).max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_split_restarts_leave_a_converging_solve_alone(cuda, precision):
    """With a reachable tolerance no cycle stagnates: no restart, and the same
    bits as without the option."""
    case, rho, (u, v, w), p_hat = _case((32, 32, 32))
    out = []
    for nres in (0, 5):
        with PressurePoisson(case.shape, case.spacing, precision=precision, split_restarts=nres,
                             stop_rule="rms", inner_cycles=1, max_cycles=100) as s:
            s.ppe_mg_solver_init(rho, 1e-3)
            uo, vo, wo = u.copy(), v.copy(), w.copy()
            p, st = s.ppe_mg_solver(uo, vo, wo, case.dt, p_hat, tol=1e-6)
            out.append((p, uo, st))
    assert out[1][2]["restarts"] == 0 and out[1][2]["cycles"] == out[0][2]["cycles"]
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


def test_split_restarts_invalid_with_krylov(cuda):
    with pytest.raises(GBMGError):
        PressurePoisson((16, 16, 16), (1 / 16,) * 3, split_restarts=2, krylov=True)
