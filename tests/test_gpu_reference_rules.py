"""The reference's own stopping rules and right-hand-side convention at the
drop-in boundary, on the GPU through the C ABI, against the oracle.

* GBMG_STOP_RMS: the DomainDecomposition driver ppe_mg_solver stops when the
  absolute RMS residual drops below p_tol*1e-3
  ("DomainDecomposition/3D/src/ns_solver/ns_ppe_mg_solver.f90:42-43").  The
  GPU stops at the same cycle as the oracle's residual history says.
* GBMG_STOP_INCREMENT: ppe_sor_solver and PRESS_POISSON stop when the largest
  change of p between iterations drops below p_tol
  ("Two phase flows/newOpenMP/3D+IBM/src/ns_solver/ns_ppe_solver.f90:143,152",
  "MPLS_RisingBubble/20190612/SOLVE_PRESSURE_POISSON.F90:158-164"); here the
  iteration is a V-cycle.  The GPU stops at the cycle where the oracle's
  iterates first change by less than p_tol.
* zero_wall_faces: MPLS_RisingBubble's RHSP zeroes the wall-normal faces of
  the velocity before its divergence ("SOLVE_PRESSURE_POISSON.F90:16-41").
  Checked in that code's array layout (ghost cells -2..N+3 per axis,
  "MPLS_RisingBubble/20190612/BC.F90:15") and density convention
  rho = ratio*H + (1 - H) ("MPLS_RisingBubble/20190612/AMURHO.F90:21-22").
"""
import numpy as np
import pytest

from fortrancfd_gb300 import PressurePoisson, inputs
from oracle import oracle as orc
from tests import cases
from tests.cases import rel_l2

pytestmark = pytest.mark.gpu


def _between(a, b):
    return float(np.sqrt(a * b))


@pytest.mark.parametrize("precision,idx,scale", [("fp64", 1, 4), ("mixed", 1, 4),
                                                 ("fp64", 0, 1), ("mixed", 1, 2)])
def test_rms_rule_stops_where_the_reference_driver_would(cuda, precision, idx, scale):
    c = cases.config(idx, scale)
    n = c.b.size
    bn = np.linalg.norm(c.b)
    _, st_or = orc.mg_solve(c.coef, c.b, tol=1e-13, max_cycles=40)
    rms = [h * bn / np.sqrt(n) for h in st_or["history"]]
    k = 8  # stop after cycle k + 1: a threshold between the RMS of cycles k and k + 1
    tol = _between(rms[k - 1], rms[k])
    with PressurePoisson(c.shape, c.spacing, precision=precision, stop_rule="rms") as s:
        s.ppe_init(c.rho)
        p, st = s.solve(c.b, tol=tol)
    assert st["status"] == 0
    assert st["rms_residual"] < tol
    if precision == "fp64":
        assert st["cycles"] == k + 1, (st["cycles"], k + 1)
    else:
        assert abs(st["cycles"] - (k + 1)) <= 1, (st["cycles"], k + 1)
    _, r2 = orc.residual(c.coef, p, c.b)
    assert np.sqrt(r2 / n) < tol


def _oracle_increments(c, kmax):
    """max |p_k - p_(k-1)| of the oracle's cycles from zero (iterates after k
    cycles, each mean-free)."""
    prev = np.zeros_like(c.b)
    out = []
    for k in range(1, kmax + 1):
        p, _ = orc.mg_solve(c.coef, c.b, tol=1e-300, max_cycles=k)
        out.append(float(np.abs(p - prev).max()))
        prev = p
    return out, prev


@pytest.mark.parametrize("precision,idx,scale", [("fp64", 1, 4), ("mixed", 1, 4),
                                                 ("fp64", 0, 1), ("mixed", 0, 1)])
def test_increment_rule_stops_where_the_reference_sweep_would(cuda, precision, idx, scale):
    c = cases.config(idx, scale)
    inc, _ = _oracle_increments(c, 12)
    k = 7
    tol = _between(inc[k - 1], inc[k])  # first below tol after cycle k + 1
    p_ref, _ = orc.mg_solve(c.coef, c.b, tol=1e-13, max_cycles=60)
    with PressurePoisson(c.shape, c.spacing, precision=precision, stop_rule="increment") as s:
        s.ppe_init(c.rho)
        p, st = s.solve(c.b, tol=tol)
    assert st["status"] == 0
    assert 0 < st["increment"] < tol
    if precision == "fp64":
        assert st["cycles"] == k + 1, (st["cycles"], k + 1)
    else:
        assert abs(st["cycles"] - (k + 1)) <= 1, (st["cycles"], k + 1)
    # a cycle contracts the error several-fold, so the error of the stopped
    # iterate is of the order of the last increment
    assert np.abs(p - p_ref).max() < 3 * tol


def test_increment_rule_needs_stationary_cycles(cuda):
    from fortrancfd_gb300 import GBMGError
    with pytest.raises(GBMGError):
        PressurePoisson((8, 8, 8), (0.125,) * 3, krylov=True, stop_rule="increment")


G = 3  # MPLS_RisingBubble's ghost width (arrays -2:N+3)


def _mp3_array(a, nan=True):
    """An MP3-layout array: ghost width 3 on every side, interior set to a
    (cell arrays; a face array's faces 0..N sit at indices 3..N+3 in its own
    axis, as U1(0:NODE_X) of the reference's -2:N+3 array)."""
    shape = tuple(m + 2 * G for m in a.shape)
    big = np.full(shape, np.nan if nan else 0.0)
    view = big[tuple(slice(G, G + m) for m in a.shape)]
    view[...] = a
    return big, view


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rhsp_wall_faces_in_the_mpls_layout(cuda, precision):
    nz, ny, nx = 16, 24, 32
    case = inputs.custom((nz, ny, nx), centers=((0.5, 0.45, 0.4),), radii=(0.2,), seed=5)
    ratio = 1000.0
    phi = inputs.level_set(case)
    # AMURHO: rho = ratio*HEAVY + (1 - HEAVY), HEAVY = 1 where phi > 0
    H = orc.heaviside(phi, case.eps)
    rho = ratio * H + (1.0 - H)
    rng = np.random.default_rng(11)
    faces = [rng.standard_normal((nz, ny, nx + 1)), rng.standard_normal((nz, ny + 1, nx)),
             rng.standard_normal((nz + 1, ny, nx))]  # wall faces NOT zero
    dt = 1e-3
    # the reference's sequence: walls zeroed, divergence, solve, correction
    want_faces = [a.copy() for a in faces]
    want_faces[0][..., 0] = want_faces[0][..., -1] = 0.0
    want_faces[1][:, 0, :] = want_faces[1][:, -1, :] = 0.0
    want_faces[2][0] = want_faces[2][-1] = 0.0
    coef = orc.face_coef(rho, case.spacing)
    b = orc.divergence(*want_faces, dt, case.spacing)
    p_or, _ = orc.mg_solve(coef, b, tol=1e-13, max_cycles=80)
    u_or, v_or, w_or = orc.correct(rho, p_or, dt, *want_faces, case.spacing)
    rho_big, rho_v = _mp3_array(rho)
    vel = [_mp3_array(a) for a in faces]
    p_big, p_v = _mp3_array(np.zeros((nz, ny, nx)))
    p_tol = 1e-9 * np.abs(p_or).max()
    with PressurePoisson(case.shape, case.spacing, precision=precision, stop_rule="increment",
                         zero_wall_faces=True, max_cycles=100) as s:
        s.ppe_init(rho_v)
        _, st = s.ppe_solver(vel[0][1], vel[1][1], vel[2][1], dt, tol=p_tol, p=p_v)
    assert st["status"] == 0 and st["increment"] < p_tol
    # the caller's wall faces were zeroed, the ghost cells left alone
    np.testing.assert_array_equal(vel[0][1][..., [0, -1]], 0.0)
    np.testing.assert_array_equal(vel[1][1][:, [0, -1], :], 0.0)
    np.testing.assert_array_equal(vel[2][1][[0, -1]], 0.0)
    assert np.isnan(p_big[0]).all() and np.isnan(vel[0][0][:, :, 0]).all()
    assert np.abs(p_v - p_or).max() < 10 * p_tol
    for got, want in zip((vel[0][1], vel[1][1], vel[2][1]), (u_or, v_or, w_or)):
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-6 * np.abs(want).max())


def test_wall_faces_read_as_given_by_default(cuda):
    """Without zero_wall_faces the divergence reads the wall faces as passed
    (the ppe_sor_solver prologue, whose callers' velbc zeroed them)."""
    c = cases.config(1, 8)
    u = c.u.copy()
    u[..., 0] = 1.0
    with PressurePoisson(c.shape, c.spacing) as s:
        got = s.divergence(u, c.v, c.w, c.case.dt)
    with PressurePoisson(c.shape, c.spacing, zero_wall_faces=True) as s:
        got0 = s.divergence(u.copy(), c.v, c.w, c.case.dt)
    want = orc.divergence(u, c.v, c.w, c.case.dt, c.spacing, remove_mean=False)
    np.testing.assert_array_equal(got, want)
    want0 = orc.divergence(c.u, c.v, c.w, c.case.dt, c.spacing, remove_mean=False)
    np.testing.assert_array_equal(got0, want0)
    assert rel_l2(got, got0) > 0
