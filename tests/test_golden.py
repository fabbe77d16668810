"""Golden fixtures (tests/golden/, made by tests/golden/make_golden.py): the
oracle on CPU and the CUDA path on GPU must reproduce the stored answers."""
import os

import numpy as np
import pytest

from fortrancfd_gb300 import inputs
from oracle import oracle as orc
from tests.cases import rel_l2

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = ["bubble2d_128.npz", "sphere3d_32.npz"]


def load(name):
    return np.load(os.path.join(HERE, name))


def build(fx):
    case = inputs.config(int(fx["index"]), int(fx["scale"]))
    phi = inputs.level_set(case)
    rho = orc.rho_from_phi(phi, case.eps, case.rho_pos, case.rho_neg)
    u, v, w = inputs.velocity(case)
    return case, phi, rho, (u, v, w)


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_reproduces_fixture(name):
    fx = load(name)
    case, phi, rho, (u, v, w) = build(fx)
    assert rho.sum() == pytest.approx(float(fx["rho_sum"]), rel=1e-14)
    coef = orc.face_coef(rho, case.spacing)
    b = orc.divergence(u, v, w, case.dt, case.spacing)
    assert np.abs(b).sum() == pytest.approx(float(fx["b_sum_abs"]), rel=1e-13)
    p, st = orc.mg_solve(coef, b, tol=1e-10)
    assert st["cycles"] == int(fx["cycles"])
    # thread-count dependent reduction order only
    assert rel_l2(p, fx["p"]) <= 1e-12
    uo, vo, wo = orc.correct(rho, p, case.dt, u, v, w, case.spacing)
    for a, key in ((uo, "u_abs"), (vo, "v_abs"), (wo, "w_abs")):
        assert np.abs(a).sum() == pytest.approx(float(fx[key]), rel=1e-10)


def test_oracle_cycle_reproduces_reference_transliteration():
    fx = load("dd3_constant_8.npz")
    h = float(fx["h"])
    coef = orc.face_coef(np.ones((8, 8, 8)), (h, h, h))
    for k in (1, 2, 3):
        p, st = orc.mg_solve(coef, fx["b"], tol=1e-300, max_cycles=k, levels=int(fx["levels"]),
                             smoother=1, record_history=0)
        ref = fx[f"p{k}"]
        np.testing.assert_allclose(p, ref, rtol=0, atol=1e-11 * np.abs(ref).max())


@pytest.mark.gpu
@pytest.mark.parametrize("name", FIXTURES)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_reproduces_fixture(cuda, name, precision):
    from fortrancfd_gb300 import PressurePoisson

    fx = load(name)
    case, phi, rho, (u, v, w) = build(fx)
    with PressurePoisson(case.shape, case.spacing, precision=precision) as s:
        s.rho_mu(phi, case.eps, case.rho_pos, case.rho_neg)
        p, st = s.ppe_solver(u, v, w, case.dt, tol=1e-10)
    assert st["status"] == 0
    if precision == "fp64":
        assert abs(st["cycles"] - int(fx["cycles"])) <= 1
        assert rel_l2(p, fx["p"]) <= 1e-9
    else:
        assert rel_l2(p, fx["p"]) <= 1e-9
    for a, key in ((u, "u_abs"), (v, "v_abs"), (w, "w_abs")):
        assert np.abs(a).sum() == pytest.approx(float(fx[key]), rel=1e-8)


def _momentum_fixture():
    return np.load(os.path.join(HERE, "momentum2d_12x10.npz"))


def _momentum_state(f):
    st = {k[3:]: f[k] for k in f.files if k.startswith("in_")}
    st["w"] = st["nrm_z"] = None
    return st


def test_momentum_oracle_equals_the_golden_loops():
    """The oracle's predictor pass and CCD gradient equal the stored outputs
    of the literal loop restatement bit for bit (curvature: its pow)."""
    from oracle import oracle as orc
    f = _momentum_fixture()
    g = int(f["ghost"])
    shape = tuple(int(x) for x in f["shape"])
    sp = tuple(float(x) for x in f["spacing"])
    st = _momentum_state(f)
    prm = orc.ns_params(ghost=g, bc=tuple(int(b) for b in f["prm_bc"]) + (1, 1),
                        dt=float(f["prm_dt"]), re=float(f["prm_re"]), fr=float(f["prm_fr"]),
                        we=float(f["prm_we"]), mu_12=float(f["prm_mu_12"]),
                        gravity=(float(f["prm_gx"]), float(f["prm_gy"]), 0.0),
                        btn_g=float(f["prm_btn_g"]), btn_sf=float(f["prm_btn_sf"]))
    dif = orc.ns_diffusion(shape, sp, prm, st)[:2]
    old = (st["u"], st["v"])
    src, vel = orc.ns_advance(shape, sp, prm, old, old, dif, (st["su_old"], st["sv_old"]))
    u, v = vel[0].copy(), vel[1].copy()
    orc.velbc(shape, prm, u, v)
    bits = lambda a: np.ascontiguousarray(a).view(np.int64)  # noqa: E731
    for got, key in ((src[0], "su"), (src[1], "sv"), (u, "u_new"), (v, "v_new")):
        assert np.array_equal(bits(got), bits(f[key])), key
    fx, fy, _, cv = orc.ns_curvature(shape, sp, g, st["phi"])
    assert np.array_equal(bits(fx), bits(f["ccd_fx"]))
    assert np.array_equal(bits(fy), bits(f["ccd_fy"]))
    np.testing.assert_allclose(cv, f["ccd_curv"], rtol=1e-15, atol=0)
