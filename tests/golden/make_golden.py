"""Regenerates the golden fixtures in tests/golden/ (run from the repo root:
python tests/golden/make_golden.py).

The reference ships no tests or fixtures for its pressure path and cannot be
built here, so these fixtures are outputs of this repo's CPU oracle on seeded
inputs (the two small benchmark geometries) plus, for the constant-coefficient
cycle, the line-by-line transliteration of the reference's multigrid in
tests/refloops.py.  They freeze the checker's answers so that the GPU tests
and later oracle changes are compared against stored numbers.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fortrancfd_gb300 import inputs  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from tests import refloops as ref  # noqa: E402


def solve_fixture(index, scale, name):
    case = inputs.config(index, scale)
    phi = inputs.level_set(case)
    rho = orc.rho_from_phi(phi, case.eps, case.rho_pos, case.rho_neg)
    coef = orc.face_coef(rho, case.spacing)
    u, v, w = inputs.velocity(case)
    b = orc.divergence(u, v, w, case.dt, case.spacing)
    p, st = orc.mg_solve(coef, b, tol=1e-10)
    uo, vo, wo = orc.correct(rho, p, case.dt, u, v, w, case.spacing)
    np.savez_compressed(os.path.join(HERE, name), index=index, scale=scale, p=p,
                        cycles=st["cycles"], history=np.array(st["history"]),
                        b_sum_abs=np.abs(b).sum(), rho_sum=rho.sum(),
                        u_sum=uo.sum(), v_sum=vo.sum(), w_sum=wo.sum(),
                        u_abs=np.abs(uo).sum(), v_abs=np.abs(vo).sum(), w_abs=np.abs(wo).sum())
    print(name, case.shape, st["cycles"], st["rel_residual"])


def dd_fixture():
    shape, levels = (8, 8, 8), 3
    h = 1.0 / 8
    rng = np.random.default_rng(3)
    b = rng.standard_normal(shape)
    b -= b.mean()
    dd = ref.DDMultigrid(8, 8, 8, h, h, h, levels, wall="folded")
    its = dd.solve(b, np.zeros(shape), 3)
    np.savez_compressed(os.path.join(HERE, "dd3_constant_8.npz"), b=b, p1=its[0], p2=its[1],
                        p3=its[2], levels=levels, h=h)
    print("dd3_constant_8", shape)


def momentum_fixture():
    """One predictor pass of the momentum step (sec_part1..3, the upwind
    advection, the AB2 predictor and velbc) and the CCD gradient and curvature
    of a small 2D state, computed by the literal loop restatement of the
    reference (tests/refloops.py).  The inputs are stored too, so the fixture
    does not depend on the platform's sin or cos."""
    g = 3
    shape, sp = (1, 10, 12), (1 / 12, 1 / 12, 1.0)
    case = inputs.custom(shape, extent=(1.0, 10 / 12, 1.0), centers=((0.5, 0.4, 0.5),),
                         radii=(0.25,), seed=21)
    st = inputs.momentum_state(case, ghost=g, amplitude=0.3)
    prm = dict(re=100.0, fr=0.5, we=2.0, mu_12=1e-2, gx=0.3, gy=-0.8, btn_g=1.0, btn_sf=1.0,
               dt=2e-3, bc=(1, 2, 1, 1))
    nx, ny = 12, 10
    tu, tv = ref.ns_ab_diff_sec_2d(st["u"], st["v"], st["rho"], st["mu"], st["delta"],
                                   st["phi"], st["nrm_x"], st["nrm_y"], st["curv"], g, nx, ny,
                                   sp[0], sp[1], prm["re"], prm["mu_12"], prm["gx"], prm["gy"],
                                   prm["btn_g"], prm["btn_sf"], prm["fr"], prm["we"])
    old = (st["u"], st["v"])
    src, vel = ref.ns_ab_adv_predictor(old, old, (tu, tv), (st["su_old"], st["sv_old"]), g,
                                       (nx, ny), sp[:2], prm["dt"])
    un, vn = vel[0].copy(), vel[1].copy()
    ref.velbc(un, vn, None, g, nx, ny, 1, prm["bc"][0:2], prm["bc"][2:4])
    fx, fy, _, cv = ref.curv(st["phi"].copy(), g, sp[0], sp[1])
    keys = ("u", "v", "su_old", "sv_old", "rho", "mu", "delta", "phi", "nrm_x", "nrm_y", "curv")
    np.savez_compressed(os.path.join(HERE, "momentum2d_12x10.npz"), ghost=g, spacing=sp,
                        shape=shape, **{"in_" + k: st[k] for k in keys},
                        **{"prm_" + k: np.asarray(v) for k, v in prm.items()},
                        su=src[0], sv=src[1], u_new=un, v_new=vn, ccd_fx=fx, ccd_fy=fy,
                        ccd_curv=cv)
    print("momentum2d_12x10", shape)


if __name__ == "__main__":
    if "--momentum" not in sys.argv:
        solve_fixture(0, 1, "bubble2d_128.npz")
        solve_fixture(1, 8, "sphere3d_32.npz")
        dd_fixture()
    momentum_fixture()
