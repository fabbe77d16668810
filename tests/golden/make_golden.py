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


if __name__ == "__main__":
    solve_fixture(0, 1, "bubble2d_128.npz")
    solve_fixture(1, 8, "sphere3d_32.npz")
    dd_fixture()
