"""torch.ops.gbmg.solve: registration (CPU) and, on the GPU, the solve against
the FP64 oracle (1e-8 relative at tol 1e-12), its gradients against the
autograd Function on the same kernels (1e-8), and its rho gradient against
central differences (2e-6 relative; forward 1e-13, adjoint 1e-10)."""
import numpy as np
import pytest
import torch

import fortrancfd_gb300.ops  # noqa: F401  registers torch.ops.gbmg
from oracle import oracle as orc
from tests import cases
from tests.cases import rel_l2


def test_operator_is_registered():
    assert hasattr(torch.ops.gbmg, "solve")
    schema = str(torch.ops.gbmg.solve.default._schema)
    assert "rho" in schema and "adjoint_tol" in schema


@pytest.mark.gpu
def test_solve_matches_oracle(cuda):
    c = cases.config(1, 8)
    rho = torch.from_numpy(c.rho).to(cuda)
    b = torch.from_numpy(c.b).to(cuda)
    p = torch.ops.gbmg.solve(rho, b, *c.spacing, 1e-12, 1e-10, "mixed")
    want, _ = orc.mg_solve(c.coef, c.b, tol=1e-13, max_cycles=400, krylov=1)
    assert rel_l2(p.cpu().numpy(), want) <= 1e-8


@pytest.mark.gpu
def test_gradients_match_the_autograd_function(cuda):
    """Same kernels as PressureSolveRho (whose gradients the adjoint tests
    check against central differences): the two agree to 1e-8."""
    from fortrancfd_gb300 import PressurePoisson
    from fortrancfd_gb300.autograd import PressureSolveRho

    c = cases.config(1, 8)
    rho0 = torch.from_numpy(c.rho).to(cuda)
    b0 = torch.from_numpy(c.b).to(cuda)
    w = torch.from_numpy(np.random.default_rng(4).standard_normal(c.shape)).to(cuda)
    grads = []
    for use_op in (True, False):
        rho = rho0.clone().requires_grad_(True)
        b = b0.clone().requires_grad_(True)
        if use_op:
            p = torch.ops.gbmg.solve(rho, b, *c.spacing, 1e-12, 1e-11, "fp64")
        else:
            s = PressurePoisson(c.shape, c.spacing, krylov=True, max_cycles=400)
            p = PressureSolveRho.apply(rho, b, s, 1e-12, 1e-11)
        (w * p).sum().backward()
        grads.append((rho.grad.cpu().numpy(), b.grad.cpu().numpy()))
    (gr0, gb0), (gr1, gb1) = grads
    assert rel_l2(gr0, gr1) <= 1e-8
    assert rel_l2(gb0, gb1) <= 1e-8


@pytest.mark.gpu
def test_rho_gradient_matches_central_differences(cuda):
    from fortrancfd_gb300 import inputs

    case = inputs.config(3, 8)
    c = cases.Built(case)
    rho0 = torch.from_numpy(c.rho).to(cuda)
    b0 = torch.from_numpy(c.b).to(cuda)
    args = (*c.spacing, 1e-13, 1e-10, "fp64")
    rho = rho0.clone().requires_grad_(True)
    (0.5 * (torch.ops.gbmg.solve(rho, b0, *args) ** 2).sum()).backward()
    v = torch.from_numpy(np.random.default_rng(3).standard_normal(c.shape)).to(cuda)
    v /= v.norm()
    h = 1e-6 * float(rho0.abs().max())
    with torch.no_grad():
        jp = 0.5 * (torch.ops.gbmg.solve(rho0 + h * v, b0, *args) ** 2).sum()
        jm = 0.5 * (torch.ops.gbmg.solve(rho0 - h * v, b0, *args) ** 2).sum()
    fd = float((jp - jm) / (2 * h))
    # as the autograd Function's rho test: 2e-6 (the adjoint's FP64 floor)
    assert abs(fd - float((rho.grad * v).sum())) <= 2e-6 * abs(fd)


@pytest.mark.gpu
def test_concurrent_calls_from_two_threads(cuda):
    """Two host threads call the operator on the same shape (one cached
    handle) with different densities: each result equals the one computed
    alone, because every call holds its handle's lock for the whole solve."""
    import threading

    c = cases.config(1, 8)
    rhos = [torch.from_numpy(c.rho).to(cuda), torch.from_numpy(c.rho[::-1].copy()).to(cuda)]
    b = torch.from_numpy(c.b).to(cuda)
    want = [torch.ops.gbmg.solve(r, b, *c.spacing, 1e-10, 1e-10, "fp64") for r in rhos]
    got = [[None] * 4 for _ in rhos]
    errors = []

    def run(i):
        try:
            torch.cuda.set_device(cuda)
            for k in range(4):
                got[i][k] = torch.ops.gbmg.solve(rhos[i], b, *c.spacing, 1e-10, 1e-10, "fp64")
        except Exception as exc:  # reported below
            errors.append(exc)

    threads = [threading.Thread(target=run, args=(i,)) for i in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for i in range(2):
        for k in range(4):
            assert torch.equal(got[i][k], want[i]), (i, k)
