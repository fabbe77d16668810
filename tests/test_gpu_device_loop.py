"""The cycle loop on the device against the loop on the host.

use_graph=True runs the whole cycle loop as one CUDA graph: a WHILE node
repeats the iteration, and a one-thread controller kernel after each cycle
applies the stopping tests (divergence, residual or increment, the mixed
solve's flat-residual test, the cycle limit) and ends the loop.
use_graph="cycle" replays one graph per cycle and tests on the host, and
use_graph=False launches every kernel.  All three run the same kernels in
the same order and the controller does the host's arithmetic, so the pressure
is bit-identical and the cycle counts are equal, for every kind of iteration
and stopping rule, for a solve that hits the cycle limit, and for warm starts
of the mixed solve (whose loop may restart after its FP64 certification)."""
import numpy as np
import pytest

from fortrancfd_gb300 import PressurePoisson
from tests import cases

pytestmark = pytest.mark.gpu

MODES = (True, "cycle", False)


def _solve_all(c, tol, p0=None, check=True, **kw):
    out = []
    for g in MODES:
        with PressurePoisson(c.shape, c.spacing, use_graph=g, **kw) as s:
            s.ppe_init(c.rho)
            p = None if p0 is None else p0.copy()
            p, st = s.solve(c.b, p=p, tol=tol, check=check)
            out.append((p, st))
    return out


def _same(out):
    (p0, s0), rest = out[0], out[1:]
    for p, st in rest:
        np.testing.assert_array_equal(p, p0)
        assert st["cycles"] == s0["cycles"]
        assert st["status"] == s0["status"]
        assert st["rel_residual"] == s0["rel_residual"]
        assert st["increment"] == s0["increment"]
    assert s0["device_loop"] == 1
    assert all(st["device_loop"] == 0 for _, st in rest)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("krylov", [False, True])
def test_device_loop_matches_host_loop(cuda, precision, krylov):
    c = cases.config(1, 4)
    _same(_solve_all(c, 1e-10, precision=precision, krylov=krylov, max_cycles=200))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
# the 128^2 bubble: max |p| is about 3e4 and the RMS of b about 2.6e5, so both
# thresholds stop near a relative residual of 1e-10
@pytest.mark.parametrize("rule,tol", [("increment", 1e-6), ("rms", 1e-4)])
def test_device_loop_stop_rules(cuda, precision, rule, tol):
    c = cases.config(0, 1)
    out = _solve_all(c, tol, precision=precision, stop_rule=rule, max_cycles=200)
    _same(out)
    if rule == "increment":
        assert 0.0 < out[0][1]["increment"] < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_device_loop_stops_at_the_cycle_limit(cuda, precision):
    c = cases.config(1, 4)
    out = _solve_all(c, 1e-14, check=False, precision=precision, max_cycles=5)
    _same(out)
    assert out[0][1]["cycles"] == 5 and out[0][1]["status"] != 0


def test_device_loop_warm_start_mixed(cuda):
    c = cases.config(1, 4)
    rng = np.random.default_rng(5)
    p0 = rng.standard_normal(c.shape)
    _same(_solve_all(c, 1e-10, p0=p0, precision="mixed", max_cycles=200))


def test_fp32_cycles_per_defect_correction(cuda):
    """inner_cycles: FP32 V-cycles per double-word defect correction.  Every
    setting reaches the tolerance in FP64 (certified) with the same solution
    to 1e-9; a fixed count tests every that many cycles; the default (four,
    the last correction as many as the last reduction predicts) takes at most
    one cycle more than one cycle per correction."""
    from fortrancfd_gb300 import GBMGError
    from tests.cases import rel_l2
    c = cases.config(1, 4)
    out = {}
    for inner in (1, 2, 3):
        with PressurePoisson(c.shape, c.spacing, precision="mixed", inner_cycles=inner,
                             max_cycles=200) as s:
            s.ppe_init(c.rho)
            out[inner] = s.solve(c.b, tol=1e-10)
    for inner in (2, 3):
        assert out[inner][1]["status"] == 0 and out[inner][1]["rel_residual"] < 1e-10
        assert rel_l2(out[inner][0], out[1][0]) <= 1e-9
        assert out[inner][1]["cycles"] % inner == 0
    with PressurePoisson(c.shape, c.spacing, precision="mixed", max_cycles=200) as s:
        s.ppe_init(c.rho)
        p, st = s.solve(c.b, tol=1e-10)
    assert st["status"] == 0 and st["rel_residual"] < 1e-10
    assert st["cycles"] <= out[1][1]["cycles"] + 1, (st["cycles"], out[1][1]["cycles"])
    assert rel_l2(p, out[1][0]) <= 1e-9
    with pytest.raises(GBMGError):
        PressurePoisson(c.shape, c.spacing, precision="mixed", inner_cycles=2,
                        stop_rule="increment")
