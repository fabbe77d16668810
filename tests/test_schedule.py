"""The adaptive schedule of the mixed-precision loop (tail_cycles in
fortrancfd_gb300/csrc/schedule.h, shared by the device-side loop controller
and the host loop), compiled as plain C++ and checked on the CPU against the
rule it states: after a correction that took the relative residual from prev
to rel in s cycles, the next correction gets the smallest k < step_max with
rel * r**k < tol for r = (rel/prev)**(1/s), else step_max.  The inputs avoid
the exact boundary, where the product form and the root form may round
apart."""
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "fortrancfd_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include "schedule.h"
int main() {
  double rel, prev, tol;
  int s, m;
  while (std::scanf("%lf %lf %lf %d %d", &rel, &prev, &tol, &s, &m) == 5)
    std::printf("%d\n", gbmg::tail_cycles(rel, prev, tol, s, m));
  return 0;
}
"""


@pytest.fixture(scope="module")
def tail(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("schedule")
    src, exe = d / "drv.cpp", d / "drv"
    src.write_text(DRIVER)
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", CSRC, str(src), "-o", str(exe)], check=True)

    def run(rows):
        inp = "".join(f"{r!r} {p!r} {t!r} {s} {m}\n" for r, p, t, s, m in rows)
        out = subprocess.run([str(exe)], input=inp, capture_output=True, text=True, check=True)
        return [int(x) for x in out.stdout.split()]

    return run


def _rule(rel, prev, tol, s, m):
    r = (rel / prev) ** (1.0 / s)
    for k in range(1, m):
        if rel * r ** k < tol:
            return k
    return m


def _margin(rel, prev, tol, s, m):
    """Distance in log10 of the nearest k from the threshold."""
    r = (rel / prev) ** (1.0 / s)
    return min(abs(math.log10(rel * r ** k / tol)) for k in range(1, m + 1))


def test_tail_cycles_follows_its_rule(tail):
    rng = np.random.default_rng(3)
    rows = []
    while len(rows) < 2000:
        s, m = int(rng.integers(1, 6)), int(rng.integers(2, 9))
        tol = 10.0 ** rng.uniform(-13, -6)
        rel = tol * 10.0 ** rng.uniform(0.01, 6)  # above the tolerance
        factor = 10.0 ** rng.uniform(-2, -0.05)   # per cycle
        prev = rel / factor ** s
        if _margin(rel, prev, tol, s, m) > 1e-9:
            rows.append((rel, prev, tol, s, m))
    got = tail(rows)
    want = [_rule(*row) for row in rows]
    assert got == want
    assert min(got) == 1 and max(got) >= 4


def test_tail_cycles_without_a_reduction_keeps_the_full_length(tail):
    rows = [(1e-6, 1e-6, 1e-10, 4, 4),          # no reduction
            (2e-6, 1e-6, 1e-10, 4, 4),          # growth
            (1e-6, float("nan"), 1e-10, 4, 4),  # no usable history
            (1e-6, 0.0, 1e-10, 4, 4)]
    assert tail(rows) == [4, 4, 4, 4]


def test_tail_cycles_at_the_256_cube_benchmark(tail):
    """The 256^3 sphere converges by about 0.3 per cycle: after four cycles
    from 1 (rel 8.1e-3), and from 4.3e-8, three cycles do not reach 1e-10,
    so a full correction follows; from 1.2e-9 three cycles do."""
    assert tail([(8.1e-3, 1.0, 1e-10, 4, 4), (4.3e-8, 4.3e-8 / 0.3 ** 4, 1e-10, 4, 4),
                 (1.2e-9, 1.2e-9 / 0.3 ** 4, 1e-10, 4, 4)]) == [4, 4, 3]
