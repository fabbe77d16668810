"""The Fortran binding (include/gbmg.f90) driven the way the reference's
solvers would call it: ghost-padded arrays (3 ghost cells per side), the two
calls that replace ppe_sor_init and ppe_sor_solver, then the divergence check.
The Fortran program's pressure and corrected velocities must equal, bit for
bit, those of the same projection made through the Python binding on dense
arrays, its ghost cells must be untouched, and the projected field must be
divergence-free to the solver tolerance.  Needs gfortran (skipped without)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from fortrancfd_gb300 import PressurePoisson, _lib
from tests import cases

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def dropin(tmp_path_factory):
    fc = shutil.which("gfortran")
    if fc is None:
        pytest.skip("gfortran not installed")
    _lib.load()
    so = _lib.library_path()
    libdir = os.path.dirname(so)
    out = tmp_path_factory.mktemp("fortran")
    exe = out / "dropin_ppe"
    cmd = [fc, "-O2", "-std=f2008", "-J", str(out),
           os.path.join(ROOT, "include", "gbmg.f90"),
           os.path.join(ROOT, "tests", "fortran", "dropin_ppe.f90"),
           "-o", str(exe), so, f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def _write_case(path, c, precision, tol):
    nz, ny, nx = c.shape
    with open(path, "wb") as f:
        np.array([nx, ny, nz, precision], np.int32).tofile(f)
        np.array([*c.spacing, c.case.dt, tol], np.float64).tofile(f)
        for a in (c.rho, c.u, c.v, c.w):
            np.ascontiguousarray(a, np.float64).tofile(f)


def _read_result(path, c):
    nz, ny, nx = c.shape
    with open(path, "rb") as f:
        status, cycles, rc_div, ghosts_ok = np.fromfile(f, np.int32, 4)
        rel, mx, mean = np.fromfile(f, np.float64, 3)
        p = np.fromfile(f, np.float64, nz * ny * nx).reshape(nz, ny, nx)
        u = np.fromfile(f, np.float64, nz * ny * (nx + 1)).reshape(nz, ny, nx + 1)
        v = np.fromfile(f, np.float64, nz * (ny + 1) * nx).reshape(nz, ny + 1, nx)
        w = np.fromfile(f, np.float64, (nz + 1) * ny * nx).reshape(nz + 1, ny, nx)
    return dict(status=int(status), cycles=int(cycles), rc_div=int(rc_div),
                ghosts_ok=int(ghosts_ok), rel=float(rel), mx=float(mx), mean=float(mean),
                p=p, u=u, v=v, w=w)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fortran_dropin_projection(cuda, dropin, tmp_path, precision):
    c = cases.config(1, 8)
    tol = 1e-10
    _write_case(tmp_path / "case.bin", c, {"fp64": 0, "mixed": 1}[precision], tol)
    r = subprocess.run([str(dropin), str(tmp_path / "case.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    f = _read_result(tmp_path / "out.bin", c)
    assert f["status"] == 0 and f["rc_div"] == 0 and f["ghosts_ok"] == 1
    assert f["rel"] < tol

    u, v, w = c.u.copy(), c.v.copy(), c.w.copy()
    with PressurePoisson(c.shape, c.spacing, precision=precision) as s:
        s.ppe_init(c.rho)
        p, st = s.ppe_solver(u, v, w, c.case.dt, tol=tol)
        mx, mean = s.div_stats(u, v, w)
    assert f["cycles"] == st["cycles"]
    np.testing.assert_array_equal(f["p"], p)
    for a, b in ((f["u"], u), (f["v"], v), (f["w"], w)):
        np.testing.assert_array_equal(a, b)
    assert f["mx"] == mx and f["mean"] == mean
