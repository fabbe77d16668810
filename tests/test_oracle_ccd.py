"""The compact-difference normals and curvature of the oracle (or_ccd_*,
or_ns_curvature) against the literal loop restatement (tests/refloops.py),
bit for bit, and against the properties of the scheme.  CPU only."""
import numpy as np
import pytest

from oracle import oracle as orc
from tests import refloops as ref


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def test_ccd_line_matches_the_loops():
    rng = np.random.default_rng(3)
    for L in (8, 17, 40):
        f = rng.standard_normal(L)
        h = 0.037
        fx, fxx = orc.ccd_line(f, h)
        gx, gxx = ref.ccd_solve(list(f), h)
        assert np.array_equal(_bits(fx), _bits(np.array(gx)))
        assert np.array_equal(_bits(fxx), _bits(np.array(gxx)))


def test_ccd_is_high_order_on_smooth_data():
    """Derivatives of sin(x) on a fine line: sixth-order interior accuracy."""
    errs = []
    for L in (64, 128):
        h = 2 * np.pi / (L - 1)
        x = np.arange(L) * h
        fx, fxx = orc.ccd_line(np.sin(x), h)
        inner = slice(L // 4, 3 * L // 4)
        errs.append(max(np.abs(fx - np.cos(x))[inner].max(), np.abs(fxx + np.sin(x))[inner].max()))
    assert errs[0] < 1e-7 and errs[1] < errs[0] / 16


def _phi(shape, g, seed=0):
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    ps = orc.padded_shape(shape, g)
    axes = [(np.arange(n) - g + 0.5) / max(nx, ny) for n in ps]
    grids = np.meshgrid(*axes, indexing="ij")
    c = 0.37
    r2 = sum((a - c) ** 2 for a in grids)
    return np.sqrt(r2) - 0.2 + 1e-3 * rng.standard_normal(ps)


@pytest.mark.parametrize("shape", [(1, 9, 11), (5, 6, 7)])
def test_curvature_matches_the_loops(shape):
    g = 3
    spacing = (0.05, 0.06, 0.07)
    phi = _phi(shape, g)
    nx, ny, nz, cv = orc.ns_curvature(shape, spacing, g, phi)
    three = shape[0] > 1
    rx, ry, rz, rc = ref.curv(phi.copy(), g, spacing[0], spacing[1], spacing[2] if three else None)
    assert np.array_equal(_bits(nx), _bits(rx))
    assert np.array_equal(_bits(ny), _bits(ry))
    if three:
        assert np.array_equal(_bits(nz), _bits(rz))
    assert np.array_equal(_bits(cv), _bits(rc))


def test_curvature_of_a_sphere_and_a_circle():
    """phi = distance d - r: the level sets are circles (spheres) of radius d,
    curvature 1/d (2D) and 2/d (3D), checked near the surface."""
    g = 3
    for shape, expect in (((1, 64, 64), 1.0), ((48, 48, 48), 2.0)):
        nz, ny, nx = shape
        h = 1.0 / nx
        ps = orc.padded_shape(shape, g)
        axes = [(np.arange(n) - g + 0.5) * h for n in ps]
        grids = np.meshgrid(*axes, indexing="ij")
        r0 = 0.3
        d = np.sqrt(sum((a - 0.5) ** 2 for a in grids))
        phi = d - r0
        _, _, _, cv = orc.ns_curvature(shape, (h, h, h), g, phi)
        band = np.abs(phi) < h
        rel = np.abs(cv[band] * d[band] - expect) / expect
        assert np.median(rel) < 1e-3 and rel.max() < 2e-2, (np.median(rel), rel.max())


def test_mass_correction_restores_the_initial_mass():
    """mass_preserving_level_set: an interface shifted by 0.3 cells (5% mass
    error) comes back to the initial mass within 2e-4 after two iterations."""
    g = 3
    shape = (1, 48, 48)
    h = 1 / 48
    ps = orc.padded_shape(shape, g)
    ys, xs = np.meshgrid(*[(np.arange(m) - g + 0.5) * h for m in ps], indexing="ij")
    phi = 0.25 - np.sqrt((xs - 0.5) ** 2 + (ys - 0.5) ** 2)
    sp = (h, h, 1.0)
    _, m0 = orc.ns_mass_correct(shape, sp, g, phi, 1.5 * h, 1e-3, 0.0, iterations=0)
    shifted = phi + 0.3 * h
    _, m1 = orc.ns_mass_correct(shape, sp, g, shifted, 1.5 * h, 1e-3, 0.0, iterations=0)
    fixed, _ = orc.ns_mass_correct(shape, sp, g, shifted, 1.5 * h, 1e-3, m0, iterations=2)
    _, m2 = orc.ns_mass_correct(shape, sp, g, fixed, 1.5 * h, 1e-3, 0.0, iterations=0)
    assert abs(m1 - m0) / m0 > 0.03
    assert abs(m2 - m0) / m0 < 2e-4


def _disc(shape, g, h, c=(0.45, 0.5, 0.5), r=0.2):
    ps = orc.padded_shape(shape, g)
    grids = np.meshgrid(*[(np.arange(m) - g + 0.5) * h for m in ps], indexing="ij")
    cen = c[:len(ps)][::-1]
    phi = r - np.sqrt(sum((a - cc) ** 2 for a, cc in zip(grids, cen)))
    vof = orc.heaviside(phi, 1.5 * h)
    return phi, vof


def test_vof_transport_conserves_and_moves_the_disc():
    """vof_wlic_solver in a uniform x velocity (walls at rest, disc away from
    them): the volume is conserved to round-off, vof stays in [0, 1] and the
    centroid moves by u dt per step."""
    g = 3
    shape = (1, 48, 48)
    h = 1 / 48
    phi, vof = _disc(shape, g, h)
    u = np.zeros_like(vof)
    u[:, g:g + 47] = 0.5          # faces 1..47 of the reference (walls 0 and 48 at rest)
    v = np.zeros_like(vof)
    dt = 0.2 * h / 0.5
    x = (np.arange(vof.shape[1]) - g + 0.5) * h
    inner = (slice(g, g + 48), slice(g, g + 48))
    vol0 = vof[inner].sum()
    cx0 = (vof[inner] * x[None, g:g + 48]).sum() / vol0
    cur = vof
    for _ in range(10):
        cur = orc.vof_wlic((1, 48, 48), (h, h, 1.0), g, cur, cur, u, v, None, phi, dt)
    vol = cur[inner].sum()
    cx = (cur[inner] * x[None, g:g + 48]).sum() / vol
    assert abs(vol - vol0) / vol0 < 1e-12
    assert cur.min() >= 0.0 and cur.max() <= 1.0
    assert cx - cx0 == pytest.approx(10 * 0.5 * dt, rel=0.02)
