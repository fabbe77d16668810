"""The momentum step's oracle (oracle/oracle.c or_ns_*) against the literal
loop restatement of the reference (tests/refloops.py), bit for bit, and the
oracle's whole step against its defining properties.  CPU only."""
import numpy as np
import pytest

from fortrancfd_gb300 import inputs
from oracle import oracle as orc
from tests import refloops as ref

CASES = [((1, 10, 12), (0.1, 0.08, 1.0)), ((4, 5, 6), (0.2, 0.25, 0.3))]


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def _state(shape, spacing, seed, ghost=3):
    case = inputs.custom(shape, extent=tuple(n * h for n, h in zip(shape[::-1], spacing)),
                         centers=((0.5 * shape[2] * spacing[0], 0.45 * shape[1] * spacing[1],
                                   0.5 * shape[0] * spacing[2]),),
                         radii=(0.3 * min(shape[1] * spacing[1], shape[2] * spacing[0]),),
                         seed=seed)
    st = inputs.momentum_state(case, ghost=ghost, amplitude=0.3)
    rng = np.random.default_rng(seed)
    for k in ("u", "v", "w"):  # ghosts as arbitrary as the interior
        if st[k] is not None:
            st[k] = st[k] + 0.01 * rng.standard_normal(st[k].shape)
    return st


def _prm(**kw):
    base = dict(ghost=3, dt=2e-3, re=100.0, fr=0.5, we=2.0, mu_12=1e-2,
                gravity=(0.3, -0.8, -0.5), btn_g=1.0, btn_sf=1.0)
    base.update(kw)
    return orc.ns_params(**base)


@pytest.mark.parametrize("shape,spacing", CASES)
@pytest.mark.parametrize("sf", [0.0, 1.0])
def test_diffusion_matches_the_loops(shape, spacing, sf):
    st = _state(shape, spacing, 5)
    prm = _prm(btn_sf=sf)
    three = shape[0] > 1
    got = orc.ns_diffusion(shape, spacing, prm, st)
    nz, ny, nx = shape
    curv = st["curv"] if sf else np.zeros_like(st["curv"])
    if three:
        want = ref.ns_ab_diff_sec_3d(st["u"], st["v"], st["w"], st["rho"], st["mu"], st["delta"],
                                     st["phi"], st["nrm_x"], st["nrm_y"], st["nrm_z"], curv, 3, nx,
                                     ny, nz, *spacing, prm.re, prm.mu_12, prm.gx, prm.gy, prm.gz,
                                     prm.btn_g, sf, prm.fr, prm.we)
    else:
        want = ref.ns_ab_diff_sec_2d(st["u"], st["v"], st["rho"], st["mu"], st["delta"],
                                     st["phi"], st["nrm_x"], st["nrm_y"], curv, 3, nx, ny,
                                     spacing[0], spacing[1], prm.re, prm.mu_12, prm.gx, prm.gy,
                                     prm.btn_g, sf, prm.fr, prm.we)
    for c in range(3 if three else 2):
        assert np.array_equal(got[c], want[c]), c
        assert np.abs(got[c]).max() > 0


@pytest.mark.parametrize("shape,spacing", CASES)
def test_advance_matches_the_loops(shape, spacing):
    st = _state(shape, spacing, 6)
    prm = _prm()
    three = shape[0] > 1
    nc = 3 if three else 2
    rng = np.random.default_rng(1)
    old = tuple(st[k] for k in ("u", "v", "w")[:nc])
    tmp = tuple(a + 0.05 * rng.standard_normal(a.shape) for a in old)
    diff = orc.ns_diffusion(shape, spacing, prm, st)[:nc]
    so = tuple(st[k] for k in ("su_old", "sv_old", "sw_old")[:nc])
    src, vel = orc.ns_advance(shape, spacing, prm, old, tmp, diff, so)
    n = shape[::-1][:nc]
    src2, vel2 = ref.ns_ab_adv_predictor(old, tmp, diff, so, 3, n, spacing[:nc], prm.dt)
    for c in range(nc):
        assert np.array_equal(_bits(src[c]), _bits(src2[c])), c
        assert np.array_equal(_bits(vel[c]), _bits(vel2[c])), c


@pytest.mark.parametrize("shape,spacing", CASES)
@pytest.mark.parametrize("bc", [(1, 1, 1, 1, 1, 1), (2, 1, 1, 2, 2, 1), (0, 2, 1, 0, 1, 3)])
def test_velbc_matches_the_loops(shape, spacing, bc):
    rng = np.random.default_rng(2)
    three = shape[0] > 1
    ps = orc.padded_shape(shape, 3)
    f = [rng.standard_normal(ps) for _ in range(3 if three else 2)]
    g = [a.copy() for a in f]
    h = [a.copy() for a in f]
    prm = _prm(bc=bc)
    orc.velbc(shape, prm, *f)
    nz, ny, nx = shape
    ref.velbc(g[0], g[1], g[2] if three else None, 3, nx, ny, nz, bc[0:2], bc[2:4], bc[4:6])
    inputs.velbc_numpy(h[0], h[1], h[2] if three else None, 3, bc)
    for c in range(len(f)):
        assert np.array_equal(_bits(f[c]), _bits(g[c])), c
        assert np.array_equal(_bits(f[c]), _bits(h[c])), c


@pytest.mark.parametrize("shape,spacing", [((1, 16, 16), (1 / 16, 1 / 16, 1.0)),
                                           ((8, 8, 8), (1 / 8, 1 / 8, 1 / 8))])
def test_step_is_divergence_free_and_consistent(shape, spacing):
    st = _state(shape, spacing, 7)
    prm = _prm(p_tol=1e-12)
    three = shape[0] > 1
    nc = 3 if three else 2
    vel = tuple(st[k] for k in ("u", "v", "w")[:nc])
    so = tuple(st[k] for k in ("su_old", "sv_old", "sw_old")[:nc])
    out = orc.ns_ab_step(shape, spacing, prm, st["rho_now"], vel, st, so, st["p"], krylov=1)
    assert out["status"] == 0
    g = 3
    nz, ny, nx = shape
    sl = (slice(g, g + nz),) if three else ()
    # interior divergence of the result (faces 0..n of each axis)
    u = out["u"][sl + (slice(g, g + ny), slice(g - 1, g + nx))]
    v = out["v"][sl + (slice(g - 1, g + ny), slice(g, g + nx))]
    div = np.diff(u, axis=-1) / spacing[0] + np.diff(v, axis=-2) / spacing[1]
    if three:
        w = out["w"][(slice(g - 1, g + nz), slice(g, g + ny), slice(g, g + nx))]
        div = div + np.diff(w, axis=0) / spacing[2]
    base = max(np.abs(np.diff(st["u"], axis=-1)).max() / spacing[0], 1.0)
    assert np.abs(div).max() < 1e-8 * base
    # ghosts obey velbc
    again = [out[k].copy() for k in ("u", "v", "w")[:nc]]
    orc.velbc(shape, prm, *again)
    for c, k in enumerate(("u", "v", "w")[:nc]):
        assert np.array_equal(_bits(again[c]), _bits(out[k]))
    # the source is that of the last pass, whose advecting velocity was the
    # third pass's result: re-running three passes reproduces it (to the
    # rounding of the OpenMP reductions inside the solves, which vary by run)
    prm3 = _prm(p_tol=1e-12, iterations=3)
    out3 = orc.ns_ab_step(shape, spacing, prm3, st["rho_now"], vel, st, so, st["p"], krylov=1)
    diff = orc.ns_diffusion(shape, spacing, prm, st)[:nc]
    src, _ = orc.ns_advance(shape, spacing, prm, vel, tuple(out3[k] for k in ("u", "v", "w")[:nc]),
                            diff, so)
    for c, k in enumerate(("su", "sv", "sw")[:nc]):
        np.testing.assert_allclose(src[c], out[k], rtol=0, atol=1e-12 * np.abs(out[k]).max())
    # velocity change statistics of ns_check_convergence_vel
    d = [out[k] - out3[k] for k in ("u", "v", "w")[:nc]]
    inner = tuple(sl) + (slice(g, g + ny), slice(g, g + nx))
    linf = max(np.abs(a[inner]).max() for a in d)
    l2 = np.sqrt(sum((a[inner] ** 2).sum() for a in d) / (nc * nx * ny * nz))
    assert out["linf"] == pytest.approx(linf, rel=1e-6)
    assert out["l2f"] == pytest.approx(l2, rel=1e-6)
    assert out["linf"] > 0


def test_quick_advection_matches_the_loops():
    shape, spacing = CASES[0]
    st = _state(shape, spacing, 8)
    prm = _prm(adv_scheme=1)
    rng = np.random.default_rng(2)
    old = (st["u"], st["v"])
    tmp = tuple(a + 0.05 * rng.standard_normal(a.shape) for a in old)
    zero = (np.zeros_like(st["u"]), np.zeros_like(st["v"]))
    src, _ = orc.ns_advance(shape, spacing, prm, old, tmp, zero, zero)
    want = ref.ns_ab_adv_source_quick_2d(old[0], old[1], tmp[0], tmp[1], 3, shape[2], shape[1],
                                         spacing[0], spacing[1])
    for c in range(2):
        assert np.array_equal(src[c], want[c]), c
        assert np.abs(src[c]).max() > 0
