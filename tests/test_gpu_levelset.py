"""Level-set advection on the GPU (gbmg_ls_advect, levelset.py) against the
CPU oracle's restatement of level_set_rk3_solver: FP64 with every product
rounded on its own on both sides, so the results are compared bit for bit."""
import numpy as np
import pytest

from fortrancfd_gb300 import GBMGError, LevelSet, node_velocity
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _case(shape, seed=5):
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    z, y, x = np.meshgrid(*[(np.arange(n) + 0.5) / n for n in shape], indexing="ij")
    phi = np.sqrt((x - 0.45) ** 2 + (y - 0.5) ** 2 + ((z - 0.55) ** 2 if nz > 1 else 0)) - 0.25
    phi = phi + 0.01 * rng.standard_normal(shape)
    u, v, w = (rng.standard_normal(shape) for _ in range(3))
    return phi, u, v, w


@pytest.mark.parametrize("shape,steps", [((1, 33, 47), 3), ((9, 10, 11), 2), ((20, 24, 28), 2),
                                         ((1, 1, 16), 2), ((5, 1, 1), 1)])
def test_advect_matches_oracle_bitwise(cuda, shape, steps):
    phi, u, v, w = _case(shape)
    spacing = (1.0 / shape[2], 1.0 / shape[1], 1.0 / shape[0])
    dt = 0.2 * min(spacing)
    want = orc.ls_advect(phi, u, v, w, dt, spacing, steps=steps)
    got = phi.copy()
    with LevelSet(shape, spacing) as ls:
        n0 = ls.kernel_launches
        ls.advect(got, u, v, w, dt=dt, steps=steps)
        assert ls.kernel_launches > n0
    np.testing.assert_array_equal(got, want)


def test_device_tensors_and_padded_host_arrays(cuda):
    import torch
    shape = (12, 14, 16)
    phi, u, v, w = _case(shape, seed=8)
    spacing = (0.1, 0.2, 0.3)
    want = orc.ls_advect(phi, u, v, w, 1e-3, spacing, steps=2)
    with LevelSet(shape, spacing) as ls:
        t = [torch.from_numpy(a).to(cuda) for a in (phi, u, v, w)]
        ls.advect(t[0], t[1], t[2], t[3], dt=1e-3, steps=2)
        np.testing.assert_array_equal(t[0].cpu().numpy(), want)
        # host arrays with 3 ghost cells per side, as the reference allocates them
        g = 3
        big = np.full((shape[0] + 2 * g, shape[1] + 2 * g, shape[2] + 2 * g), np.nan)
        view = big[g:-g, g:-g, g:-g]
        view[...] = phi
        ls.advect(view, u, v, w, dt=1e-3, steps=2)
        np.testing.assert_array_equal(view, want)
        assert np.isnan(big[0]).all() and np.isnan(big[:, :, 0]).all()


def test_node_velocity_and_translation(cuda):
    """MAC faces of a uniform flow averaged to the cells (node_vel) carry a
    smooth bump along the box: the GPU result is the oracle's, and both stay
    close to the exact translation."""
    n = 64
    h = 1.0 / n
    x = (np.arange(n) + 0.5) * h
    X, Y = np.meshgrid(x, x, indexing="xy")
    phi0 = np.exp(-((X - 0.35) ** 2 + (Y - 0.5) ** 2) / 0.01)[None]
    uf = np.full((1, n, n + 1), 1.0)
    vf = np.zeros((1, n + 1, n))
    un, vn, _ = node_velocity(uf, vf)
    dt = 0.25 * h
    steps = int(round(0.3 / dt))
    with LevelSet((1, n, n), (h, h)) as ls:
        phi = ls.advect(phi0.copy(), un, vn, None, dt=dt, steps=steps)
    np.testing.assert_array_equal(phi, orc.ls_advect(phi0, un, vn, None, dt, (h, h, 1.0), steps))
    exact = np.exp(-((X - 0.35 - steps * dt) ** 2 + (Y - 0.5) ** 2) / 0.01)[None]
    assert np.abs(phi - exact).max() < 2e-3


def test_errors_and_no_op(cuda):
    shape = (4, 5, 6)
    phi, u, v, w = _case(shape)
    with LevelSet(shape, (0.1, 0.1, 0.1)) as ls:
        with pytest.raises(GBMGError):
            ls.advect(phi.copy(), u, v, w, dt=-1.0)
        same = ls.advect(phi.copy(), u, v, w, dt=1e-3, steps=0)
        np.testing.assert_array_equal(same, phi)
        with pytest.raises(ValueError):
            ls.advect(phi.copy(), u[:, :, :-1], v, w, dt=1e-3)


def _stretched(shape, h, seed=4):
    rng = np.random.default_rng(seed)
    nz = shape[0]
    z, y, x = np.meshgrid(*[(np.arange(n) + 0.5) * h for n in shape], indexing="ij")
    r = np.sqrt((x - 0.5) ** 2 + (y - 0.45) ** 2 + ((z - 0.25) ** 2 if nz > 1 else 0))
    return (r - 0.3) * 1.7 + 0.01 * rng.standard_normal(shape)


@pytest.mark.parametrize("shape", [(1, 40, 48), (16, 18, 20)])
def test_redistance_initial_matches_oracle_bitwise(cuda, shape):
    """btn = 0 (S = phi, no Heaviside): no transcendental function on the
    path, so GPU and oracle agree bit for bit, iteration count included."""
    h = 1.0 / shape[2]
    phi = _stretched(shape, h)
    want, it_w, ch_w = orc.ls_redistance(phi, 1.5 * h, 0.1 * h, (h, h, h), btn=0, max_iter=12)
    got = phi.copy()
    with LevelSet(shape, (h, h, h)) as ls:
        _, it, ch = ls.redistance(got, 1.5 * h, 0.1 * h, btn=0, max_iter=12)
    assert it == it_w and ch == ch_w
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("shape", [(1, 64, 64), (24, 24, 24)])
def test_redistance_with_mass_correction_matches_oracle(cuda, shape):
    """btn = 1: the sign and the mass correction use sin and cos (CUDA's on
    the GPU, the C library's in the oracle), so the comparison is to 1e-12 of
    max |phi|; the iteration count is the same."""
    h = 1.0 / shape[2]
    phi = _stretched(shape, h)
    want, it_w, _ = orc.ls_redistance(phi, 1.5 * h, 0.1 * h, (h, h, h), btn=1)
    got = phi.copy()
    with LevelSet(shape, (h, h, h)) as ls:
        _, it, _ = ls.redistance(got, 1.5 * h, 0.1 * h, btn=1)
    assert it == it_w
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * np.abs(phi).max())


def test_redistance_device_tensor(cuda):
    import torch
    shape = (1, 32, 40)
    h = 1.0 / 40
    phi = _stretched(shape, h)
    want, _, _ = orc.ls_redistance(phi, 1.5 * h, 0.1 * h, (h, h, h), btn=0, max_iter=5)
    t = torch.from_numpy(phi).to(cuda)
    with LevelSet(shape, (h, h, h)) as ls:
        ls.redistance(t, 1.5 * h, 0.1 * h, btn=0, max_iter=5)
        with pytest.raises(GBMGError):
            ls.redistance(t, -1.0, 0.1 * h)
    np.testing.assert_array_equal(t.cpu().numpy(), want)
