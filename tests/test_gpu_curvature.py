"""Interface normals and curvature on the GPU (gbmg_ns_curvature, momentum.curv)
against the oracle's compact-difference restatement: the derivatives are FP64
in the reference's operand order on both sides and compared bit for bit; the
curvature divides by s^1.5, s = |grad phi|^2 + 1e-12, which the GPU forms as
s*sqrt(s) (correctly rounded sqrt, so within about two roundings of exact)
and the oracle with glibc's pow (within about one), so it is compared to
1e-14 relative."""
import numpy as np
import pytest

from fortrancfd_gb300 import NSParams, PressurePoisson, curv
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

G = 3


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def _phi(shape, seed=2):
    rng = np.random.default_rng(seed)
    ps = orc.padded_shape(shape, G)
    n = max(shape)
    axes = [(np.arange(m) - G + 0.5) / n for m in ps]
    grids = np.meshgrid(*axes, indexing="ij")
    d = np.sqrt(sum((a - 0.45) ** 2 for a in grids))
    return d - 0.25 + 1e-3 * rng.standard_normal(ps)


def _check(got, want, three):
    for c in range(3 if three else 2):
        assert np.array_equal(_bits(got[c]), _bits(want[c])), c
    np.testing.assert_allclose(got[3], want[3], rtol=1e-14, atol=1e-14 * np.abs(want[3]).max())


@pytest.mark.parametrize("shape", [(1, 24, 32), (1, 64, 40), (8, 12, 16), (16, 16, 16)])
def test_curvature_matches_oracle(cuda, shape):
    import torch
    spacing = (1.0 / shape[2], 1.0 / shape[1], 1.0 / max(shape[0], 1))
    phi = _phi(shape)
    want = orc.ns_curvature(shape, spacing, G, phi)
    three = shape[0] > 1
    prm = NSParams(dt=1.0, ghost=G)
    with PressurePoisson(shape, spacing) as pp:
        # host arrays through the C ABI
        out = [np.zeros_like(phi) for _ in range(4)]
        curv(pp, prm, phi, out[0], out[1], out[2] if three else None, out[3])
        _check(out, want, three)
        # device tensors in place
        t = [torch.zeros(phi.shape, dtype=torch.float64, device=cuda) for _ in range(4)]
        n0 = pp.kernel_launches
        curv(pp, prm, torch.from_numpy(phi).to(cuda), t[0], t[1], t[2] if three else None, t[3])
        assert pp.kernel_launches > n0
        _check([a.cpu().numpy() for a in t], want, three)


def test_curvature_of_a_sphere(cuda):
    import torch
    shape = (64, 64, 64)
    h = 1.0 / 64
    ps = orc.padded_shape(shape, G)
    axes = [(np.arange(m) - G + 0.5) * h for m in ps]
    grids = np.meshgrid(*axes, indexing="ij")
    d = np.sqrt(sum((a - 0.5) ** 2 for a in grids))
    phi = torch.from_numpy(d - 0.3).to(cuda)
    out = [torch.zeros_like(phi) for _ in range(4)]
    with PressurePoisson(shape, (h, h, h)) as pp:
        curv(pp, NSParams(dt=1.0, ghost=G), phi, *out)
    cv = out[3].cpu().numpy()
    band = np.abs(d - 0.3) < h
    rel = np.abs(cv[band] * d[band] - 2.0) / 2.0
    assert np.median(rel) < 1e-3 and rel.max() < 2e-2
