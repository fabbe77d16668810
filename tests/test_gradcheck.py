"""CPU checks of the cancellation-free central difference's operator apply
(fortrancfd_gb300.gradcheck.operator_apply) against the oracle's operator."""
import numpy as np
import pytest
import torch

from fortrancfd_gb300.gradcheck import operator_apply
from oracle import oracle as orc
from tests import cases


@pytest.mark.parametrize("idx,scale", [(0, 4), (1, 16), (4, 16)])
def test_operator_apply_matches_oracle(idx, scale):
    c = cases.config(idx, scale)
    p = np.random.default_rng(5).standard_normal(c.shape)
    want = orc.apply(c.coef, p)
    got = operator_apply([torch.from_numpy(a) for a in c.coef], torch.from_numpy(p)).numpy()
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * np.abs(want).max())
    assert abs(got.sum()) <= 1e-9 * np.abs(got).sum()  # the constants are its null space
