"""gbmg_div_stats_noalloc, the divergence statistics with static scratch.

GPU: two calls in a row agree with gbmg_div_stats (the handle's entry point)
on the same device arrays to 1e-14 relative; both run the same reduction
kernel with the same block count, so the tolerance only guards against a
changed summation order.  The second call also shows that the first left the
static completion counter at zero.  CPU: sizes beyond the limit and invalid
grids are rejected before any CUDA call.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from fortrancfd_gb300 import GBMGError, PressurePoisson, _lib, inputs
from fortrancfd_gb300.ppe import div_stats_noalloc


def _velocity(case, device, pad=0):
    """Face velocities as CUDA tensors; pad > 0 places them in ghost-padded
    storage (views with y and z strides larger than the extents)."""
    out = []
    for a in inputs.velocity(case):
        t = torch.from_numpy(np.ascontiguousarray(a)).to(device)
        if pad:
            big = torch.full((t.shape[0] + 2 * pad, t.shape[1] + 2 * pad, t.shape[2] + 2 * pad),
                             7.0, dtype=t.dtype, device=device)
            big[pad:-pad, pad:-pad, pad:-pad] = t
            t = big[pad:-pad, pad:-pad, pad:-pad]
        out.append(t)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("idx,scale,pad", [(0, 2, 0), (1, 8, 0), (4, 8, 2), (1, 1, 0)])
def test_two_calls_match_the_handle_entry_point(cuda, idx, scale, pad):
    case = inputs.config(idx, scale)
    u, v, w = _velocity(case, cuda, pad)
    if case.shape[0] == 1:
        u, v, w = u[0], v[0], None
    with PressurePoisson(case.shape, case.spacing) as s:
        want = s.div_stats(u, v, w)
    assert want[0] > 0 and want[1] > 0
    for _ in range(2):
        got = div_stats_noalloc(u, v, w, case.spacing)
        np.testing.assert_allclose(got, want, rtol=1e-14, atol=0)


def _call(grid, err):
    L = _lib.load()
    f = _lib.Field(None, 0, 0)
    mx, mean = C.c_double(), C.c_double()
    return L.gbmg_div_stats_noalloc(C.byref(grid) if grid is not None else None, f, f, f,
                                    C.byref(mx), C.byref(mean), -1, None, err, len(err))


def test_rejects_sizes_beyond_the_limit_and_invalid_arguments():
    L = _lib.load()
    err = C.create_string_buffer(256)
    assert _call(None, err) == _lib.GBMG_INVALID_ARG
    assert b"invalid grid" in err.value
    assert _call(_lib.Grid(0, 4, 4, 1.0, 1.0, 1.0), err) == _lib.GBMG_INVALID_ARG
    # fields are checked before sizes: give u and v a dummy address
    buf = (C.c_double * 4)()
    f = _lib.Field(C.addressof(buf), 1, 1)
    mx, mean = C.c_double(), C.c_double()
    big = _lib.Grid(8, 65536, 65536, 1.0, 1.0, 1.0)  # 2^32 rows of cells
    rc = L.gbmg_div_stats_noalloc(C.byref(big), f, f, f, C.byref(mx), C.byref(mean), -1, None,
                                  err, len(err))
    assert rc == _lib.GBMG_INVALID_ARG
    assert b"exceed the limit" in err.value
    assert _call(_lib.Grid(4, 4, 4, 1.0, 1.0, 1.0), err) == _lib.GBMG_INVALID_ARG
    assert b"invalid field" in err.value


def test_python_wrapper_needs_cuda_tensors():
    with pytest.raises(TypeError):
        div_stats_noalloc(np.zeros((2, 2, 3)), np.zeros((2, 3, 2)), np.zeros((3, 2, 2)),
                          (1.0, 1.0, 1.0))
    assert issubclass(GBMGError, RuntimeError)
