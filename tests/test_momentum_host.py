"""Host-side logic of the momentum-step binding (no GPU, no kernel launch):
the addresses and strides momentum.py hands to the C ABI for ghost-padded
arrays, its shape and memory checks, and the time-step driver's pseudo-time
iteration count."""
import numpy as np
import pytest

from fortrancfd_gb300 import momentum


@pytest.mark.parametrize("shape", [(1, 6, 8), (4, 5, 6)])
@pytest.mark.parametrize("g", [2, 3])
def test_padded_field_addresses(shape, g):
    ps = momentum.padded_shape(shape, g)
    a = np.zeros(ps)
    base = a.ctypes.data
    st = [s // 8 for s in a.strides]
    three = len(ps) == 3
    # cell arrays at the reference's (1,1,1); faces at face 0 of their axis
    want = {"phi": (g, g, g), "u": (g, g, g - 1), "v": (g, g - 1, g), "w": (g - 1, g, g)}
    for name, (k, j, i) in want.items():
        if name == "w" and not three:
            continue
        f, mem = momentum._padded_field(a, name, shape, g)
        off = (k * st[0] if three else 0) + j * st[-2] + i * st[-1]
        if not three:
            off = j * st[0] + i
        assert f.data == base + 8 * off, name
        assert f.sy == ps[-1]
        assert f.sz == (st[0] if three else ps[-1] * ps[0])
        assert mem == 0


def test_padded_field_rejects_wrong_input():
    with pytest.raises(ValueError, match="padded shape"):
        momentum._padded_field(np.zeros((5, 5)), "phi", (1, 4, 4), 3)
    with pytest.raises(TypeError):
        momentum._padded_field(np.zeros((10, 10), np.float32), "phi", (1, 4, 4), 3)
    with pytest.raises(ValueError, match="contiguous"):
        momentum._padded_field(np.zeros((10, 20))[:, ::2], "phi", (1, 4, 4), 3)
    assert momentum._padded_field(None, "phi", (1, 4, 4), 3)[1] is None


def test_one_memory_and_params():
    with pytest.raises(ValueError, match="same memory"):
        momentum._one_memory((None, 0), (None, 1))
    c = momentum.NSParams(dt=0.5, bc=(1, 2, 1, 2, 0, 3), iterations=2).c_struct()
    assert list(c.bc) == [1, 2, 1, 2, 0, 3] and c.iterations == 2 and c.dt == 0.5


def test_recon_iteration_count_matches_the_reference_loop():
    """clsvof_recon redistances until the accumulated pseudo time exceeds
    3 dx: with rdt = 0.25 dx that is 13 steps (the accumulation of 0.25
    is exact, so 12 steps reach 3 dx without exceeding it)."""
    dx = 1.0 / 64
    rdt = 0.25 * dx
    n, t = 0, 0.0
    while True:
        n += 1
        t += rdt
        if t > 3.0 * dx:
            break
    assert n == 13
