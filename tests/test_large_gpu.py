"""Tensors of more than 2^31 elements on the device: the element-wise kernel's
64-bit index decomposition, a strided copy of that size, and whole-array
reductions whose winning index lies beyond 2^31 (a 32-bit signed index would
wrap). u8 / i8 data keep each tensor at about 2 GB; results are compared with
numpy exactly."""

import numpy as np
import pytest

import rstsr_gb300 as rt

pytestmark = pytest.mark.gpu

BIG = (1 << 31) + 4099


def test_binary_add_past_2_31(dev):
    rng = np.random.default_rng(1)
    a = rng.integers(0, 256, BIG, dtype=np.uint8)
    b = rng.integers(0, 256, BIG, dtype=np.uint8)
    got = (rt.asarray(a, dev) + rt.asarray(b, dev)).to_numpy()
    np.testing.assert_array_equal(got, a + b)  # wrapping u8 arithmetic


def test_strided_copy_past_2_31(dev):
    """A [2, 2^30 + 3] view transposed to a C-contiguous [2^30 + 3, 2] copy."""
    rng = np.random.default_rng(2)
    n = (1 << 30) + 3
    x = rng.integers(-128, 128, (2, n), dtype=np.int8)
    got = rt.asarray(x, dev).t().to_contig("C").to_numpy()
    assert got.shape == (n, 2)
    np.testing.assert_array_equal(got, x.T)


def test_whole_array_reductions_past_2_31(dev):
    rng = np.random.default_rng(3)
    x = rng.integers(0, 200, BIG, dtype=np.uint8)
    x[BIG - 77] = 255  # the only maximum, beyond index 2^31
    x[(1 << 31) + 5] = 0
    t = rt.asarray(x, dev)
    assert t.argmax_all() == BIG - 77
    assert t.max_all() == 255
    assert t.sum_all() == int(x.sum(dtype=np.uint8))  # u8 sums wrap, as in the reference
    del t
    y = rng.integers(-100, 100, BIG, dtype=np.int8)
    y[BIG - 3] = -128  # the only minimum, beyond 2^31
    ty = rt.asarray(y, dev)
    assert ty.argmin_all() == BIG - 3
    assert ty.min_all() == -128
