"""Host-side helpers of the Python mirror (no GPU): the bf16 rounding of host
scalars passed to fill / scalar operators, the element bounds of a strided
layout and the contiguous stride helpers."""

import itertools
import struct

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _bf16_bits_torch(x: float) -> int:
    t = torch.tensor([x], dtype=torch.float32).to(torch.bfloat16)
    return int(t.view(torch.int16).item()) & 0xFFFF


def test_bf16_scalar_rounding_matches_torch():
    from rstsr_gb300 import _lib
    from rstsr_gb300.tensor import _scalar_bytes

    rng = np.random.default_rng(0)
    values = [0.0, -0.0, 1.0, -1.0, 1.00390625, 1.01171875, 3.0e38, 3.4028235e38, -3.4028235e38, 1e-40, -1e-45,
              float("inf"), float("-inf"), 65504.0, 1 / 3]
    # exact ties of the bf16 grid (the lower 16 bits 0x8000) with even and odd upper halves
    for hi in (0x3F80, 0x3F81, 0x4049, 0xC2F7):
        values.append(struct.unpack("<f", struct.pack("<I", (hi << 16) | 0x8000))[0])
    values += list(rng.standard_normal(2000) * 10.0 ** rng.integers(-30, 30, 2000))
    for v in values:
        buf = _scalar_bytes(v, _lib.BF16)
        got = buf[0] | (buf[1] << 8)
        assert got == _bf16_bits_torch(v), (v, hex(got), hex(_bf16_bits_torch(v)))
    nan = _scalar_bytes(float("nan"), _lib.BF16)
    bits = nan[0] | (nan[1] << 8)
    assert (bits & 0x7F80) == 0x7F80 and (bits & 0x007F) != 0  # still a NaN


def test_bounds_cover_exactly_the_addressed_elements():
    from rstsr_gb300.tensor import _bounds

    rng = np.random.default_rng(1)
    for _ in range(500):
        nd = int(rng.integers(0, 4))
        shape = tuple(int(v) for v in rng.integers(0, 4, nd))
        stride = tuple(int(v) for v in rng.integers(-7, 8, nd))
        off = 100
        lo, hi = _bounds(shape, stride, off)
        idx = [off + sum(i * s for i, s in zip(ix, stride)) for ix in itertools.product(*[range(d) for d in shape])]
        if not idx:
            assert lo == hi
        else:
            assert (lo, hi) == (min(idx), max(idx) + 1), (shape, stride)


@pytest.mark.parametrize("shape", [(), (5,), (3, 4), (2, 0, 3), (1, 7, 1, 2)])
def test_contiguous_strides_match_numpy(shape):
    from rstsr_gb300.tensor import _c_strides, _f_strides

    c = np.zeros(shape, dtype=np.int8, order="C")
    f = np.zeros(shape, dtype=np.int8, order="F")
    if 0 not in shape:
        assert _c_strides(shape) == c.strides
        assert _f_strides(shape) == f.strides
    else:  # zero-size axes: the reference's strides treat the extent as 1
        assert len(_c_strides(shape)) == len(shape) and len(_f_strides(shape)) == len(shape)
