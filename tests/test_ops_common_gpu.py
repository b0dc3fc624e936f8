"""The element-wise math family, predicates, comparisons and isclose on the
GPU against oracle/elementwise.py and numpy (exact where the operation is
exact; transcendental functions within a few ulp of CUDA's math library)."""

import numpy as np
import pytest

import rstsr_gb300 as rt
from oracle import elementwise as E
from rstsr_gb300._lib import RstsrError

pytestmark = pytest.mark.gpu

SPECIAL = [0.0, -0.0, 0.5, -0.5, 1.5, -1.5, 2.5, -2.5, 1.0, -1.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324,
           0.49999999999999994, 1e300, -1e300, 3.75, -7.25]


def values(dtype, n=400, seed=0, lo=-3.0, hi=3.0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(lo, hi, n)
    x = np.concatenate([x, np.array(SPECIAL)])
    with np.errstate(all="ignore"):
        return x.astype(dtype)


MATH = {
    "acos": (np.arccos, -1, 1), "acosh": (np.arccosh, 1, 50), "asin": (np.arcsin, -1, 1),
    "asinh": (np.arcsinh, -50, 50), "atan": (np.arctan, -50, 50), "atanh": (np.arctanh, -1, 1),
    "cosh": (np.cosh, -20, 20), "expm1": (np.expm1, -20, 20), "log1p": (np.log1p, -0.99, 50),
    "log2": (np.log2, 1e-3, 1e3), "log10": (np.log10, 1e-3, 1e3), "sinh": (np.sinh, -20, 20),
    "tan": (np.tan, -1.5, 1.5),
}


@pytest.mark.parametrize("op", sorted(MATH))
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_transcendental_within_ulps(dev, op, dtype):
    f, lo, hi = MATH[op]
    x = values(dtype, lo=lo, hi=hi)[:400]
    got = getattr(rt, op)(rt.asarray(x, dev)).to_numpy()
    with np.errstate(all="ignore"):
        want = f(x.astype(np.float64))
    finite = np.isfinite(want)
    rtol = 4e-15 if dtype == np.float64 else 2e-6
    np.testing.assert_allclose(got[finite].astype(np.float64), want[finite], rtol=rtol, atol=1e-300)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(want.astype(dtype)))


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.float16])
def test_exact_unary_ops(dev, dtype):
    x = values(dtype, lo=-10, hi=10)
    t = rt.asarray(x, dev)
    np.testing.assert_array_equal(rt.round(t).to_numpy(), E.rust_round(x))
    np.testing.assert_array_equal(rt.trunc(t).to_numpy(), np.trunc(x))
    np.testing.assert_array_equal(rt.unary("sign", t).to_numpy(), E.ext_sign(x))
    np.testing.assert_array_equal(rt.conj(t).to_numpy(), x)
    np.testing.assert_array_equal(rt.real(t).to_numpy(), x)
    np.testing.assert_array_equal(rt.imag(t).to_numpy(), np.zeros_like(x))
    with np.errstate(all="ignore"):
        np.testing.assert_array_equal(rt.inv(t).to_numpy(), (np.float64(1) / x.astype(np.float64)).astype(dtype)
                                      if dtype != np.float64 else 1.0 / x)
    # sign of zeros is 0 (the reference's ext_sign), NaN stays NaN
    z = rt.unary("sign", rt.asarray(np.array([0.0, -0.0, np.nan, -3.0], dtype=dtype), dev)).to_numpy()
    assert z[0] == 0 and z[1] == 0 and np.isnan(z[2]) and z[3] == -1


@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.uint16, np.int8])
def test_integer_unary_ops(dev, dtype):
    info = np.iinfo(dtype)
    x = np.array([0, 1, 5, info.max, info.min, info.min + 1] + ([-1, -7] if info.min < 0 else [3, 9]), dtype=dtype)
    t = rt.asarray(x, dev)
    np.testing.assert_array_equal(rt.unary("sign", t).to_numpy(), E.ext_sign(x))
    np.testing.assert_array_equal(rt.conj(t).to_numpy(), x)
    np.testing.assert_array_equal(rt.imag(t).to_numpy(), np.zeros_like(x))
    with pytest.raises(RstsrError):
        rt.log1p(t)


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.float16])
def test_predicates(dev, dtype):
    x = values(dtype)
    t = rt.asarray(x, dev)
    np.testing.assert_array_equal(rt.isfinite(t).to_numpy(), np.isfinite(x))
    np.testing.assert_array_equal(rt.isinf(t).to_numpy(), np.isinf(x))
    np.testing.assert_array_equal(rt.isnan(t).to_numpy(), np.isnan(x))
    np.testing.assert_array_equal(rt.signbit(t).to_numpy(), E.signbit_is_positive(x))


def test_predicates_integers_and_bf16(dev):
    xi = np.array([-3, 0, 4, np.iinfo(np.int32).min], dtype=np.int32)
    np.testing.assert_array_equal(rt.signbit(rt.asarray(xi, dev)).to_numpy(), xi > 0)
    with pytest.raises(RstsrError):
        rt.isnan(rt.asarray(xi, dev))
    f = np.array([1.0, -0.0, np.inf, np.nan, -2.0], dtype=np.float32)
    bits = (f.view(np.uint32) >> 16).astype(np.uint16)
    t = rt.asarray(bits, dev)
    t = rt.Tensor(t.storage, t.shape, t.stride, t.offset, rt._lib.BF16)
    np.testing.assert_array_equal(rt.isnan(t).to_numpy(), np.isnan(f))
    np.testing.assert_array_equal(rt.signbit(t).to_numpy(), ~np.signbit(f))


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.float16])
def test_binary_float_ops(dev, dtype):
    a = values(dtype, seed=1)
    b = values(dtype, seed=2)[::-1].copy()
    ta, tb = rt.asarray(a, dev), rt.asarray(b, dev)
    np.testing.assert_array_equal(rt.copysign(ta, tb).to_numpy(), np.copysign(a, b))
    np.testing.assert_array_equal(rt.nextafter(ta, tb).to_numpy(), np.nextafter(a, b))
    np.testing.assert_array_equal(rt.floor_divide(ta, tb).to_numpy(), E.floor_divide(a, b))
    rtol = {np.float64: 4e-16, np.float32: 2.4e-7, np.float16: 1e-3}[dtype]
    for name, f in (("atan2", np.arctan2), ("hypot", np.hypot), ("logaddexp", E.logaddexp_naive)):
        got = getattr(rt, name)(ta, tb).to_numpy()
        with np.errstate(all="ignore"):
            want = f(a, b)
        fin = np.isfinite(want) & (np.abs(want) > 1e-30)
        # absolute term: log near 1 (logaddexp) turns a 1-ulp difference of exp into a larger relative one
        np.testing.assert_allclose(got[fin].astype(np.float64), want[fin].astype(np.float64), rtol=4 * rtol,
                                   atol=8 * rtol)
        np.testing.assert_array_equal(np.isnan(got), np.isnan(want))


def test_nextafter_bf16_bits(dev):
    a = np.array([1.0, 1.0, 0.0, -0.0, 2.0, np.inf], dtype=np.float32)
    b = np.array([2.0, 0.0, -1.0, 1.0, 2.0, 0.0], dtype=np.float32)
    ab = (a.view(np.uint32) >> 16).astype(np.uint16)
    bb = (b.view(np.uint32) >> 16).astype(np.uint16)
    ta, tb = rt.asarray(ab, dev), rt.asarray(bb, dev)
    ta = rt.Tensor(ta.storage, ta.shape, ta.stride, ta.offset, rt._lib.BF16)
    tb = rt.Tensor(tb.storage, tb.shape, tb.stride, tb.offset, rt._lib.BF16)
    got = rt.nextafter(ta, tb).to_numpy()
    assert got.tolist() == [0x3F81, 0x3F7F, 0x8001, 0x0001, 0x4000, 0x7F7F]


@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.uint8, np.int8])
def test_floor_divide_integers(dev, dtype):
    info = np.iinfo(dtype)
    rng = np.random.default_rng(3)
    a = rng.integers(info.min, info.max, 300, dtype=dtype, endpoint=True)
    b = rng.integers(-9 if info.min < 0 else 0, 10, 300).astype(dtype)
    a[:3] = [info.min, info.max, 7]
    b[:3] = [-1 if info.min < 0 else 1, 0, 3]
    got = rt.floor_divide(rt.asarray(a, dev), rt.asarray(b, dev)).to_numpy()
    np.testing.assert_array_equal(got, E.floor_divide(a, b))


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.uint16, np.bool_])
def test_comparisons_with_broadcast_and_scalars(dev, dtype):
    rng = np.random.default_rng(4)
    if dtype == np.bool_:
        a = rng.integers(0, 2, (6, 1, 5)).astype(bool)
        b = rng.integers(0, 2, (3, 5)).astype(bool)
    elif np.dtype(dtype).kind == "f":
        a = rng.integers(-3, 4, (6, 1, 5)).astype(dtype)
        b = rng.integers(-3, 4, (3, 5)).astype(dtype)
        a[0, 0, 0] = np.nan
        b[1, 2] = np.nan
    else:
        a = rng.integers(0, 6, (6, 1, 5)).astype(dtype)
        b = rng.integers(0, 6, (3, 5)).astype(dtype)
    ta, tb = rt.asarray(a, dev), rt.asarray(b, dev)
    for name, f in (("equal", np.equal), ("not_equal", np.not_equal), ("greater", np.greater),
                    ("greater_equal", np.greater_equal), ("less", np.less), ("less_equal", np.less_equal)):
        got = getattr(rt, name)(ta, tb)
        assert got.dtype_code == rt._lib.BOOL
        np.testing.assert_array_equal(got.to_numpy(), f(a, b))
        if dtype != np.bool_:
            s = dtype(2)
            np.testing.assert_array_equal(getattr(rt, name)(ta, s).to_numpy(), f(a, s))
            np.testing.assert_array_equal(getattr(rt, name)(s, tb).to_numpy(), f(s, b))


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.float16, np.int32])
def test_isclose_matches_reference_formula(dev, dtype):
    rng = np.random.default_rng(5)
    if np.dtype(dtype).kind == "f":
        a = rng.standard_normal(500).astype(dtype)
        b = (a * (1 + rng.choice([0, 1e-9, 1e-6, 1e-4, 1e-2], 500))).astype(dtype)
        a[:6] = [np.nan, np.nan, np.inf, np.inf, 0.0, 1e-9]
        b[:6] = [np.nan, 1.0, np.inf, -np.inf, 1e-9, 0.0]
    else:
        a = rng.integers(-100, 100, 500).astype(dtype)
        b = (a + rng.integers(-1, 2, 500)).astype(dtype)
    ta, tb = rt.asarray(a, dev), rt.asarray(b, dev)
    for rtol, atol, en in ((1e-5, 1e-8, False), (1e-3, 0.0, True), (0.0, 1.0, False)):
        got = rt.isclose(ta, tb, rtol, atol, en).to_numpy()
        np.testing.assert_array_equal(got, E.isclose(a, b, rtol, atol, en))
