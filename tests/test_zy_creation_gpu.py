"""arange / linspace / tril / triu on the GPU: the reference's creation
known-answer tests, and bit-exact agreement with the oracle
(oracle/creation.py) on value sweeps, strided and batched layouts; and
allclose_all against all(oracle isclose). The module is collected after the
element-wise, GEMM, reduction and indexing modules (pytest orders files by
name), before the allocation-free module that must run last."""

import numpy as np
import pytest

import rstsr_gb300 as rt
from oracle import creation as OC
from oracle import elementwise as E
from rstsr_gb300._lib import RstsrError
from tests.test_creation_oracle import CASES, DT, arange_args, check_values

pytestmark = pytest.mark.gpu


def bits(x):
    x = np.asarray(x)
    return x.view(f"u{x.itemsize}") if x.dtype.kind == "f" else x


def run_case(case, dev):
    dt = DT[case["dtype"]]
    if case["op"] == "arange":
        s, e, st = arange_args(case["args"])
        return rt.arange(s, e, st, dtype=dt, device=dev)
    if case["op"] == "linspace":
        start, stop, num = case["args"]
        return rt.linspace(start, stop, num, endpoint=case["endpoint"], dtype=dt, device=dev)
    t = rt.asarray(np.array(case["a"], dtype=dt), dev)
    return (rt.triu if case["op"] == "triu" else rt.tril)(t, case["k"])


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['op']}-{c['src'].split(':')[1]}")
def test_device_reproduces_reference_kat(dev, case):
    if "error" in case:
        with pytest.raises(rt.RstsrError) as err:
            run_case(case, dev)
        assert err.value.kind == case["error"]
        return
    check_values(case, run_case(case, dev).to_numpy())


@pytest.mark.parametrize("start,stop,step,dtype", [
    (0.0, 1.0, 0.1, np.float64), (0.0, 1.0, 0.1, np.float32), (1.0, 0.0, -0.1, np.float64),
    (-3.5, 40000.0, 0.37, np.float64), (-3.5, 40000.0, 0.37, np.float32), (0.0, 0.3, 0.1, np.float64),
    (0, 10, 3, np.int32), (10, 0, -2, np.int32), (-7, 300007, 7, np.int64), (0, 2 ** 32 - 1, 65536, np.uint32),
    (2 ** 63, 2 ** 63 + 100, 7, np.uint64), (0, 100, 7, np.int8), (200, 255, 11, np.uint8),
    (0, 1000, 333, np.int16), (64000, 65000, 500, np.uint16), (5, 5, 1, np.int64), (1.0, 0.0, 0.5, np.float64),
])
def test_arange_matches_oracle(dev, start, stop, step, dtype):
    want = OC.arange(start, stop, step, dtype)
    got = rt.arange(start, stop, step, dtype=dtype, device=dev).to_numpy()
    assert got.dtype == want.dtype and got.shape == want.shape
    np.testing.assert_array_equal(bits(got), bits(want))


def test_arange_refusals(dev):
    with pytest.raises(rt.RstsrError) as err:
        rt.arange(0, 10, 0, dtype=np.int32, device=dev)
    assert err.value.kind == "InvalidValue"
    with pytest.raises(rt.RstsrError) as err:
        rt.arange(0, 5, -100, dtype=np.int8, device=dev)  # the reference's repeated addition wraps
    assert err.value.kind == "ValueOutOfRange"
    with pytest.raises(rt.RstsrError) as err:
        rt.arange(0.0, 1.0, 0.5, dtype=np.float16, device=dev)
    assert err.value.kind == "UnImplemented"
    assert rt.arange(3, dtype=np.int32, device=dev).to_numpy().tolist() == [0, 1, 2]


@pytest.mark.parametrize("start,stop,num,endpoint,dtype", [
    (0.0, 1.0, 11, True, np.float64), (0.0, 1.0, 11, True, np.float32), (2.0, 10.0, 100, False, np.float64),
    (-5.0, 5.0, 100003, True, np.float32), (-5.0, 5.0, 100003, True, np.float64), (3.0, 3.0, 1, True, np.float64),
    (1.0, 2.0, 0, True, np.float64), (1e10, -1e10, 7, False, np.float32),
])
def test_linspace_matches_oracle(dev, start, stop, num, endpoint, dtype):
    want = OC.linspace(start, stop, num, dtype, endpoint=endpoint)
    got = rt.linspace(start, stop, num, endpoint=endpoint, dtype=dtype, device=dev).to_numpy()
    assert got.shape == want.shape
    np.testing.assert_array_equal(bits(got), bits(want))


def test_linspace_refuses_integers(dev):
    with pytest.raises(rt.RstsrError) as err:
        rt.linspace(0, 10, 5, dtype=np.int32, device=dev)
    assert err.value.kind == "InvalidValue"


@pytest.mark.parametrize("shape", [(5, 5), (3, 7), (7, 3), (4, 1, 6), (2, 3, 4, 5), (1, 300, 257), (0, 4)])
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int8, np.bool_, np.float16])
@pytest.mark.parametrize("upper", [False, True])
def test_tri_mask_copy_matches_oracle(dev, shape, dtype, upper):
    rng = np.random.default_rng(5)
    x = (rng.integers(1, 100, shape) if dtype != np.bool_ else rng.integers(0, 2, shape)).astype(dtype)
    t = rt.asarray(x, dev)
    for k in (-300, -2, -1, 0, 1, 3, 300):
        got = (rt.triu if upper else rt.tril)(t, k).to_numpy()
        np.testing.assert_array_equal(got, OC.tri_mask(x, k, upper))
    np.testing.assert_array_equal(t.to_numpy(), x)  # the input is not modified


@pytest.mark.parametrize("kind", ["f", "perm", "flip"])
def test_tri_mask_in_place_on_strided_views(dev, kind):
    rng = np.random.default_rng(6)
    base_shape = (3, 9, 8)
    base = rng.standard_normal(int(np.prod(base_shape)))
    if kind == "f":
        shape, stride, off = base_shape, (1, 3, 27), 0
    elif kind == "perm":
        shape, stride, off = (9, 3, 8), (8, 72, 1), 0
    else:
        shape, stride, off = base_shape, (72, 8, -1), 7
    t = rt.from_host_layout(base, shape, stride, off, dev)
    before = t.to_numpy()
    rt.tril(t, -1, inplace=True)
    np.testing.assert_array_equal(t.to_numpy(), OC.tri_mask(before, -1, False))
    whole = rt.Tensor(t.storage, (base.size,), (1,), 0, t.dtype_code).to_numpy()
    assert np.count_nonzero(whole == 0) == np.count_nonzero(OC.tri_mask(before, -1, False) == 0)


def test_tri_mask_needs_two_axes(dev):
    with pytest.raises(rt.RstsrError) as err:
        rt.tril(rt.asarray(np.ones(4), dev))
    assert err.value.kind == "InvalidLayout"


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32])
def test_allclose_is_all_of_isclose(dev, dtype):
    """allclose_all (auto_impl/reduction.rs:717-749) against all(oracle isclose),
    with broadcasting, NaN handling and the zero-size error."""
    rng = np.random.default_rng(9)
    x = (rng.standard_normal((64, 33)) * 100).astype(dtype)
    for y, rtol, atol in [(x, 1e-5, 1e-8), ((x * (1 + 1e-7)).astype(dtype), 1e-5, 1e-8),
                          ((x * (1 + 1e-7)).astype(dtype), 1e-9, 0.0), ((x + 1).astype(dtype), 1e-5, 1e-8),
                          ((x + 1).astype(dtype), 0.0, 1.0)]:
        want = bool(E.isclose(x, y, rtol, atol).all())
        assert rt.allclose(rt.asarray(x, dev), rt.asarray(y, dev), rtol, atol) is want
    rows = np.broadcast_to(x[0], (5, 33)).copy()
    assert rt.allclose(rt.asarray(rows, dev), rt.asarray(x[0], dev)) is True
    if dtype != np.int32:
        xn = x.copy()
        xn[3, 4] = np.nan
        tn = rt.asarray(xn, dev)
        assert rt.allclose(tn, tn) is False
        assert rt.allclose(tn, tn, equal_nan=True) is True
    with pytest.raises(RstsrError) as err:
        rt.allclose(rt.asarray(np.zeros((0, 3), dtype=dtype), dev), rt.asarray(np.zeros((0, 3), dtype=dtype), dev))
    assert err.value.kind == "InvalidValue"
