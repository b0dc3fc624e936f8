"""Axis reductions and arg reductions on the GPU against the oracle:
integers and arg indices bit-exact, f64 within 1e-13 relative, f32 within 1e-5."""

import numpy as np
import pytest

import rstsr_gb300 as rt
from oracle import layout as OL
from oracle import oracle as O
from tests.helpers import NP, rand, strided_case, values

pytestmark = pytest.mark.gpu

KINDS = ["c", "f", "perm", "slice", "slice2", "flip"]
F64_TOL = 1e-13
F32_TOL = 1e-5


def up(dev, buf, shape, stride, off):
    return rt.from_host_layout(buf, shape, stride, off, dev)


def oracle_reduce(op, case, axes, out_dtype):
    buf, shape, stride, off = case
    oshape, ostride, _ = OL.reduce_output_layout((shape, stride, off), axes)
    out = O.empty_strided(oshape, ostride, out_dtype)
    O.reduce_axes(op, O.Strided(buf, shape, stride, off), axes, out, nthreads=4)
    return out.values(), (oshape, ostride)


def check_close(got, want, dtype, op):
    if np.dtype(dtype).kind in "iub" or op in ("min", "max", "count_nonzero"):
        np.testing.assert_array_equal(got, want, err_msg=op)
    else:
        # normwise relative error: summation order changes rounding, and a
        # single output that cancels to ~0 has no meaningful elementwise error
        tol = F64_TOL if np.dtype(dtype) == np.float64 else F32_TOL
        if op == "std":
            # sqrt amplifies the rounding of a small one-pass variance; compare variances
            got, want = np.square(got.astype(np.float64)), np.square(want.astype(np.float64))
        err = np.max(np.abs(got - want)) / max(np.max(np.abs(want)), 1e-300) if want.size else 0.0
        assert err <= tol, f"{op}: normwise rel err {err}"


AXES = [(1, 3), (3,), (0,), (1,), (0, 1, 2, 3), (2, 0)]


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("axes", AXES)
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int64])
def test_reduce_axes_matches_oracle(dev, kind, axes, dtype):
    case = strided_case(kind, (3, 10, 6, 40), dtype, seed=21)
    t = up(dev, *case)
    ops = ["sum", "min", "max", "count_nonzero"]
    if np.dtype(dtype).kind == "f":
        ops += ["mean", "var", "std", "l2_norm"]
    for op in ops:
        out_dt = np.uint64 if op == "count_nonzero" else dtype
        want, lo = oracle_reduce(op, case, list(axes), out_dt)
        got = rt.reduce_axes(op, t, list(axes))
        assert (got.shape, got.stride) == lo, op
        check_close(got.to_numpy(), want, dtype, op)


@pytest.mark.parametrize("dtype", [np.int32, np.int64])
def test_integer_sum_and_prod_wrap(dev, dtype):
    info = np.iinfo(dtype)
    x = np.full((3, 5000), info.max // 3, dtype=dtype)
    t = rt.asarray(x, dev)
    with np.errstate(over="ignore"):
        want = x.sum(axis=1, dtype=dtype)
    np.testing.assert_array_equal(t.sum_axes(1).to_numpy(), want)
    y = np.full((2, 70), 3, dtype=dtype)
    with np.errstate(over="ignore"):
        wantp = np.prod(y, axis=1, dtype=dtype)
    np.testing.assert_array_equal(rt.asarray(y, dev).prod_axes(1).to_numpy(), wantp)


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int64])
@pytest.mark.parametrize("axes", [(3,), (1,), (1, 3), (2, 0)])
def test_argmax_argmin_match_oracle(dev, kind, dtype, axes):
    case = strided_case(kind, (3, 10, 6, 40), dtype, seed=31)
    buf = case[0]
    if np.dtype(dtype).kind == "i":
        buf[:] = buf % 7  # many ties
    t = up(dev, *case)
    for is_max in (True, False):
        oshape, ostride, _ = OL.reduce_output_layout(case[1:], list(axes))
        out = O.empty_strided(oshape, ostride, np.uint64)
        O.argreduce_axes(is_max, O.Strided(*case), list(axes), out, nthreads=4)
        got = rt.argreduce_axes(is_max, t, list(axes))
        assert (got.shape, got.stride) == (oshape, ostride)
        np.testing.assert_array_equal(got.to_numpy(), out.values())


def test_argmax_all_and_nan_rule(dev):
    x = np.array([[np.nan, 1.0, 5.0], [1.0, np.nan, 5.0], [2.0, 7.0, np.nan]])
    t = rt.asarray(x, dev)
    assert t.argmax_axes(1).to_numpy().tolist() == [0, 2, 1]
    assert t.argmax_all() == 0  # NaN at flat index 0
    y = rt.asarray(np.array([1.0, np.nan, 3.0, 3.0]), dev)
    assert y.argmax_all() == 2
    z = rt.asarray(np.array([], dtype=np.float64), dev)
    with pytest.raises(rt.RstsrError) as e:
        z.argmax_all()
    assert e.value.kind == "InvalidLayout"


def test_reduce_all_scalars(dev):
    x = rand((37, 129), np.float64, seed=41)
    t = rt.asarray(x, dev)
    assert abs(t.sum_all() - x.sum()) <= 1e-13 * np.abs(x).sum()
    assert t.max_all() == x.max() and t.min_all() == x.min()
    xi = rand((1000, 17), np.int32, seed=42)
    ti = rt.asarray(xi, dev).permute_dims(1, 0)
    assert ti.sum_all() == int(xi.sum(dtype=np.int32))
    assert ti.argmax_all() == int(np.argmax(xi.T))
    assert ti.argmin_all() == int(np.argmin(xi.T))


def test_zero_size_rules(dev):
    e = rt.zeros((0, 4), np.float64, dev)
    assert e.sum_all() == 0.0
    s = e.sum_axes(0)
    assert s.shape == (4,) and s.to_numpy().tolist() == [0.0] * 4
    with pytest.raises(rt.RstsrError) as err:
        e.max_all()
    assert err.value.kind == "InvalidValue"


def test_bool_reductions(dev):
    y = np.array([[False, False, True], [False, True, True], [True, True, True]])
    t = rt.asarray(y, dev)
    assert t.all_axes(0).to_numpy().tolist() == [False, False, True]
    assert t.any_axes(1).to_numpy().tolist() == [True, True, True]
    assert t.sum_all() == 6 and t.count_nonzero_all() == 6
    assert not t.all_all() and t.any_all()


def test_small_dtypes_widened(dev):
    x = rand((4, 300), np.int8, seed=43)
    t = rt.asarray(x, dev)
    with np.errstate(over="ignore"):
        np.testing.assert_array_equal(t.sum_axes(1).to_numpy(), x.sum(axis=1, dtype=np.int8))
    np.testing.assert_array_equal(t.argmax_axes(1).to_numpy(), np.argmax(x, axis=1))
    h = rand((3, 64), np.float16, seed=44)
    th = rt.asarray(h, dev)
    np.testing.assert_allclose(th.sum_axes(1).to_numpy().astype(np.float64), h.astype(np.float64).sum(axis=1),
                               rtol=2e-3)


def test_broadcast_stride0_input(dev):
    x = rand((1, 50), np.float64, seed=45)
    t = rt.asarray(x, dev).broadcast_to((8, 50))
    np.testing.assert_allclose(t.sum_axes(0).to_numpy(), 8 * x[0], rtol=1e-15)
    np.testing.assert_allclose(t.sum_axes(1).to_numpy(), np.full(8, x.sum()), rtol=1e-14)


def test_large_reduction_uses_split_path(dev):
    """Few outputs, long reduced runs: exercises the chunked two-pass path."""
    x = rand((4, 1 << 20), np.float64, seed=46)
    t = rt.asarray(x, dev)
    got = t.sum_axes(1).to_numpy()
    ref = x.sum(axis=1)
    assert np.max(np.abs(got - ref) / np.abs(x).sum(axis=1)) < 1e-15 * 64
    xc = rand((1 << 18, 8), np.int32, seed=47)
    tc = rt.asarray(xc, dev)
    np.testing.assert_array_equal(tc.sum_axes(0).to_numpy(), xc.sum(axis=0, dtype=np.int32))
    np.testing.assert_array_equal(tc.argmax_axes(0).to_numpy(), np.argmax(xc, axis=0))


def test_kat_reductions(dev, kats):
    for case in kats:
        op = case["op"]
        if not (op.endswith("_all") or op.endswith("_axes")):
            continue
        arr = np.array(case["a"], dtype=NP[case["dtype"]])
        if "shape" in case:
            arr = arr.reshape(case["shape"])
        t = rt.asarray(arr, dev)
        if op.startswith("arg"):
            if op.endswith("_all"):
                got = (t.argmax_all() if "max" in op else t.argmin_all())
                assert got == case["expect"], case["src"]
            else:
                got = (t.argmax_axes(case["axes"]) if "max" in op else t.argmin_axes(case["axes"]))
                assert got.to_numpy().tolist() == case["expect"], case["src"]
            continue
        if op.endswith("_all"):
            got = getattr(t, op)()
            np.testing.assert_allclose(float(got), float(case["expect"]), rtol=1e-13, err_msg=case["src"])
        else:
            got = getattr(t, op)(case["axes"]).to_numpy()
            np.testing.assert_allclose(got.astype(np.float64), np.array(case["expect"], dtype=np.float64), rtol=1e-13,
                                       err_msg=case["src"])


# reduced lengths that select every group size of the row regime (one thread
# per output up to 256 threads per output, several outputs per CTA) and the
# column regime, with a few outputs each, against the oracle
@pytest.mark.parametrize("nred", [7, 100, 1000, 2500, 5000, 8192, 20000, 70001])
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int64])
@pytest.mark.parametrize("order", ["C", "F"])
def test_group_sizes_match_oracle(dev, nred, dtype, order):
    shape = (5, nred)
    stride = OL.c_stride(shape) if order == "C" else OL.f_stride(shape)
    buf = rand(shape, dtype, seed=nred).ravel()
    if np.dtype(dtype).kind == "i":
        buf[:] = buf % 17  # ties for the arg reductions
    case = (buf, shape, stride, 0)
    t = up(dev, *case)
    for op in ("sum", "max"):
        want, lo = oracle_reduce(op, case, [1], dtype)
        got = rt.reduce_axes(op, t, [1])
        assert (got.shape, got.stride) == lo
        check_close(got.to_numpy(), want, dtype, op)
    for is_max in (True, False):
        out = O.empty_strided((5,), (1,), np.uint64)
        O.argreduce_axes(is_max, O.Strided(*case), [1], out, nthreads=4)
        np.testing.assert_array_equal(rt.argreduce_axes(is_max, t, [1]).to_numpy(), out.values())


def test_f64_sum_wide_range_and_specials(dev):
    """f64 sums and means accumulate in fixed point on the device: values
    spread over 600 binades, subnormals, cancellation and huge magnitudes stay
    within 1e-13 of the oracle; NaN and +-inf follow IEEE addition."""
    rng = np.random.default_rng(5)
    n = 9000
    rows = [
        rng.uniform(-1, 1, n) * 10.0 ** rng.uniform(-300, 300, n),       # wide dynamic range
        rng.uniform(0, 1, n) * 1e-310,                                   # subnormals only
        np.concatenate([np.full(n // 2, 1e17), np.full(n - n // 2, -1e17)]) + rng.uniform(-1, 1, n),
        rng.uniform(0.5, 1.0, n) * 1e305,                                # the sum overflows to +inf
        rng.uniform(-1, 1, n),
    ]
    x = np.stack(rows)
    t = rt.asarray(x, dev)
    for op in ("sum", "mean"):
        case = (x.ravel(), x.shape, OL.c_stride(x.shape), 0)
        want, _ = oracle_reduce(op, case, [1], np.float64)
        got = rt.reduce_axes(op, t, [1]).to_numpy()
        assert np.isinf(got[3]) and np.isinf(want[3]) and got[3] > 0
        fin = np.isfinite(want)
        for i in np.nonzero(fin)[0]:
            # per row: the scale of that row's own terms
            scale = max(abs(want[i]), np.max(np.abs(x[i])) * (1 if op == "sum" else 1.0 / n), 1e-320)
            assert abs(got[i] - want[i]) <= 1e-13 * scale, (op, i, got[i], want[i])
    y = np.array([[1.0, np.inf, 2.0], [np.inf, -np.inf, 1.0], [np.nan, 1.0, 2.0], [-np.inf, -1.0, 5.0]])
    g = rt.asarray(y, dev).sum_axes(1).to_numpy()
    assert g[0] == np.inf and np.isnan(g[1]) and np.isnan(g[2]) and g[3] == -np.inf
    # the column regime and the split partials take the same accumulator
    z = rng.uniform(-1, 1, (1 << 16, 6)) * 10.0 ** rng.uniform(-30, 30, (1 << 16, 6))
    gz = rt.asarray(z, dev).sum_axes(0).to_numpy()
    wz = np.array([float(sum(map(__import__("fractions").Fraction, z[:, j]))) for j in range(6)])
    assert np.all(np.abs(gz - wz) <= 1e-13 * np.max(np.abs(z), axis=0))


@pytest.mark.parametrize("n", [4, 6, 96, 4096])
@pytest.mark.parametrize("dtype", [np.float32, np.int32, np.float64])
def test_step2_rows_reaching_the_buffer_end(dev, n, dtype):
    """Rows of a step-2 view whose last element is the last element of its
    buffer (no element after it): the 16-byte loads of the step-2 walk stop
    at the view's end. Against the oracle."""
    R = 5
    buf = rand((R * 2 * n - 1,), dtype, seed=n)
    if np.dtype(dtype).kind == "i":
        buf[:] = buf % 13
    case = (buf, (R, n), (2 * n, 2), 0)
    t = up(dev, *case)
    for op in ("sum", "max"):
        want, lo = oracle_reduce(op, case, [1], dtype)
        got = rt.reduce_axes(op, t, [1])
        assert (got.shape, got.stride) == lo
        check_close(got.to_numpy(), want, dtype, op)
    for is_max in (True, False):
        out = O.empty_strided((R,), (1,), np.uint64)
        O.argreduce_axes(is_max, O.Strided(*case), [1], out, nthreads=4)
        np.testing.assert_array_equal(rt.argreduce_axes(is_max, t, [1]).to_numpy(), out.values())
