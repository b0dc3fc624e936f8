"""Row-regime reductions of 16 MB to 134 MB against the oracle.

At these sizes the planner's choices differ from the small cases of
test_reduce_gpu.py: groups of 2 to 32 threads per output with full rounds of
vector loads, the chunk split of the reduced range with its combine pass
(chunk boundaries falling inside runs of the reduced dim 0), partial last
CTAs, negative strides and offsets. Also every value kind, the arg
reductions' first-index and NaN rules on ties, and a non-monotone arg layout
(reduced axes whose memory order differs from their logical order). Integers
and indices bit-exact; f64 within 1e-13 and f32 within 1e-5 normwise relative
(f32 sums against an f64 oracle).
"""

import numpy as np
import pytest

import rstsr_gb300 as rt
from oracle import layout as OL
from oracle import oracle as O

pytestmark = pytest.mark.gpu

F64_TOL = 1e-13
F32_TOL = 1e-5


def make(dtype, n, seed, lo=-1.0, hi=1.0):
    rng = np.random.default_rng(seed)
    if np.dtype(dtype).kind == "f":
        return rng.uniform(lo, hi, n).astype(dtype)
    return rng.integers(-1000, 1001, n).astype(dtype)


def oracle_reduce(op, buf, shape, stride, off, axes, out_dtype):
    if buf.dtype == np.float32 and op in ("sum", "mean", "var", "std", "l2_norm", "prod"):
        buf, out_dtype = buf.astype(np.float64), np.float64
    oshape, ostride, _ = OL.reduce_output_layout((shape, stride, off), axes)
    out = O.empty_strided(oshape, ostride, out_dtype)
    O.reduce_axes(op, O.Strided(buf, shape, stride, off), axes, out, nthreads=O.max_threads())
    return out.values(), (tuple(oshape), tuple(ostride))


def oracle_arg(is_max, buf, shape, stride, off, axes):
    oshape, ostride, _ = OL.reduce_output_layout((shape, stride, off), axes)
    out = O.empty_strided(oshape, ostride, np.uint64)
    O.argreduce_axes(is_max, O.Strided(buf, shape, stride, off), axes, out, nthreads=O.max_threads())
    return out.values(), (tuple(oshape), tuple(ostride))


def check(got, want, dtype, op):
    if np.dtype(dtype).kind in "iub" or op in ("min", "max", "count_nonzero"):
        np.testing.assert_array_equal(got, want, err_msg=op)
        return
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    if op == "std":
        got, want = np.square(got), np.square(want)
    tol = F64_TOL if np.dtype(dtype) == np.float64 else F32_TOL
    err = float(np.max(np.abs(got - want)) / max(float(np.max(np.abs(want))), 1e-300))
    assert err <= tol, f"{op}: normwise rel err {err}"


def run_case(dev, buf, shape, stride, off, axes, ops, args=(True, False)):
    t = rt.from_host_layout(buf, shape, stride, off, dev)
    for op in ops:
        out_dt = np.uint64 if op == "count_nonzero" else buf.dtype
        want, lo = oracle_reduce(op, buf, shape, stride, off, list(axes), out_dt)
        got = rt.reduce_axes(op, t, list(axes))
        assert (got.shape, got.stride) == lo, op
        check(got.to_numpy(), want, buf.dtype, op)
    for is_max in args:
        want, lo = oracle_arg(is_max, buf, shape, stride, off, list(axes))
        got = rt.argreduce_axes(is_max, t, list(axes))
        assert (got.shape, got.stride) == lo
        np.testing.assert_array_equal(got.to_numpy(), want, err_msg=f"arg{'max' if is_max else 'min'}")


# (rows, run length): groups of 2 threads (128 outputs per CTA, a partial
# last CTA), 16 threads, and 32 threads with the reduced range split in three
ROWS = [(262147, 128), (32771, 128), (4099, 1024), (1031, 4096)]


@pytest.mark.parametrize("rows,n", ROWS, ids=[f"{r}x{n}" for r, n in ROWS])
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32])
def test_contiguous_rows(dev, rows, n, dtype):
    if np.dtype(dtype).itemsize == 8 and n != 4096:
        rows = rows // 2 + 1  # the same bytes
    buf = make(dtype, rows * n, seed=rows + n)
    if np.dtype(dtype).kind == "i":
        buf %= 7  # many ties
    run_case(dev, buf, (rows, n), (n, 1), 0, (1,), ["sum"])


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int64])
def test_runs_cut_by_chunks(dev, dtype):
    """Runs of 96 elements (rows of 128, the first 96 used), 6144 per output:
    the chunks of the split reduced range end inside runs."""
    outer = 1024 if np.dtype(dtype).itemsize == 4 else 512
    base = make(dtype, outer * 64 * 128, seed=5)
    shape, stride = (outer, 64, 96), (64 * 128, 128, 1)
    run_case(dev, base, shape, stride, 0, (1, 2), ["sum", "max"])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_negative_strides_and_offset(dev, dtype):
    """Kept axis 0 and reduced axis 1 reversed; runs of 96."""
    outer = 1024 if dtype == np.float32 else 512
    base = make(dtype, outer * 64 * 128, seed=6)
    shape, stride = (outer, 64, 96), (-64 * 128, -128, 1)
    off = (outer - 1) * 64 * 128 + 63 * 128
    run_case(dev, base, shape, stride, off, (1, 2), ["sum", "min"])


def test_aligned_offset_rows(dev):
    """Rows of 2040 of a [2049, 2048] f32 buffer starting 4 elements in."""
    base = make(np.float32, 2049 * 2048, seed=7)
    run_case(dev, base, (2049, 2040), (2048, 1), 4, (1,), ["sum", "mean"])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_value_kinds(dev, dtype):
    """Every value reduction on [4099, 1024] (f32) / [2053, 1024] (f64), a zero
    at the start of every third row for count_nonzero; the product on values
    near 1 so that it stays finite."""
    rows = 4099 if dtype == np.float32 else 2053
    buf = make(dtype, rows * 1024, seed=8)
    buf[::3 * 1024] = 0
    run_case(dev, buf, (rows, 1024), (1024, 1), 0, (1,),
             ["sum", "mean", "var", "std", "l2_norm", "min", "max", "count_nonzero"], args=())
    near1 = make(dtype, rows * 1024, seed=12, lo=0.999, hi=1.001)
    run_case(dev, near1, (rows, 1024), (1024, 1), 0, (1,), ["prod"], args=())


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_arg_nan_rules(dev, dtype):
    """A NaN at logical index 0 answers 0; other NaNs are never taken; ties
    resolve to the first index."""
    rows, n = 65539, 128
    buf = make(dtype, rows * n, seed=9)
    buf = np.round(buf * 8) / 8  # ties
    x = buf.reshape(rows, n)
    x[::5, 0] = np.nan
    x[1::7, 37] = np.nan
    x[2::11, :] = np.nan
    x[3::13, :] = 0.5
    run_case(dev, buf, (rows, n), (n, 1), 0, (1,), [])


def test_non_monotone_arg_layout(dev):
    """Reduced axes (1, 2) of a view whose memory-inner axis is logically
    outer: the arg reductions carry logical indices through the walk."""
    nout = 2048
    base = make(np.float32, nout * 64 * 128, seed=10)
    base = np.round(base * 16) / 16
    shape, stride = (nout, 128, 64), (64 * 128, 1, 128)
    run_case(dev, base, shape, stride, 0, (1, 2), ["sum"])


def test_workload_sum_axes_1_3(dev):
    """The [32,64,128,128] sum over axes (1, 3): 4096 outputs of 64 runs of 128."""
    shape = (32, 64, 128, 128)
    buf = make(np.float32, int(np.prod(shape)), seed=11)
    run_case(dev, buf, shape, OL.c_stride(shape), 0, (1, 3), ["sum"], args=())
