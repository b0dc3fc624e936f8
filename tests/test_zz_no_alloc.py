"""The allocation-free sum over axes (rstsr_cuda_sum_axes_noalloc).

Callers that cannot let this library allocate device memory -- hosts that
own all GPU memory through their own arena, latency-critical loops that
cannot take cudaMalloc's synchronisation, plugin hosts that forbid foreign
allocations -- use this entry point: it takes a stream instead of a context
and keeps its scratch in a fixed static device array. These tests call it
through the C ABI and check it against the regular entry point,
rstsr_cuda_reduce_axes_into, and against the CPU oracle, on two calls in a
row, in C and F layouts, including plans whose default split would need more
than the fixed scratch. This file is collected
last so that a failure here stops a -x run only after every other test.
"""

import ctypes as C

import numpy as np
import pytest

import rstsr_gb300 as rt
from oracle import layout as OL
from oracle import oracle as O
from rstsr_gb300._lib import call, lib

pytestmark = pytest.mark.gpu

F64_TOL = 1e-13


def regular_sum(dev, t, axes, out):
    ax = (C.c_int64 * len(axes))(*axes)
    call("rstsr_cuda_reduce_axes_into", dev.ctx, 0, t.dtype_code, C.c_void_p(t.ptr), C.byref(t.layout()), ax,
         len(axes), C.c_void_p(out.ptr), C.byref(out.layout()))


def noalloc_sum(dev, t, axes, out):
    ax = (C.c_int64 * len(axes))(*axes)
    rc = lib().rstsr_cuda_sum_axes_noalloc(C.c_void_p(dev.stream()), t.dtype_code, C.c_void_p(t.ptr),
                                           C.byref(t.layout()), ax, len(axes), C.c_void_p(out.ptr),
                                           C.byref(out.layout()))
    assert rc == 0, lib().rstsr_cuda_last_error().decode()


def oracle_sum(buf, shape, stride, axes, dtype):
    """The oracle's sum; f32 inputs are summed in f64 (the oracle's own f32
    sum of 2^19 elements carries about 1e-5 of rounding)."""
    if dtype == np.float32:
        buf, dtype = buf.astype(np.float64), np.float64
    kept = [d for i, d in enumerate(shape) if i not in axes]
    out = O.empty_strided(kept, OL.c_stride(kept), dtype)
    O.reduce_axes("sum", O.Strided(buf, shape, stride, 0), list(axes), out, nthreads=O.max_threads())
    return out.values()


def check(got, want, dtype, what):
    if np.dtype(dtype).kind == "f":
        tol = F64_TOL if dtype == np.float64 else 1e-5
        err = np.max(np.abs(got - want)) / max(np.max(np.abs(want)), 1e-300)
        assert err <= tol, f"{what}: normwise rel err {err}"
    else:
        np.testing.assert_array_equal(got, want, err_msg=what)


@pytest.mark.parametrize(
    "shape,axes,dtype,order",
    [
        ((4, 1 << 20), [1], np.float64, "C"),      # few outputs, long rows: split partials in the static scratch
        ((1 << 18, 8), [0], np.float64, "C"),      # column regime with split partials
        ((32, 64, 128, 128), [1, 3], np.float64, "C"),  # the workload's sum over axes (1, 3)
        ((32, 64, 128, 128), [1, 3], np.float32, "F"),  # the same on the F-ordered layout
        ((6, 1 << 19), [1], np.float32, "C"),
        ((1 << 17, 5), [0], np.int32, "C"),
        # column regime whose default split needs more than the fixed scratch
        # (about 4.9 MB of partials): it runs with fewer chunks instead
        ((8192, 4096), [0], np.float64, "C"),
        ((4096, 6000), [1], np.float32, "F"),       # F order, 4096 outputs along the contiguous axis
    ],
)
def test_noalloc_matches_regular_and_oracle_twice(dev, shape, axes, dtype, order):
    rng = np.random.default_rng(123)
    stride = OL.c_stride(shape) if order == "C" else OL.f_stride(shape)
    for call_no in range(2):
        n = int(np.prod(shape))
        if np.dtype(dtype).kind == "f":
            buf = rng.uniform(-1, 1, n).astype(dtype)
        else:
            buf = rng.integers(-1000, 1001, n).astype(dtype)
        t = rt.from_host_layout(buf, shape, stride, 0, dev)
        kept = [d for i, d in enumerate(shape) if i not in axes]
        want = rt.empty(kept, dtype, dev)
        got = rt.empty(kept, dtype, dev)
        rt.fill(got, 7)  # stale contents must not leak into the result
        regular_sum(dev, t, axes, want)
        noalloc_sum(dev, t, axes, got)
        dev.sync()
        g = got.to_numpy()
        check(g, want.to_numpy(), dtype, f"call {call_no} vs the regular entry point")
        check(g, oracle_sum(buf, shape, stride, axes, dtype), dtype, f"call {call_no} vs the oracle")


def test_noalloc_rejects_unsupported_dtype(dev):
    x = rt.zeros((64, 1), np.float16, dev)
    ax = (C.c_int64 * 1)(0)
    out = rt.empty((1,), np.float16, dev)
    rc = lib().rstsr_cuda_sum_axes_noalloc(C.c_void_p(dev.stream()), x.dtype_code, C.c_void_p(x.ptr),
                                           C.byref(x.layout()), ax, 1, C.c_void_p(out.ptr), C.byref(out.layout()))
    assert rc == 7  # UnImplemented: dtype outside f64/f32/i32/i64
    assert b"supports" in lib().rstsr_cuda_last_error()
