"""The allocation-free sum over axes (rstsr_cuda_sum_axes_noalloc).

Callers that cannot let this library allocate device memory -- hosts that
own all GPU memory through their own arena, latency-critical loops that
cannot take cudaMalloc's synchronisation, plugin hosts that forbid foreign
allocations -- use this entry point: it takes a stream instead of a context
and keeps its scratch in a fixed static device array. These tests call it
through the C ABI and check it against the regular entry point,
rstsr_cuda_reduce_axes_into, on two calls in a row. This file is collected
last so that a failure here stops a -x run only after every other test.
"""

import ctypes as C

import numpy as np
import pytest

import rstsr_gb300 as rt
from rstsr_gb300._lib import Layout, call, lib

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


@pytest.mark.parametrize(
    "shape,axes,dtype",
    [
        ((4, 1 << 20), [1], np.float64),      # few outputs, long rows: split partials in the static scratch
        ((1 << 18, 8), [0], np.float64),      # column regime with split partials
        ((32, 64, 128, 128), [1, 3], np.float64),  # the workload's sum over axes (1, 3)
        ((6, 1 << 19), [1], np.float32),
        ((1 << 17, 5), [0], np.int32),
    ],
)
def test_noalloc_matches_regular_twice(dev, shape, axes, dtype):
    rng = np.random.default_rng(123)
    for call_no in range(2):
        if np.dtype(dtype).kind == "f":
            x = rng.uniform(-1, 1, shape).astype(dtype)
        else:
            x = rng.integers(-1000, 1001, shape).astype(dtype)
        t = rt.asarray(x, dev)
        kept = [d for i, d in enumerate(shape) if i not in axes]
        want = rt.empty(kept, dtype, dev)
        got = rt.empty(kept, dtype, dev)
        rt.fill(got, 7)  # stale contents must not leak into the result
        regular_sum(dev, t, axes, want)
        noalloc_sum(dev, t, axes, got)
        dev.sync()
        w, g = want.to_numpy(), got.to_numpy()
        if np.dtype(dtype).kind == "f":
            tol = F64_TOL if dtype == np.float64 else 1e-5
            err = np.max(np.abs(g - w)) / max(np.max(np.abs(w)), 1e-300)
            assert err <= tol, f"call {call_no}: normwise rel err {err}"
        else:
            np.testing.assert_array_equal(g, w)


def test_noalloc_rejects_unsupported_dtype(dev):
    x = rt.zeros((64, 1), np.float16, dev)
    ax = (C.c_int64 * 1)(0)
    out = rt.empty((1,), np.float16, dev)
    rc = lib().rstsr_cuda_sum_axes_noalloc(C.c_void_p(dev.stream()), x.dtype_code, C.c_void_p(x.ptr),
                                           C.byref(x.layout()), ax, 1, C.c_void_p(out.ptr), C.byref(out.layout()))
    assert rc == 7  # UnImplemented: dtype outside f64/f32/i32/i64
    assert b"supports" in lib().rstsr_cuda_last_error()
