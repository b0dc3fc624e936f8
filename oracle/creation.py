"""Python restatement of the reference's device creation algorithms
(TEST INFRASTRUCTURE ONLY: what the device's arange / linspace / tril / triu
are compared with, never the product).

  arange    rstsr-native-impl/src/cpu_rayon/creation.rs:8-104 (the rayon device's
            arange_impl, rstsr-core/src/feature_rayon/auto_impl/creation.rs:74-86):
            f64 / f32 through `start + i * step` in f64 (cpu_rayon/creation.rs:36-55),
            i32 / i64 / u32 / u64 through isize arithmetic (:8-34), each with
            n = ceil((end - start) / step) in f64 and the last element dropped when it
            is not strictly inside the interval; other element types, and the cases
            those conversions reject, by repeated addition while `current < end`
            (cpu_serial/creation.rs:7-19).
  linspace  cpu_rayon/creation.rs:108-128: step = (end - start) / (n - 1) (or / n
            without the endpoint) in the element type, element i = start + i * step.
  tril/triu cpu_serial/op_tri.rs:524-591 over the last two axes: tril zeroes
            j >= i + k + 1, triu zeroes j < i + k (clipped to the row here; the
            reference indexes past the row when i + k > ncol).

`arange` returns None where the reference's repeated addition does not end
(more than `cap` elements, or a value that stops changing).
"""

from __future__ import annotations

import math

import numpy as np

FLOAT_ACCEL = (np.float64, np.float32)
INT_ACCEL = (np.int32, np.int64, np.uint32, np.uint64)
INT_LOOP = (np.int8, np.int16, np.uint8, np.uint16)
ISIZE_MIN, ISIZE_MAX = -(2 ** 63), 2 ** 63 - 1


def _f64_to_usize(x: float):
    """num's ToPrimitive::to_usize for f64: Some(trunc) within (-1, 2^64)."""
    if math.isnan(x) or not (-1.0 < x < 18446744073709551616.0):
        return None
    return int(x)


def _f64_to_isize(x: float):
    if math.isnan(x) or not (-9223372036854777856.0 < x < 9223372036854775808.0):
        return None
    return int(x)


def _wrap(v: int, dtype) -> int:
    info = np.iinfo(dtype)
    span = info.max - info.min + 1
    return (v - info.min) % span + info.min


def _loop(start, end, step, dtype, cap):
    """while current < end { push(current); current = current + step } in the type."""
    out = []
    cur = np.array(start, dtype=dtype)[()]
    endv = np.array(end, dtype=dtype)[()]
    stepv = np.array(step, dtype=dtype)[()]
    with np.errstate(over="ignore"):
        while cur < endv:
            if len(out) >= cap:
                return None
            out.append(cur)
            nxt = np.array(cur + stepv, dtype=dtype)[()]  # wrapping / rounding in the type
            if nxt == cur:
                return None
            cur = nxt
    return np.array(out, dtype=dtype)


def _loop_len(start, end, step, dtype, cap):
    got = _loop(start, end, step, dtype, cap)
    return None if got is None else ("loop", got)


def arange_len(start, end, step, dtype, cap=1 << 20):
    """('accel', n, first, step, kind) for the closed-form paths (no values
    built), ('loop', values) for repeated addition, or None where that
    addition does not finish within `cap` elements."""
    dtype = np.dtype(dtype).type
    if step == 0:
        raise ValueError("step must not be zero")
    if dtype in FLOAT_ACCEL:
        s, e, st = float(dtype(start)), float(dtype(end)), float(dtype(step))
        q = (e - s) / st if st else float("nan")
        n = _f64_to_usize(math.ceil(q)) if math.isfinite(q) else None
        if n is None:
            return _loop_len(start, end, step, dtype, cap)
        if n:
            last = dtype(np.float64(s + float(n - 1) * st))
            endv = dtype(end)
            if (st > 0 and last >= endv) or (st < 0 and last <= endv):
                n -= 1
        return ("accel", n, s, st, "float")
    if dtype in INT_ACCEL:
        s, e, st = int(start), int(end), int(step)
        if all(ISIZE_MIN <= x <= ISIZE_MAX for x in (s, e, st)):
            diff = _wrap(e - s, np.int64)
            n = _f64_to_isize(math.ceil(float(diff) / float(st)))
            if n is None:
                return _loop_len(start, end, step, dtype, cap)
            n = max(n, 0)
            if n:
                last = _wrap(s + (n - 1) * st, np.int64)
                info = np.iinfo(dtype)
                if s + (n - 1) * st != last or not info.min <= last <= info.max:
                    raise OverflowError("value does not fit the element type")
                if (st > 0 and last >= e) or (st < 0 and last <= e):
                    n -= 1
            return ("accel", n, s, st, "int")
        return _loop_len(start, end, step, dtype, cap)
    if dtype in INT_LOOP:
        return _loop_len(start, end, step, dtype, cap)
    raise TypeError(f"arange is not defined for {np.dtype(dtype).name} here")


def arange(start, end, step, dtype, cap=1 << 20):
    """The values of arange(start, end, step) in `dtype`, or None (see arange_len)."""
    dtype = np.dtype(dtype).type
    r = arange_len(start, end, step, dtype, cap)
    if r is None or r[0] == "loop":
        return None if r is None else r[1]
    _, n, s, st, kind = r
    if kind == "float":
        return np.array([s + float(i) * st for i in range(n)], dtype=np.float64).astype(dtype)
    return np.array([s + i * st for i in range(n)], dtype=dtype)


def linspace(start, end, n, dtype, endpoint=True):
    dtype = np.dtype(dtype).type
    if n == 0:
        return np.zeros(0, dtype=dtype)
    if n == 1:
        return np.array([start], dtype=dtype)
    s, e = dtype(start), dtype(end)
    div = dtype(n - 1) if endpoint else dtype(n)
    with np.errstate(all="ignore"):
        step = dtype(dtype(e - s) / div)
        return np.array([dtype(s + dtype(dtype(i) * step)) for i in range(n)], dtype=dtype)


def tri_mask(x: np.ndarray, k: int, upper: bool) -> np.ndarray:
    """tril (upper=False) / triu (upper=True) of the last two axes of a copy of x."""
    out = np.array(x, copy=True)
    nrow, ncol = out.shape[-2], out.shape[-1]
    for i in range(nrow):
        if upper:
            out[..., i, : min(max(i + k, 0), ncol)] = 0
        else:
            out[..., i, max(i + k + 1, 0):] = 0
    return out
