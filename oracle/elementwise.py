"""numpy restatement of the reference's element-wise operator semantics
(TEST INFRASTRUCTURE ONLY: the results the device kernels are compared with,
never the product). Each function follows the closure the reference applies per element:

  round        Rust f64::round (half away from zero), auto_impl/op_binary_common.rs:30
  sign         ExtNum::ext_sign, rstsr-dtype-traits/src/ext_num.rs:83-89, :125-134, :166-178
  signbit      Signed::is_positive, auto_impl/op_binary_common.rs:97 (floats: sign bit clear)
  floor_divide ExtReal::ext_floor_divide, rstsr-dtype-traits/src/ext_real.rs (floor(a / b);
               integers Integer::div_floor)
  logaddexp    (a.exp() + b.exp()).ln(), auto_impl/op_ternary_common.rs:13 (no rescaling)
  isclose      rstsr-dtype-traits/src/isclose.rs:92-105 (|a - b| <= atol + rtol |b|)
Integer division by zero gives 0 here where the reference panics; integer
MIN / -1 wraps.
"""

from __future__ import annotations

import numpy as np


def rust_round(x):
    x = np.asarray(x)
    w = x.astype(np.float64)
    r = np.trunc(w)
    f = w - r
    out = np.where(np.abs(f) >= 0.5, r + np.sign(w), r)
    return out.astype(x.dtype)


def ext_sign(x):
    x = np.asarray(x)
    if x.dtype.kind == "f":
        return np.where(np.isnan(x), x, np.where(x > 0, 1, np.where(x < 0, -1, 0))).astype(x.dtype)
    if x.dtype.kind == "u":
        return (x != 0).astype(x.dtype)
    return np.sign(x).astype(x.dtype)


def signbit_is_positive(x):
    x = np.asarray(x)
    if x.dtype.kind == "f":
        return ~np.signbit(x)
    return x > 0


def floor_divide(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype.kind == "f":
        with np.errstate(all="ignore"):
            return np.floor((a / b).astype(a.dtype)).astype(a.dtype)
    with np.errstate(all="ignore"):
        q = np.floor_divide(a, np.where(b == 0, 1, b))
        q = np.where(b == 0, 0, q)
        if a.dtype.kind == "i":
            mn = np.iinfo(a.dtype).min
            q = np.where((a == mn) & (b == -1), mn, q)
    return q.astype(a.dtype)


def logaddexp_naive(a, b):
    with np.errstate(all="ignore"):
        return np.log(np.exp(a) + np.exp(b))


def isclose(a, b, rtol=1e-5, atol=1e-8, equal_nan=False):
    a, b = np.asarray(a), np.asarray(b)
    with np.errstate(all="ignore"):
        if a.dtype.kind == "f":
            diff = np.abs((a - b).astype(a.dtype)).astype(np.float64)
            absb = np.abs(b).astype(np.float64)
            nan = np.isnan(a) & np.isnan(b)
        else:
            d = np.where(a >= b, a - b, b - a)  # wrapping in the integer type
            diff = d.astype(np.float64)
            absb = np.where(b < 0, -b, b).astype(np.float64) if a.dtype.kind == "i" else b.astype(np.float64)
            nan = np.zeros(np.broadcast(a, b).shape, dtype=bool)
        return (diff <= atol + rtol * absb) | (equal_nan & nan)
