"""Pins oracle/elementwise.py to the semantics the reference states for its
element-wise closures (CPU only)."""

import numpy as np

from oracle import elementwise as E


def test_round_is_half_away_from_zero():
    # Rust f64::round: rstsr-core/src/feature_rayon/auto_impl/op_binary_common.rs:30
    x = np.array([0.5, 1.5, 2.5, -0.5, -2.5, 0.49999999999999994, -0.0, 3.0])
    assert E.rust_round(x).tolist() == [1.0, 2.0, 3.0, -1.0, -3.0, 0.0, -0.0, 3.0]


def test_sign_zero_and_nan():
    # rstsr-dtype-traits/src/ext_num.rs:166-178: NaN -> NaN, +-inf -> +-1, both zeros -> 0
    s = E.ext_sign(np.array([0.0, -0.0, np.nan, np.inf, -np.inf, -2.0]))
    assert s[0] == 0 and s[1] == 0 and np.isnan(s[2]) and s[3:].tolist() == [1.0, -1.0, -1.0]
    assert E.ext_sign(np.array([0, 5], dtype=np.uint8)).tolist() == [0, 1]
    assert E.ext_sign(np.array([-128, 0, 9], dtype=np.int8)).tolist() == [-1, 0, 1]


def test_signbit_is_is_positive():
    # auto_impl/op_binary_common.rs:97 writes b.is_positive()
    assert E.signbit_is_positive(np.array([0.0, -0.0, 1.0, -np.inf, np.nan])).tolist() == \
        [True, False, True, False, True]
    assert E.signbit_is_positive(np.array([-1, 0, 1])).tolist() == [False, False, True]


def test_floor_divide():
    assert E.floor_divide(np.array([7, -7, 7, -7], np.int32), np.array([2, 2, -2, -2], np.int32)).tolist() == \
        [3, -4, -4, 3]
    assert E.floor_divide(np.array([-7.0]), np.array([2.0])).tolist() == [-4.0]


def test_isclose_is_asymmetric_and_keeps_inf_unequal():
    # rstsr-dtype-traits/src/isclose.rs:92-105: |a - b| <= atol + rtol |b|; inf - inf is NaN
    assert E.isclose(np.array([1.0]), np.array([1.0 + 1e-6]), 1e-6, 0.0).tolist() == [True]
    assert E.isclose(np.array([np.inf]), np.array([np.inf])).tolist() == [False]
    assert E.isclose(np.array([np.nan]), np.array([np.nan]), equal_nan=True).tolist() == [True]
