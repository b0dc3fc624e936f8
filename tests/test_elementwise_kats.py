"""The element-wise oracle reproduces the reference's own element-wise
known-answer tests (CPU only).

The fixture tests/golden/elementwise_kats.json holds the cases of
rstsr-core/tests/core_func/operators/test_comparison.rs and
rstsr-core/tests/core_func/math/test_unary_math.rs. The oracle is
oracle/elementwise.py where the reference's closures differ from numpy (sign)
and numpy elsewhere: the functions the GPU tests compare the device with.
"""

import json
from pathlib import Path

import numpy as np
import pytest

from oracle import elementwise as E

CASES = json.loads((Path(__file__).resolve().parent / "golden" / "elementwise_kats.json").read_text())
DTYPES = {"f64": np.float64, "i32": np.int32, "u8": np.uint8}

ORACLE = {
    "gt": np.greater, "ge": np.greater_equal, "lt": np.less, "le": np.less_equal, "eq": np.equal,
    "ne": np.not_equal, "maximum": np.maximum, "minimum": np.minimum,
    "abs": np.abs, "sqrt": np.sqrt, "sign": E.ext_sign, "floor": np.floor, "ceil": np.ceil, "trunc": np.trunc,
    "exp": np.exp, "log": np.log, "sin": np.sin, "cos": np.cos, "tanh": np.tanh,
    "isnan": np.isnan, "isfinite": np.isfinite, "isinf": np.isinf,
}


def decode(values, dtype=None):
    """JSON values with "nan" / "inf" / "-inf" / "-0.0" strings as an array."""
    out = [float(v) if isinstance(v, str) else v for v in values]
    return np.array(out, dtype=dtype)


def operands(case):
    dt = DTYPES[case["dtype"]]
    ops = [decode(case["a"], dt)]
    if "b" in case:
        ops.append(decode(case["b"], dt))
    return ops


def check(case, got):
    """The reference's own comparison: to_vec() equality ("exact"), values with the
    sign of zero and NaN-ness ("bits"), or rt::allclose(rtol 1e-5, atol 1e-8)."""
    got = np.asarray(got)
    want = decode(case["expect"])
    if case["cmp"] == "exact":
        assert got.tolist() == want.tolist(), (case["src"], got, want)
    elif case["cmp"] == "bits":
        nan = np.isnan(want)
        assert np.array_equal(np.isnan(got), nan), (case["src"], got)
        assert np.array_equal(got[~nan], want[~nan]), (case["src"], got)
        assert np.array_equal(np.signbit(got[~nan]), np.signbit(want[~nan])), (case["src"], got)
    else:
        assert np.allclose(got.astype(np.float64), want.astype(np.float64), rtol=1e-5, atol=1e-8), \
            (case["src"], got, want)


def test_fixture_covers_the_reference_files():
    srcs = {c["src"].split(":")[0] for c in CASES}
    assert srcs == {"rstsr-core/tests/core_func/operators/test_comparison.rs",
                    "rstsr-core/tests/core_func/math/test_unary_math.rs"}
    assert len(CASES) == 25
    assert {c["op"] for c in CASES} == set(ORACLE)


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['op']}-{c['dtype']}-{c['src'].split(':')[1]}")
def test_oracle_reproduces_reference_kat(case):
    with np.errstate(all="ignore"):
        check(case, ORACLE[case["op"]](*operands(case)))
