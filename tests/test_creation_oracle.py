"""Creation (arange / linspace / tril / triu) on the CPU: the oracle
(oracle/creation.py) reproduces the reference's own known-answer tests
(tests/golden/creation_kats.json), and the library's host-side arange length
(rstsr_cuda_arange_len) equals the oracle's on edge cases and a seeded sweep."""

import ctypes as C
import json
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import creation as OC

CASES = json.loads((Path(__file__).resolve().parent / "golden" / "creation_kats.json").read_text())
DT = {"f64": np.float64, "f32": np.float32, "i32": np.int32}


def arange_args(args):
    if len(args) == 1:
        return 0, args[0], 1
    if len(args) == 2:
        return args[0], args[1], 1
    return tuple(args)


def check_values(case, got):
    """The reference's comparison for each case kind."""
    got = np.asarray(got)
    if "expect" in case:
        assert got.tolist() == case["expect"], case["src"]
    if "expect_len" in case:
        assert len(got) == case["expect_len"], case["src"]
    if "last_close" in case:
        assert abs(float(got[-1]) - case["last_close"]) < 1e-9, case["src"]
    if "last_below" in case:
        assert float(got[-1]) < case["last_below"], case["src"]


def oracle_case(case):
    dt = DT[case["dtype"]]
    if case["op"] == "arange":
        return OC.arange(*arange_args(case["args"]), dt)
    if case["op"] == "linspace":
        start, stop, num = case["args"]
        return OC.linspace(start, stop, num, dt, endpoint=case["endpoint"])
    return OC.tri_mask(np.array(case["a"], dtype=dt), case["k"], case["op"] == "triu")


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['op']}-{c['src'].split(':')[1]}")
def test_oracle_reproduces_reference_kat(case):
    if "error" in case:
        with pytest.raises(ValueError):
            oracle_case(case)
        return
    check_values(case, oracle_case(case))


# ------------------------------------------------------- library arange length


def library_len(lib, start, stop, step, dtype):
    from rstsr_gb300 import _lib
    from rstsr_gb300.tensor import _scalar_bytes

    code = _lib.dtype_code(dtype)
    n = C.c_int64(-1)
    rc = lib.rstsr_cuda_arange_len(code, *(_scalar_bytes(v, code) for v in (start, stop, step)), C.byref(n))
    return rc, n.value


def expected(start, stop, step, dtype):
    """('len', n) | ('error', code): the library refuses what the reference
    cannot finish (repeated addition that wraps, runs away or stalls)."""
    try:
        r = OC.arange_len(start, stop, step, dtype, cap=4096)
    except ValueError:
        return ("error", 2)
    except OverflowError:
        return ("error", 3)
    if r is None:
        return ("error", 3)
    if r[0] == "accel":
        return ("len", r[1])
    got = r[1]
    if len(got) and np.dtype(dtype).kind in "iu":
        # refused where the repeated addition wraps, the step after the last
        # element included (the reference then stops on, or goes on with,
        # wrapped values)
        vals = [int(v) for v in got]
        info = np.iinfo(dtype)
        nxt = vals[-1] + int(step)
        if any(b <= a for a, b in zip(vals, vals[1:])) or not info.min <= nxt <= info.max:
            return ("error", 3)
    return ("len", len(got))


EDGE = [
    (0, 10, 3, np.int32), (10, 0, -2, np.int32), (0, 10, -1, np.int32), (5, 5, 1, np.int64), (5, 4, 1, np.int64),
    (-7, 7, 2, np.int64), (0, 1, 7, np.uint32), (3, 2, 1, np.uint32), (0, 100, 1, np.uint64),
    (2 ** 63, 2 ** 63 + 10, 3, np.uint64), (2 ** 64 - 10, 2 ** 64 - 1, 4, np.uint64),
    (2 ** 64 - 10, 2 ** 64 - 1, 8, np.uint64),
    (0, 100, 7, np.int8), (120, 127, 5, np.int8), (0, 5, -100, np.int8), (5, 0, -1, np.int8), (100, 127, 9, np.int8),
    (0, 255, 16, np.uint8), (250, 255, 2, np.uint8), (0, 1000, 333, np.int16), (65000, 65535, 500, np.uint16),
    (0.0, 1.0, 0.1, np.float64), (0.0, 1.0, 0.1, np.float32), (1.0, 0.0, -0.1, np.float64), (0.0, 1.0, -0.1, np.float64),
    (1.0, 0.0, 0.1, np.float64), (0.0, 0.3, 0.1, np.float64), (0.0, 0.3, 0.1, np.float32), (0.5, 0.5, 1.0, np.float64),
    (-1e300, 1e300, 1e-300, np.float64), (0.0, float("inf"), 1.0, np.float64), (float("-inf"), 0.0, 1.0, np.float64),
    (float("nan"), 1.0, 1.0, np.float64), (0.0, float("nan"), 1.0, np.float64), (0.0, 10.0, float("inf"), np.float64),
    (0.0, 1e-300, 1e-310, np.float64), (1e16, 1e16 + 8, 1.0, np.float64), (0.0, 0.0, 1.0, np.float32),
    (0, 10, 0, np.int32), (0.0, 1.0, 0.0, np.float64),
]


@pytest.mark.parametrize("start,stop,step,dtype", EDGE)
def test_library_arange_length_matches_oracle(built_lib, start, stop, step, dtype):
    kind, want = expected(start, stop, step, dtype)
    rc, n = library_len(built_lib, start, stop, step, dtype)
    if kind == "error":
        assert rc == want, (rc, n)
    else:
        assert rc == 0 and n == want, (rc, n, want)


def test_library_arange_length_sweep(built_lib):
    rng = np.random.default_rng(8)
    for _ in range(3000):
        dt = [np.float64, np.float32, np.int32, np.int64, np.uint32, np.int8, np.int16, np.uint8][rng.integers(8)]
        if dt in (np.float64, np.float32):
            start, stop = (float(v) for v in rng.uniform(-50, 50, 2))
            step = float(rng.choice([-1, 1]) * rng.uniform(0.01, 7))
        else:
            info = np.iinfo(dt)
            lo, hi = max(info.min, -3000), min(info.max, 3000)
            start, stop = (int(v) for v in rng.integers(lo, hi + 1, 2))
            step = int(rng.integers(1, min(300, info.max)))
            if info.min < 0 and rng.random() < 0.5:
                step = -step
        kind, want = expected(start, stop, step, dt)
        rc, n = library_len(built_lib, start, stop, step, dt)
        if kind == "error":
            assert rc == want, (start, stop, step, dt, rc, n)
        else:
            assert rc == 0 and n == want, (start, stop, step, dt, rc, n, want)


def test_library_refuses_what_it_does_not_provide(built_lib):
    from rstsr_gb300 import _lib

    assert library_len(built_lib, 0.0, 10.0, float("nan"), np.float64)[0] == 7
    n = C.c_int64()
    buf = (C.c_uint8 * 8)()
    assert built_lib.rstsr_cuda_arange_len(_lib.F16, buf, buf, buf, C.byref(n)) == 7
    assert built_lib.rstsr_cuda_arange_len(_lib.BOOL, buf, buf, buf, C.byref(n)) == 7
    assert built_lib.rstsr_cuda_arange_len(99, buf, buf, buf, C.byref(n)) == 2


def test_oracle_linspace_and_tri_edges():
    assert OC.linspace(0.0, 1.0, 0, np.float64).tolist() == []
    assert OC.linspace(3.0, 9.0, 1, np.float32).tolist() == [3.0]
    x = np.arange(24).reshape(2, 3, 4)
    assert (OC.tri_mask(x, 0, False) == np.tril(x)).all() and (OC.tri_mask(x, 2, True) == np.triu(x, 2)).all()
    assert (OC.tri_mask(x, 10, True) == 0).all() and (OC.tri_mask(x, -10, False) == 0).all()
    assert math.isclose(float(OC.linspace(0.0, 1.0, 11, np.float64)[3]), 0.3)


def test_oracle_tri_mask_matches_numpy():
    """numpy's tril / triu mask the last two axes with the same k convention: an
    independent check of the oracle's masks on random shapes and offsets."""
    rng = np.random.default_rng(12)
    for _ in range(300):
        nd = int(rng.integers(2, 5))
        shape = tuple(int(v) for v in rng.integers(0, 6, nd))
        x = rng.integers(1, 9, shape)
        k = int(rng.integers(-7, 8))
        np.testing.assert_array_equal(OC.tri_mask(x, k, False), np.tril(x, k))
        np.testing.assert_array_equal(OC.tri_mask(x, k, True), np.triu(x, k))
