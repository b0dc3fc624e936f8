"""Pins the oracle's pack_tri / unpack_tri / index_select against the
reference's own unit tests (tests/golden/tri_index_kats.json), plus property
checks of the restatement (CPU only)."""

import json
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

CASES = json.loads((Path(__file__).resolve().parent / "golden" / "tri_index_kats.json").read_text())


def fingerprint(x: np.ndarray, order: str) -> float:
    """rstsr-core/src/dev_utilities/mod.rs:48-68 (flattening in the device order)."""
    v = np.asarray(x, dtype=np.float64).ravel(order=order)
    return float(np.dot(v, np.cos(np.arange(v.size, dtype=np.float64))))


def strides(shape, kind):
    return O.c_strides(shape) if kind in ("c", "C") else O.f_strides(shape)


def _slice(arr, spec):
    return arr[tuple(slice(None) if s is None else s for s in spec)]


def oracle_index_select(arr_buf, shape, st, axis, indices):
    idx = [i + shape[axis] if i < 0 else i for i in indices]
    src = O.Strided(arr_buf, shape, st)
    oshape = list(shape)
    oshape[axis] = len(idx)
    out = O.empty_strided(oshape, O.c_strides(oshape), arr_buf.dtype)
    O.index_select(out, src, axis, idx)
    return out.values()


@pytest.mark.parametrize("case", CASES, ids=[f"{c['op']}-{i}" for i, c in enumerate(CASES)])
def test_oracle_matches_reference_tri_index_kat(case):
    op = case["op"]
    if op == "pack_unpack":
        order = 0 if case["order"] == "C" else 1
        shape = case["shape"]
        buf = np.arange(48.0)
        src = O.Strided(buf, shape, strides(shape, case["layout"]))
        n = shape[-1] if order == 0 else shape[0]
        ntp = n * (n + 1) // 2
        pshape = shape[:-2] + [ntp] if order == 0 else [ntp] + shape[2:]
        dst = O.empty_strided(pshape, strides(pshape, case["layout"]), np.float64)
        O.pack_tri(dst, src, case["uplo"] == "L", order)
        assert _slice(dst.values(), case["packed_slice"]).tolist() == case["expect_packed"], case["src"]
        mat = O.empty_strided(shape, strides(shape, case["layout"]), np.float64)
        O.unpack_tri(mat, dst, case["uplo"] == "L", case["symm"], order)
        assert _slice(mat.values(), case["unpacked_slice"]).tolist() == case["expect_unpacked"], case["src"]
    elif op == "pack_tril_c_vs_f":
        base = np.arange(16.0).reshape(4, 4)
        for kind in ("c", "f"):
            src = O.Strided(base.ravel(order=kind.upper()), [4, 4], strides([4, 4], kind))
            dst = O.empty_strided([10], [1], np.float64)
            O.pack_tri(dst, src, True, 0)
            assert dst.values().tolist() == case["expect_packed"], case["src"]
    elif op == "index_select_fingerprint":
        lo, hi, num = case["linspace"]
        lin = np.linspace(lo, hi, int(num))
        order = case["order"]
        shape = case["shape"]
        a = lin.reshape(shape, order=order)
        got = oracle_index_select(a.ravel(), list(a.shape), O.c_strides(a.shape), case["axis"], case["indices"])
        assert abs(fingerprint(got, order) - case["expect"]) < case["tol"], case["src"]
    elif op == "index_select":
        a = np.array(case["a"], dtype={"f64": np.float64, "i32": np.int32}[case["dtype"]])
        got = oracle_index_select(a, [a.size], [1], case["axis"], case["indices"])
        assert got.tolist() == case["expect"], case["src"]
    else:
        raise AssertionError(op)


@pytest.mark.parametrize("n", [1, 2, 5, 33])
@pytest.mark.parametrize("lower", [True, False])
def test_oracle_pack_unpack_round_trip_and_symmetries(n, lower):
    rng = np.random.default_rng(n)
    m = rng.standard_normal((3, n, n))
    ntp = n * (n + 1) // 2
    src = O.Strided(m.ravel(), [3, n, n], O.c_strides([3, n, n]))
    packed = O.empty_strided([3, ntp], O.c_strides([3, ntp]), np.float64)
    O.pack_tri(packed, src, lower, 0)
    tri = np.tril(m) if lower else np.triu(m)
    for symm, want in [("Sy", tri + np.swapaxes(tri, 1, 2) - np.eye(n) * m),
                       ("He", tri + np.swapaxes(tri, 1, 2) - np.eye(n) * m),
                       ("Ay", tri - np.swapaxes(tri, 1, 2)),
                       ("Ah", tri - np.swapaxes(tri, 1, 2))]:
        out = O.empty_strided([3, n, n], O.c_strides([3, n, n]), np.float64)
        O.unpack_tri(out, packed, lower, symm, 0)
        np.testing.assert_array_equal(out.values(), want)
    out = O.empty_strided([3, n, n], O.c_strides([3, n, n]), np.float64)
    O.unpack_tri(out, packed, lower, "N", 0)
    np.testing.assert_array_equal(out.values(), tri)


def test_oracle_index_select_matches_numpy_take():
    rng = np.random.default_rng(7)
    a = rng.integers(-100, 100, (5, 7, 9)).astype(np.int64)
    for axis in range(3):
        idx = rng.integers(0, a.shape[axis], 11).tolist()
        got = oracle_index_select(a.ravel(), list(a.shape), O.c_strides(a.shape), axis, idx)
        np.testing.assert_array_equal(got, np.take(a, idx, axis=axis))
