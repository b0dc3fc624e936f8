"""Pins the CPU oracle against the reference's own known-answer tests (CPU only)."""

import numpy as np
import pytest

from oracle import layout as OL
from oracle import oracle as O
from tests.helpers import NP, strided_case, values


def _red(case, op, arr, axes):
    a = O.Strided(arr.ravel(), arr.shape, OL.c_stride(arr.shape), 0)
    axes = [x + arr.ndim if x < 0 else x for x in axes]
    oshape, ostride, _ = OL.reduce_output_layout((arr.shape, OL.c_stride(arr.shape), 0), axes)
    out_dt = np.uint64 if op in ("count_nonzero",) or (op == "sum" and arr.dtype == np.bool_) else arr.dtype
    out = O.empty_strided(oshape, ostride, out_dt)
    O.reduce_axes(op, a, axes, out)
    return out.values()


def _arg(is_max, arr, axes):
    a = O.Strided(arr.ravel(), arr.shape, OL.c_stride(arr.shape), 0)
    oshape, ostride, _ = OL.reduce_output_layout((arr.shape, OL.c_stride(arr.shape), 0), axes)
    out = O.empty_strided(oshape, ostride, np.uint64)
    O.argreduce_axes(is_max, a, axes, out)
    return out.values()


def _arr(case):
    arr = np.array(case["a"], dtype=NP[case["dtype"]])
    if "shape" in case:
        arr = arr.reshape(case["shape"])
    return arr


def test_kat_count(kats):
    assert len(kats) >= 60


@pytest.mark.parametrize("idx", range(68))
def test_oracle_matches_reference_kat(kats, idx):
    case = kats[idx]
    op = case["op"]
    if op.endswith("_all") and op.startswith("arg"):
        arr = _arr(case)
        got = _arg(op == "argmax_all", arr.ravel(), [0])
        assert int(got) == case["expect"], case["src"]
    elif op.endswith("_axes") and op.startswith("arg"):
        arr = _arr(case)
        got = _arg(op == "argmax_axes", arr, case["axes"])
        assert got.tolist() == case["expect"], case["src"]
    elif op.endswith("_all"):
        arr = _arr(case)
        red = op[: -len("_all")]
        got = _red(case, red, arr, list(range(arr.ndim)))
        np.testing.assert_allclose(np.asarray(got, dtype=np.float64), case["expect"], rtol=1e-12, err_msg=case["src"])
    elif op.endswith("_axes"):
        arr = _arr(case)
        red = op[: -len("_axes")]
        got = _red(case, red, arr, case["axes"])
        np.testing.assert_allclose(np.asarray(got, dtype=np.float64), case["expect"], rtol=1e-12, err_msg=case["src"])
    elif op == "to_contig":
        arr = _arr(case)
        shape, stride, off = arr.shape, OL.c_stride(arr.shape), 0
        v = case["view"]
        if "transpose" in v:
            shape = tuple(shape[i] for i in v["transpose"])
            stride = tuple(stride[i] for i in v["transpose"])
        if "slice" in v:
            shape = tuple((d + 1) // 2 for d in shape)
            stride = tuple(s * 2 for s in stride)
            assert list(stride) == case["view_stride"]
        if "flip" in v:
            ax = v["flip"]
            off += stride[ax] * (shape[ax] - 1)
            stride = tuple(-s if i == ax else s for i, s in enumerate(stride))
        src = O.Strided(arr.ravel(), shape, stride, off)
        dst = O.empty_strided(shape, OL.c_stride(shape), arr.dtype)
        O.assign_arbitrary(dst, src, 0)
        assert dst.values().tolist() == case["expect"], case["src"]
    elif op in ("add", "sub", "mul", "div"):
        a = np.array(case["a"], dtype=NP[case["dtype"]])
        b = np.array(case["b"], dtype=NP[case["dtype"]])
        la, lb = OL.broadcast_layout((a.shape, OL.c_stride(a.shape), 0), (b.shape, OL.c_stride(b.shape), 0))
        lc = OL.layout_for_binary_op(la, lb)
        c = O.empty_strided(lc[0], lc[1], a.dtype)
        O.binary(op, c, O.Strided(a.ravel(), *la), O.Strided(b.ravel(), *lb))
        assert c.values().tolist() == case["expect"], case["src"]
    elif op == "rem":
        a = np.array(case["a"], dtype=np.int64)
        b = np.array(case["b"], dtype=np.int64)
        assert np.fmod(a, b).tolist() == case["expect"]
    elif op == "matmul":
        a = np.array(case["a"], dtype=np.int64)
        b = np.array(case["b"], dtype=np.int64)
        assert OL.matmul_shape(a.shape, b.shape) == np.array(case["expect"]).shape
        assert np.matmul(a, b).tolist() == case["expect"], case["src"]
    elif op == "matmul_from":
        a = np.array(case["a"]).reshape(case["shape_a"])
        b = np.array(case["b"]).reshape(case["shape_b"])
        c = np.array(case["c"]).reshape(case["shape_c"])
        got = case["alpha"] * (a @ b) + case["beta"] * c
        np.testing.assert_allclose(got.ravel(), case["expect"], rtol=1e-14)
    elif op == "batched_linspace_stats":
        n = case["n"]
        a = np.linspace(*case["a_range"], n).reshape(case["shape"])
        b = np.linspace(*case["b_range"], n).reshape(case["shape"])
        c = a @ b
        assert abs(c.mean() - case["expect"]["mean_all"]) < case["tol"]
        assert abs(c.std() - case["expect"]["std_all"]) < case["tol"]
    elif op == "greedy_layout":
        (shape, stride, _), _ = OL.greedy_layout((tuple(case["shape"]), tuple(case["stride"]), 0), case["keep_shape"])
        assert list(shape) == case["expect"]["shape"]
        assert list(stride) == case["expect"]["stride"]
    else:
        pytest.fail(f"unhandled KAT op {op}")


@pytest.mark.parametrize("kind", ["c", "f", "perm", "slice", "slice2", "flip"])
def test_oracle_assign_matches_numpy(kind):
    buf, shape, stride, off = strided_case(kind, (3, 4, 5, 6), np.float64, seed=1)
    want = values(buf, shape, stride, off)
    dst = O.empty_strided(shape, OL.c_stride(shape), np.float64)
    O.assign(dst, O.Strided(buf, shape, stride, off))
    np.testing.assert_array_equal(dst.values(), want)
    dst2 = O.empty_strided(shape, OL.f_stride(shape), np.float64)
    O.assign(dst2, O.Strided(buf, shape, stride, off), nthreads=4)
    np.testing.assert_array_equal(dst2.values(), want)


def test_oracle_reductions_match_numpy():
    buf, shape, stride, off = strided_case("perm", (4, 5, 6, 7), np.float64, seed=2)
    x = values(buf, shape, stride, off)
    a = O.Strided(buf, shape, stride, off)
    for op, fn in [("sum", np.sum), ("max", np.max), ("min", np.min), ("mean", np.mean), ("var", np.var),
                   ("std", np.std)]:
        oshape, ostride, _ = OL.reduce_output_layout((shape, stride, off), [1, 3])
        out = O.empty_strided(oshape, ostride, np.float64)
        O.reduce_axes(op, a, [1, 3], out, nthreads=3)
        np.testing.assert_allclose(out.values(), fn(x, axis=(1, 3)), rtol=1e-12, err_msg=op)
    oshape, ostride, _ = OL.reduce_output_layout((shape, stride, off), [3])
    out = O.empty_strided(oshape, ostride, np.uint64)
    O.argreduce_axes(True, a, [3], out)
    np.testing.assert_array_equal(out.values(), np.argmax(x, axis=3))


def test_oracle_argmax_nan_rule():
    # serial fold: a NaN first element is kept, later NaNs are skipped
    x = np.array([[np.nan, 1.0, 5.0], [1.0, np.nan, 5.0], [2.0, 7.0, np.nan]])
    a = O.Strided(x.ravel(), x.shape, OL.c_stride(x.shape), 0)
    out = O.empty_strided((3,), (1,), np.uint64)
    O.argreduce_axes(True, a, [1], out)
    assert out.values().tolist() == [0, 2, 1]


def test_oracle_fma_two_roundings():
    rng = np.random.default_rng(3)
    a, b, c = (rng.standard_normal(1000) for _ in range(3))
    d = O.empty_strided((1000,), (1,), np.float64)
    O.fma(d, *(O.Strided(x, (1000,), (1,), 0) for x in (a, b, c)))
    np.testing.assert_array_equal(d.values(), (a * b) + c)
