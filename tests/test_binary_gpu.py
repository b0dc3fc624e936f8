"""Binary operators with broadcasting, in-place forms, scalars, unary ops and
the fused a*b+c on the GPU against the oracle (bit-exact values and layouts)."""

import numpy as np
import pytest

import rstsr_gb300 as rt
from oracle import layout as OL
from oracle import oracle as O
from tests.helpers import NP, rand, strided_case, values

pytestmark = pytest.mark.gpu

KINDS = ["c", "f", "perm", "slice", "flip"]


def up(dev, buf, shape, stride, off):
    return rt.from_host_layout(buf, shape, stride, off, dev)


def oracle_binary(op, a_case, b_case):
    (abuf, ash, ast, aoff), (bbuf, bsh, bst, boff) = a_case, b_case
    la, lb = OL.broadcast_layout((ash, ast, aoff), (bsh, bst, boff))
    lc = OL.layout_for_binary_op(la, lb)
    c = O.empty_strided(lc[0], lc[1], abuf.dtype)
    O.binary(op, c, O.Strided(abuf, *la), O.Strided(bbuf, *lb))
    return c, lc


@pytest.mark.parametrize("op", ["add", "sub", "mul", "div"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int64])
@pytest.mark.parametrize("kind", KINDS)
def test_binary_same_layout(dev, op, dtype, kind):
    a_case = strided_case(kind, (3, 8, 5, 34), dtype, seed=1)
    b_case = strided_case(kind, (3, 8, 5, 34), dtype, seed=2)
    if op == "div" and np.dtype(dtype).kind == "i":
        b_case[0][b_case[0] == 0] = 7
    want, lc = oracle_binary(op, a_case, b_case)
    got = rt.binary(op, up(dev, *a_case), up(dev, *b_case))
    assert (got.shape, got.stride) == (lc[0], lc[1])
    np.testing.assert_array_equal(got.to_numpy(), want.values())


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32])
@pytest.mark.parametrize("kind", KINDS)
def test_binary_broadcast_workload_shape(dev, dtype, kind):
    """a (4 layouts) * c[1,64,1,128]-style broadcast operand, reduced sizes."""
    a_case = strided_case(kind, (2, 16, 3, 32), dtype, seed=3)
    cb = rand((1, 16, 1, 32), dtype, seed=4).ravel()
    c_case = (cb, (1, 16, 1, 32), OL.c_stride((1, 16, 1, 32)), 0)
    for op in ("add", "mul"):
        want, lc = oracle_binary(op, a_case, c_case)
        got = rt.binary(op, up(dev, *a_case), up(dev, *c_case))
        assert (got.shape, got.stride) == (lc[0], lc[1])
        np.testing.assert_array_equal(got.to_numpy(), want.values())


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int64])
@pytest.mark.parametrize("kind", KINDS)
def test_fma_matches_two_pass_reference(dev, dtype, kind):
    """d = a*b + c (c broadcast [1,n1,1,n3]) equals the reference's two passes
    bit for bit, in the layout `&a * &b` gives."""
    a_case = strided_case(kind, (3, 8, 5, 34), dtype, seed=5)
    b_case = strided_case(kind, (3, 8, 5, 34), dtype, seed=6)
    cb = rand((1, 8, 1, 34), dtype, seed=7).ravel()
    ab, lab = oracle_binary("mul", a_case, b_case)
    lcb, _ = OL.broadcast_layout(((1, 8, 1, 34), OL.c_stride((1, 8, 1, 34)), 0), (lab[0], lab[1], 0))
    d = O.empty_strided(lab[0], lab[1], np.dtype(dtype))
    O.fma(d, O.Strided(a_case[0], *OL.broadcast_layout(a_case[1:], b_case[1:])[0]),
          O.Strided(b_case[0], *OL.broadcast_layout(a_case[1:], b_case[1:])[1]), O.Strided(cb, *lcb))
    # same as the two-pass oracle
    two = O.empty_strided(lab[0], lab[1], np.dtype(dtype))
    O.binary("add", two, ab, O.Strided(cb, *lcb))
    np.testing.assert_array_equal(d.values(), two.values())
    c_dev = rt.asarray(cb.reshape(1, 8, 1, 34), dev)
    got = rt.fma(up(dev, *a_case), up(dev, *b_case), c_dev)
    assert (got.shape, got.stride) == (lab[0], lab[1])
    np.testing.assert_array_equal(got.to_numpy(), d.values())


def test_inplace_and_consuming(dev):
    x = rand((6, 40), np.float64, seed=8)
    y = rand((40,), np.float64, seed=9)
    a = rt.asarray(x, dev)
    b = rt.asarray(y, dev)
    a += b
    np.testing.assert_array_equal(a.to_numpy(), x + y)
    a -= b
    np.testing.assert_array_equal(a.to_numpy(), (x + y) - y)
    # RConsume: a = b (op) a
    a2 = rt.asarray(x, dev)
    rt.binary_inplace("sub", a2, b, reversed_=True)
    np.testing.assert_array_equal(a2.to_numpy(), y - x)


def test_scalar_operands(dev):
    x = rand((5, 33), np.float32, seed=10)
    a = rt.asarray(x, dev)
    np.testing.assert_array_equal((a * 3.0).to_numpy(), x * np.float32(3.0))
    np.testing.assert_array_equal((2.0 - a).to_numpy(), np.float32(2.0) - x)
    xi = rand((7, 9), np.int32, seed=11)
    ai = rt.asarray(xi, dev)
    np.testing.assert_array_equal((ai + 5).to_numpy(), xi + 5)
    np.testing.assert_array_equal((ai << 3).to_numpy(), xi << 3)


def test_integer_wrapping_and_division_rules(dev):
    big = np.array([2**31 - 1, -(2**31), 7, -7, 0], dtype=np.int32)
    one = np.array([1, -1, 2, -2, 0], dtype=np.int32)
    a, b = rt.asarray(big, dev), rt.asarray(one, dev)
    assert (a + b).to_numpy().tolist() == [-(2**31), 2**31 - 1, 9, -9, 0]
    # division truncates; x / -1 wraps; x / 0 is defined as 0 here (Rust panics)
    assert rt.binary("div", a, b).to_numpy().tolist() == [2**31 - 1, -(2**31), 3, 3, 0]
    assert rt.binary("rem", a, b).to_numpy().tolist() == [0, 0, 1, -1, 0]


@pytest.mark.parametrize("op", ["neg", "abs", "sqrt", "exp", "square", "floor", "sign", "recip"])
def test_unary_float(dev, op):
    x = rand((4, 50), np.float64, seed=12) * 3
    if op == "sqrt":
        x = np.abs(x)
    a = rt.asarray(x, dev)
    got = rt.unary(op, a).to_numpy()
    ref = {"neg": -x, "abs": np.abs(x), "sqrt": np.sqrt(x), "exp": np.exp(x), "square": x * x,
           "floor": np.floor(x), "sign": np.sign(x), "recip": 1.0 / x}[op]
    if op == "exp":
        np.testing.assert_allclose(got, ref, rtol=2e-16 * 4)
    else:
        np.testing.assert_array_equal(got, ref)


def test_unary_int_and_bool(dev):
    xi = np.array([-3, 0, 5, -(2**31)], dtype=np.int32)
    a = rt.asarray(xi, dev)
    assert (-a).to_numpy().tolist() == [3, 0, -5, -(2**31)]
    assert (~a).to_numpy().tolist() == (~xi).tolist()
    xb = np.array([True, False, True])
    assert (~rt.asarray(xb, dev)).to_numpy().tolist() == [False, True, False]


def test_kat_arithmetic(dev, kats):
    for case in kats:
        if case["op"] not in ("add", "sub", "mul", "div", "rem"):
            continue
        dt = NP[case["dtype"]]
        a = rt.asarray(np.array(case["a"], dtype=dt), dev)
        b = rt.asarray(np.array(case["b"], dtype=dt), dev)
        got = a.rem(b) if case["op"] == "rem" else rt.binary(case["op"], a, b)
        assert got.to_numpy().tolist() == case["expect"], case["src"]


def test_broadcast_error_and_dtype_mismatch(dev):
    a = rt.asarray(np.zeros((3, 4)), dev)
    b = rt.asarray(np.zeros((5,)), dev)
    with pytest.raises(rt.RstsrError):
        a + b
    c = rt.asarray(np.zeros((3, 4), np.float32), dev)
    with pytest.raises(rt.RstsrError):
        a + c
