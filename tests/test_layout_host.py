"""The library's C++ layout planner agrees with the oracle's independent
restatement and with the reference's layout unit tests (host-only, CPU)."""

import ctypes as C
import random

import pytest

from oracle import layout as OL


def L(shape, stride, offset=0):
    from rstsr_gb300._lib import Layout

    return Layout.make(shape, stride, offset)


def T(l):
    return (l.shape_t, l.stride_t, l.offset)


def random_layout(rng, ndim):
    shape = [rng.choice([1, 2, 3, 4, 5]) for _ in range(ndim)]
    perm = list(range(ndim))
    rng.shuffle(perm)
    base = OL.c_stride([shape[p] for p in perm])
    stride = [0] * ndim
    for i, p in enumerate(perm):
        stride[p] = base[i] * rng.choice([1, 1, 2])
    for i in range(ndim):
        if rng.random() < 0.15:
            stride[i] = 0
        if rng.random() < 0.15:
            stride[i] = -stride[i]
    off = sum(-s * (d - 1) for s, d in zip(stride, shape) if s < 0)
    return tuple(shape), tuple(stride), off


@pytest.mark.parametrize("seed", range(40))
def test_greedy_and_copy_layout_match_oracle(built_lib, seed):
    rng = random.Random(seed)
    shp, st, off = random_layout(rng, rng.randint(0, 6))
    for keep in (0, 1):
        out = L((), ())
        perm = (C.c_int32 * 8)()
        assert built_lib.rstsr_cuda_layout_greedy(C.byref(L(shp, st, off)), keep, C.byref(out), perm) == 0
        want, wperm = OL.greedy_layout((shp, st, off), bool(keep))
        assert T(out) == (tuple(want[0]), tuple(want[1]), want[2])
        assert list(perm)[: len(shp)] == wperm
    for order in (b"C", b"F", b"K"):
        out = L((), ())
        assert built_lib.rstsr_cuda_layout_for_array_copy(C.byref(L(shp, st, off)), order, C.byref(out)) == 0
        assert T(out) == OL.layout_for_array_copy((shp, st, off), order.decode())


@pytest.mark.parametrize("seed", range(40))
def test_binary_layouts_match_oracle(built_lib, seed):
    rng = random.Random(100 + seed)
    sa, ta, oa = random_layout(rng, rng.randint(1, 5))
    # b: a broadcast-compatible shape
    sb = tuple(d if rng.random() < 0.6 else 1 for d in sa[rng.randint(0, len(sa) - 1):])
    tb = OL.c_stride(sb) if rng.random() < 0.5 else OL.f_stride(sb)
    for order, oc in ((0, "C"), (1, "F")):
        if oc == "F":
            # col-major broadcasting aligns leading axes
            sb_o = tuple(d if rng.random() < 0.6 else 1 for d in sa[: len(sb)])
            tb_o = OL.f_stride(sb_o)
        else:
            sb_o, tb_o = sb, tb
        oa_l, ob_l = L((), ()), L((), ())
        rc = built_lib.rstsr_cuda_layout_broadcast(C.byref(L(sa, ta, oa)), C.byref(L(sb_o, tb_o)), order,
                                                   C.byref(oa_l), C.byref(ob_l))
        assert rc == 0
        wa, wb = OL.broadcast_layout((sa, ta, oa), (sb_o, tb_o, 0), oc)
        assert T(oa_l) == wa and T(ob_l) == wb
        lc = L((), ())
        assert built_lib.rstsr_cuda_layout_binary_op(C.byref(oa_l), C.byref(ob_l), order, C.byref(lc)) == 0
        assert T(lc) == OL.layout_for_binary_op(wa, wb, oc)


@pytest.mark.parametrize("seed", range(30))
def test_reduce_output_layout_matches_oracle(built_lib, seed):
    rng = random.Random(200 + seed)
    shp, st, off = random_layout(rng, rng.randint(1, 6))
    axes = sorted(rng.sample(range(len(shp)), rng.randint(1, len(shp))))
    if rng.random() < 0.5:
        axes = [a - len(shp) for a in axes]
    ax = (C.c_int64 * 8)(*axes)
    out = L((), ())
    assert built_lib.rstsr_cuda_reduce_axes_layout(C.byref(L(shp, st, off)), ax, len(axes), C.byref(out)) == 0
    assert T(out) == OL.reduce_output_layout((shp, st, off), axes)


@pytest.mark.parametrize("sa,sb", [((5,), (5,)), ((3, 5), (5, 4)), ((5,), (2, 5, 4)), ((2, 3, 5), (5,)),
                                   ((3, 5), (2, 5, 4)), ((2, 3, 5), (5, 4)), ((2, 1, 3, 5), (4, 5, 6)),
                                   ((64, 1, 8, 16), (1, 32, 16, 8))])
def test_matmul_layout_matches_oracle(built_lib, sa, sb):
    for order, oc in ((0, "C"), (1, "F")):
        # col-major matmul contracts the leading axes: the row-major pair
        # (A, B) corresponds to the col-major pair (B reversed, A reversed)
        a_shape, b_shape = (sa, sb) if oc == "C" else (tuple(reversed(sb)), tuple(reversed(sa)))
        lc = L((), ())
        la = L(a_shape, OL.c_stride(a_shape))
        lb = L(b_shape, OL.c_stride(b_shape))
        rc = built_lib.rstsr_cuda_matmul_layout(C.byref(la), C.byref(lb), order, C.byref(lc))
        assert rc == 0
        want = OL.matmul_shape(a_shape, b_shape, oc)
        assert lc.shape_t == want
        assert lc.stride_t == (OL.c_stride(want) if oc == "C" else OL.f_stride(want))


def test_reference_greedy_kats(built_lib, kats):
    for case in kats:
        if case["op"] != "greedy_layout":
            continue
        out = L((), ())
        perm = (C.c_int32 * 8)()
        assert built_lib.rstsr_cuda_layout_greedy(C.byref(L(case["shape"], case["stride"])), int(case["keep_shape"]),
                                                  C.byref(out), perm) == 0
        assert list(out.shape_t) == case["expect"]["shape"], case["src"]
        assert list(out.stride_t) == case["expect"]["stride"], case["src"]


def test_contiguity_flags(built_lib):
    assert built_lib.rstsr_cuda_layout_flags(C.byref(L((2, 3), (3, 1)))) & 1
    assert built_lib.rstsr_cuda_layout_flags(C.byref(L((2, 3), (1, 2)))) & 2
    assert built_lib.rstsr_cuda_layout_flags(C.byref(L((2, 3), (6, 2)))) & 3 == 0


def test_reduce_output_dtypes_follow_reference(built_lib):
    """Element type of each reduction's result: T for sum/min/max/prod, T (real) for
    mean/var/std/l2_norm on float types, usize for count_nonzero and for the sum of a
    bool array, bool for all/any on bool arrays (the TOut of
    rstsr-core/src/feature_rayon/auto_impl/reduction.rs:7-716); undefined pairs are
    InvalidValue errors."""
    from rstsr_gb300._lib import RED

    F64, F32, F16, BF16, I8, I16, I32, I64, U8, U16, U32, U64, BOOL = range(13)
    floats = (F64, F32, F16, BF16)
    ints = (I8, I16, I32, I64, U8, U16, U32, U64)

    def out(op, t):
        r = C.c_int(-1)
        rc = built_lib.rstsr_cuda_reduce_out_dtype(RED[op], t, C.byref(r))
        return r.value if rc == 0 else ("err", rc)

    for t in floats + ints:
        for op in ("sum", "min", "max", "prod"):
            assert out(op, t) == t, (op, t)
        assert out("count_nonzero", t) == U64
        assert out("all", t) == ("err", 2) and out("any", t) == ("err", 2)
    for t in floats:
        for op in ("mean", "var", "std", "l2_norm"):
            assert out(op, t) == t, (op, t)
    for t in ints:
        for op in ("mean", "var", "std", "l2_norm"):
            assert out(op, t) == ("err", 2), (op, t)
    assert out("sum", BOOL) == U64
    assert out("count_nonzero", BOOL) == U64
    assert out("all", BOOL) == BOOL and out("any", BOOL) == BOOL
    for op in ("min", "max", "prod", "mean"):
        assert out(op, BOOL) == ("err", 2), op
    assert out("sum", 99) == ("err", 2)


def test_unravel_index_matches_reference_and_numpy(built_lib):
    """unravel_index_c / unravel_index_f (rstsr-common/src/layout/layoutbase.rs:988-996:
    shape [3, 2, 6], flat 16 -> [1, 0, 4] in C order, [1, 1, 2] in F order), then a
    sweep against numpy.unravel_index; an index outside the shape is refused."""
    import numpy as np

    import rstsr_gb300 as rt

    assert rt.unravel_index((3, 2, 6), 0, "C") == (0, 0, 0)
    assert rt.unravel_index((3, 2, 6), 16, "C") == (1, 0, 4)
    assert rt.unravel_index((3, 2, 6), 0, "F") == (0, 0, 0)
    assert rt.unravel_index((3, 2, 6), 16, "F") == (1, 1, 2)
    assert rt.unravel_index((), 0, "C") == ()
    rng = random.Random(4)
    for _ in range(300):
        shape = tuple(rng.randint(1, 6) for _ in range(rng.randint(1, 5)))
        idx = rng.randrange(int(np.prod(shape)))
        for order in ("C", "F"):
            want = tuple(int(v) for v in np.unravel_index(idx, shape, order=order))
            assert rt.unravel_index(shape, idx, order) == want
    with pytest.raises(rt.RstsrError) as err:
        rt.unravel_index((3, 2), 6, "C")
    assert err.value.kind == "ValueOutOfRange"
