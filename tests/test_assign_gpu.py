"""assign / assign_arbitrary / to_contig / fill on the GPU against the oracle (bit-exact)."""

import numpy as np
import pytest

import rstsr_gb300 as rt
from oracle import layout as OL
from oracle import oracle as O
from tests.helpers import rand, strided_case, values

pytestmark = pytest.mark.gpu

KINDS = ["c", "f", "perm", "slice", "slice2", "flip"]
DTYPES = [np.float64, np.float32, np.int32, np.int64, np.float16, np.int8, np.bool_]


def up(dev, buf, shape, stride, off):
    return rt.from_host_layout(buf, shape, stride, off, dev)


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("order", ["C", "F"])
def test_to_contig_matches_oracle(dev, kind, dtype, order):
    buf, shape, stride, off = strided_case(kind, (4, 6, 5, 33), dtype, seed=11)
    t = up(dev, buf, shape, stride, off)
    c = t.to_contig(order)
    if order == "C":
        assert c.c_contig()
    else:
        assert c.f_contig()
    want_st = OL.c_stride(shape) if order == "C" else OL.f_stride(shape)
    dst = O.empty_strided(shape, want_st, dtype)
    O.assign_arbitrary(dst, O.Strided(buf, shape, stride, off), 0)
    np.testing.assert_array_equal(c.to_numpy(), dst.values())


@pytest.mark.parametrize("shape,axes", [((32, 64, 128, 128), (0, 2, 1, 3)), ((64, 48), (1, 0)), ((7, 33, 65), (2, 0, 1)),
                                        ((3, 1, 130, 2), (2, 3, 0, 1)), ((300, 129), (1, 0))])
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int8])
def test_permute_to_contig_transpose_paths(dev, shape, axes, dtype):
    """Axis-permuted copies (the tile-transpose path) at sizes incl. the
    memory-bound workload's [32,64,128,128] permute(0,2,1,3)."""
    if np.prod(shape) > 1e6 and dtype != np.float64:
        shape = (8, 64, 128, 128)
    base = rand(shape, dtype, seed=5)
    for src_order in ("C", "F"):
        st = OL.c_stride(shape) if src_order == "C" else OL.f_stride(shape)
        flat = base.ravel(order=src_order)
        t = rt.from_host_layout(flat, shape, st, 0, dev).permute_dims(axes)
        got = t.to_contig("C").to_numpy()
        np.testing.assert_array_equal(got, np.transpose(base, axes))


@pytest.mark.parametrize("shape", [(16, 6, 50, 40), (32, 3, 70), (32, 64, 9, 130), (16, 2, 17, 64)])
@pytest.mark.parametrize("dtype", [np.float32, np.int32])
def test_transpose_folds_short_source_runs(dev, shape, dtype):
    """F-ordered 4-byte sources whose contiguous leading extent (16 or 32) is
    shorter than the 64-wide pair tile, copied to C order: the tile folds the
    next source dim into its columns (partial last column tiles included)."""
    base = rand(shape, dtype, seed=6)
    t = rt.from_host_layout(base.ravel(order="F"), shape, OL.f_stride(shape), 0, dev)
    np.testing.assert_array_equal(t.to_contig("C").to_numpy(), base)
    # the same through a permuted view, and from an offset (even) start
    perm = (1, 0) + tuple(range(2, len(shape)))
    np.testing.assert_array_equal(t.permute_dims(perm).to_contig("C").to_numpy(), np.transpose(base, perm))
    big = rand((shape[0] + 2,) + shape[1:], dtype, seed=7)
    tb = rt.from_host_layout(big.ravel(order="F"), big.shape, OL.f_stride(big.shape), 0, dev)
    v = tb.i((slice(2, None),))
    np.testing.assert_array_equal(v.to_contig("C").to_numpy(), big[2:])


def test_assign_same_shape_all_layout_pairs(dev):
    for ka in KINDS:
        for kc in ["c", "f", "flip"]:
            buf, shape, stride, off = strided_case(ka, (3, 5, 4, 9), np.float64, seed=3)
            cbuf, _, cst, coff = strided_case(kc, (3, 5, 4, 9), np.float64, seed=4)
            a = up(dev, buf, shape, stride, off)
            c = up(dev, cbuf, shape, cst, coff)
            rt.assign(c, a)
            np.testing.assert_array_equal(c.to_numpy(), values(buf, shape, stride, off))


def test_assign_arbitrary_reshape_walk(dev):
    """Different shapes, same size: elements correspond in C (or F) walk order
    (cpu_serial/assignment.rs:28-67)."""
    x = rand((4, 6, 10), np.int32, seed=7)
    src = up(dev, x.ravel(), (4, 6, 10), OL.c_stride((4, 6, 10)), 0).permute_dims(2, 0, 1)  # (10,4,6) strided
    for order, npord in ((rt.ROW_MAJOR, "C"), (rt.COL_MAJOR, "F")):
        dst = rt.empty((12, 20), np.int32, dev, order="F")
        from rstsr_gb300._lib import call
        import ctypes as C

        call("rstsr_cuda_assign_arbitrary", dev.ctx, C.c_void_p(dst.ptr), C.byref(dst.layout()), dst.dtype_code,
             C.c_void_p(src.ptr), C.byref(src.layout()), src.dtype_code, order)
        want = np.transpose(x, (2, 0, 1)).reshape((12, 20), order=npord)
        np.testing.assert_array_equal(dst.to_numpy(), want)


@pytest.mark.parametrize("src_dt,dst_dt", [(np.float64, np.float32), (np.float32, np.float64), (np.int32, np.float64),
                                           (np.float64, np.int32), (np.int64, np.int8), (np.float32, np.bool_),
                                           (np.bool_, np.float32), (np.int32, np.uint64)])
def test_assign_casts_like_rust_as(dev, src_dt, dst_dt):
    vals = np.array([0, 1, -1, 2.5, -2.5, 127.9, 300, -300, 1e10, -1e10], dtype=np.float64)
    if np.dtype(src_dt).kind == "b":
        x = np.array([True, False, True, True, False, False, True, False, True, True])
    else:
        with np.errstate(all="ignore"):
            x = vals.astype(src_dt) if np.dtype(src_dt).kind == "f" else np.clip(vals, -1000, 1000).astype(src_dt)
    a = rt.asarray(x, dev)
    c = rt.empty(x.shape, dst_dt, dev)
    rt.assign(c, a)
    got = c.to_numpy()
    dk = np.dtype(dst_dt)
    if dk.kind == "b":
        want = x != 0
    elif dk.kind in "iu" and np.dtype(src_dt).kind == "f":
        info = np.iinfo(dk)
        want = np.where(np.isnan(x), 0, np.clip(np.trunc(x.astype(np.float64)), info.min, info.max)).astype(dk)
    else:
        with np.errstate(all="ignore"):
            want = x.astype(dst_dt)
    np.testing.assert_array_equal(got, want)


def test_cast_nan_inf_saturation(dev):
    x = np.array([np.nan, np.inf, -np.inf, 3e9, -3e9, 0.5], dtype=np.float64)
    a = rt.asarray(x, dev)
    c = rt.empty(x.shape, np.int32, dev)
    rt.assign(c, a)
    assert c.to_numpy().tolist() == [0, 2147483647, -2147483648, 2147483647, -2147483648, 0]


@pytest.mark.parametrize("dtype", [np.float64, np.int32, np.uint8, np.float16])
def test_fill_and_zero_size(dev, dtype):
    t = rt.full((3, 7, 5), 3, dtype, dev)
    assert (t.to_numpy() == 3).all()
    z = rt.zeros((0, 5), dtype, dev)
    assert z.to_contig("C").shape == (0, 5)
    s = rt.asarray(np.array(42, dtype=dtype), dev)
    assert s.to_contig("F").to_scalar() == 42


def test_kat_to_contig(dev, kats):
    for case in kats:
        if case["op"] != "to_contig":
            continue
        arr = np.array(case["a"], dtype=np.int32).reshape(case["shape"])
        t = rt.asarray(arr, dev)
        v = case["view"]
        if "transpose" in v:
            t = t.permute_dims(v["transpose"])
        if "slice" in v:
            t = t.i((slice(None, None, 2), slice(None, None, 2)))
            assert list(t.stride) == case["view_stride"]
        if "flip" in v:
            t = t.flip(v["flip"])
        c = t.to_contig("C")
        assert c.c_contig() and c.stride[-1] == 1
        assert c.to_numpy().tolist() == case["expect"], case["src"]


def test_errors_are_reported(dev):
    a = rt.asarray(np.zeros((3, 4)), dev)
    b = rt.empty((4, 3), np.float64, dev)
    with pytest.raises(rt.RstsrError) as e:
        rt.assign(b, a)
    assert e.value.kind == "InvalidLayout"
