"""pack_tri / unpack_tri / index_select on the GPU against the oracle
(bit-exact: these ops move element bits) and the reference's own unit tests."""

import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

import rstsr_gb300 as rt
from oracle import oracle as O
from rstsr_gb300 import _lib
from rstsr_gb300._lib import RstsrError
from tests.helpers import rand

pytestmark = pytest.mark.gpu

CASES = json.loads((Path(__file__).resolve().parent / "golden" / "tri_index_kats.json").read_text())


def fingerprint(x: np.ndarray, order: str) -> float:
    v = np.asarray(x, dtype=np.float64).ravel(order=order)
    return float(np.dot(v, np.cos(np.arange(v.size, dtype=np.float64))))


def _slice(arr, spec):
    return arr[tuple(slice(None) if s is None else s for s in spec)]


def with_order(dev, order):
    dev.set_default_order(order)
    return dev


@pytest.fixture
def cdev(dev):
    yield dev
    dev.set_default_order("C")


@pytest.mark.parametrize("case", CASES, ids=[f"{c['op']}-{i}" for i, c in enumerate(CASES)])
def test_device_matches_reference_tri_index_kat(cdev, case):
    op = case["op"]
    dev = with_order(cdev, case.get("order", "C"))
    if op == "pack_unpack":
        shape = case["shape"]
        st = O.c_strides(shape) if case["layout"] == "c" else O.f_strides(shape)
        t = rt.from_host_layout(np.arange(48.0), shape, st, 0, dev)
        p = rt.pack_tri(t, case["uplo"])
        assert _slice(p.to_numpy(), case["packed_slice"]).tolist() == case["expect_packed"], case["src"]
        m = rt.unpack_tri(p, case["uplo"], case["symm"])
        assert _slice(m.to_numpy(), case["unpacked_slice"]).tolist() == case["expect_unpacked"], case["src"]
    elif op == "pack_tril_c_vs_f":
        t = rt.asarray(np.arange(16.0).reshape(4, 4), dev)
        assert t.pack_tril().to_vec() == case["expect_packed"]
        assert t.to_contig("F").pack_tril().to_vec() == case["expect_packed"]
    elif op == "index_select_fingerprint":
        lo, hi, num = case["linspace"]
        order = case["order"]
        a = np.linspace(lo, hi, int(num)).reshape(case["shape"], order=order)
        t = rt.from_host_layout(a.ravel(order=order), a.shape,
                                O.c_strides(a.shape) if order == "C" else O.f_strides(a.shape), 0, dev)
        b = rt.index_select(t, case["axis"], case["indices"])
        assert b.c_contig() if order == "C" else b.f_contig()
        assert abs(fingerprint(b.to_numpy(), order) - case["expect"]) < case["tol"], case["src"]
    elif op == "index_select":
        a = np.array(case["a"], dtype={"f64": np.float64, "i32": np.int32}[case["dtype"]])
        b = rt.index_select(rt.asarray(a, dev), case["axis"], case["indices"])
        assert b.to_vec() == case["expect"], case["src"]
    else:
        raise AssertionError(op)


# ------------------------------------------------------------------ pack_tri

MAT_KINDS = ["c", "f", "tr", "batch_slice", "flip"]


def matrix_case(kind, batch, n, dtype, seed):
    """Host buffer + layout of a (batch..., n, n) tensor in one of several
    layouts: C, F, matrix axes swapped, every other batch element, flipped."""
    shape = tuple(batch) + (n, n)
    if kind == "c":
        return rand(shape, dtype, seed).ravel(), shape, O.c_strides(shape), 0
    if kind == "f":
        return rand(shape, dtype, seed).ravel(), shape, O.f_strides(shape), 0
    if kind == "tr":
        st = list(O.c_strides(shape))
        st[-1], st[-2] = st[-2], st[-1]
        return rand(shape, dtype, seed).ravel(), shape, tuple(st), 0
    if kind == "batch_slice":
        if not batch:
            return matrix_case("c", batch, n, dtype, seed)
        base = (batch[0] * 2,) + tuple(batch[1:]) + (n, n)
        st = list(O.c_strides(base))
        st[0] *= 2
        return rand(base, dtype, seed).ravel(), shape, tuple(st), 0
    if kind == "flip":
        st = list(O.c_strides(shape))
        off = st[-1] * (n - 1) + st[-2] * (n - 1)
        st[-1], st[-2] = -st[-1], -st[-2]
        return rand(shape, dtype, seed).ravel(), shape, tuple(st), off
    raise ValueError(kind)


def oracle_pack(buf, shape, st, off, lower, order, out_shape, out_st):
    dst = O.empty_strided(out_shape, out_st, buf.dtype)
    O.pack_tri(dst, O.Strided(buf, shape, st, off), lower, order)
    return dst.values()


@pytest.mark.parametrize("kind", MAT_KINDS)
@pytest.mark.parametrize("n", [1, 2, 31, 33, 70])
@pytest.mark.parametrize("batch", [(), (3,), (2, 3)])
@pytest.mark.parametrize("uplo", ["L", "U"])
def test_pack_tri_matches_oracle(cdev, kind, n, batch, uplo):
    buf, shape, st, off = matrix_case(kind, batch, n, np.float64, seed=n + len(batch))
    t = rt.from_host_layout(buf, shape, st, off, cdev)
    p = rt.pack_tri(t, uplo)
    want = oracle_pack(buf, shape, st, off, uplo == "L", 0, p.shape, p.stride)
    np.testing.assert_array_equal(p.to_numpy(), want)


@pytest.mark.parametrize("dtype", [np.float32, np.float16, np.int8, np.int16, np.int32, np.int64, np.bool_, np.uint64])
@pytest.mark.parametrize("order", ["C", "F"])
def test_pack_tri_dtypes_and_orders(cdev, dtype, order):
    dev = with_order(cdev, order)
    for n in (45, 100):  # the shared-tile kernel and the row kernel
        shape = (4, n, n) if order == "C" else (n, n, 4)
        buf = rand(shape, dtype, seed=3).ravel()
        st = O.c_strides(shape)
        t = rt.from_host_layout(buf, shape, st, 0, dev)
        for uplo in ("L", "U"):
            p = rt.pack_tri(t, uplo)
            want = oracle_pack(buf, shape, st, 0, uplo == "L", 0 if order == "C" else 1, p.shape, p.stride)
            np.testing.assert_array_equal(p.to_numpy(), want)


def test_pack_tri_large_matches_numpy(cdev):
    """(6, 1500, 1500) f64: many tiles per matrix, both triangles."""
    m = rand((6, 1500, 1500), np.float64, seed=9)
    t = rt.asarray(m, cdev)
    il = np.tril_indices(1500)
    iu = np.triu_indices(1500)
    np.testing.assert_array_equal(rt.pack_tri(t, "L").to_numpy(), m[:, il[0], il[1]])
    np.testing.assert_array_equal(rt.pack_tri(t, "U").to_numpy(), m[:, iu[0], iu[1]])


# ---------------------------------------------------------------- unpack_tri

def packed_case(batch, n, dtype, seed, kind):
    ntp = n * (n + 1) // 2
    shape = tuple(batch) + (ntp,)
    if kind == "c":
        return rand(shape, dtype, seed).ravel(), shape, O.c_strides(shape), 0
    if kind == "f":
        return rand(shape, dtype, seed).ravel(), shape, O.f_strides(shape), 0
    base = tuple(batch) + (2 * ntp,)  # every other packed element
    st = list(O.c_strides(base))
    st[-1] = 2
    return rand(base, dtype, seed).ravel(), shape, tuple(st), 0


def bits(dtype):
    return np.uint16 if dtype == "bf16" else dtype


@pytest.mark.parametrize("symm", ["Sy", "He", "Ay", "Ah", "N"])
@pytest.mark.parametrize("n", [1, 2, 32, 33, 97])
@pytest.mark.parametrize("kind", ["c", "f", "step2"])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("out_order", ["C", "F"])
def test_unpack_tri_matches_oracle(cdev, symm, n, kind, uplo, out_order):
    batch = (3,)
    buf, shape, st, off = packed_case(batch, n, np.float64, seed=n, kind=kind)
    t = rt.from_host_layout(buf, shape, st, off, cdev)
    out = rt.empty(batch + (n, n), np.float64, cdev, order=out_order)
    rt.fill(out, 7.25)  # the N form must leave the other triangle as it was
    _lib.call("rstsr_cuda_unpack_tri", cdev.ctx, t.dtype_code, C.c_void_p(out.ptr), C.byref(out.layout()),
              C.c_void_p(t.ptr), C.byref(t.layout()), uplo.encode(), rt.tensor.SYMM[symm], 0)
    want = O.Strided(np.full(out.size, 7.25), out.shape, out.stride)
    O.unpack_tri(want, O.Strided(buf, shape, st, off), uplo == "L", symm, 0)
    np.testing.assert_array_equal(out.to_numpy(), want.values())


@pytest.mark.parametrize("dtype", [np.float32, np.float16, "bf16"])
@pytest.mark.parametrize("symm", ["Sy", "Ay", "N"])
@pytest.mark.parametrize("order", ["C", "F"])
def test_unpack_tri_float_widths(cdev, dtype, symm, order):
    dev = with_order(cdev, order)
    n = 40
    ntp = n * (n + 1) // 2
    shape = (5, ntp) if order == "C" else (ntp, 5)
    vals = rand(shape, np.float32, seed=2)
    if dtype == "bf16":
        hbuf = (vals.view(np.uint32) >> 16).astype(np.uint16).ravel()
    else:
        hbuf = vals.astype(dtype).ravel()
    t = rt.from_host_layout(hbuf, shape, O.c_strides(shape), 0, dev)
    if dtype == "bf16":
        t = rt.Tensor(t.storage, t.shape, t.stride, t.offset, _lib.BF16)
    m = rt.unpack_tri(t, "L", symm)
    want = O.Strided(np.zeros(m.size, dtype=bits(dtype)), m.shape, m.stride)
    O.unpack_tri(want, O.Strided(hbuf, shape, O.c_strides(shape)), True, symm, 0 if order == "C" else 1)
    got = m.to_numpy()
    np.testing.assert_array_equal(got.view(bits(dtype)) if dtype != "bf16" else got, want.values())


def test_unpack_tri_rejects_integers_and_bad_lengths(cdev):
    t = rt.asarray(np.arange(10, dtype=np.int32), cdev)
    with pytest.raises(RstsrError, match="float"):
        rt.unpack_tri(t, "L", "Sy")
    with pytest.raises(RstsrError, match="triangular"):
        rt.unpack_tri(rt.asarray(np.zeros(9), cdev), "L", "Sy")
    with pytest.raises(RstsrError, match="same"):
        rt.pack_tri(rt.asarray(np.zeros((3, 4)), cdev), "L")


def test_pack_unpack_round_trip_full_size(cdev):
    """Size-independent property at electronic-structure size: unpack(pack(S)) == S
    for a symmetric batch (40, 700, 700), and the anti-symmetric form."""
    rng = np.random.default_rng(5)
    m = rng.standard_normal((40, 700, 700))
    s = m + np.swapaxes(m, 1, 2)
    t = rt.asarray(s, cdev)
    back = rt.unpack_tri(rt.pack_tri(t, "L"), "L", "Sy").to_numpy()
    np.testing.assert_array_equal(back, s)
    a = m - np.swapaxes(m, 1, 2)
    back = rt.unpack_tri(rt.pack_tri(rt.asarray(a, cdev), "U"), "U", "Ay").to_numpy()
    np.testing.assert_array_equal(back, a)


# ------------------------------------------------------------- index_select

def isel_oracle(buf, shape, st, off, axis, idx, out_shape, out_st):
    nidx = [i + shape[axis] if i < 0 else i for i in idx]
    dst = O.empty_strided(out_shape, out_st, buf.dtype)
    O.index_select(dst, O.Strided(buf, shape, st, off), axis, nidx)
    return dst.values()


SEL_KINDS = ["c", "f", "perm", "slice", "flip"]


def sel_case(kind, shape, dtype, seed):
    from tests.helpers import strided_case

    if kind == "perm" and len(shape) < 3:
        kind = "c"
    return strided_case(kind, shape, dtype, seed=seed)


@pytest.mark.parametrize("kind", SEL_KINDS)
@pytest.mark.parametrize("axis", [0, 1, 2, -1])
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.float16, np.int8, np.int64, np.bool_])
def test_index_select_matches_oracle(cdev, kind, axis, dtype):
    shape = (9, 12, 34)
    buf, shape, st, off = sel_case(kind, shape, dtype, seed=4)
    t = rt.from_host_layout(buf, shape, st, off, cdev)
    ax = axis % 3
    rng = np.random.default_rng(ax)
    idx = rng.integers(-shape[ax], shape[ax], 17).tolist()
    b = rt.index_select(t, axis, idx)
    want = isel_oracle(buf, shape, st, off, ax, idx, b.shape, b.stride)
    np.testing.assert_array_equal(b.to_numpy(), want)


@pytest.mark.parametrize("kind", SEL_KINDS)
@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("dtype", [np.float64, np.int16])
def test_index_select_long_rows_matches_oracle(cdev, kind, axis, dtype):
    """Innermost extents of a CTA width and more (the row kernel), odd sizes
    that defeat the vector word, repeated and negative indices."""
    shape = (5, 300, 301)
    buf, shape, st, off = sel_case(kind, shape, dtype, seed=8)
    t = rt.from_host_layout(buf, shape, st, off, cdev)
    rng = np.random.default_rng(axis + 10)
    idx = rng.integers(-shape[axis], shape[axis], 300).tolist()
    b = rt.index_select(t, axis, idx)
    want = isel_oracle(buf, shape, st, off, axis, idx, b.shape, b.stride)
    np.testing.assert_array_equal(b.to_numpy(), want)


@pytest.mark.parametrize("shape,nidx,dtype,row_step", [
    ((300, 1024), 600, np.float64, 1),    # 8 KiB rows, four row buffers, inline indices
    ((64, 12288), 4000, np.float64, 1),   # 96 KiB rows, two row buffers, uploaded indices
    ((100, 2048), 513, np.float32, 2),    # every other source row
    ((3, 40, 4096), 1024, np.int16, 1),   # two outer dims
    ((50, 1001), 700, np.float64, 1),     # row not a multiple of 16 bytes (register staging)
    ((20, 16384), 9000, np.float32, 1),   # index list too long for shared memory
])
def test_index_select_dense_columns(cdev, shape, nidx, dtype, row_step):
    """Dense selections along a contiguous innermost axis (the staged-row
    kernels: bulk copies into shared memory, or register staging)."""
    base = list(shape)
    base[-2] *= row_step
    a = rand(tuple(base), dtype, seed=nidx)
    st = list(O.c_strides(base))
    st[-2] *= row_step
    view = a[..., ::row_step, :] if row_step > 1 else a
    t = rt.from_host_layout(a.ravel(), shape, st, 0, cdev)
    rng = np.random.default_rng(nidx)
    cols = rng.integers(0, shape[-1], nidx)
    np.testing.assert_array_equal(rt.index_select(t, len(shape) - 1, cols).to_numpy(), np.take(view, cols, axis=-1))


@pytest.mark.parametrize("nidx", [1, 2, 511, 512, 513, 5000])
def test_index_select_index_counts(cdev, nidx):
    """Inline (<= 512) and uploaded index lists, rows (vector path) and columns."""
    a = rand((700, 96), np.float32, seed=nidx)
    t = rt.asarray(a, cdev)
    rng = np.random.default_rng(nidx)
    rows = rng.integers(0, 700, nidx)
    np.testing.assert_array_equal(rt.index_select(t, 0, rows).to_numpy(), a[rows])
    cols = rng.integers(0, 96, nidx)
    np.testing.assert_array_equal(rt.index_select(t, 1, cols).to_numpy(), a[:, cols])


def test_index_select_col_major_device_and_take_bool_select(cdev):
    dev = with_order(cdev, "F")
    a = rand((6, 7, 8), np.float64, seed=1)
    t = rt.from_host_layout(a.ravel(order="F"), a.shape, O.f_strides(a.shape), 0, dev)
    b = t.index_select(1, [6, 0, -1, 3])
    assert b.f_contig()
    np.testing.assert_array_equal(b.to_numpy(), a[:, [6, 0, 6, 3]])
    np.testing.assert_array_equal(t.take([1, 1], 2).to_numpy(), a[:, :, [1, 1]])
    mask = [True, False, True, True, False, False]
    np.testing.assert_array_equal(t.bool_select(0, mask).to_numpy(), a[np.array(mask)])


def test_index_select_errors(cdev):
    t = rt.asarray(np.zeros((3, 4)), cdev)
    with pytest.raises(RstsrError) as e:
        rt.index_select(t, 1, [4])
    assert e.value.code == 9
    with pytest.raises(RstsrError) as e:
        rt.index_select(t, 2, [0])
    assert e.value.code == 10
    # the device entry point checks on its own as well
    out = rt.empty((3, 1), np.float64, cdev)
    idx = (C.c_uint64 * 1)(4)
    rc = _lib.lib().rstsr_cuda_index_select(cdev.ctx, _lib.F64, C.c_void_p(out.ptr), C.byref(out.layout()),
                                            C.c_void_p(t.ptr), C.byref(t.layout()), 1, idx, 1)
    assert rc == 9


def test_index_select_large_rows_property(cdev):
    """Full-size gather (8192 x 4096 f64 = 256 MiB, 4096 rows selected): the
    selected rows' sums equal the source rows' sums, checked exactly against
    numpy on the host copy."""
    rng = np.random.default_rng(3)
    a = rng.integers(-1000, 1000, (8192, 4096)).astype(np.float64)
    t = rt.asarray(a, cdev)
    rows = rng.integers(0, 8192, 4096)
    b = rt.index_select(t, 0, rows).to_numpy()
    np.testing.assert_array_equal(b, a[rows])


def test_index_select_graph_capture(cdev):
    a = rand((64, 32), np.float64, seed=6)
    t = rt.asarray(a, cdev)
    out = rt.empty((64, 5), np.float64, cdev)
    idx = np.array([3, 1, 31, 0, 3], dtype=np.uint64)
    with rt.Graph(cdev) as g:
        _lib.call("rstsr_cuda_index_select", cdev.ctx, _lib.F64, C.c_void_p(out.ptr), C.byref(out.layout()),
                  C.c_void_p(t.ptr), C.byref(t.layout()), 1, idx.ctypes.data_as(C.POINTER(C.c_uint64)), 5)
    rt.fill(out, 0.0)
    g.launch()
    cdev.sync()
    np.testing.assert_array_equal(out.to_numpy(), a[:, [3, 1, 31, 0, 3]])
    big = np.zeros(600, dtype=np.uint64)
    out2 = rt.empty((64, 600), np.float64, cdev)
    with pytest.raises(RstsrError, match="captured"):
        with rt.Graph(cdev):
            _lib.call("rstsr_cuda_index_select", cdev.ctx, _lib.F64, C.c_void_p(out2.ptr), C.byref(out2.layout()),
                      C.c_void_p(t.ptr), C.byref(t.layout()), 1, big.ctypes.data_as(C.POINTER(C.c_uint64)), 600)
