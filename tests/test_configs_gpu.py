"""The benchmark's workloads at their stated sizes, checked against the oracle.

Each test runs the same calls `bench.py` times, on the same seeded inputs,
and compares every output with the CPU oracle (or an FP64 product for the
floating-point GEMMs):

* the small f64 case (seed 0): A [64,128] + b [128], sum_axes(C, 1),
  argmax_axes(C, 1), A % B with B [128,96];
* the memory-bound workload: f64 / f32 / i32 [32,64,128,128] in the C, F,
  axis-permuted and step-2-sliced layouts; permute(0,2,1,3) + to_contig,
  a*b+c with c [1,64,1,128], sum over axes (1, 3), argmax over the last axis;
* the f64 contraction Bm^T Bm (Bm = B[1000, 50, 300] reshaped to 1000 x 15000);
* the f32 three-term split on 8192^3 and 65536x256x256 with spread exponents;
* 512 uneven f64 problems in one grouped call, the broadcast batch
  [64,1,256,256] % [1,32,256,256], and the graph-captured chain.

Bars: copies, integers, the fused a*b+c (two roundings) and argmax indices
bit-exact, output strides equal to the oracle's; float sums <= 1e-13 (f64) /
1e-5 (f32) normwise relative; the f64 Ozaki GEMMs <= 1e-12 relative Frobenius
(the small case <= 1e-13); the f32 split <= 1e-6.
"""

import numpy as np
import pytest

import bench
import rstsr_gb300 as rt
from oracle import layout as OL
from oracle import oracle as O

pytestmark = pytest.mark.gpu

F64_SUM_TOL = 1e-13
F32_SUM_TOL = 1e-5
OZAKI_TOL = 1e-12
SPLIT_F32_TOL = 1e-6


def normwise(got, want):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    return float(np.max(np.abs(got - want)) / max(float(np.max(np.abs(want))), 1e-300))


def frob(got, want):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    return float(np.linalg.norm((got - want).ravel()) / np.linalg.norm(want.ravel()))


# ------------------------------------------------------------- small f64


def test_small_f64_seed0(dev):
    rng = np.random.default_rng(0)
    A = rng.uniform(-1, 1, (64, 128))
    b = rng.uniform(-1, 1, (128,))
    B = rng.uniform(-1, 1, (128, 96))
    tA, tb, tB = rt.asarray(A, dev), rt.asarray(b, dev), rt.asarray(B, dev)
    Cd = tA + tb
    # C = A + b (b broadcast with stride 0), bit-exact
    cref = O.empty_strided((64, 128), OL.c_stride((64, 128)), np.float64)
    O.binary("add", cref, O.Strided(A.ravel(), (64, 128), (128, 1)), O.Strided(b, (64, 128), (0, 1)))
    assert (Cd.shape, Cd.stride) == ((64, 128), (128, 1))
    np.testing.assert_array_equal(Cd.to_numpy(), cref.values())
    Cv = cref.values()
    # sum_axes(C, 1)
    sref = O.empty_strided((64,), (1,), np.float64)
    O.reduce_axes("sum", O.Strided(Cv.ravel(), (64, 128), (128, 1)), [1], sref)
    s = Cd.sum_axes(1)
    assert (s.shape, s.stride) == ((64,), (1,))
    assert normwise(s.to_numpy(), sref.values()) <= F64_SUM_TOL
    # argmax_axes(C, 1)
    gref = O.empty_strided((64,), (1,), np.uint64)
    O.argreduce_axes(True, O.Strided(Cv.ravel(), (64, 128), (128, 1)), [1], gref)
    np.testing.assert_array_equal(Cd.argmax_axes(1).to_numpy(), gref.values())
    # A % B through the Ozaki split, against an FP64 product (k = 128)
    m = rt.matmul(tA, tB)
    assert (m.shape, m.stride) == ((64, 96), (96, 1))
    assert frob(m.to_numpy(), A @ B) <= 1e-13


def test_small_f64_graph_replayed(dev):
    """The same four operations captured into one CUDA graph (the benchmark's
    replayed latency figure) and replayed twice into caller-owned outputs."""
    rng = np.random.default_rng(0)
    A = rng.uniform(-1, 1, (64, 128))
    b = rng.uniform(-1, 1, (128,))
    B = rng.uniform(-1, 1, (128, 96))
    tA, tb, tB = rt.asarray(A, dev), rt.asarray(b, dev), rt.asarray(B, dev)
    g, (cbuf, s_out, g_out, m_out) = bench.capture_small_ops(dev, tA, tb, tB)
    for t in (cbuf, s_out, m_out):
        rt.fill(t, 0.0)
    rt.fill(g_out, 7)
    g.launch()
    g.launch()
    Cv = A + b
    np.testing.assert_array_equal(cbuf.to_numpy(), Cv)
    sref = O.empty_strided((64,), (1,), np.float64)
    O.reduce_axes("sum", O.Strided(Cv.ravel(), (64, 128), (128, 1)), [1], sref)
    assert normwise(s_out.to_numpy(), sref.values()) <= F64_SUM_TOL
    gref = O.empty_strided((64,), (1,), np.uint64)
    O.argreduce_axes(True, O.Strided(Cv.ravel(), (64, 128), (128, 1)), [1], gref)
    np.testing.assert_array_equal(g_out.to_numpy(), gref.values())
    assert frob(m_out.to_numpy(), A @ B) <= 1e-13


# ---------------------------------------------------- memory-bound workload


@pytest.mark.parametrize("kind", bench.LAYOUTS)
@pytest.mark.parametrize("dname", [d for d, _ in bench.DTYPES])
def test_strided_workload_full_size(dev, dname, kind):
    """All four operations of one (dtype, layout) case of the benchmark step,
    through the same C-ABI calls, against the oracle on all host cores."""
    wl = bench.Workload(dev, rt.lib(), seed=0, dtypes=[dname], layouts=[kind])
    (c,) = wl.cases
    for op in ("to_contig", "fma", "sum", "argmax"):
        wl.run_op(c, op)
    dev.sync()
    dt = dict(bench.DTYPES)[dname]
    nth = O.max_threads()
    _, stride, off = bench.layout_of(kind, bench.SHAPE)
    a = O.Strided(c["ha"], bench.SHAPE, stride, off)
    b = O.Strided(c["hb"], bench.SHAPE, stride, off)
    cst = O.Strided(c["hc"], bench.SHAPE, (0, bench.CSHAPE[3], 0, 1), 0)

    # permute(0, 2, 1, 3) + to_contig: a C-contiguous copy of the permuted view
    pshape, pstride = bench.permuted_view(bench.SHAPE, stride)
    if c["copy"]:
        pref = O.empty_strided(pshape, OL.c_stride(pshape), dt)
        O.assign_arbitrary(pref, O.Strided(c["ha"], pshape, pstride, off), 0, nth)
        out = c["out_perm"]
        assert (out.shape, out.stride) == (pshape, OL.c_stride(pshape))
        np.testing.assert_array_equal(out.to_numpy(), pref.values())
    else:
        # the permuted view of this layout is already C-contiguous: to_contig is a view
        assert tuple(pstride) == OL.c_stride(pshape)

    # a*b+c in the binary-op output layout, two roundings as the reference's two passes
    lab = OL.layout_for_binary_op((bench.SHAPE, stride, off), (bench.SHAPE, stride, off))
    d = c["d"]
    assert (d.shape, d.stride) == (tuple(lab[0]), tuple(lab[1]))
    dref = O.empty_strided(lab[0], lab[1], dt)
    O.fma(dref, a, b, cst, nth)
    np.testing.assert_array_equal(d.to_numpy(), dref.values())
    del dref

    # sum over axes (1, 3)
    osh, ost, _ = OL.reduce_output_layout((bench.SHAPE, stride, off), [1, 3])
    s = c["sum_out"]
    assert (s.shape, s.stride) == (tuple(osh), tuple(ost))
    sref = O.empty_strided(osh, ost, dt)
    O.reduce_axes("sum", a, [1, 3], sref, nth)
    if np.dtype(dt).kind == "i":
        np.testing.assert_array_equal(s.to_numpy(), sref.values())
    else:
        tol = F64_SUM_TOL if dt == np.float64 else F32_SUM_TOL
        assert normwise(s.to_numpy(), sref.values()) <= tol

    # argmax over the last axis (i32 in [-1000, 1000]: many ties)
    osh, ost, _ = OL.reduce_output_layout((bench.SHAPE, stride, off), [3])
    g = c["arg_out"]
    assert (g.shape, g.stride) == (tuple(osh), tuple(ost))
    gref = O.empty_strided(osh, ost, np.uint64)
    O.argreduce_axes(True, a, [3], gref, nth)
    np.testing.assert_array_equal(g.to_numpy(), gref.values())


# ---------------------------------------------------------------- GEMMs


def test_ozaki_contraction_15000x1000(dev):
    """C = Bm^T Bm, Bm [1000, 15000] with entries N(0,1) exp(-0.01 P), seed 0
    (the SYRK path), against cuBLAS's native FP64 product, whose own error is
    bounded by exact rational dot products of sampled entries."""
    torch = pytest.importorskip("torch")
    from fractions import Fraction

    rng = np.random.default_rng(0)
    P, Q = 1000, 15000
    bm = rng.standard_normal((P, Q)) * np.exp(-0.01 * np.arange(P))[:, None]
    t = rt.asarray(bm, dev)
    c = rt.empty((Q, Q), np.float64, dev)
    rt.matmul_into(c, t.t(), t, 1.0, 0.0)
    got = torch.as_tensor(c.to_numpy()).cuda()
    del c
    tb = torch.from_numpy(bm).cuda()
    ref = tb.T @ tb
    err = (torch.linalg.norm(got - ref) / torch.linalg.norm(ref)).item()
    assert err <= OZAKI_TOL, err
    assert torch.equal(got, got.T), "the SYRK result must be exactly symmetric"
    pairs = [tuple(int(v) for v in rng.integers(0, Q, 2)) for _ in range(16)]
    cols = {j: [Fraction(float(x)) for x in bm[:, j]] for pair in pairs for j in pair}
    exact = np.array([float(sum(x * y for x, y in zip(cols[i], cols[j]))) for i, j in pairs])
    g = np.array([got[i, j].item() for i, j in pairs])
    r = np.array([ref[i, j].item() for i, j in pairs])
    assert np.linalg.norm(g - exact) / np.linalg.norm(exact) <= OZAKI_TOL
    assert np.linalg.norm(r - exact) / np.linalg.norm(exact) <= 1e-14  # the FP64 oracle itself
    del got, ref, tb
    torch.cuda.empty_cache()


@pytest.mark.parametrize("m,n,k", [(8192, 8192, 8192), (65536, 256, 256)])
def test_split_f32_spread_exponents(dev, m, n, k):
    """f32 three-term bf16 split, entries U(-1,1) 2^U(-8,8), against FP64."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    a = (rng.uniform(-1, 1, (m, k)) * 2.0 ** rng.uniform(-8, 8, (m, k))).astype(np.float32)
    b = (rng.uniform(-1, 1, (k, n)) * 2.0 ** rng.uniform(-8, 8, (k, n))).astype(np.float32)
    c = rt.matmul(rt.asarray(a, dev), rt.asarray(b, dev))
    assert (c.shape, c.stride) == ((m, n), (n, 1))
    got = torch.as_tensor(c.to_numpy()).cuda().double()
    ref = torch.from_numpy(a).cuda().double() @ torch.from_numpy(b).cuda().double()
    err = (torch.linalg.norm(got - ref) / torch.linalg.norm(ref)).item()
    assert err <= SPLIT_F32_TOL, err
    del got, ref
    torch.cuda.empty_cache()


def test_grouped_512_uneven_f64(dev):
    """512 f64 problems, m, n, k uniform in [16, 512] (seed 0), one grouped call."""
    import ctypes as C

    from rstsr_gb300._lib import GemmProblem, call

    rng = np.random.default_rng(0)
    dims = rng.integers(16, 513, (512, 3))
    keep, probs = [], []
    for m, n, k in dims:
        m, n, k = int(m), int(n), int(k)
        a = rng.uniform(-1, 1, (m, k))
        b = rng.uniform(-1, 1, (k, n))
        ta, tb = rt.asarray(a, dev), rt.asarray(b, dev)
        tc = rt.empty((m, n), np.float64, dev)
        keep.append((a, b, ta, tb, tc))
        probs.append(GemmProblem(m, n, k, k, n, n, ta.ptr, tb.ptr, tc.ptr, 1.0, 0.0))
    arr = (GemmProblem * len(probs))(*probs)
    call("rstsr_cuda_gemm_grouped", dev.ctx, 0, arr, len(probs), None)
    dev.sync()
    worst = 0.0
    for a, b, _, _, tc in keep:
        worst = max(worst, frob(tc.to_numpy(), a @ b))
    assert worst <= OZAKI_TOL, worst


def test_broadcast_batch_64x32_256(dev):
    """[64,1,256,256] % [1,32,256,256] f64 (matmul rule 7) against FP64."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    a = rng.uniform(-1, 1, (64, 1, 256, 256))
    b = rng.uniform(-1, 1, (1, 32, 256, 256))
    c = rt.matmul(rt.asarray(a, dev), rt.asarray(b, dev))
    assert c.shape == (64, 32, 256, 256)
    got = torch.as_tensor(c.to_numpy()).cuda()
    ref = torch.matmul(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda())
    # every one of the 2048 products, not only the whole
    num = torch.linalg.norm((got - ref).reshape(2048, -1), dim=1)
    den = torch.linalg.norm(ref.reshape(2048, -1), dim=1)
    assert (num / den).max().item() <= OZAKI_TOL
    del got, ref
    torch.cuda.empty_cache()


def test_graph_chain_replayed(dev):
    """matmul [256,256] % [256,256] -> + bias[256] -> sum_axes(1), captured
    once and replayed 1000 times, against FP64 on the host."""
    rng = np.random.default_rng(0)
    a = rng.uniform(-1, 1, (256, 256))
    b = rng.uniform(-1, 1, (256, 256))
    bias = rng.uniform(-1, 1, (256,))
    ta, tb, tbias = rt.asarray(a, dev), rt.asarray(b, dev), rt.asarray(bias, dev)
    c = rt.empty((256, 256), np.float64, dev)
    o = rt.empty((256,), np.float64, dev)

    def chain():
        rt.matmul_into(c, ta, tb, 1.0, 0.0, slices=7)
        rt.binary_inplace("add", c, tbias)
        rt.reduce_axes_into("sum", c, [1], o)

    with rt.Graph(dev) as g:
        chain()
    for _ in range(1000):
        g.launch()
    dev.sync()
    want = (a @ b + bias).sum(axis=1)
    assert frob(o.to_numpy(), want) <= OZAKI_TOL
