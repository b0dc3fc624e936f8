"""Matmul / GEMM on the GPU: the Ozaki split (f64) against an FP64 oracle
at <= 1e-12 relative Frobenius error, the three-term bf16 split (f32) at
<= 1e-6, integer matmul bit-exact, the broadcasting rules, SYRK symmetry and
the reference's known answers."""

import ctypes as C

import numpy as np
import pytest

import rstsr_gb300 as rt
from rstsr_gb300._lib import GemmOpts, call
from tests.helpers import NP, rel_err

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12
F32_TOL = 1e-6


def ref64(a, b):
    """FP64 oracle with compensated accumulation (exact products split into
    hi/lo by numpy's float64 matmul of the error-free parts is not needed at
    these sizes: use extended-precision dot via math.fsum on a few rows)."""
    return np.asarray(a, np.float64) @ np.asarray(b, np.float64)


@pytest.mark.parametrize("m,n,k", [(64, 96, 128), (128, 128, 64), (200, 130, 77), (257, 300, 1000), (33, 17, 2050)])
def test_ozaki_f64_matmul(dev, m, n, k):
    rng = np.random.default_rng(m * 7 + n)
    a = rng.uniform(-1, 1, (m, k))
    b = rng.uniform(-1, 1, (k, n))
    ta, tb = rt.asarray(a, dev), rt.asarray(b, dev)
    c = (ta % tb).to_numpy()
    assert rel_err(c, ref64(a, b)) <= F64_TOL
    assert rt.lib().rstsr_cuda_last_ozaki_slices() >= 4


@pytest.mark.parametrize("m,n,k,want", [(512, 512, 512, 8), (1024, 1024, 1024, 8), (1024, 1024, 1025, 0)])
def test_ozaki_slice_count_rule(dev, m, n, k, want):
    """Calls of at most 2^30 multiply-adds take 8 slices without measuring the
    exponent spread; larger ones choose from the spread (4-8). Rows scaled by
    2^U(-30, 30) and a decaying K profile keep the spread wide."""
    rng = np.random.default_rng(m + k)
    a = rng.standard_normal((m, k)) * 2.0 ** rng.uniform(-30, 30, (m, 1)) * np.exp(-0.004 * np.arange(k))
    b = rng.standard_normal((k, n)) * 2.0 ** rng.uniform(-30, 30, (1, n))
    c = (rt.asarray(a, dev) % rt.asarray(b, dev)).to_numpy()
    got = rt.lib().rstsr_cuda_last_ozaki_slices()
    if want:
        assert got == want
    else:
        assert 4 <= got <= 8
    assert rel_err(c, ref64(a, b)) <= F64_TOL


def test_ozaki_exponent_spread_and_signs(dev):
    rng = np.random.default_rng(1)
    m, n, k = 150, 140, 300
    a = rng.standard_normal((m, k)) * np.exp(rng.uniform(-20, 20, (m, 1)))  # row scales
    b = rng.standard_normal((k, n)) * np.exp(-0.01 * np.arange(k))[:, None]
    c = (rt.asarray(a, dev) % rt.asarray(b, dev)).to_numpy()
    assert rel_err(c, ref64(a, b)) <= F64_TOL


def test_ozaki_syrk_symmetric(dev):
    """B^T B with B = A's own buffer viewed transposed: the SYRK shortcut."""
    rng = np.random.default_rng(2)
    p, q = 300, 260
    bm = rng.standard_normal((p, q)) * np.exp(-0.01 * np.arange(p))[:, None]
    t = rt.asarray(bm, dev)
    c = (t.t() % t).to_numpy()
    assert np.array_equal(c, c.T)
    assert rel_err(c, bm.T @ bm) <= F64_TOL


@pytest.mark.parametrize("order", ["C", "F"])
def test_ozaki_strided_operands_alpha_beta(dev, order):
    rng = np.random.default_rng(3)
    m, n, k = 190, 150, 210
    a = rng.uniform(-1, 1, (k, m)).T  # transposed view
    b = rng.uniform(-1, 1, (n, k)).T
    c0 = rng.uniform(-1, 1, (m, n))
    dev.set_default_order(order)
    try:
        ta = rt.asarray(np.ascontiguousarray(a.T), dev).t()
        tb = rt.asarray(np.ascontiguousarray(b.T), dev).t()
        tc = rt.asarray(c0, dev)
        if order == "F":
            tc = tc.to_contig("F")
        rt.matmul_into(tc, ta, tb, 2.0, 1.5)
        want = 2.0 * (a @ b) + 1.5 * c0
        assert rel_err(tc.to_numpy(), want) <= F64_TOL
    finally:
        dev.set_default_order("C")


@pytest.mark.parametrize("m,n,k", [(64, 96, 128), (300, 200, 500), (128, 256, 2048)])
def test_split_f32_matmul(dev, m, n, k):
    rng = np.random.default_rng(k)
    a = (rng.uniform(-1, 1, (m, k)) * 2.0 ** rng.uniform(-8, 8, (m, k))).astype(np.float32)
    b = (rng.uniform(-1, 1, (k, n)) * 2.0 ** rng.uniform(-8, 8, (k, n))).astype(np.float32)
    c = (rt.asarray(a, dev) % rt.asarray(b, dev)).to_numpy()
    assert c.dtype == np.float32
    assert rel_err(c, ref64(a, b)) <= F32_TOL


def test_native_precision_f64(dev):
    rng = np.random.default_rng(4)
    a = rng.uniform(-1, 1, (70, 50))
    b = rng.uniform(-1, 1, (50, 30))
    c = rt.matmul(rt.asarray(a, dev), rt.asarray(b, dev), precision=1).to_numpy()
    assert rel_err(c, a @ b) <= 1e-14


@pytest.mark.parametrize("sa,sb", [((5,), (5,)), ((3, 5), (5, 4)), ((5,), (2, 5, 4)), ((2, 3, 5), (5,)),
                                   ((3, 5), (2, 5, 4)), ((2, 3, 5), (5, 4)), ((2, 1, 3, 5), (4, 5, 6)),
                                   ((4, 1, 9, 16), (1, 3, 16, 7))])
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int64])
def test_matmul_rules_match_numpy(dev, sa, sb, dtype):
    rng = np.random.default_rng(len(sa) * 10 + len(sb))
    if np.dtype(dtype).kind == "f":
        a = rng.uniform(-1, 1, sa).astype(dtype)
        b = rng.uniform(-1, 1, sb).astype(dtype)
    else:
        a = rng.integers(-50, 50, sa).astype(dtype)
        b = rng.integers(-50, 50, sb).astype(dtype)
    got = rt.matmul(rt.asarray(a, dev), rt.asarray(b, dev)).to_numpy()
    want = np.matmul(a.astype(np.float64) if a.dtype.kind == "f" else a, b.astype(np.float64) if b.dtype.kind == "f" else b)
    assert got.shape == want.shape
    if np.dtype(dtype).kind == "f":
        tol = F64_TOL if dtype == np.float64 else F32_TOL
        assert rel_err(got, want) <= tol
    else:
        np.testing.assert_array_equal(got, want)


def test_col_major_matmul_rules(dev):
    rng = np.random.default_rng(5)
    dev.set_default_order("F")
    try:
        # col-major: matrix axes first, batch axes trailing
        a = rng.uniform(-1, 1, (3, 5, 4))
        b = rng.uniform(-1, 1, (5, 6, 4))
        got = rt.matmul(rt.asarray(a, dev), rt.asarray(b, dev)).to_numpy()
        want = np.einsum("ikb,kjb->ijb", a, b)
        assert got.shape == (3, 6, 4)
        assert rel_err(got, want) <= F64_TOL
    finally:
        dev.set_default_order("C")


def test_kat_matmul(dev, kats):
    for case in kats:
        if case["op"] == "matmul":
            a = rt.asarray(np.array(case["a"], dtype=np.int32), dev)
            b = rt.asarray(np.array(case["b"], dtype=np.int32), dev)
            assert (a % b).to_numpy().tolist() == case["expect"], case["src"]
        elif case["op"] == "matmul_from":
            a = rt.asarray(np.array(case["a"]).reshape(case["shape_a"]), dev)
            b = rt.asarray(np.array(case["b"]).reshape(case["shape_b"]), dev)
            c = rt.asarray(np.array(case["c"]).reshape(case["shape_c"]), dev)
            rt.matmul_into(c, a, b, case["alpha"], case["beta"])
            np.testing.assert_allclose(c.to_numpy().ravel(), case["expect"], rtol=1e-13)
        elif case["op"] == "batched_linspace_stats":
            n = case["n"]
            a = rt.asarray(np.linspace(*case["a_range"], n).reshape(case["shape"]), dev)
            b = rt.asarray(np.linspace(*case["b_range"], n).reshape(case["shape"]), dev)
            c = a % b
            assert abs(c.mean_all() - case["expect"]["mean_all"]) < case["tol"]
            assert abs(c.std_all() - case["expect"]["std_all"]) < case["tol"]


@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
def test_driver_gemm_blas_semantics(dev, order, ta, tb):
    rng = np.random.default_rng(6)
    m, n, k = 70, 90, 110
    opa = rng.uniform(-1, 1, (m, k))
    opb = rng.uniform(-1, 1, (k, n))
    c0 = rng.uniform(-1, 1, (m, n))
    # store op(A), op(B), C in `order` with the trans flags applied
    def store(x, trans):
        s = x.T if trans == "T" else x
        return np.ascontiguousarray(s) if order == 0 else np.asfortranarray(s)
    A, B = store(opa, ta), store(opb, tb)
    Cm = np.ascontiguousarray(c0) if order == 0 else np.asfortranarray(c0)
    lda = A.shape[1] if order == 0 else A.shape[0]
    ldb = B.shape[1] if order == 0 else B.shape[0]
    ldc = n if order == 0 else m
    da = rt.asarray(A.ravel(order="K"), dev)
    db = rt.asarray(B.ravel(order="K"), dev)
    dc = rt.asarray(Cm.ravel(order="K"), dev)
    call("rstsr_cuda_gemm", dev.ctx, order, ta.encode(), tb.encode(), m, n, k, C.c_double(0.5), C.c_void_p(da.ptr), lda,
         C.c_void_p(db.ptr), ldb, C.c_double(-2.0), C.c_void_p(dc.ptr), ldc, 0, None)
    got = dc.to_numpy().reshape((m, n) if order == 0 else (n, m))
    if order == 1:
        got = got.T
    assert rel_err(got, 0.5 * opa @ opb - 2.0 * c0) <= F64_TOL


def test_grouped_gemm_uneven(dev):
    rng = np.random.default_rng(7)
    from rstsr_gb300._lib import GemmProblem

    probs, keep = [], []
    for i in range(12):
        m, n, k = (int(x) for x in rng.integers(16, 200, 3))
        a = rng.uniform(-1, 1, (m, k))
        b = rng.uniform(-1, 1, (k, n))
        ta, tb = rt.asarray(a, dev), rt.asarray(b, dev)
        tc = rt.zeros((m, n), np.float64, dev)
        keep.append((a, b, ta, tb, tc))
        probs.append(GemmProblem(m, n, k, k, n, n, ta.ptr, tb.ptr, tc.ptr, 1.0, 0.0))
    arr = (GemmProblem * len(probs))(*probs)
    call("rstsr_cuda_gemm_grouped", dev.ctx, 0, arr, len(probs), None)
    for a, b, _, _, tc in keep:
        assert rel_err(tc.to_numpy(), a @ b) <= F64_TOL


def test_zero_k_scales_c(dev):
    c = rt.full((4, 5), 2.0, np.float64, dev)
    a = rt.zeros((4, 0), np.float64, dev)
    b = rt.zeros((0, 5), np.float64, dev)
    rt.matmul_into(c, a, b, 1.0, 0.5)
    assert (c.to_numpy() == 1.0).all()


def test_broadcast_batched_matmul_one_launch(dev):
    """Rule 7 broadcast batch [8,1,96,64] % [1,5,64,80] (40 products) runs as
    one grouped split GEMM; every product within the f64 bar."""
    rng = np.random.default_rng(8)
    a = rng.uniform(-1, 1, (8, 1, 96, 64))
    b = rng.uniform(-1, 1, (1, 5, 64, 80))
    l0 = dev.launch_count()
    got = (rt.asarray(a, dev) % rt.asarray(b, dev)).to_numpy()
    launches = dev.launch_count() - l0
    assert launches <= 12, f"{launches} launches for one batched matmul"
    assert got.shape == (8, 5, 96, 80)
    assert rel_err(got, np.matmul(a, b)) <= F64_TOL
    af = a.astype(np.float32)
    bf = b.astype(np.float32)
    gotf = (rt.asarray(af, dev) % rt.asarray(bf, dev)).to_numpy()
    assert rel_err(gotf, np.matmul(af.astype(np.float64), bf.astype(np.float64))) <= F32_TOL


def test_grouped_uneven_f32_and_transposed_outputs(dev):
    rng = np.random.default_rng(9)
    from rstsr_gb300._lib import GemmProblem

    probs, keep = [], []
    for i in range(9):
        m, n, k = (int(x) for x in rng.integers(16, 300, 3))
        a = rng.uniform(-1, 1, (m, k)).astype(np.float32)
        b = rng.uniform(-1, 1, (k, n)).astype(np.float32)
        ta, tb = rt.asarray(a, dev), rt.asarray(b, dev)
        tc = rt.full((m, n), 1.0, np.float32, dev)
        keep.append((a, b, ta, tb, tc))
        probs.append(GemmProblem(m, n, k, k, n, n, ta.ptr, tb.ptr, tc.ptr, 2.0, -1.0))
    arr = (GemmProblem * len(probs))(*probs)
    call("rstsr_cuda_gemm_grouped", dev.ctx, 1, arr, len(probs), None)
    for a, b, _, _, tc in keep:
        want = 2.0 * (a.astype(np.float64) @ b.astype(np.float64)) - 1.0
        assert rel_err(tc.to_numpy(), want) <= F32_TOL


def test_graph_captured_chain_matches_eager(dev):
    """matmul -> broadcast bias add -> sum_axes captured once, replayed."""
    rng = np.random.default_rng(10)
    a = rng.uniform(-1, 1, (256, 256))
    b = rng.uniform(-1, 1, (256, 256))
    bias = rng.uniform(-1, 1, (256,))
    ta, tb, tbias = rt.asarray(a, dev), rt.asarray(b, dev), rt.asarray(bias, dev)
    c = rt.empty((256, 256), np.float64, dev)
    out = rt.empty((256,), np.float64, dev)

    def chain():
        rt.matmul_into(c, ta, tb, 1.0, 0.0, slices=7)
        rt.binary_inplace("add", c, tbias)
        rt.reduce_axes_into("sum", c, [1], out)

    chain()  # eager warm-up
    eager = out.to_numpy().copy()
    with rt.Graph(dev) as g:
        chain()
    rt.fill(out, 0.0)
    n0 = dev.launch_count()
    for _ in range(5):
        g.launch()
    dev.sync()
    assert dev.launch_count() - n0 >= 5 * 3
    np.testing.assert_array_equal(out.to_numpy(), eager)
    want = (a @ b + bias).sum(axis=1)
    assert rel_err(eager, want) <= F64_TOL


@pytest.mark.parametrize("dtype,tol,slices", [(np.float64, F64_TOL, 7), (np.float32, F32_TOL, 0)])
def test_autotune_picks_config_and_results_stay_correct(dev, tmp_path, dtype, tol, slices):
    code = rt.autotune_gemm(dev, dtype, 512, 512, 512, slices=slices)
    kt, group = code & 0xFF, code >> 8
    assert kt in (16, 32, 64) and group in (4, 8, 16, 32)
    # a problem of the same shape class (log2 extents rounded up: 9, 9, 9) runs with that config
    rng = np.random.default_rng(11)
    a = rng.uniform(-1, 1, (500, 480)).astype(dtype)
    b = rng.uniform(-1, 1, (480, 300)).astype(dtype)
    c = rt.matmul(rt.asarray(a, dev), rt.asarray(b, dev), slices=slices).to_numpy()
    assert rel_err(c, ref64(a, b)) <= tol
    path = tmp_path / "tuned.txt"
    rt.autotune_save(path)
    mode = "ozaki" if dtype == np.float64 else "bf16x3"
    nsl = "7" if dtype == np.float64 else "3"
    assert [mode, nsl, "9", "9", "9", str(kt), str(group)] in [l.split() for l in path.read_text().splitlines()]
    rt.autotune_load(path)  # round trip through the file


def test_ozaki_against_exact_dot_products(dev):
    """Sampled entries of the C3-shaped SYRK against exact rational sums."""
    from fractions import Fraction

    rng = np.random.default_rng(0)
    P, Q = 1000, 512
    bm = rng.standard_normal((P, Q)) * np.exp(-0.01 * np.arange(P))[:, None]
    t = rt.asarray(bm, dev)
    c = rt.matmul(t.t(), t).to_numpy()
    pairs = [tuple(int(v) for v in rng.integers(0, Q, 2)) for _ in range(24)]
    cols = {j: [Fraction(float(x)) for x in bm[:, j]] for pair in pairs for j in pair}
    exact = np.array([float(sum(a * b for a, b in zip(cols[i], cols[j]))) for i, j in pairs])
    got = np.array([c[i, j] for i, j in pairs])
    assert np.linalg.norm(got - exact) / np.linalg.norm(exact) <= F64_TOL
