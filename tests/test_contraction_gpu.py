"""einsum / tensordot / vecdot on the GPU against the einsum oracle and the
reference's own tensordot / vecdot unit tests.

Tolerances: integer types exact; f64 <= 1e-12 relative Frobenius (every
contraction is an Ozaki-split GEMM), or, where the result cancels (a single
dot product), <= 1e-13 relative to the same contraction of the absolute
values, the scale the split's error bound is stated on; f32 <= 1e-5 on the
same two scales (bf16-split GEMMs and FP32 sums)."""

import json
from pathlib import Path

import numpy as np
import pytest

import rstsr_gb300 as rt
from oracle import oracle as O
from rstsr_gb300._lib import RstsrError
from tests.helpers import rel_err
from tests.test_contraction_oracle import operand, oracle_vecdot, strided, tensordot_subscripts

pytestmark = pytest.mark.gpu

CASES = json.loads((Path(__file__).resolve().parent / "golden" / "contraction_kats.json").read_text())
TOL = {np.float64: 1e-12, np.float32: 1e-5}


@pytest.fixture
def cdev(dev):
    yield dev
    dev.set_default_order("C")


def make(rng, shape, dtype, kind):
    """A device tensor of `shape` in layout `kind` and its host values."""
    if np.dtype(dtype).kind == "f":
        x = rng.standard_normal(shape).astype(dtype)
    else:
        x = rng.integers(-9, 10, shape).astype(dtype)
    shape = tuple(shape)
    n = len(shape)
    if kind == "c" or n == 0:
        return rt.from_host_layout(x.ravel(), shape, O.c_strides(shape), 0, DEV[0]), x
    if kind == "f":
        return rt.from_host_layout(x.ravel(order="F"), shape, O.f_strides(shape), 0, DEV[0]), x
    if kind == "rev":  # axes reversed view of a C-contiguous buffer
        base = x.transpose(tuple(range(n))[::-1]).copy()
        st = O.c_strides(base.shape)[::-1]
        return rt.from_host_layout(base.ravel(), shape, st, 0, DEV[0]), x
    if kind == "step2":  # every other element along the last axis
        base = np.zeros(shape[:-1] + (2 * shape[-1],), dtype=dtype)
        base[..., ::2] = x
        st = list(O.c_strides(base.shape))
        st[-1] *= 2
        return rt.from_host_layout(base.ravel(), shape, tuple(st), 0, DEV[0]), x
    if kind == "flip":
        base = x[..., ::-1].copy()
        st = list(O.c_strides(shape))
        off = st[-1] * (shape[-1] - 1)
        st[-1] = -st[-1]
        return rt.from_host_layout(base.ravel(), shape, tuple(st), off, DEV[0]), x
    raise ValueError(kind)


DEV = [None]


@pytest.fixture(autouse=True)
def _bind_dev(dev):
    DEV[0] = dev


def oracle_einsum(sub, arrs):
    acc = np.float64 if arrs[0].dtype.kind == "f" else np.int64
    return O.einsum(sub, *[strided(np.ascontiguousarray(x.astype(acc))) for x in arrs]).values()


def check(got, want, dtype, sub=None, arrs=None):
    if np.dtype(dtype).kind == "f":
        e = rel_err(got, want)
        if e > TOL[dtype] and sub is not None:
            scale = oracle_einsum(sub, [np.abs(x) for x in arrs])
            e_abs = np.linalg.norm(np.ravel(got - want)) / np.linalg.norm(np.ravel(scale))
            assert e_abs <= TOL[dtype] / 10, (e, e_abs)
        else:
            assert e <= TOL[dtype], e
    else:
        np.testing.assert_array_equal(got.astype(np.int64), want.astype(np.int64))


EINSUM_CASES = [
    ("ij,jk->ik", [(64, 48), (48, 40)]),
    ("ij,jk->ki", [(33, 20), (20, 17)]),
    ("bij,bjk->bik", [(4, 33, 20), (4, 20, 17)]),
    ("bij,bjk->ibk", [(4, 33, 20), (4, 20, 17)]),
    ("ij,kj->ik", [(30, 25), (19, 25)]),
    ("ijk,jkl->il", [(7, 6, 5), (6, 5, 9)]),
    ("ijk,kjl->li", [(7, 6, 5), (5, 6, 9)]),
    ("i,j->ij", [(40,), (30,)]),
    ("bi,bj->bij", [(5, 40), (5, 30)]),
    ("ij,ij->ij", [(20, 30), (20, 30)]),
    ("ab,ab->", [(31, 17), (31, 17)]),
    ("ii->", [(50, 50)]),
    ("ii->i", [(50, 50)]),
    ("ij->ji", [(50, 40)]),
    ("ij->i", [(50, 40)]),
    ("ij->", [(50, 40)]),
    ("iij,jk->ik", [(12, 12, 20), (20, 7)]),
    ("ij,jk,kl->il", [(20, 30), (30, 40), (40, 10)]),
    ("ijk,ikl->ijl", [(6, 20, 15), (6, 15, 11)]),
    ("ij,jk", [(16, 24), (24, 8)]),
    ("Pmn,mi,na->Pia", [(12, 30, 30), (30, 5), (30, 20)]),
    ("μi,νa,μνκλ,κj,λb->iajb", [(6, 3), (6, 3), (6, 6, 6, 6), (6, 3), (6, 3)]),
]


@pytest.mark.parametrize("sub,shapes", EINSUM_CASES, ids=[c[0] for c in EINSUM_CASES])
@pytest.mark.parametrize("dtype", [np.float64, np.int64, np.float32, np.int32])
def test_einsum_matches_oracle(cdev, sub, shapes, dtype):
    rng = np.random.default_rng(len(sub) + len(shapes))
    kinds = ["c", "rev", "step2", "flip", "f"]
    ts, xs = zip(*[make(rng, s, dtype, kinds[k % len(kinds)]) for k, s in enumerate(shapes)])
    got = rt.einsum(sub, *ts).to_numpy()
    check(got, oracle_einsum(sub, list(xs)), dtype, sub, list(xs))


@pytest.mark.parametrize("kind", ["c", "f", "rev", "step2", "flip"])
def test_einsum_operand_layouts(cdev, kind):
    rng = np.random.default_rng(3)
    a, xa = make(rng, (37, 29), np.float64, kind)
    b, xb = make(rng, (29, 23), np.float64, kind)
    c, xc = make(rng, (5, 37, 23), np.float64, kind)
    check(rt.einsum("ij,jk->ik", a, b).to_numpy(), oracle_einsum("ij,jk->ik", [xa, xb]), np.float64)
    check(rt.einsum("bik,ij->bjk", c, a).to_numpy(), oracle_einsum("bik,ij->bjk", [xc, xa]), np.float64)


def test_einsum_col_major_output_and_zero_extents(cdev):
    dev = cdev
    dev.set_default_order("F")
    rng = np.random.default_rng(4)
    a, xa = make(rng, (9, 7), np.float64, "f")
    b, xb = make(rng, (7, 5), np.float64, "f")
    c = rt.einsum("ij,jk->ik", a, b)
    assert c.f_contig()
    check(c.to_numpy(), xa @ xb, np.float64)
    dev.set_default_order("C")
    z1 = rt.einsum("ij,jk->ik", rt.asarray(np.zeros((4, 0)), dev), rt.asarray(np.zeros((0, 3)), dev))
    np.testing.assert_array_equal(z1.to_numpy(), np.zeros((4, 3)))
    z2 = rt.einsum("ij,jk->ik", rt.asarray(np.zeros((0, 5)), dev), rt.asarray(np.ones((5, 3)), dev))
    assert z2.shape == (0, 3)


def test_einsum_errors(cdev):
    a = rt.asarray(np.ones((3, 4)), cdev)
    b = rt.asarray(np.ones((5, 4)), cdev)
    with pytest.raises(RstsrError) as e:
        rt.einsum("ij,jk->ik", a, b)
    assert e.value.code == 1
    with pytest.raises(RstsrError):
        rt.einsum("ij,jk,kl->il", a, b)
    with pytest.raises(RstsrError) as e:
        rt.einsum("...j->j", a)
    assert e.value.code == 7
    with pytest.raises(RstsrError):
        rt.einsum("ij->ij", rt.asarray(np.ones((3, 4), dtype=np.float16), cdev))


def test_einsum_three_index_transform_large(cdev):
    """The 3-index AO -> MO step at moderate size: B[P, m, n] C1[m, i] C2[n, a]
    (both contractions on the tensor cores), against FP64 numpy."""
    rng = np.random.default_rng(9)
    B = rng.standard_normal((64, 120, 120))
    C1 = rng.standard_normal((120, 20))
    C2 = rng.standard_normal((120, 90))
    got = rt.einsum("Pmn,mi,na->Pia", rt.asarray(B, cdev), rt.asarray(C1, cdev), rt.asarray(C2, cdev)).to_numpy()
    want = np.einsum("Pmn,mi,na->Pia", B, C1, C2, optimize=True)
    assert rel_err(got, want) <= 1e-12


# ---------------------------------------------------------------- tensordot

@pytest.mark.parametrize("case", [c for c in CASES if c["op"] == "tensordot"],
                         ids=lambda c: c["src"].split("/")[-1])
def test_tensordot_reference_kat(cdev, case):
    a = rt.asarray(operand(case, "a", np.float64), cdev)
    b = rt.asarray(operand(case, "b", np.float64), cdev)
    axes = case["axes"] if isinstance(case["axes"], int) else tuple(case["axes"])
    np.testing.assert_allclose(rt.tensordot(a, b, axes).to_numpy(), np.array(case["expect"], dtype=np.float64),
                               rtol=1e-15, atol=0)


@pytest.mark.parametrize("sa,sb,axes", [
    ((6, 7, 8), (8, 5), 1),
    ((6, 7, 8), (7, 8, 5), 2),
    ((6, 7, 8), (8, 7, 5), ([1, 2], [1, 0])),
    ((4, 5, 6), (6, 4, 3), ([-1, 0], [0, 1])),
    ((3, 4), (5, 6), 0),
    ((3, 4, 5), (3, 4, 5), 3),
])
@pytest.mark.parametrize("dtype", [np.float64, np.int64])
def test_tensordot_matches_oracle(cdev, sa, sb, axes, dtype):
    rng = np.random.default_rng(len(sa) * 10 + len(sb))
    a, xa = make(rng, sa, dtype, "rev")
    b, xb = make(rng, sb, dtype, "c")
    got = rt.tensordot(a, b, axes).to_numpy()
    sub = tensordot_subscripts(len(sa), len(sb), axes if isinstance(axes, int) else (list(axes[0]), list(axes[1])))
    want = oracle_einsum(sub, [xa, xb])
    check(got, want, dtype)
    if np.dtype(dtype).kind == "f":
        assert rel_err(got, np.tensordot(xa, xb, axes)) <= 1e-12


# ------------------------------------------------------------------- vecdot

@pytest.mark.parametrize("case", [c for c in CASES if c["op"] == "vecdot"], ids=lambda c: c["src"].split("/")[-1])
def test_vecdot_reference_kat(cdev, case):
    dt = {"f64": np.float64, "i64": np.int64, "i32": np.int32}[case["dtype"]]
    a = rt.asarray(operand(case, "a", dt), cdev)
    b = rt.asarray(operand(case, "b", dt), cdev)
    got = rt.vecdot(a, b).to_numpy()
    np.testing.assert_allclose(got.astype(np.float64), np.array(case["expect"], dtype=np.float64),
                               rtol=case.get("tol", 0), atol=0)


@pytest.mark.parametrize("sa,sb", [((40, 300), (40, 300)), ((5, 1, 70), (3, 70)), ((70,), (6, 70)),
                                   ((4, 3, 200), (4, 3, 200))])
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32])
def test_vecdot_broadcast_matches_oracle(cdev, sa, sb, dtype):
    rng = np.random.default_rng(sum(sa))
    a, xa = make(rng, sa, dtype, "c")
    b, xb = make(rng, sb, dtype, "step2")
    got = rt.vecdot(a, b).to_numpy()
    want = oracle_vecdot(xa, xb)
    if np.dtype(dtype).kind == "f":
        assert rel_err(got, want) <= (1e-13 if dtype == np.float64 else 1e-5)
    else:
        np.testing.assert_array_equal(got, want.astype(dtype))


def test_vecdot_axes_forms(cdev):
    rng = np.random.default_rng(2)
    xa = rng.standard_normal((6, 5, 4))
    xb = rng.standard_normal((6, 5, 4))
    a, b = rt.asarray(xa, cdev), rt.asarray(xb, cdev)
    np.testing.assert_allclose(rt.vecdot(a, b, 0).to_numpy(), np.einsum("ijk,ijk->jk", xa, xb), rtol=1e-13)
    np.testing.assert_allclose(rt.vecdot(a, b, -2).to_numpy(), np.einsum("ijk,ijk->ik", xa, xb), rtol=1e-13)
    np.testing.assert_allclose(rt.vecdot(a, b, ([0, 2], [0, 2])).to_numpy(), np.einsum("ijk,ijk->j", xa, xb),
                               rtol=1e-13)
    with pytest.raises(RstsrError):
        rt.vecdot(a, rt.asarray(np.ones((6, 5, 3)), cdev))


@pytest.mark.parametrize("sa,sb,order", [((300, 257), (300, 257), "C"), ((5, 1, 100), (3, 100), "C"),
                                         ((64, 4096), (4096,), "C"), ((33, 40), (33, 40), "F")])
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int64])
def test_vecdot_fused_rows(cdev, sa, sb, order, dtype):
    """Contracted axis contiguous in both operands (the one-warp-per-output
    kernel), with broadcasting and a column-major device."""
    dev = cdev
    dev.set_default_order(order)
    rng = np.random.default_rng(len(sa) + sa[-1])
    xa = rng.standard_normal(sa).astype(dtype) if np.dtype(dtype).kind == "f" else \
        rng.integers(-50, 50, sa).astype(dtype)
    xb = rng.standard_normal(sb).astype(dtype) if np.dtype(dtype).kind == "f" else \
        rng.integers(-50, 50, sb).astype(dtype)
    if order == "C":
        a, b = rt.asarray(xa, dev), rt.asarray(xb, dev)
        got = rt.vecdot(a, b).to_numpy()
        want = oracle_vecdot(xa, xb)
    else:  # column-major: the first axis is contiguous; contract it
        a = rt.from_host_layout(xa.ravel(order="F"), xa.shape, O.f_strides(xa.shape), 0, dev)
        b = rt.from_host_layout(xb.ravel(order="F"), xb.shape, O.f_strides(xb.shape), 0, dev)
        got = rt.vecdot(a, b, 0).to_numpy()
        want = oracle_vecdot(np.ascontiguousarray(xa.T), np.ascontiguousarray(xb.T))
    if np.dtype(dtype).kind == "f":
        assert rel_err(got, want) <= (1e-13 if dtype == np.float64 else 1e-5)
    else:
        np.testing.assert_array_equal(got, want.astype(dtype))
