"""Pins the einsum oracle against the reference's tensordot / vecdot unit
tests (tests/golden/contraction_kats.json) and numpy, and checks the
library's host-side subscript parsing (CPU only)."""

import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

CASES = json.loads((Path(__file__).resolve().parent / "golden" / "contraction_kats.json").read_text())
LETTERS = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"


def operand(case, key, dtype):
    if key in case:
        return np.array(case[key], dtype=dtype)
    r = case[key + "_arange"]
    lo, hi = (0, r) if isinstance(r, int) else r
    return np.arange(lo, hi, dtype=dtype).reshape(case[key + "_shape"])


def strided(x):
    return O.Strided(np.ascontiguousarray(x).ravel(), x.shape, O.c_strides(x.shape))


def tensordot_subscripts(nda, ndb, axes):
    """The labelling of rstsr-common/src/tensordot_to_einsum.rs:18-112."""
    if isinstance(axes, int):
        xa, xb = list(range(nda - axes, nda)), list(range(axes))
    else:
        xa, xb = [a % nda for a in axes[0]], [b % ndb for b in axes[1]]
    gen = iter(LETTERS)
    la, lb = [None] * nda, [None] * ndb
    for i, j in zip(xa, xb):
        la[i] = lb[j] = next(gen)
    for i in range(nda):
        if la[i] is None:
            la[i] = next(gen)
    for j in range(ndb):
        if lb[j] is None:
            lb[j] = next(gen)
    out = [la[i] for i in range(nda) if i not in xa] + [lb[j] for j in range(ndb) if j not in xb]
    return "".join(la) + "," + "".join(lb) + "->" + "".join(out)


def oracle_vecdot(a, b):
    """Last-axis vecdot with numpy broadcasting of the remaining axes."""
    a64, b64 = np.broadcast_arrays(a.astype(np.float64 if a.dtype.kind == "f" else np.int64),
                                   b.astype(np.float64 if b.dtype.kind == "f" else np.int64))
    n = a64.shape[-1]
    lab = LETTERS[: a64.ndim]
    return O.einsum(f"{lab},{lab}->{lab[:-1]}", strided(np.ascontiguousarray(a64)),
                    strided(np.ascontiguousarray(b64))).values() if n else np.zeros(a64.shape[:-1])


@pytest.mark.parametrize("case", CASES, ids=[f"{c['op']}-{i}" for i, c in enumerate(CASES)])
def test_oracle_matches_reference_contraction_kat(case):
    dt = {"f64": np.float64, "i64": np.int64, "i32": np.int64}[case["dtype"]]
    a, b = operand(case, "a", dt), operand(case, "b", dt)
    if case["op"] == "tensordot":
        got = O.einsum(tensordot_subscripts(a.ndim, b.ndim, case["axes"]), strided(a), strided(b)).values()
    else:
        got = oracle_vecdot(a, b)
    np.testing.assert_allclose(got, np.array(case["expect"], dtype=np.float64), rtol=case.get("tol", 0), atol=0,
                               err_msg=case["src"])


@pytest.mark.parametrize("sub,shapes", [
    ("ij,jk->ik", [(5, 7), (7, 3)]),
    ("bij,bjk->bik", [(3, 4, 5), (3, 5, 2)]),
    ("ij,jk,kl->il", [(3, 4), (4, 5), (5, 2)]),
    ("ii->", [(6, 6)]),
    ("ii->i", [(6, 6)]),
    ("iij,jk->ik", [(3, 3, 4), (4, 2)]),
    ("ij->", [(4, 5)]),
    ("i,j->ij", [(4,), (3,)]),
    ("ij,kj", [(3, 4), (5, 4)]),
])
def test_oracle_einsum_matches_numpy(sub, shapes):
    rng = np.random.default_rng(len(sub))
    arrs = [rng.standard_normal(s) for s in shapes]
    got = O.einsum(sub, *[strided(x) for x in arrs]).values()
    np.testing.assert_allclose(got, np.einsum(sub, *arrs), rtol=1e-13, atol=1e-13)


def test_tensordot_labels_follow_the_reference_doc_example():
    # rstsr-common/src/tensordot_to_einsum.rs:13-15: (2, 2, ([1], [0])) -> "ba,ac->bc"
    assert tensordot_subscripts(2, 2, ([1], [0])) == "ba,ac->bc"


def _shape(lib, sub, layouts):
    from rstsr_gb300._lib import MAX_NDIM, Layout

    n = len(layouts)
    lays = (Layout * n)(*[Layout.make(s, O.c_strides(s)) for s in layouts])
    nd = C.c_int32()
    shp = (C.c_int64 * MAX_NDIM)()
    rc = lib.rstsr_cuda_einsum_output_shape(sub.encode("utf-8"), n, lays, C.byref(nd), shp)
    return rc, tuple(shp[i] for i in range(nd.value))


def test_library_parses_subscripts(built_lib):
    assert _shape(built_lib, "ij,jk->ik", [(2, 3), (3, 4)]) == (0, (2, 4))
    assert _shape(built_lib, "ij,jk", [(2, 3), (3, 4)]) == (0, (2, 4))          # implicit: i, k
    assert _shape(built_lib, "ji,jk", [(3, 2), (3, 4)]) == (0, (2, 4))
    assert _shape(built_lib, " ab , bc -> ca ", [(2, 3), (3, 5)]) == (0, (5, 2))
    assert _shape(built_lib, "μi,νa,μνκλ,κj,λb->iajb", [(3, 2)] * 2 + [(3, 3, 3, 3)] + [(3, 2)] * 2) == \
        (0, (2, 2, 2, 2))
    assert _shape(built_lib, "ii->i", [(4, 4)]) == (0, (4,))
    assert _shape(built_lib, "ij,jk->ik", [(2, 3), (4, 4)])[0] == 1               # extents disagree
    assert _shape(built_lib, "ij,jk->iq", [(2, 3), (3, 4)])[0] == 2               # label in no operand
    assert _shape(built_lib, "ij,jk->ii", [(2, 3), (3, 4)])[0] == 2               # repeated output label
    assert _shape(built_lib, "ij->ij", [(2, 3), (3, 4)])[0] == 2                  # operand count
    assert _shape(built_lib, "...i->i", [(2, 3)])[0] == 7                         # ellipsis
