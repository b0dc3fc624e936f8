"""The library's layout algebra (host-only exports) and the oracle's
restatement (oracle/layout.py) reproduce the reference's own layout unit tests
(tests/golden/layout_kats.json, from rstsr-common/src/layout/{layoutbase,
matmul, broadcast}.rs and rstsr-core/src/device_faer/matmul.rs): contiguity
and preference flags, matmul output layouts in both orders, broadcast shapes,
strides and failures (CPU only)."""

import ctypes as C
import json
from pathlib import Path

import pytest

from oracle import layout as OL

CASES = json.loads((Path(__file__).resolve().parent / "golden" / "layout_kats.json").read_text())
FLAG_BIT = {"c_contig": 1, "f_contig": 2, "c_prefer": 4, "f_prefer": 8}
ORACLE_FLAG = {"c_contig": OL.c_contig, "f_contig": OL.f_contig, "c_prefer": OL.c_prefer, "f_prefer": OL.f_prefer}


def L(lay):
    from rstsr_gb300._lib import Layout

    return Layout.make(lay[0], lay[1], lay[2])


def T(l):
    return [list(l.shape_t), list(l.stride_t), l.offset]


def _ids(c):
    return f"{c['op']}-{c.get('flag', c.get('order', ''))}-{c['src'].split(':')[1]}"


def test_fixture_size():
    assert len(CASES) == 62
    assert {c["op"] for c in CASES} == {"flag", "matmul_layout", "broadcast"}


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_library_reproduces_reference_layout_kat(built_lib, case):
    order = 0 if case.get("order", "C") == "C" else 1
    if case["op"] == "flag":
        got = built_lib.rstsr_cuda_layout_flags(C.byref(L(case["layout"])))
        assert bool(got & FLAG_BIT[case["flag"]]) is case["expect"], (case["src"], got)
    elif case["op"] == "matmul_layout":
        lc = L([[], [], 0])
        rc = built_lib.rstsr_cuda_matmul_layout(C.byref(L(case["la"])), C.byref(L(case["lb"])), order, C.byref(lc))
        if "expect" in case:
            assert rc == 0 and T(lc) == case["expect"], (case["src"], rc, T(lc))
        else:
            assert rc == 0 and T(lc)[0] == case["expect_shape"], (case["src"], rc, T(lc))
    else:
        oa, ob = L([[], [], 0]), L([[], [], 0])
        rc = built_lib.rstsr_cuda_layout_broadcast(C.byref(L(case["la"])), C.byref(L(case["lb"])), order,
                                                   C.byref(oa), C.byref(ob))
        if case["expect_shape"] is None:
            assert rc != 0, case["src"]
            return
        assert rc == 0 and T(oa)[0] == case["expect_shape"] and T(ob)[0] == case["expect_shape"], case["src"]
        if "expect_a" in case:
            assert T(oa)[1] == case["expect_a"] and T(ob)[1] == case["expect_b"], (case["src"], T(oa), T(ob))


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_oracle_reproduces_reference_layout_kat(case):
    if case["op"] == "flag":
        shape, stride, _ = case["layout"]
        assert bool(ORACLE_FLAG[case["flag"]](tuple(shape), tuple(stride))) is case["expect"], case["src"]
    elif case["op"] == "matmul_layout":
        shape = OL.matmul_shape(tuple(case["la"][0]), tuple(case["lb"][0]), case["order"])
        assert list(shape) == case.get("expect", [case.get("expect_shape")])[0], case["src"]
    else:
        la = tuple(case["la"][0]), tuple(case["la"][1]), 0
        lb = tuple(case["lb"][0]), tuple(case["lb"][1]), 0
        if case["expect_shape"] is None:
            with pytest.raises(ValueError):
                OL.broadcast_layout(la, lb, case["order"])
            return
        wa, wb = OL.broadcast_layout(la, lb, case["order"])
        assert list(wa[0]) == case["expect_shape"], case["src"]
        if "expect_a" in case:
            assert list(wa[1]) == case["expect_a"] and list(wb[1]) == case["expect_b"], case["src"]
