"""The oracle's assign_arbitrary (the C- or F-order walk the device's
rstsr_cuda_assign_arbitrary is compared with) and numpy's ordered reshape (the
reference the GPU reshape-walk test uses) both reproduce the reference's
reshape-through-copy known-answer tests (tests/golden/reshape_kats.json, from
rstsr-core/tests/core_func/manipulation/test_reshape.rs) (CPU only)."""

import json
from pathlib import Path

import numpy as np
import pytest

from oracle import layout as OL
from oracle import oracle as O

CASES = json.loads((Path(__file__).resolve().parent / "golden" / "reshape_kats.json").read_text())


def _ids(c):
    return f"{c['order']}-{c['src'].split(':')[1]}"


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_oracle_walk_reproduces_reference_reshape(case):
    buf = np.array(case["buf"], dtype=np.int32)
    shape, stride, off = case["view"]
    src = O.Strided(buf, tuple(shape), tuple(stride), off)
    order = 0 if case["order"] == "C" else 1
    st = OL.c_stride(case["shape"]) if order == 0 else OL.f_stride(case["shape"])
    dst = O.empty_strided(tuple(case["shape"]), st, np.int32)
    O.assign_arbitrary(dst, src, order)
    assert dst.values().tolist() == case["expect"], case["src"]


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_numpy_ordered_reshape_reproduces_reference_reshape(case):
    buf = np.array(case["buf"], dtype=np.int32)
    shape, stride, off = case["view"]
    view = np.lib.stride_tricks.as_strided(buf[off:], shape=shape, strides=[s * buf.itemsize for s in stride])
    got = np.reshape(view, case["shape"], order=case["order"])
    assert got.tolist() == case["expect"], case["src"]
