"""The reference's reshape-through-copy and vecdot known-answer tests run on the
device: tests/golden/reshape_kats.json (rstsr-core/tests/core_func/
manipulation/test_reshape.rs, C and F walks of contiguous, transposed and
strided sources through rstsr_cuda_assign_arbitrary) and
tests/golden/vecdot_kats.json (rstsr-core/tests/core_func/linalg/
test_vecdot.rs: broadcasting of the remaining axes, a contracted axis other
than the last, the empty contraction, step-2 operands). Integer results are
compared exactly with the reference's expected values."""

import json
from pathlib import Path

import numpy as np
import pytest

import rstsr_gb300 as rt

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
RESHAPE = json.loads((GOLDEN / "reshape_kats.json").read_text())
VECDOT = json.loads((GOLDEN / "vecdot_kats.json").read_text())


@pytest.mark.parametrize("case", RESHAPE, ids=lambda c: f"{c['order']}-{c['src'].split(':')[1]}")
def test_device_reshape_kat(dev, case):
    buf = np.array(case["buf"], dtype=np.int32)
    shape, stride, off = case["view"]
    t = rt.from_host_layout(buf, tuple(shape), tuple(stride), off, dev)
    got = t.reshape(case["shape"], order=case["order"])
    assert got.to_numpy().tolist() == case["expect"], case["src"]


def _operand(dev, case, key):
    start, stop, shape = case[key]
    x = rt.asarray(np.arange(start, stop, dtype=np.int64).reshape(shape), dev)
    if case.get(key + "_view") == "step2":
        x = x.i((Ellipsis, slice(None, None, 2)))
    if case.get("transpose"):
        x = x.t()
    return x


@pytest.mark.parametrize("case", VECDOT, ids=lambda c: c["src"].split(":")[1])
def test_device_vecdot_kat(dev, case):
    a, b = _operand(dev, case, "a"), _operand(dev, case, "b")
    got = rt.vecdot(a, b, case["axis"]).to_numpy()
    assert np.asarray(got).astype(np.int64).tolist() == case["expect"], case["src"]
