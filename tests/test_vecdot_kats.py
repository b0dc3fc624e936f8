"""The vecdot oracle (oracle_vecdot: the einsum oracle over numpy-broadcast
operands, which the GPU vecdot tests compare the device with) reproduces the
reference's vecdot known-answer tests (tests/golden/vecdot_kats.json, from
rstsr-core/tests/core_func/linalg/test_vecdot.rs): broadcasting of the
remaining axes, a contracted axis other than the last, the empty contraction
and strided operands (CPU only)."""

import json
from pathlib import Path

import numpy as np
import pytest

from tests.test_contraction_oracle import oracle_vecdot

CASES = json.loads((Path(__file__).resolve().parent / "golden" / "vecdot_kats.json").read_text())


def _operand(case, key):
    start, stop, shape = case[key]
    x = np.arange(start, stop, dtype=np.int32).reshape(shape)
    if case.get(key + "_view") == "step2":
        x = x[..., ::2]
    if case.get("transpose"):
        x = x.T
    return x


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["src"].split(":")[1])
def test_oracle_vecdot_reproduces_reference_kat(case):
    a, b = _operand(case, "a"), _operand(case, "b")
    ax = case["axis"]
    a, b = np.moveaxis(a, ax, -1), np.moveaxis(b, ax, -1)
    got = oracle_vecdot(a, b)
    assert np.asarray(got).astype(np.int64).tolist() == case["expect"], case["src"]
