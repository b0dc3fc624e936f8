"""The device's element-wise operators reproduce the reference's own
known-answer tests (tests/golden/elementwise_kats.json, from
rstsr-core/tests/core_func/{operators/test_comparison.rs, math/test_unary_math.rs}),
with the reference's own comparisons."""

import pytest

import rstsr_gb300 as rt
from tests.test_elementwise_kats import CASES, check, operands

pytestmark = pytest.mark.gpu

CMP = {"gt": "greater", "ge": "greater_equal", "lt": "less", "le": "less_equal", "eq": "equal", "ne": "not_equal"}
PRED = ("isnan", "isfinite", "isinf")


def run(case, dev):
    ts = [rt.asarray(x, dev) for x in operands(case)]
    op = case["op"]
    if op in CMP:
        return rt.compare(CMP[op], ts[0], ts[1])
    if op in ("maximum", "minimum"):
        return rt.binary(op, ts[0], ts[1])
    if op in PRED:
        return rt.predicate(op, ts[0])
    return rt.unary(op, ts[0])


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['op']}-{c['dtype']}-{c['src'].split(':')[1]}")
def test_device_reproduces_reference_kat(dev, case):
    check(case, run(case, dev).to_numpy())
