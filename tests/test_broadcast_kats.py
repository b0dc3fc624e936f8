"""The library's broadcasting rule (rstsr_cuda_layout_broadcast, the planner
every element-wise operator uses) and the oracle's both reproduce the
reference's broadcast_shapes known-answer tests
(tests/golden/broadcast_kats.json, from
rstsr-core/tests/core_func/manipulation/test_broadcast_shapes.rs), row- and
column-major (host-only, CPU).

broadcast_shapes folds the shapes pairwise with broadcast_shape
(rstsr-core/src/tensor/manipulation/broadcast.rs:104-120); the folds below do
the same through each implementation.
"""

import ctypes as C
import json
from pathlib import Path

import pytest

from oracle import layout as OL

CASES = json.loads((Path(__file__).resolve().parent / "golden" / "broadcast_kats.json").read_text())


def _contig(shape, order):
    return OL.c_stride(shape) if order == "C" else OL.f_stride(shape)


def fold(shapes, order, pair):
    if not shapes:
        return ()
    result = tuple(shapes[0])
    for s in shapes[1:]:
        result = pair(tuple(s), result, order)
    return result


def oracle_pair(sa, sb, order):
    out, _ = OL.broadcast_layout((sa, _contig(sa, order), 0), (sb, _contig(sb, order), 0), order)
    return out[0]


def library_pair(lib):
    from rstsr_gb300._lib import Layout

    def pair(sa, sb, order):
        oa, ob = Layout.make((), ()), Layout.make((), ())
        rc = lib.rstsr_cuda_layout_broadcast(C.byref(Layout.make(sa, _contig(sa, order))),
                                             C.byref(Layout.make(sb, _contig(sb, order))),
                                             0 if order == "C" else 1, C.byref(oa), C.byref(ob))
        if rc != 0:
            raise ValueError(f"broadcast failed ({rc})")
        assert oa.shape_t == ob.shape_t
        return oa.shape_t

    return pair


def _ids(c):
    return f"{c['order']}-{len(c['shapes'])}-{c['src'].split(':')[1]}"


def test_fixture_size():
    assert len(CASES) == 43
    assert sum(c["expect"] is None for c in CASES) == 8


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_oracle_broadcast_shapes(case):
    if case["expect"] is None:
        with pytest.raises(ValueError):
            fold(case["shapes"], case["order"], oracle_pair)
    else:
        assert fold(case["shapes"], case["order"], oracle_pair) == tuple(case["expect"])


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_library_broadcast_shapes(built_lib, case):
    pair = library_pair(built_lib)
    if case["expect"] is None:
        with pytest.raises(ValueError):
            fold(case["shapes"], case["order"], pair)
    else:
        assert fold(case["shapes"], case["order"], pair) == tuple(case["expect"])
