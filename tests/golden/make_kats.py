"""Writes reference_kats.json and the fixtures beside it (tri_index,
contraction, elementwise, broadcast, reshape, vecdot, creation, layout):
known-answer cases transcribed from the reference's own test suite (RESTGroup/rstsr, paths relative to its workspace).

Each case names the file:line it comes from. Integer literals in the
reference's `tensor_from_nested!` are i32; `arange` defaults to i32 for integer
ranges in these tests. Run:  python tests/golden/make_kats.py
"""

import json
import math
from pathlib import Path

B3 = [[3, 6, 9], [4, 10, 5], [8, 3, 2]]
A23 = [[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]]
P34 = [[1, 2, 3, 4], [5, 6, 7, 9], [10, 3, 4, 5]]
CN = [[0, 1, 7, 0, 0], [3, 0, 0, 2, 19]]

CASES = [
    # ----------------------------------------------------------- argmax / argmin
    *[
        dict(src="rstsr-core/tests/core_func/reduction/test_argmax.rs:24-38", op="argmax_all", dtype="i32", a=a, expect=e)
        for a, e in [
            ([1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0], 0),
            ([3, 3, 3, 3, 2, 2, 2, 2], 0),
            ([0, 1, 2, 3, 4, 5, 6, 7], 7),
            ([7, 6, 5, 4, 3, 2, 1, 0], 0),
        ]
    ],
    dict(src="rstsr-core/tests/core_func/reduction/test_argmax.rs:72-78", op="argmax_axes", dtype="i32", a=B3, axes=[0],
         expect=[2, 1, 0]),
    dict(src="rstsr-core/tests/core_func/reduction/test_argmax.rs:72-78", op="argmax_axes", dtype="i32", a=B3, axes=[1],
         expect=[2, 1, 0]),
    *[
        dict(src="rstsr-core/tests/core_func/reduction/test_argmin.rs:20-34", op="argmin_all", dtype="i32", a=a, expect=e)
        for a, e in [
            ([1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0], 8),
            ([3, 3, 3, 3, 2, 2, 2, 2], 4),
            ([0, 1, 2, 3, 4, 5, 6, 7], 0),
            ([7, 6, 5, 4, 3, 2, 1, 0], 7),
        ]
    ],
    dict(src="rstsr-core/tests/core_func/reduction/test_argmin.rs:46-52", op="argmin_axes", dtype="i32", a=B3, axes=[1],
         expect=[0, 0, 2]),
    # ----------------------------------------------------------------- sums
    dict(src="rstsr-core/tests/core_func/reduction/test_sum.rs:24-33", op="sum_axes", dtype="i32",
         a=[[1, 2, 3], [4, 5, 6], [7, 8, 9]], axes=[1], expect=[6, 15, 24]),
    dict(src="rstsr-core/tests/core_func/reduction/test_sum.rs:44-50", op="sum_all", dtype="i32",
         a=[[1, 2, 3], [4, 5, 6], [7, 8, 9]], expect=45),
    dict(src="rstsr-core/tests/core_func/reduction/test_sum.rs:52-62", op="sum_axes", dtype="i32",
         a=list(range(24)), shape=[2, 3, 4], axes=[-2, -1], expect=[66, 210]),
    dict(src="rstsr-core/tests/core_func/reduction/test_sum.rs:64-73", op="sum_all", dtype="i32",
         a=[[1, 2, 3], [4, 5, 6]], expect=21),
    # ------------------------------------------------------------ mean/var/std
    dict(src="rstsr-core/tests/core_func/reduction/test_mean.rs:19-30", op="mean_all", dtype="f64", a=A23, expect=3.5),
    dict(src="rstsr-core/tests/core_func/reduction/test_mean.rs:19-30", op="mean_axes", dtype="f64", a=A23, axes=[0],
         expect=[2.5, 3.5, 4.5]),
    dict(src="rstsr-core/tests/core_func/reduction/test_mean.rs:19-30", op="mean_axes", dtype="f64", a=A23, axes=[1],
         expect=[2.0, 5.0]),
    dict(src="rstsr-core/tests/core_func/reduction/test_var.rs:20-33", op="var_all", dtype="f64", a=A23,
         expect=2.9166666666666665),
    dict(src="rstsr-core/tests/core_func/reduction/test_var.rs:20-33", op="var_axes", dtype="f64", a=A23, axes=[0],
         expect=[2.25, 2.25, 2.25]),
    dict(src="rstsr-core/tests/core_func/reduction/test_var.rs:20-33", op="var_axes", dtype="f64", a=A23, axes=[1],
         expect=[0.6666666666666666, 0.6666666666666666]),
    dict(src="rstsr-core/tests/core_func/reduction/test_std.rs:20-33", op="std_all", dtype="f64", a=A23,
         expect=1.707825127659933),
    dict(src="rstsr-core/tests/core_func/reduction/test_std.rs:20-33", op="std_axes", dtype="f64", a=A23, axes=[0],
         expect=[1.5, 1.5, 1.5]),
    dict(src="rstsr-core/tests/core_func/reduction/test_std.rs:20-33", op="std_axes", dtype="f64", a=A23, axes=[1],
         expect=[0.816496580927726, 0.816496580927726]),
    # ------------------------------------------------------------- min / max
    dict(src="rstsr-core/tests/core_func/reduction/test_max.rs:18-32", op="max_all", dtype="f64",
         a=[3.0, 4.0, 5.0, 10.0, -3.0, -5.0, 6.0], expect=10.0),
    dict(src="rstsr-core/tests/core_func/reduction/test_max.rs:18-32", op="max_axes", dtype="f64",
         a=[[3.0, 6.0, 9.0], [4.0, 10.0, 5.0], [8.0, 3.0, 2.0]], axes=[0], expect=[8.0, 10.0, 9.0]),
    dict(src="rstsr-core/tests/core_func/reduction/test_max.rs:18-32", op="max_axes", dtype="f64",
         a=[[3.0, 6.0, 9.0], [4.0, 10.0, 5.0], [8.0, 3.0, 2.0]], axes=[1], expect=[9.0, 10.0, 8.0]),
    dict(src="rstsr-core/tests/core_func/reduction/test_min.rs:18-32", op="min_all", dtype="f64",
         a=[3.0, 4.0, 5.0, 10.0, -3.0, -5.0, 6.0], expect=-5.0),
    dict(src="rstsr-core/tests/core_func/reduction/test_min.rs:18-32", op="min_axes", dtype="f64",
         a=[[3.0, 6.0, 9.0], [4.0, 10.0, 5.0], [8.0, 3.0, 2.0]], axes=[0], expect=[3.0, 3.0, 2.0]),
    dict(src="rstsr-core/tests/core_func/reduction/test_min.rs:18-32", op="min_axes", dtype="f64",
         a=[[3.0, 6.0, 9.0], [4.0, 10.0, 5.0], [8.0, 3.0, 2.0]], axes=[1], expect=[3.0, 4.0, 2.0]),
    # ------------------------------------------------------------------ prod
    dict(src="rstsr-core/tests/core_func/reduction/test_prod.rs:18-28", op="prod_axes", dtype="i32", a=P34, axes=[-1],
         expect=[24, 1890, 600]),
    dict(src="rstsr-core/tests/core_func/reduction/test_prod.rs:31-46", op="prod_all", dtype="i32",
         a=[1, 2, 10, 11, 6, 5, 4], expect=26400),
    dict(src="rstsr-core/tests/core_func/reduction/test_prod.rs:31-46", op="prod_axes", dtype="i32", a=P34, axes=[0],
         expect=[50, 36, 84, 180]),
    dict(src="rstsr-core/tests/core_func/reduction/test_prod.rs:55-63", op="prod_all", dtype="i32",
         a=[[1, 2, 3], [4, 5, 6]], expect=720),
    # ------------------------------------------------------------- all / any
    dict(src="rstsr-core/tests/core_func/reduction/test_all.rs:19-34", op="all_all", dtype="bool",
         a=[False, True, True, False], expect=False),
    dict(src="rstsr-core/tests/core_func/reduction/test_all.rs:19-34", op="all_all", dtype="bool",
         a=[True, True, True, True], expect=True),
    dict(src="rstsr-core/tests/core_func/reduction/test_all.rs:19-34", op="all_all", dtype="bool",
         a=[False, False, False, False], expect=False),
    dict(src="rstsr-core/tests/core_func/reduction/test_all.rs:38-50", op="all_axes", dtype="bool",
         a=[[False, False, True], [False, True, True], [True, True, True]], axes=[0], expect=[False, False, True]),
    dict(src="rstsr-core/tests/core_func/reduction/test_all.rs:38-50", op="all_axes", dtype="bool",
         a=[[False, False, True], [False, True, True], [True, True, True]], axes=[1], expect=[False, False, True]),
    dict(src="rstsr-core/tests/core_func/reduction/test_any.rs:19-31", op="any_all", dtype="bool",
         a=[False, False, True, False], expect=True),
    dict(src="rstsr-core/tests/core_func/reduction/test_any.rs:19-31", op="any_all", dtype="bool",
         a=[False, False, False, False], expect=False),
    dict(src="rstsr-core/tests/core_func/reduction/test_any.rs:35-47", op="any_axes", dtype="bool",
         a=[[False, False, False], [False, True, False], [True, True, False]], axes=[0], expect=[True, True, False]),
    dict(src="rstsr-core/tests/core_func/reduction/test_any.rs:35-47", op="any_axes", dtype="bool",
         a=[[False, False, False], [False, True, False], [True, True, False]], axes=[1], expect=[False, True, True]),
    # --------------------------------------------------------- count_nonzero
    dict(src="rstsr-core/tests/core_func/reduction/test_count_nonzero.rs:18-28", op="count_nonzero_axes", dtype="i32",
         a=CN, axes=[1], expect=[2, 3]),
    dict(src="rstsr-core/tests/core_func/reduction/test_count_nonzero.rs:36-44", op="count_nonzero_all", dtype="i32",
         a=CN, expect=5),
    # ------------------------------------------------------------- to_contig
    dict(src="rstsr-core/tests/core_func/manipulation/test_to_contig.rs:56-80", op="to_contig", dtype="i32",
         a=list(range(12)), shape=[3, 4], view=dict(transpose=[1, 0]),
         expect=[[0, 4, 8], [1, 5, 9], [2, 6, 10], [3, 7, 11]]),
    dict(src="rstsr-core/tests/core_func/manipulation/test_to_contig.rs:82-101", op="to_contig", dtype="i32",
         a=list(range(24)), shape=[4, 6], view=dict(slice=[[None, None, 2], [None, None, 2]]),
         view_stride=[12, 2], expect=[[0, 2, 4], [12, 14, 16]]),
    dict(src="rstsr-core/tests/core_func/manipulation/test_to_contig.rs:270-287", op="to_contig", dtype="i32",
         a=list(range(12)), shape=[3, 4], view=dict(flip=0),
         expect=[[8, 9, 10, 11], [4, 5, 6, 7], [0, 1, 2, 3]]),
    # ------------------------------------------------------------ arithmetic
    dict(src="rstsr-core/tests/core_func/operators/test_arithmetic.rs:14-22", op="add", dtype="i32",
         a=[[1, 2], [3, 4]], b=[[10, 20], [30, 40]], expect=[[11, 22], [33, 44]]),
    dict(src="rstsr-core/tests/core_func/operators/test_arithmetic.rs:24-31", op="add", dtype="i32",
         a=[[1, 2, 3], [4, 5, 6]], b=[10, 20, 30], expect=[[11, 22, 33], [14, 25, 36]]),
    dict(src="rstsr-core/tests/core_func/operators/test_arithmetic.rs:36-44", op="sub", dtype="i32",
         a=[[10, 20], [30, 40]], b=[[1, 2], [3, 4]], expect=[[9, 18], [27, 36]]),
    dict(src="rstsr-core/tests/core_func/operators/test_arithmetic.rs:49-57", op="mul", dtype="i32",
         a=[[1, 2], [3, 4]], b=[10, 100], expect=[[10, 200], [30, 400]]),
    dict(src="rstsr-core/tests/core_func/operators/test_arithmetic.rs:62-72", op="div", dtype="f64",
         a=[[10.0, 20.0], [30.0, 40.0]], b=[[2.0, 4.0], [5.0, 8.0]], expect=[[5.0, 5.0], [6.0, 5.0]]),
    dict(src="rstsr-core/tests/core_func/operators/test_arithmetic.rs:77-92", op="rem", dtype="i32",
         a=[[10, 21], [33, 44]], b=[[3, 4], [5, 7]], expect=[[1, 1], [3, 2]]),
    # ---------------------------------------------------------------- matmul
    dict(src="rstsr-core/tests/core_func/operators/test_arithmetic.rs:77-92", op="matmul", dtype="i32",
         a=[[10, 21], [33, 44]], b=[[3, 4], [5, 7]], expect=[[135, 187], [319, 440]]),
    dict(src="rstsr-core/tests/core_func/linalg/test_matmul.rs:17-31", op="matmul", dtype="i32",
         a=[1, 2], b=[[3], [4]], expect=[11]),
    dict(src="rstsr-core/tests/core_func/linalg/test_matmul.rs:17-31", op="matmul", dtype="i32",
         a=[[3], [4]], b=[[1, 2]], expect=[[3, 6], [4, 8]]),
    dict(src="rstsr-core/tests/core_func/linalg/test_matmul.rs:34-43", op="matmul", dtype="i32",
         a=[1, 2], b=[[1, 2], [3, 4]], expect=[7, 10]),
    dict(src="rstsr-core/tests/core_func/linalg/test_matmul.rs:46-55", op="matmul", dtype="i32",
         a=[[1, 2], [3, 4]], b=[1, 2], expect=[5, 11]),
    dict(src="rstsr-core/tests/core_func/linalg/test_matmul.rs:58-70", op="matmul", dtype="i32",
         a=[[1, 2], [3, 4]], b=[[1, 0], [1, 1]], expect=[[3, 2], [7, 4]]),
    dict(src="rstsr-core/tests/core_func/linalg/test_matmul.rs:58-70", op="matmul", dtype="i32",
         a=[[1, 0], [1, 1]], b=[[1, 2], [3, 4]], expect=[[1, 2], [4, 6]]),
    dict(src="rstsr-core/tests/core_func/linalg/test_matmul.rs:75-90", op="matmul", dtype="i32",
         a=[[[1, 2], [3, 4]], [[1, 0], [1, 1]]], b=[[1, 2], [3, 4]], expect=[[[7, 10], [15, 22]], [[1, 2], [4, 6]]]),
    dict(src="rstsr-core/src/tensor/linalg/matmul.rs:366-374", op="matmul_from", dtype="f64",
         a=[float(x) for x in range(15)], shape_a=[3, 5], b=[float(x) for x in range(20)], shape_b=[5, 4],
         c=[float(x) for x in range(12)], shape_c=[3, 4], alpha=2.0, beta=1.5,
         expect=[240.0, 261.5, 283.0, 304.5, 646.0, 717.5, 789.0, 860.5, 1052.0, 1173.5, 1295.0, 1416.5]),
    dict(src="crates-device/rstsr-openblas/tests/test_workable.rs:14-27", op="batched_linspace_stats", dtype="f64",
         n=1048576, shape=[16, 256, 256], a_range=[0.0, 1.0], b_range=[1.0, 2.0],
         expect=dict(mean_all=213.2503660477036, std_all=148.88523481701804), tol=1e-6),
    # ---------------------------------------------------------- layout algebra
    dict(src="rstsr-common/src/layout/rearrangement.rs:466-496", op="greedy_layout", keep_shape=False,
         shape=[5, 1, 2, 1, 3, 6], stride=[1000, 10, 10, 40, 0, 100],
         expect=dict(shape=[2, 6, 5, 1, 1, 1], stride=[10, 100, 1000, 0, 0, 0])),
    dict(src="rstsr-common/src/layout/rearrangement.rs:466-496", op="greedy_layout", keep_shape=True,
         shape=[5, 1, 2, 1, 3, 6], stride=[1000, 10, 10, 40, 0, 100],
         expect=dict(shape=[1, 1, 3, 2, 6, 5], stride=[10, 40, 0, 10, 100, 1000])),
    dict(src="rstsr-common/src/layout/rearrangement.rs:466-496", op="greedy_layout", keep_shape=True,
         shape=[2, 3, 4], stride=[12, 4, 1], expect=dict(shape=[4, 3, 2], stride=[1, 4, 12])),
    dict(src="rstsr-common/src/layout/rearrangement.rs:466-496", op="greedy_layout", keep_shape=False,
         shape=[2, 3, 4], stride=[1, 2, 6], expect=dict(shape=[2, 3, 4], stride=[1, 2, 6])),
]


# Triangular packing and index selection (the reference's own unit tests).
# `fingerprint` is rstsr-core/src/dev_utilities/mod.rs:48-68: the row-major
# flattening x of the result dotted with cos(0), cos(1), ..., cos(size-1).
SEL = [1, 2, 3, 5, 8, 13, 21, 34, 55, 89, 144, 233]
TRI_INDEX_CASES = [
    dict(src="rstsr-core/src/tensor/operators/op_tri.rs:192-208", op="pack_unpack", order="C", uplo="L",
         buf="arange48", shape=[3, 4, 4], layout="f", packed_slice=[1],
         expect_packed=[1.0, 4.0, 16.0, 7.0, 19.0, 31.0, 10.0, 22.0, 34.0, 46.0],
         symm="Sy", unpacked_slice=[0, 1], expect_unpacked=[3.0, 15.0, 18.0, 21.0]),
    dict(src="rstsr-core/src/tensor/operators/op_tri.rs:210-226", op="pack_unpack", order="F", uplo="U",
         buf="arange48", shape=[4, 4, 3], layout="c", packed_slice=[None, 1],
         expect_packed=[1.0, 4.0, 16.0, 7.0, 19.0, 31.0, 10.0, 22.0, 34.0, 46.0],
         symm="Sy", unpacked_slice=[None, 1, 0], expect_unpacked=[3.0, 15.0, 18.0, 21.0]),
    dict(src="rstsr-core/src/tensor/operators/op_tri.rs:253-268", op="pack_tril_c_vs_f", order="C",
         buf="arange16", shape=[4, 4], expect_packed=[0.0, 4.0, 5.0, 8.0, 9.0, 10.0, 12.0, 13.0, 14.0, 15.0]),
    *[
        dict(src="rstsr-core/src/tensor/adv_indexing.rs:209-219", op="index_select_fingerprint", order="C",
             linspace=[1.0, 24.0, 24], shape=[2, 3, 4], axis=ax, indices=[0, 0, 1, -1], expect=e, tol=1e-8)
        for ax, e in [(0, -31.94175930917264), (1, 3.5719025258942088), (2, -25.648600916145096)]
    ],
    *[
        dict(src="rstsr-core/src/tensor/adv_indexing.rs:220-231", op="index_select_fingerprint", order="F",
             linspace=[1.0, 24.0, 24], shape=[4, 3, 2], axis=ax, indices=[0, 0, 1, -1], expect=e, tol=1e-8)
        for ax, e in [(2, -31.94175930917264), (1, 3.5719025258942088), (0, -25.648600916145096)]
    ],
    *[
        dict(src="rstsr-core/src/tensor/adv_indexing.rs:242-254", op="index_select_fingerprint", order="C",
             linspace=[1.0, 2.0, 256 * 256 * 256], shape=[256, 256, 256], axis=ax, indices=SEL, expect=e, tol=1e-10)
        for ax, e in [(0, 0.9357016252766746), (1, 1.012193909979973), (2, 1.010735112247236)]
    ],
    dict(src="rstsr-core/src/tensor/adv_indexing.rs:233-238", op="index_select", dtype="f64",
         a=[1.0, 2.0, 3.0, 4.0], axis=0, indices=[], expect=[]),
    dict(src="rstsr-core/tests/core_func/indexing/test_indexing.rs:96-107", op="index_select", dtype="i32",
         a=list(range(10)), axis=0, indices=[2, 4, 8], expect=[2, 4, 8]),
]


# Contractions: tensordot (through TBLIS in the reference) and vecdot.
CONTRACTION_CASES = [
    dict(src="crates-plugin/rstsr-tblis/src/tensordot_impl.rs:81-92", op="tensordot", dtype="f64",
         a=[[1.0, 2.0], [3.0, 4.0]], b=[[5.0, 6.0], [7.0, 8.0]], axes=0,
         expect=[[[[5, 6], [7, 8]], [[10, 12], [14, 16]]], [[[15, 18], [21, 24]], [[20, 24], [28, 32]]]]),
    dict(src="crates-plugin/rstsr-tblis/src/tensordot_impl.rs:94-105", op="tensordot", dtype="f64",
         a_arange=60, a_shape=[3, 4, 5], b_arange=24, b_shape=[4, 3, 2], axes=[[1, 0], [0, 1]],
         expect=[[4400.0, 4730.0], [4532.0, 4874.0], [4664.0, 5018.0], [4796.0, 5162.0], [4928.0, 5306.0]]),
    dict(src="rstsr-core/src/tensor/linalg/vecdot.rs:418-424", op="vecdot", dtype="i64",
         a_arange=[0, 6], a_shape=[2, 3], b_arange=[6, 12], b_shape=[2, 3], expect=[23, 122]),
    dict(src="rstsr-core/src/tensor/linalg/vecdot.rs:426-430", op="vecdot", dtype="f64",
         a=[[0.0, 5.0, 0.0], [0.0, 0.0, 10.0], [0.0, 6.0, 8.0]], b=[0.0, 0.6, 0.8], expect=[3.0, 8.0, 10.0],
         tol=1e-12),
    dict(src="rstsr-core/tests/doc_draft/linalg/test_vecdot.rs:18-23", op="vecdot", dtype="i32",
         a=[1, 2, 3], b=[4, 5, 6], expect=32),
    dict(src="rstsr-core/tests/doc_draft/linalg/test_vecdot.rs:25-32", op="vecdot", dtype="i32",
         a=[[1, 2], [3, 4]], b=[[5, 6], [7, 8]], expect=[17, 53]),
]

# Element-wise family (comparisons, maximum / minimum, unary math, classification).
# Non-finite values and negative zero are written as strings ("nan", "inf", "-inf",
# "-0.0") so the file stays plain JSON. `cmp`: "exact" for the reference's `to_vec()`
# equality, "bits" for exact values including the sign of zero and NaN-ness, "close"
# for its `assert_equal` (rt::allclose, rtol 1e-5, atol 1e-8).
_CMP = "rstsr-core/tests/core_func/operators/test_comparison.rs"
_UM = "rstsr-core/tests/core_func/math/test_unary_math.rs"
ELEMENTWISE_CASES = [
    *[
        dict(src=f"{_CMP}:{line}", op=op, dtype="i32", a=[1, 2, 3, 4], b=[2, 2, 2, 2], expect=e, cmp="exact")
        for op, line, e in [
            ("gt", 30, [False, False, True, True]),
            ("ge", 32, [False, True, True, True]),
            ("lt", 34, [True, False, False, False]),
            ("le", 36, [True, True, False, False]),
            ("eq", 38, [False, True, False, False]),
            ("ne", 40, [True, False, True, True]),
        ]
    ],
    dict(src=f"{_CMP}:58-61", op="maximum", dtype="i32", a=[1, 5, 3], b=[4, 2, 6], expect=[4, 5, 6], cmp="close"),
    dict(src=f"{_CMP}:58-63", op="minimum", dtype="i32", a=[1, 5, 3], b=[4, 2, 6], expect=[1, 2, 3], cmp="close"),
    dict(src=f"{_UM}:27-28", op="abs", dtype="i32", a=[-1, 2, -3], expect=[1, 2, 3], cmp="close"),
    dict(src=f"{_UM}:31-32", op="sqrt", dtype="f64", a=[0.0, 1.0, 4.0, 9.0], expect=[0.0, 1.0, 2.0, 3.0], cmp="close"),
    dict(src=f"{_UM}:35-36", op="sign", dtype="f64", a=[-2.0, 0.0, 3.0], expect=[-1.0, 0.0, 1.0], cmp="close"),
    dict(src=f"{_UM}:39-40", op="sign", dtype="i32", a=[-2, 0, 3], expect=[-1, 0, 1], cmp="exact"),
    dict(src=f"{_UM}:43-44", op="sign", dtype="u8", a=[0, 5], expect=[0, 1], cmp="exact"),
    dict(src=f"{_UM}:47-48", op="floor", dtype="f64", a=[-1.5, 0.5, 2.4], expect=[-2.0, 0.0, 2.0], cmp="close"),
    dict(src=f"{_UM}:47-49", op="ceil", dtype="f64", a=[-1.5, 0.5, 2.4], expect=[-1.0, 1.0, 3.0], cmp="close"),
    dict(src=f"{_UM}:47-50", op="trunc", dtype="f64", a=[-1.5, 0.5, 2.4], expect=[-1.0, 0.0, 2.0], cmp="close"),
    dict(src=f"{_UM}:62-69", op="sign", dtype="f64", a=["nan", "inf", "-inf", "-0.0", 0.0],
         expect=["nan", 1.0, -1.0, 0.0, 0.0], cmp="bits"),
    dict(src=f"{_UM}:87-93", op="exp", dtype="f64", a=[0.0, 1.0, 2.0], expect=[1.0, math.e, math.e * math.e],
         cmp="close"),
    dict(src=f"{_UM}:87-95", op="log", dtype="f64", a=[1.0, math.e, math.e * math.e], expect=[0.0, 1.0, 2.0],
         cmp="close"),
    dict(src=f"{_UM}:98-99", op="sin", dtype="f64", a=[0.0, math.pi / 2, math.pi], expect=[0.0, 1.0, 0.0],
         cmp="close"),
    dict(src=f"{_UM}:98-100", op="cos", dtype="f64", a=[0.0, math.pi / 2, math.pi], expect=[1.0, 0.0, -1.0],
         cmp="close"),
    dict(src=f"{_UM}:103-105", op="tanh", dtype="f64", a=[-1.0, 0.0, 1.0],
         expect=[-math.tanh(1.0), 0.0, math.tanh(1.0)], cmp="close"),
    *[
        dict(src=f"{_UM}:{line}", op=op, dtype="f64", a=[0.0, "nan", "inf", "-inf"], expect=e, cmp="exact")
        for op, line, e in [
            ("isnan", "122-123", [False, True, False, False]),
            ("isfinite", "122-124", [True, False, False, False]),
            ("isinf", "122-125", [False, False, True, True]),
        ]
    ],
]


# broadcast_shapes: the shape rule the element-wise operators broadcast by
# (order "C" aligns trailing axes, "F" leading axes); expect None = an error.
_BS = "rstsr-core/tests/core_func/manipulation/test_broadcast_shapes.rs"
BROADCAST_CASES = [
    *[
        dict(src=f"{_BS}:18-80", order="C", shapes=s, expect=e)
        for s, e in [
            ([], []), ([[]], []), ([[7]], [7]), ([[1, 2], [2]], [1, 2]), ([[1, 1]], [1, 1]),
            ([[1, 1], [3, 4]], [3, 4]), ([[6, 7], [5, 6, 1], [7], [5, 1, 7]], [5, 6, 7]), ([[5, 6, 1]], [5, 6, 1]),
            ([[1, 3], [3, 1]], [3, 3]), ([[1, 0], [0, 0]], [0, 0]), ([[0, 1], [0, 0]], [0, 0]),
            ([[1, 0], [0, 1]], [0, 0]), ([[1, 1], [0, 0]], [0, 0]), ([[1, 1], [1, 0]], [1, 0]),
            ([[1, 1], [0, 1]], [0, 1]), ([[], [0]], [0]), ([[0], [0, 0]], [0, 0]), ([[0], [0, 1]], [0, 0]),
            ([[1], [0, 0]], [0, 0]), ([[], [0, 0]], [0, 0]), ([[1, 1], [0]], [1, 0]), ([[1], [0, 1]], [0, 1]),
            ([[1], [1, 0]], [1, 0]), ([[], [1, 0]], [1, 0]), ([[], [0, 1]], [0, 1]), ([[1], [3]], [3]),
            ([[2], [3, 2]], [3, 2]),
        ]
    ],
    dict(src=f"{_BS}:84-87", order="C", shapes=[[1, 2]] * 32, expect=[1, 2]),
    dict(src=f"{_BS}:89-92", order="C", shapes=[[1, 2]] * 100, expect=[1, 2]),
    dict(src=f"{_BS}:94-97", order="C", shapes=[[2]] * 32, expect=[2]),
    *[
        dict(src=f"{_BS}:106-123", order="C", shapes=s, expect=None)
        for s in [
            [[3], [4]], [[2, 3], [2]], [[3], [3], [4]], [[1, 3, 4], [2, 3, 3]], [[1, 2], [3, 1], [3, 2], [10, 5]],
            [[2], [2, 3]],
        ]
    ],
    dict(src=f"{_BS}:126-130", order="C", shapes=[[2]] * 32 + [[3]] * 32, expect=None),
    dict(src=f"{_BS}:167-171", order="C", shapes=[[2]] * 32 + [[]], expect=[2]),
    dict(src=f"{_BS}:190-192", order="F", shapes=[[1, 6, 1, 8], [5, 1, 7]], expect=[5, 6, 7, 8]),
    dict(src=f"{_BS}:198-200", order="F", shapes=[[4, 5], [4]], expect=[4, 5]),
    dict(src=f"{_BS}:206-208", order="F", shapes=[[5, 3, 15], [5, 1, 15]], expect=[5, 3, 15]),
    dict(src=f"{_BS}:214-216", order="F", shapes=[[5, 3, 15], [5, 3]], expect=[5, 3, 15]),
    dict(src=f"{_BS}:220-222", order="F", shapes=[[3], [2, 1]], expect=None),
]


# reshape through a copy: the values of a (strided) source walked in C or F
# order into the target shape (assign_arbitrary). `buf` is the source storage,
# `view` = (shape, stride, offset) over it; `expect` is indexed [i][j].
_RS = "rstsr-core/tests/core_func/manipulation/test_reshape.rs"
_A43 = list(range(1, 13))
RESHAPE_CASES = [
    dict(src=f"{_RS}:22-27", buf=_A43, view=[[4, 3], [3, 1], 0], shape=[2, 6], order="C",
         expect=[[1, 2, 3, 4, 5, 6], [7, 8, 9, 10, 11, 12]]),
    dict(src=f"{_RS}:30-32", buf=_A43, view=[[4, 3], [3, 1], 0], shape=[3, 4], order="C",
         expect=[[1, 2, 3, 4], [5, 6, 7, 8], [9, 10, 11, 12]]),
    dict(src=f"{_RS}:35-37", buf=_A43, view=[[4, 3], [3, 1], 0], shape=[3, 4], order="F",
         expect=[[1, 10, 8, 6], [4, 2, 11, 9], [7, 5, 3, 12]]),
    dict(src=f"{_RS}:40-42", buf=_A43, view=[[3, 4], [1, 3], 0], shape=[3, 4], order="C",
         expect=[[1, 4, 7, 10], [2, 5, 8, 11], [3, 6, 9, 12]]),
    dict(src=f"{_RS}:55-59", buf=list(range(6)), view=[[6], [1], 0], shape=[2, 3], order="F",
         expect=[[0, 2, 4], [1, 3, 5]]),
    dict(src=f"{_RS}:63-67", buf=list(range(1, 9)), view=[[4], [2], 1], shape=[2, 2], order="F",
         expect=[[2, 6], [4, 8]]),
]


# vecdot along one axis with the remaining axes broadcast: `a` / `b` as
# (start, stop, shape) aranges or explicit nested lists, `a_view` / `b_view` a
# step-2 slice of the last axis, `axis` counted from the end.
_VD = "rstsr-core/tests/core_func/linalg/test_vecdot.rs"
VECDOT_CASES = [
    dict(src=f"{_VD}:25-29", a=[0, 6, [2, 3]], b=[0, 3, [1, 3]], axis=-1, expect=[5, 14]),
    dict(src=f"{_VD}:31-34", a=[0, 6, [2, 3]], b=[0, 3, [1, 3]], transpose=True, axis=-2, expect=[5, 14]),
    dict(src=f"{_VD}:49-53", a=[0, 4, [2, 1, 2]], b=[0, 4, [1, 2, 2]], axis=-1, expect=[[1, 3], [3, 13]]),
    dict(src=f"{_VD}:58-61", a=[0, 4, [2, 1, 2]], b=[0, 4, [2, 2]], axis=-1, expect=[[1, 3], [3, 13]]),
    dict(src=f"{_VD}:144-149", a=[0, 0, [0]], b=[0, 0, [0]], axis=-1,
         expect=0),
    dict(src=f"{_VD}:160-169", a=[0, 12, [3, 4]], b=[8, 20, [3, 4]], a_view="step2", b_view="step2", axis=-1,
         expect=[20, 132, 308]),
]


# Creation: arange (`args` = [stop] | [start, stop] | [start, stop, step]),
# linspace (`args` = [start, stop, num], `endpoint`), tril / triu (`k`).
# `expect` values, `expect_len`, `last_close` (|last - v| < 1e-9),
# `last_below` (last < v) or `error` (the reference's error kind).
_AR = "rstsr-core/tests/core_func/creation/test_arange.rs"
_LS = "rstsr-core/tests/core_func/creation/test_linspace.rs"
_TT = "rstsr-core/tests/core_func/creation/test_tril_triu.rs"
_TSER = "rstsr-core/src/device_cpu_serial/creation.rs"
_ONES2 = [[1, 1], [1, 1]]
_ONES3 = [[1, 1, 1], [1, 1, 1], [1, 1, 1]]
_A3D = [[[1, 1], [1, 1]], [[1, 1], [1, 0]], [[1, 1], [0, 0]]]
_M9 = [[1, 2, 3], [4, 5, 6], [7, 8, 9]]
CREATION_CASES = [
    dict(src=f"{_AR}:26-28", op="arange", dtype="i32", args=[3], expect_len=3),
    dict(src=f"{_AR}:27-30", op="arange", dtype="i32", args=[0, 3], expect_len=3),
    dict(src=f"{_AR}:31-32", op="arange", dtype="i32", args=[3, 9], expect_len=6),
    dict(src=f"{_AR}:45", op="arange", dtype="i32", args=[0, 10, 0], error="InvalidValue"),
    dict(src=f"{_AR}:46", op="arange", dtype="f64", args=[0.0, 10.0, 0.0], error="InvalidValue"),
    dict(src=f"{_AR}:62-63", op="arange", dtype="i32", args=[2, 10], expect=[2, 3, 4, 5, 6, 7, 8, 9]),
    dict(src=f"{_AR}:65-66", op="arange", dtype="i32", args=[1, 10, 3], expect=[1, 4, 7]),
    dict(src=f"{_AR}:68-69", op="arange", dtype="i32", args=[10, 0, -2], expect=[10, 8, 6, 4, 2]),
    dict(src="rstsr-core/src/feature_rayon/auto_impl/creation.rs:126-130", op="linspace", dtype="f64",
         args=[1.0, 5.0, 5], endpoint=True, expect=[1.0, 2.0, 3.0, 4.0, 5.0]),
    dict(src=f"{_LS}:23-25", op="linspace", dtype="f64", args=[0.0, 10.0, 50], endpoint=True, expect_len=50),
    dict(src=f"{_LS}:27-30", op="linspace", dtype="f64", args=[2.0, 10.0, 100], endpoint=True, last_close=10.0),
    dict(src=f"{_LS}:32-35", op="linspace", dtype="f64", args=[2.0, 10.0, 100], endpoint=False, last_below=10.0),
    dict(src=f"{_LS}:50-52", op="linspace", dtype="f64", args=[0.0, 1.0, 1], endpoint=True, expect=[0.0]),
    dict(src=f"{_LS}:69-71", op="linspace", dtype="f64", args=[0.0, 1.0, 5], endpoint=True,
         expect=[0.0, 0.25, 0.5, 0.75, 1.0]),
    dict(src=f"{_TT}:26-28", op="tril", dtype="i32", a=_ONES2, k=0, expect=[[1, 0], [1, 1]]),
    dict(src=f"{_TT}:26-30", op="triu", dtype="i32", a=_ONES2, k=0, expect=[[1, 1], [0, 1]]),
    dict(src=f"{_TT}:42-47", op="tril", dtype="i32", a=_A3D, k=0,
         expect=[[[1, 0], [1, 1]], [[1, 0], [1, 0]], [[1, 0], [0, 0]]]),
    dict(src=f"{_TT}:42-48", op="triu", dtype="i32", a=_A3D, k=0,
         expect=[[[1, 1], [0, 1]], [[1, 1], [0, 0]], [[1, 1], [0, 0]]]),
    dict(src=f"{_TT}:60-62", op="tril", dtype="i32", a=_ONES3, k=1, expect=[[1, 1, 0], [1, 1, 1], [1, 1, 1]]),
    dict(src=f"{_TT}:60-66", op="triu", dtype="i32", a=_ONES3, k=-1, expect=[[1, 1, 1], [1, 1, 1], [0, 1, 1]]),
    dict(src=f"{_TSER}:160-165", op="tril", dtype="i32", a=_M9, k=-1, expect=[[0, 0, 0], [4, 0, 0], [7, 8, 0]]),
    dict(src=f"{_TSER}:166-169", op="triu", dtype="i32", a=_M9, k=-1, expect=[[1, 2, 3], [4, 5, 6], [0, 8, 9]]),
]


# Layout algebra (rstsr-common/src/layout): contiguity / preference flags,
# matmul output layouts and broadcast layouts. Layouts are [shape, stride, offset].
_LB = "rstsr-common/src/layout/layoutbase.rs"
_LM = "rstsr-common/src/layout/matmul.rs"
_BR = "rstsr-common/src/layout/broadcast.rs"


def _cs(shape):
    st, acc = [], 1
    for d in reversed(shape):
        st.append(acc)
        acc *= max(d, 1)
    return st[::-1]


def _fs(shape):
    st, acc = [], 1
    for d in shape:
        st.append(acc)
        acc *= max(d, 1)
    return st


def _c(shape):
    return [list(shape), _cs(shape), 0]


def _f(shape):
    return [list(shape), _fs(shape), 0]


def _swap(lay, i, j):
    sh, st, off = [list(x) if isinstance(x, list) else x for x in lay]
    sh[i], sh[j] = sh[j], sh[i]
    st[i], st[j] = st[j], st[i]
    return [sh, st, off]


_S357 = [3, 5, 7]
LAYOUT_CASES = [
    *[dict(src=f"{_LB}:755-779", op="flag", flag="f_prefer", layout=lay, expect=e) for lay, e in [
        ([_S357, [1, 10, 100], 0], True), ([_S357, [1, 3, 15], 0], True), ([_S357, [1, 3, -15], 1000], False),
        ([_S357, [1, 21, 3], 0], False), ([_S357, [35, 7, 1], 0], False), ([_S357, [2, 6, 30], 0], False),
        ([[], [], 0], True), ([[2, 0, 4], [1, 10, 100], 0], True), ([[2, 1, 4], [1, 1, 2], 0], True)]],
    *[dict(src=f"{_LB}:782-806", op="flag", flag="c_prefer", layout=lay, expect=e) for lay, e in [
        ([_S357, [100, 10, 1], 0], True), ([_S357, [35, 7, 1], 0], True), ([_S357, [-35, 7, 1], 1000], False),
        ([_S357, [7, 21, 1], 0], False), ([_S357, [1, 3, 15], 0], False), ([_S357, [70, 14, 2], 0], False),
        ([[], [], 0], True), ([[2, 0, 4], [1, 10, 100], 0], True), ([[2, 1, 4], [4, 1, 1], 0], True)]],
    *[dict(src=f"{_LB}:809-825", op="flag", flag="f_contig", layout=lay, expect=e) for lay, e in [
        ([_S357, [1, 3, 15], 0], True), ([_S357, [1, 4, 20], 0], False), ([[], [], 0], True),
        ([[2, 0, 4], [1, 10, 100], 0], True), ([[2, 1, 4], [1, 1, 2], 0], True)]],
    *[dict(src=f"{_LB}:828-844", op="flag", flag="c_contig", layout=lay, expect=e) for lay, e in [
        ([_S357, [35, 7, 1], 0], True), ([_S357, [36, 7, 1], 0], False), ([[], [], 0], True),
        ([[2, 0, 4], [1, 10, 100], 0], True), ([[2, 1, 4], [4, 1, 1], 0], True)]],
    dict(src=f"{_LM}:563-570", op="matmul_layout", order="C", la=_c([4]), lb=_c([4]), expect=[[], [], 0]),
    dict(src=f"{_LM}:572-575", op="matmul_layout", order="C", la=_c([5]), lb=_swap(_f([3, 4, 5, 6]), 0, 1),
         expect=_c([4, 3, 6])),
    dict(src=f"{_LM}:577-580", op="matmul_layout", order="C", la=_swap(_f([3, 4, 5, 6]), 0, 1), lb=_c([6]),
         expect=_c([4, 3, 5])),
    dict(src=f"{_LM}:582-585", op="matmul_layout", order="C", la=_c([7, 6]), lb=_swap(_f([2, 3, 4, 5, 6]), -1, -2),
         expect=_c([2, 3, 4, 7, 5])),
    dict(src=f"{_LM}:587-590", op="matmul_layout", order="C", la=_swap(_f([2, 3, 4, 5, 6]), -1, -2), lb=_c([5, 7]),
         expect=_c([2, 3, 4, 6, 7])),
    dict(src=f"{_LM}:592-595", op="matmul_layout", order="C", la=_swap(_f([4, 1, 2, 5, 6]), 0, 2),
         lb=_swap(_f([4, 3, 1, 6, 7]), 0, 2), expect=_c([2, 3, 4, 5, 7])),
    dict(src=f"{_LM}:597-600", op="matmul_layout", order="C", la=_swap(_f([4, 3, 2, 5, 6]), 0, 2),
         lb=_swap(_f([4, 3, 2, 6, 7]), 0, 2), expect=_c([2, 3, 4, 5, 7])),
    dict(src=f"{_LM}:602-607", op="matmul_layout", order="F", la=_f([5, 6]), lb=_f([6, 7]), expect=_f([5, 7])),
    dict(src=f"{_LM}:609-613", op="matmul_layout", order="F", la=_f([5]), lb=_f([5, 6, 3, 4]), expect=_f([6, 3, 4])),
    dict(src=f"{_LM}:615-619", op="matmul_layout", order="F", la=_f([5, 6, 3, 4]), lb=_f([6]), expect=_f([5, 3, 4])),
    dict(src=f"{_LM}:621-626", op="matmul_layout", order="F", la=_f([5, 6, 2, 1, 4]), lb=_f([6, 7, 1, 3, 4]),
         expect=_f([5, 7, 2, 3, 4])),
    *[dict(src=f"{_BR}:{line}", op="broadcast", order="C", la=_c(a), lb=_c(b), expect_shape=e) for a, b, e, line in [
        ([8, 1, 6, 1], [7, 1, 5], [8, 7, 6, 5], "287-294"), ([5, 4], [1], [5, 4], "299-306"),
        ([5, 4], [4], [5, 4], "311-318"), ([15, 3, 5], [15, 1, 5], [15, 3, 5], "323-330"),
        ([15, 3, 5], [3, 5], [15, 3, 5], "335-342"), ([15, 3, 5], [3, 1], [15, 3, 5], "347-354"),
        ([1, 1, 2], [1, 2], [1, 1, 2], "357-364"), ([1, 2], [1, 1, 2], [1, 1, 2], "367-374"),
        ([3], [4], None, "381-384"), ([2, 1], [8, 4, 3], None, "387-390"), ([15, 3, 5], [15, 3], None, "394-397")]],
    dict(src=f"{_BR}:406-414", op="broadcast", order="C", la=_c([8, 1, 6, 3, 1]), lb=_f([7, 1, 3, 5]),
         expect_shape=[8, 7, 6, 3, 5], expect_a=[18, 0, 3, 1, 0], expect_b=[0, 1, 0, 7, 21]),
    # output shapes of `%` on contiguous operands (rstsr-core/src/device_faer/matmul.rs)
    *[dict(src=f"rstsr-core/src/device_faer/matmul.rs:{line}", op="matmul_layout", order=o,
           la=(_c if o == "C" else _f)(a), lb=(_c if o == "C" else _f)(b), expect_shape=e) for a, b, o, e, line in [
        ([3], [2, 3, 5], "C", [2, 5], "264-268"), ([2, 3, 5], [5], "C", [2, 3], "270-274"),
        ([5, 3], [2, 3, 5], "C", [2, 5, 5], "276-280"), ([2, 3, 5], [5, 3], "C", [2, 3, 3], "282-286"),
        ([5, 3, 2], [3], "F", [5, 2], "293-297"), ([5], [5, 3, 2], "F", [3, 2], "299-303"),
        ([5, 3, 2], [3, 5], "F", [5, 5, 2], "305-309"), ([3, 5], [5, 3, 2], "F", [3, 3, 2], "311-315"),
        ([1, 3, 5], [2, 5, 3], "C", [2, 3, 3], "328-331"), ([2, 3, 5], [1, 5, 3], "C", [2, 3, 3], "337-340"),
        ([1, 3, 5], [1, 5, 3], "C", [1, 3, 3], "347-350")]],
]


def main() -> None:
    here = Path(__file__).resolve().parent
    out = here / "reference_kats.json"
    out.write_text(json.dumps(CASES, indent=1) + "\n")
    print(f"wrote {len(CASES)} cases to {out}")
    out = here / "tri_index_kats.json"
    out.write_text(json.dumps(TRI_INDEX_CASES, indent=1) + "\n")
    print(f"wrote {len(TRI_INDEX_CASES)} cases to {out}")
    out = here / "contraction_kats.json"
    out.write_text(json.dumps(CONTRACTION_CASES, indent=1) + "\n")
    print(f"wrote {len(CONTRACTION_CASES)} cases to {out}")
    out = here / "elementwise_kats.json"
    out.write_text(json.dumps(ELEMENTWISE_CASES, indent=1) + "\n")
    print(f"wrote {len(ELEMENTWISE_CASES)} cases to {out}")
    out = here / "broadcast_kats.json"
    out.write_text(json.dumps(BROADCAST_CASES, indent=1) + "\n")
    print(f"wrote {len(BROADCAST_CASES)} cases to {out}")
    out = here / "reshape_kats.json"
    out.write_text(json.dumps(RESHAPE_CASES, indent=1) + "\n")
    print(f"wrote {len(RESHAPE_CASES)} cases to {out}")
    out = here / "vecdot_kats.json"
    out.write_text(json.dumps(VECDOT_CASES, indent=1) + "\n")
    print(f"wrote {len(VECDOT_CASES)} cases to {out}")
    out = here / "creation_kats.json"
    out.write_text(json.dumps(CREATION_CASES, indent=1) + "\n")
    print(f"wrote {len(CREATION_CASES)} cases to {out}")
    out = here / "layout_kats.json"
    out.write_text(json.dumps(LAYOUT_CASES, indent=1) + "\n")
    print(f"wrote {len(LAYOUT_CASES)} cases to {out}")


if __name__ == "__main__":
    main()
