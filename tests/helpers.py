"""Shared helpers of the test suite: seeded inputs, strided layouts and the
oracle-side evaluation of a KAT case."""

from __future__ import annotations

import numpy as np

from oracle import layout as OL
from oracle import oracle as O

NP = {"f64": np.float64, "f32": np.float32, "i32": np.int32, "i64": np.int64, "bool": np.bool_, "u64": np.uint64}


def rand(shape, dtype, seed=0, lo=-1.0, hi=1.0):
    rng = np.random.default_rng(seed)
    dt = np.dtype(dtype)
    n = int(np.prod(shape)) if len(shape) else 1
    if dt.kind == "f":
        return rng.uniform(lo, hi, n).astype(dt).reshape(shape)
    if dt.kind == "b":
        return (rng.integers(0, 2, n) == 1).reshape(shape)
    return rng.integers(-1000, 1001, n).astype(dt).reshape(shape)


def strided_case(kind: str, shape, dtype, seed=0):
    """A host buffer and a view layout of `shape` in one of the layouts of the
    memory-bound workload: 'c', 'f', 'perm' (C-contiguous base with axes 1,2
    swapped, viewed back), 'slice' (step-2 innermost slice of a wider base),
    'slice2' (step-2 slice on axis 2), 'flip' (negative strides)."""
    shape = tuple(shape)
    n = len(shape)
    if kind == "c":
        buf = rand(shape, dtype, seed).ravel()
        return buf, shape, OL.c_stride(shape), 0
    if kind == "f":
        buf = rand(shape, dtype, seed).ravel()
        return buf, shape, OL.f_stride(shape), 0
    if kind == "perm":
        assert n >= 3
        base = list(shape)
        base[1], base[2] = base[2], base[1]
        buf = rand(base, dtype, seed).ravel()
        st = list(OL.c_stride(base))
        st[1], st[2] = st[2], st[1]
        return buf, shape, tuple(st), 0
    if kind == "slice":
        base = list(shape)
        base[-1] *= 2
        buf = rand(base, dtype, seed).ravel()
        st = list(OL.c_stride(base))
        st[-1] *= 2
        return buf, shape, tuple(st), 0
    if kind == "slice2":
        assert n >= 3
        base = list(shape)
        base[2] *= 2
        buf = rand(base, dtype, seed).ravel()
        st = list(OL.c_stride(base))
        st[2] *= 2
        return buf, shape, tuple(st), 0
    if kind == "flip":
        buf = rand(shape, dtype, seed).ravel()
        st = list(OL.c_stride(shape))
        off = 0
        for ax in (0, n - 1):
            off += st[ax] * (shape[ax] - 1)
            st[ax] = -st[ax]
        return buf, shape, tuple(st), off
    raise ValueError(kind)


def values(buf, shape, stride, offset):
    return O.Strided(buf, shape, stride, offset).values()


def rel_err(got, ref):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    den = np.linalg.norm(ref.ravel())
    num = np.linalg.norm((got - ref).ravel())
    return num / den if den > 0 else num
