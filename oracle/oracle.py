"""ctypes front of the C oracle (TEST INFRASTRUCTURE ONLY).

Buffers are flat numpy arrays; layouts are (shape, stride, offset) in
elements, the same convention as the device C ABI. ``build()`` compiles
``rstsr_oracle.c`` with OpenMP into ``oracle/_build/liboracle.so``.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "rstsr_oracle.c"
LIB = HERE / "_build" / "liboracle.so"

MAXD = 8


class OLayout(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32),
        ("reserved", C.c_int32),
        ("offset", C.c_int64),
        ("shape", C.c_int64 * MAXD),
        ("stride", C.c_int64 * MAXD),
    ]


def olayout(shape, stride, offset=0) -> OLayout:
    l = OLayout()
    l.ndim = len(shape)
    l.offset = int(offset)
    for i, (d, s) in enumerate(zip(shape, stride)):
        l.shape[i] = int(d)
        l.stride[i] = int(s)
    return l


DT = {np.dtype(np.float64): 0, np.dtype(np.float32): 1, np.dtype(np.int32): 6, np.dtype(np.int64): 7,
      np.dtype(np.uint64): 11, np.dtype(np.bool_): 12}
OPS = dict(add=0, sub=1, mul=2, div=3)
REDS = dict(sum=0, mean=1, var=2, std=3, min=4, max=5, prod=6, l2_norm=7, all=8, any=9, count_nonzero=10)

_lib = None


def build(force: bool = False) -> Path:
    LIB.parent.mkdir(exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        cc = os.environ.get("CC", "gcc")
        subprocess.run([cc, "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-o", str(LIB), str(SRC), "-lm"],
                       check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P, LP, I = C.c_void_p, C.POINTER(OLayout), C.c_int
        L.oracle_assign.argtypes = [P, LP, P, LP, I, I]
        L.oracle_assign_arbitrary.argtypes = [P, LP, P, LP, I, I, I]
        L.oracle_binary.argtypes = [I, I, P, LP, P, LP, P, LP, I]
        L.oracle_fma.argtypes = [I, P, LP, P, LP, P, LP, P, LP, I]
        L.oracle_reduce_axes.argtypes = [I, I, P, LP, C.POINTER(C.c_int64), I, P, LP, I]
        L.oracle_argreduce_axes.argtypes = [I, I, P, LP, C.POINTER(C.c_int64), I, C.POINTER(C.c_uint64), LP, I]
        L.oracle_max_threads.argtypes = []
        L.oracle_pack_tri.argtypes = [P, LP, P, LP, I, I, I]
        L.oracle_unpack_tri.argtypes = [P, LP, P, LP, I, I, I, I]
        L.oracle_index_select.argtypes = [P, LP, P, LP, I, C.POINTER(C.c_uint64), C.c_int64, I]
        L.oracle_einsum.argtypes = [I, I, C.POINTER(P), LP, C.POINTER(C.c_int32), P, LP, C.POINTER(C.c_int32), I,
                                    C.POINTER(C.c_int64)]
        for f in (L.oracle_assign, L.oracle_assign_arbitrary, L.oracle_binary, L.oracle_fma, L.oracle_reduce_axes,
                  L.oracle_argreduce_axes, L.oracle_max_threads, L.oracle_pack_tri, L.oracle_unpack_tri,
                  L.oracle_index_select, L.oracle_einsum):
            f.restype = C.c_int
        _lib = L
    return _lib


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _ok(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with code {rc}")


class Strided:
    """A host tensor: flat buffer + layout (elements)."""

    def __init__(self, buf: np.ndarray, shape, stride, offset=0):
        self.buf = np.ascontiguousarray(buf).ravel()
        self.shape = tuple(int(s) for s in shape)
        self.stride = tuple(int(s) for s in stride)
        self.offset = int(offset)

    @property
    def layout(self) -> OLayout:
        return olayout(self.shape, self.stride, self.offset)

    def values(self) -> np.ndarray:
        """The logical array (numpy view resolved to a copy)."""
        isz = self.buf.itemsize
        if any(d == 0 for d in self.shape):
            return np.zeros(self.shape, self.buf.dtype)
        return np.array(np.lib.stride_tricks.as_strided(
            self.buf[self.offset:], shape=self.shape, strides=tuple(s * isz for s in self.stride)))


def c_strides(shape):
    st, acc = [], 1
    for d in reversed(shape):
        st.append(acc)
        acc *= max(int(d), 1)
    return tuple(reversed(st))


def f_strides(shape):
    st, acc = [], 1
    for d in shape:
        st.append(acc)
        acc *= max(int(d), 1)
    return tuple(st)


def empty_strided(shape, stride, dtype, offset=0) -> Strided:
    lo, hi = offset, offset + 1
    if any(d == 0 for d in shape):
        hi = offset
    else:
        for d, s in zip(shape, stride):
            if s > 0:
                hi += s * (d - 1)
            else:
                lo += s * (d - 1)
    return Strided(np.zeros(max(hi, 1), dtype=dtype), shape, stride, offset)


def assign(dst: Strided, src: Strided, nthreads: int = 1) -> None:
    _ok(lib().oracle_assign(_p(dst.buf), C.byref(dst.layout), _p(src.buf), C.byref(src.layout), dst.buf.itemsize,
                            nthreads), "assign")


def assign_arbitrary(dst: Strided, src: Strided, order: int = 0, nthreads: int = 1) -> None:
    _ok(lib().oracle_assign_arbitrary(_p(dst.buf), C.byref(dst.layout), _p(src.buf), C.byref(src.layout),
                                      dst.buf.itemsize, order, nthreads), "assign_arbitrary")


def binary(op: str, c: Strided, a: Strided, b: Strided, nthreads: int = 1) -> None:
    _ok(lib().oracle_binary(OPS[op], DT[c.buf.dtype], _p(c.buf), C.byref(c.layout), _p(a.buf), C.byref(a.layout),
                            _p(b.buf), C.byref(b.layout), nthreads), "binary")


def fma(d: Strided, a: Strided, b: Strided, c: Strided, nthreads: int = 1) -> None:
    _ok(lib().oracle_fma(DT[d.buf.dtype], _p(d.buf), C.byref(d.layout), _p(a.buf), C.byref(a.layout), _p(b.buf),
                         C.byref(b.layout), _p(c.buf), C.byref(c.layout), nthreads), "fma")


def reduce_axes(op: str, a: Strided, axes, out: Strided, nthreads: int = 1) -> None:
    ax = (C.c_int64 * max(len(axes), 1))(*axes)
    _ok(lib().oracle_reduce_axes(REDS[op], DT[a.buf.dtype], _p(a.buf), C.byref(a.layout), ax, len(axes), _p(out.buf),
                                 C.byref(out.layout), nthreads), "reduce_axes")


def argreduce_axes(is_max: bool, a: Strided, axes, out: Strided, nthreads: int = 1) -> None:
    ax = (C.c_int64 * max(len(axes), 1))(*axes)
    _ok(lib().oracle_argreduce_axes(1 if is_max else 0, DT[a.buf.dtype], _p(a.buf), C.byref(a.layout), ax, len(axes),
                                    out.buf.ctypes.data_as(C.POINTER(C.c_uint64)), C.byref(out.layout), nthreads),
        "argreduce_axes")


def pack_tri(dst: Strided, src: Strided, lower: bool, order: int = 0) -> None:
    """dst (.., n(n+1)/2) <- the lower / upper triangle of src (.., n, n)."""
    _ok(lib().oracle_pack_tri(_p(dst.buf), C.byref(dst.layout), _p(src.buf), C.byref(src.layout), dst.buf.itemsize,
                              1 if lower else 0, order), "pack_tri")


SYMM = {"Sy": 0, "He": 1, "Ay": 2, "Ah": 3, "N": 4}


def unpack_tri(dst: Strided, src: Strided, lower: bool, symm: str = "Sy", order: int = 0) -> None:
    """dst (.., n, n) <- packed triangle src (.., n(n+1)/2) and its mirror."""
    _ok(lib().oracle_unpack_tri(_p(dst.buf), C.byref(dst.layout), _p(src.buf), C.byref(src.layout), dst.buf.itemsize,
                                1 if lower else 0, SYMM[symm], order), "unpack_tri")


def index_select(dst: Strided, src: Strided, axis: int, indices) -> None:
    """dst[.., k, ..] = src[.., indices[k], ..] along `axis`."""
    idx = np.ascontiguousarray(np.asarray(indices, dtype=np.uint64))
    _ok(lib().oracle_index_select(_p(dst.buf), C.byref(dst.layout), _p(src.buf), C.byref(src.layout), int(axis),
                                  idx.ctypes.data_as(C.POINTER(C.c_uint64)), C.c_int64(idx.size), dst.buf.itemsize),
        "index_select")


def _parse_einsum(subscripts: str, nops: int):
    """Subscripts -> (input label lists, output labels); numpy's implicit output."""
    s = "".join(ch for ch in subscripts if not ch.isspace())
    lhs, arrow, rhs = s.partition("->")
    ins = lhs.split(",")
    if len(ins) != nops:
        raise ValueError("operand count")
    if not arrow:
        from collections import Counter
        cnt = Counter("".join(ins))
        rhs = "".join(sorted(c for c, n in cnt.items() if n == 1))
    return ins, rhs


def einsum(subscripts: str, *ops: Strided, out: Strided | None = None) -> Strided:
    """Einstein summation by its definition (f64 with compensated sums, or
    wrapping i64); ops are Strided f64 or i64 host tensors."""
    ins, outl = _parse_einsum(subscripts, len(ops))
    labels = sorted(set("".join(ins)))
    lid = {c: i for i, c in enumerate(labels)}
    ext = [0] * len(labels)
    for sub, t in zip(ins, ops):
        for c, d in zip(sub, t.shape):
            ext[lid[c]] = d
    dt = ops[0].buf.dtype
    code = 0 if dt == np.float64 else 7
    if out is None:
        shape = [ext[lid[c]] for c in outl]
        out = empty_strided(shape, c_strides(shape), dt)
    n = len(ops)
    ptrs = (C.c_void_p * n)(*[t.buf.ctypes.data for t in ops])
    lays = (OLayout * n)(*[t.layout for t in ops])
    labs = (C.c_int32 * max(sum(len(x) for x in ins), 1))(*[lid[c] for x in ins for c in x])
    olabs = (C.c_int32 * max(len(outl), 1))(*[lid[c] for c in outl])
    exts = (C.c_int64 * max(len(ext), 1))(*ext)
    _ok(lib().oracle_einsum(code, n, ptrs, lays, labs, _p(out.buf), C.byref(out.layout), olabs, len(labels), exts),
        "einsum")
    return out
