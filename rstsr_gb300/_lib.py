"""ctypes binding of ``librstsr_cuda.so`` (the C ABI declared in ``include/rstsr_cuda.h``).

The library must have been built (``rstsr_gb300.build.build()``); loading fails
loudly otherwise: there is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

MAX_NDIM = 8

_LIB_PATH = Path(os.environ.get("RSTSR_CUDA_LIB", Path(__file__).resolve().parent / "_build" / "librstsr_cuda.so"))


class RstsrError(RuntimeError):
    """A non-zero rstsr_status; ``code`` is the status, the message is the library's."""

    NAMES = {
        1: "InvalidLayout",
        2: "InvalidValue",
        3: "ValueOutOfRange",
        4: "DeviceMismatch",
        5: "DeviceError",
        6: "RuntimeError",
        7: "UnImplemented",
        8: "Timeout",
        9: "IndexError",
        10: "AxisError",
    }

    def __init__(self, code: int, msg: str):
        self.code = code
        self.kind = self.NAMES.get(code, f"Status{code}")
        super().__init__(f"{self.kind}: {msg}")


class Layout(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32),
        ("_reserved", C.c_int32),
        ("offset", C.c_int64),
        ("shape", C.c_int64 * MAX_NDIM),
        ("stride", C.c_int64 * MAX_NDIM),
    ]

    @classmethod
    def make(cls, shape, stride, offset=0) -> "Layout":
        shape = tuple(int(s) for s in shape)
        stride = tuple(int(s) for s in stride)
        if len(shape) != len(stride):
            raise ValueError("shape and stride ranks differ")
        if len(shape) > MAX_NDIM:
            raise ValueError(f"at most {MAX_NDIM} dimensions are supported")
        lay = cls()
        lay.ndim = len(shape)
        lay.offset = int(offset)
        for i, (d, s) in enumerate(zip(shape, stride)):
            lay.shape[i] = d
            lay.stride[i] = s
        return lay

    @property
    def shape_t(self) -> tuple:
        return tuple(self.shape[i] for i in range(self.ndim))

    @property
    def stride_t(self) -> tuple:
        return tuple(self.stride[i] for i in range(self.ndim))

    def __repr__(self) -> str:  # pragma: no cover - debugging aid
        return f"Layout(shape={self.shape_t}, stride={self.stride_t}, offset={self.offset})"


class GemmOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("ozaki_slices", C.c_int32), ("reserved", C.c_int32 * 6)]


class GemmProblem(C.Structure):
    _fields_ = [
        ("m", C.c_int64),
        ("n", C.c_int64),
        ("k", C.c_int64),
        ("lda", C.c_int64),
        ("ldb", C.c_int64),
        ("ldc", C.c_int64),
        ("a", C.c_void_p),
        ("b", C.c_void_p),
        ("c", C.c_void_p),
        ("alpha", C.c_double),
        ("beta", C.c_double),
    ]


# dtype codes (rstsr_dtype)
F64, F32, F16, BF16, I8, I16, I32, I64, U8, U16, U32, U64, BOOL = range(13)

_NP2CODE = {
    np.dtype(np.float64): F64,
    np.dtype(np.float32): F32,
    np.dtype(np.float16): F16,
    np.dtype(np.int8): I8,
    np.dtype(np.int16): I16,
    np.dtype(np.int32): I32,
    np.dtype(np.int64): I64,
    np.dtype(np.uint8): U8,
    np.dtype(np.uint16): U16,
    np.dtype(np.uint32): U32,
    np.dtype(np.uint64): U64,
    np.dtype(np.bool_): BOOL,
}
_CODE2NP = {v: k for k, v in _NP2CODE.items()}
_CODE2NP[BF16] = np.dtype(np.uint16)  # raw bits on the host


def dtype_code(dt) -> int:
    if isinstance(dt, str) and dt == "bf16":
        return BF16
    return _NP2CODE[np.dtype(dt)]


def np_dtype(code: int) -> np.dtype:
    return _CODE2NP[code]


# binary ops (rstsr_binary_op)
OP = dict(add=0, sub=1, mul=2, div=3, rem=4, bitand=5, bitor=6, bitxor=7, shl=8, shr=9, maximum=10, minimum=11, pow=12,
          atan2=13, copysign=14, hypot=15, logaddexp=16, nextafter=17, floor_divide=18)
UOP = dict(neg=0, not_=1, abs=2, sqrt=3, exp=4, log=5, sin=6, cos=7, tanh=8, square=9, floor=10, ceil=11, sign=12, recip=13,
           acos=14, acosh=15, asin=16, asinh=17, atan=18, atanh=19, cosh=20, expm1=21, log1p=22, log2=23, log10=24,
           round=25, sinh=26, tan=27, trunc=28, inv=29, conj=30, real=31, imag=32)
PRED = dict(isfinite=0, isinf=1, isnan=2, signbit=3)
CMP = dict(equal=0, not_equal=1, greater=2, greater_equal=3, less=4, less_equal=5)
RED = dict(sum=0, mean=1, var=2, std=3, min=4, max=5, prod=6, l2_norm=7, all=8, any=9, count_nonzero=10)

_P = C.c_void_p
_L = C.POINTER(Layout)
_I = C.c_int32
_SIGS = {
    "rstsr_cuda_ctx_create": ([_I, C.POINTER(_P)], C.c_int),
    "rstsr_cuda_ctx_destroy": ([_P], C.c_int),
    "rstsr_cuda_ctx_sync": ([_P], C.c_int),
    "rstsr_cuda_ctx_set_stream": ([_P, _P], C.c_int),
    "rstsr_cuda_ctx_get_stream": ([_P], _P),
    "rstsr_cuda_ctx_device": ([_P], C.c_int32),
    "rstsr_cuda_ctx_launch_count": ([_P], C.c_uint64),
    "rstsr_cuda_last_error": ([], C.c_char_p),
    "rstsr_cuda_version": ([], C.c_char_p),
    "rstsr_cuda_layout_broadcast": ([_L, _L, _I, _L, _L], C.c_int),
    "rstsr_cuda_layout_binary_op": ([_L, _L, _I, _L], C.c_int),
    "rstsr_cuda_layout_for_array_copy": ([_L, C.c_char, _L], C.c_int),
    "rstsr_cuda_layout_greedy": ([_L, _I, _L, C.POINTER(C.c_int32)], C.c_int),
    "rstsr_cuda_layout_flags": ([_L], C.c_int32),
    "rstsr_cuda_unravel_index": ([C.POINTER(C.c_int64), _I, C.c_uint64, _I, C.POINTER(C.c_int64)], C.c_int),
    "rstsr_cuda_malloc": ([_P, C.c_size_t, C.POINTER(_P)], C.c_int),
    "rstsr_cuda_free": ([_P, _P], C.c_int),
    "rstsr_cuda_memcpy_h2d": ([_P, _P, _P, C.c_size_t], C.c_int),
    "rstsr_cuda_memcpy_d2h": ([_P, _P, _P, C.c_size_t], C.c_int),
    "rstsr_cuda_memcpy_d2d": ([_P, _P, _P, C.c_size_t], C.c_int),
    "rstsr_cuda_memcpy_h2d_async": ([_P, _P, _P, C.c_size_t], C.c_int),
    "rstsr_cuda_memcpy_d2h_async": ([_P, _P, _P, C.c_size_t], C.c_int),
    "rstsr_cuda_assign": ([_P, _P, _L, _I, _P, _L, _I], C.c_int),
    "rstsr_cuda_assign_arbitrary": ([_P, _P, _L, _I, _P, _L, _I, _I], C.c_int),
    "rstsr_cuda_fill": ([_P, _P, _L, _I, _P], C.c_int),
    "rstsr_cuda_arange_len": ([_I, _P, _P, _P, C.POINTER(C.c_int64)], C.c_int),
    "rstsr_cuda_arange": ([_P, _I, _P, C.c_int64, _P, _P], C.c_int),
    "rstsr_cuda_linspace": ([_P, _I, _P, C.c_int64, _P, _P, C.c_int32], C.c_int),
    "rstsr_cuda_tril": ([_P, _I, _P, _L, C.c_int64, C.c_int32], C.c_int),
    "rstsr_cuda_binary": ([_P, _I, _I, _P, _L, _P, _L, _P, _L], C.c_int),
    "rstsr_cuda_binary_scalar": ([_P, _I, _I, _P, _L, _P, _L, _P, _I], C.c_int),
    "rstsr_cuda_binary_inplace": ([_P, _I, _I, _P, _L, _P, _L, _I], C.c_int),
    "rstsr_cuda_unary": ([_P, _I, _I, _P, _L, _P, _L], C.c_int),
    "rstsr_cuda_unary_predicate": ([_P, _I, _I, _P, _L, _P, _L], C.c_int),
    "rstsr_cuda_compare": ([_P, _I, _I, _P, _L, _P, _L, _P, _L], C.c_int),
    "rstsr_cuda_compare_scalar": ([_P, _I, _I, _P, _L, _P, _L, _P, _I], C.c_int),
    "rstsr_cuda_isclose": ([_P, _I, _P, _L, _P, _L, _P, _L, C.c_double, C.c_double, _I], C.c_int),
    "rstsr_cuda_allclose_all": ([_P, _I, _P, _L, _P, _L, C.c_double, C.c_double, C.c_int32, C.POINTER(C.c_uint8)], C.c_int),
    "rstsr_cuda_fma": ([_P, _I, _P, _L, _P, _L, _P, _L, _P, _L], C.c_int),
    "rstsr_cuda_reduce_out_dtype": ([_I, _I, C.POINTER(C.c_int)], C.c_int),
    "rstsr_cuda_reduce_all": ([_P, _I, _I, _P, _L, _P], C.c_int),
    "rstsr_cuda_reduce_axes_layout": ([_L, C.POINTER(C.c_int64), _I, _L], C.c_int),
    "rstsr_cuda_reduce_axes": ([_P, _I, _I, _P, _L, C.POINTER(C.c_int64), _I, C.POINTER(_P), _L], C.c_int),
    "rstsr_cuda_reduce_axes_into": ([_P, _I, _I, _P, _L, C.POINTER(C.c_int64), _I, _P, _L], C.c_int),
    "rstsr_cuda_sum_axes_noalloc": ([_P, _I, _P, _L, C.POINTER(C.c_int64), _I, _P, _L], C.c_int),
    "rstsr_cuda_argreduce_all": ([_P, _I, _I, _P, _L, C.POINTER(C.c_uint64)], C.c_int),
    "rstsr_cuda_argreduce_axes": ([_P, _I, _I, _P, _L, C.POINTER(C.c_int64), _I, C.POINTER(_P), _L], C.c_int),
    "rstsr_cuda_argreduce_axes_into": ([_P, _I, _I, _P, _L, C.POINTER(C.c_int64), _I, _P, _L], C.c_int),
    "rstsr_cuda_pack_tri": ([_P, _I, _P, _L, _P, _L, C.c_char, _I], C.c_int),
    "rstsr_cuda_unpack_tri": ([_P, _I, _P, _L, _P, _L, C.c_char, _I, _I], C.c_int),
    "rstsr_cuda_index_select": (
        [_P, _I, _P, _L, _P, _L, C.c_int32, C.POINTER(C.c_uint64), C.c_int64],
        C.c_int,
    ),
    "rstsr_cuda_einsum": ([_P, _I, C.c_char_p, _I, C.POINTER(_P), _L, _P, _L, C.POINTER(GemmOpts)], C.c_int),
    "rstsr_cuda_einsum_output_shape": ([C.c_char_p, _I, _L, C.POINTER(C.c_int32), C.POINTER(C.c_int64)], C.c_int),
    "rstsr_cuda_tensordot": (
        [_P, _I, _P, _L, _P, _L, _P, _L, C.POINTER(C.c_int64), C.POINTER(C.c_int64), _I, C.POINTER(GemmOpts)],
        C.c_int,
    ),
    "rstsr_cuda_vecdot": (
        [_P, _I, _P, _L, _P, _L, _P, _L, C.POINTER(C.c_int64), C.POINTER(C.c_int64), _I, _I],
        C.c_int,
    ),
    "rstsr_cuda_gemm": (
        [_P, _I, C.c_char, C.c_char, C.c_int64, C.c_int64, C.c_int64, C.c_double, _P, C.c_int64, _P, C.c_int64,
         C.c_double, _P, C.c_int64, _I, C.POINTER(GemmOpts)],
        C.c_int,
    ),
    "rstsr_cuda_matmul": ([_P, _I, _P, _L, _P, _L, _P, _L, C.c_double, C.c_double, _I, C.POINTER(GemmOpts)], C.c_int),
    "rstsr_cuda_matmul_layout": ([_L, _L, _I, _L], C.c_int),
    "rstsr_cuda_syrk": (
        [_P, _I, C.c_char, C.c_char, C.c_int64, C.c_int64, C.c_double, _P, C.c_int64, C.c_double, _P, C.c_int64,
         _I, C.POINTER(GemmOpts)],
        C.c_int,
    ),
    "rstsr_cuda_symm": (
        [_P, _I, C.c_char, C.c_char, C.c_int64, C.c_int64, C.c_double, _P, C.c_int64, _P, C.c_int64, C.c_double,
         _P, C.c_int64, _I, C.POINTER(GemmOpts)],
        C.c_int,
    ),
    "rstsr_cuda_trsm": (
        [_P, _I, C.c_char, C.c_char, C.c_char, C.c_char, C.c_int64, C.c_int64, C.c_double, _P, C.c_int64, _P,
         C.c_int64, _I, C.POINTER(GemmOpts)],
        C.c_int,
    ),
    "rstsr_cuda_gemm_grouped": ([_P, _I, C.POINTER(GemmProblem), _I, C.POINTER(GemmOpts)], C.c_int),
    "rstsr_cuda_last_ozaki_slices": ([], C.c_int32),
    "rstsr_cuda_graph_begin": ([_P], C.c_int),
    "rstsr_cuda_graph_end": ([_P, C.POINTER(_P)], C.c_int),
    "rstsr_cuda_graph_launch": ([_P, _P], C.c_int),
    "rstsr_cuda_graph_destroy": ([_P], C.c_int),
    "rstsr_cuda_autotune_gemm": (
        [_P, _I, C.c_int64, C.c_int64, C.c_int64, C.POINTER(GemmOpts), C.POINTER(C.c_int32)],
        C.c_int,
    ),
    "rstsr_cuda_autotune_save": ([C.c_char_p], C.c_int),
    "rstsr_cuda_autotune_load": ([C.c_char_p], C.c_int),
}

_lib = None


def lib() -> C.CDLL:
    """Load (once) and return the library with every signature declared."""
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise RuntimeError(
                f"{_LIB_PATH} is missing: build the CUDA backend first (python -m rstsr_gb300.build); "
                "there is no CPU fallback"
            )
        L = C.CDLL(str(_LIB_PATH))
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def exported_names() -> list[str]:
    return list(_SIGS)


def check(status: int) -> None:
    if status != 0:
        msg = lib().rstsr_cuda_last_error().decode(errors="replace")
        raise RstsrError(status, msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))
