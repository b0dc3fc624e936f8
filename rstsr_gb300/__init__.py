"""rstsr_gb300: the GB300 (sm_103a) CUDA device backend for RSTSR.

The product is the C-ABI library ``librstsr_cuda.so`` (``include/rstsr_cuda.h``),
built in-tree by ``rstsr_gb300.build``. This package holds its Python binding
and a host-side mirror of rstsr's tensor layer used by the tests and the
benchmark.
"""

from ._lib import RstsrError, lib  # noqa: F401
from .tensor import (  # noqa: F401
    COL_MAJOR,
    ROW_MAJOR,
    DeviceCuda,
    Graph,
    Tensor,
    arange,
    allclose,
    argreduce_all,
    argreduce_axes,
    asarray,
    assign,
    autotune_gemm,
    autotune_load,
    autotune_save,
    binary,
    binary_inplace,
    binary_scalar,
    compare,
    bool_select,
    einsum,
    empty,
    fill,
    fma,
    from_host_layout,
    full,
    index_select,
    isclose,
    linspace,
    matmul,
    matmul_into,
    pack_tri,
    predicate,
    reduce_all,
    reduce_axes,
    reduce_axes_into,
    symm,
    syrk,
    take,
    tensordot,
    tril,
    triu,
    trsm,
    to_contig,
    unary,
    unpack_tri,
    unravel_index,
    unraveled_argmax_all,
    unraveled_argmin_all,
    vecdot,
    zeros,
)

from . import _lib as _l


def _install_op_functions():
    """rt.isnan(a), rt.less(a, b), rt.atan2(a, b), rt.log1p(a), ... as module
    functions named after rstsr's (the predicates, comparisons and the
    element-wise math family)."""
    g = globals()
    for name in _l.PRED:
        g[name] = (lambda n: lambda a: predicate(n, a))(name)
    for name in _l.CMP:
        g[name] = (lambda n: lambda a, b: compare(n, a, b))(name)
    for name in ("atan2", "copysign", "hypot", "logaddexp", "nextafter", "floor_divide"):
        g[name] = (lambda n: lambda a, b: binary(n, a, b) if isinstance(b, Tensor) else binary_scalar(n, a, b))(name)
    for name in ("acos", "acosh", "asin", "asinh", "atan", "atanh", "cosh", "expm1", "log1p", "log2", "log10",
                 "round", "sinh", "tan", "trunc", "inv", "conj", "real", "imag"):
        g[name] = (lambda n: lambda a: unary(n, a))(name)


_install_op_functions()

__version__ = "0.1.0"
