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
    bool_select,
    einsum,
    empty,
    fill,
    fma,
    from_host_layout,
    full,
    index_select,
    matmul,
    matmul_into,
    pack_tri,
    reduce_all,
    reduce_axes,
    reduce_axes_into,
    take,
    tensordot,
    to_contig,
    unary,
    unpack_tri,
    vecdot,
    zeros,
)

__version__ = "0.1.0"
