"""CPU oracle of the rstsr hot path (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` use this package, and only as the reference results the device is
compared with / the timed reference CPU path; the CUDA backend never imports it.

  rstsr_oracle.c  assign / assign_arbitrary walks, element-wise arithmetic, the
                  reductions and arg-reductions, pack / unpack of triangles,
                  index_select and einsum over explicit layouts (serial and
                  OpenMP), built by oracle.py
  oracle.py       ctypes wrapper of that library (``Strided`` operands)
  layout.py       the layout algebra (flags, greedy / K order, broadcasting,
                  binary-op and reduction output layouts, matmul shapes)
  elementwise.py  the element-wise closures where the reference differs from
                  numpy (round, sign, signbit, floor_divide, logaddexp, isclose)
  creation.py     arange (lengths and values), linspace, tril / triu
"""
