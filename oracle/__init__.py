"""CPU oracle of the rstsr hot path (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` use this package, and only as the reference results the device is
compared with / the timed reference CPU path; the CUDA backend never imports it.
"""
