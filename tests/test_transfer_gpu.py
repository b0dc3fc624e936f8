"""Host <-> device moves of DeviceChangeAPI (to_cpu_vec / from_cpu_vec,
rstsr-core/src/storage/conversion.rs:3-21) through rstsr_cuda_memcpy_h2d_async
and rstsr_cuda_memcpy_d2h_async: pageable host memory (numpy arrays, as a Rust
Vec<T> would be) goes through the context's staging ring in 8 MiB chunks,
page-locked memory (torch's pin_memory) is one stream-ordered copy. Round
trips must return every byte unchanged, for sizes around the chunk and ring
boundaries and for host pointers at odd byte offsets."""

import ctypes as C

import numpy as np
import pytest

import rstsr_gb300 as rt
from rstsr_gb300._lib import call, lib

pytestmark = pytest.mark.gpu

CHUNK = 8 << 20


def dev_buf(dev, nbytes):
    return rt.empty((max(nbytes, 1),), np.uint8, dev)


@pytest.mark.parametrize("nbytes", [0, 1, 7, 4096 + 3, CHUNK - 1, CHUNK, CHUNK + 1, 4 * CHUNK + 5, 9 * CHUNK + 123,
                                    48 * CHUNK])
@pytest.mark.parametrize("host_offset", [0, 3])
def test_pageable_round_trip(dev, nbytes, host_offset):
    rng = np.random.default_rng(nbytes + host_offset)
    backing = rng.integers(0, 256, nbytes + host_offset + 1, dtype=np.uint8)
    src = backing[host_offset:host_offset + nbytes]
    d = dev_buf(dev, nbytes)
    call("rstsr_cuda_memcpy_h2d_async", dev.ctx, C.c_void_p(d.ptr), src.ctypes.data_as(C.c_void_p),
         C.c_size_t(nbytes))
    # the source may be reused as soon as the call returns
    backing[:] = 0
    out_backing = np.full(nbytes + host_offset + 1, 0xAB, dtype=np.uint8)
    out = out_backing[host_offset:host_offset + nbytes]
    call("rstsr_cuda_memcpy_d2h_async", dev.ctx, out.ctypes.data_as(C.c_void_p), C.c_void_p(d.ptr),
         C.c_size_t(nbytes))
    # the pageable destination holds the data when the call returns
    want = np.random.default_rng(nbytes + host_offset).integers(0, 256, nbytes + host_offset + 1,
                                                                  dtype=np.uint8)[host_offset:host_offset + nbytes]
    np.testing.assert_array_equal(out, want)
    assert out_backing[:host_offset].tolist() == [0xAB] * host_offset  # nothing written outside
    assert out_backing[host_offset + nbytes] == 0xAB


def test_pageable_transfers_are_stream_ordered(dev):
    """An h2d_async into a buffer a kernel is still reading, then a d2h_async
    of a kernel's output: both wait for the work queued before them."""
    n = 3 * CHUNK // 8 + 11
    x = np.arange(n, dtype=np.float64)
    a = rt.asarray(x, dev)
    b = a + a  # queued
    y = np.full(n, -1.0)
    call("rstsr_cuda_memcpy_h2d_async", dev.ctx, C.c_void_p(a.ptr), y.ctypes.data_as(C.c_void_p),
         C.c_size_t(y.nbytes))
    c = a * 3.0
    got_b = np.empty(n)
    got_c = np.empty(n)
    call("rstsr_cuda_memcpy_d2h_async", dev.ctx, got_b.ctypes.data_as(C.c_void_p), C.c_void_p(b.ptr),
         C.c_size_t(got_b.nbytes))
    call("rstsr_cuda_memcpy_d2h_async", dev.ctx, got_c.ctypes.data_as(C.c_void_p), C.c_void_p(c.ptr),
         C.c_size_t(got_c.nbytes))
    np.testing.assert_array_equal(got_b, 2 * x)
    np.testing.assert_array_equal(got_c, np.full(n, -3.0))


def test_pinned_round_trip_is_asynchronous(dev):
    torch = pytest.importorskip("torch")
    n = 5 * CHUNK + 17
    src = torch.randint(0, 256, (n,), dtype=torch.uint8).pin_memory()
    dst = torch.zeros((n,), dtype=torch.uint8).pin_memory()
    d = dev_buf(dev, n)
    call("rstsr_cuda_memcpy_h2d_async", dev.ctx, C.c_void_p(d.ptr), C.c_void_p(src.data_ptr()), C.c_size_t(n))
    call("rstsr_cuda_memcpy_d2h_async", dev.ctx, C.c_void_p(dst.data_ptr()), C.c_void_p(d.ptr), C.c_size_t(n))
    dev.sync()  # page-locked copies complete in stream order
    assert torch.equal(src, dst)


def test_staged_copy_refused_inside_graph_capture(dev):
    x = np.ones(1024)
    d = rt.empty((1024,), np.float64, dev)
    with pytest.raises(rt.RstsrError) as e:
        with rt.Graph(dev):
            call("rstsr_cuda_memcpy_h2d_async", dev.ctx, C.c_void_p(d.ptr), x.ctypes.data_as(C.c_void_p),
                 C.c_size_t(x.nbytes))
    assert "graph" in str(e.value)


def test_null_pointers_rejected(dev):
    rc = lib().rstsr_cuda_memcpy_h2d_async(dev.ctx, None, None, C.c_size_t(8))
    assert rc == 2
    rc = lib().rstsr_cuda_memcpy_d2h_async(dev.ctx, None, None, C.c_size_t(0))
    assert rc == 0
