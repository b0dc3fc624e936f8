"""Host-side mirror of rstsr's tensor layer over the CUDA device.

``DeviceCuda`` plays the role of rstsr's device type and ``Tensor`` the role of
``TensorBase<Storage<..., DeviceCuda>, Layout<IxD>>``: every view operation
(permute, slice, broadcast, flip, reshape of a contiguous tensor) is layout
algebra on the host, and every data operation is one C-ABI call with
``(device pointer, Layout)`` pairs, exactly the split the reference makes
between ``rstsr-core/src/tensor`` (host) and the device traits of
``rstsr-core/src/operators`` (device). Method names follow ``rt::`` and
``TensorBase`` (``to_contig``, ``sum_axes``, ``argmax_axes``, ``%`` = matmul).
"""

from __future__ import annotations

import ctypes as C
import numbers
from typing import Iterable, Sequence

import numpy as np

from . import _lib
from ._lib import Layout, RstsrError, call, check, dtype_code, lib, np_dtype

ROW_MAJOR, COL_MAJOR = 0, 1


def _order_code(order) -> int:
    if order in ("C", "c", ROW_MAJOR, "RowMajor"):
        return ROW_MAJOR
    if order in ("F", "f", COL_MAJOR, "ColMajor"):
        return COL_MAJOR
    raise ValueError(f"unknown order {order!r}")


class DeviceCuda:
    """One CUDA device, its stream and memory pool (the C-ABI context)."""

    def __init__(self, device_id: int = 0, default_order="C"):
        ctx = C.c_void_p()
        call("rstsr_cuda_ctx_create", int(device_id), C.byref(ctx))
        self._ctx = ctx
        self.device_id = int(device_id)
        self.default_order = _order_code(default_order)

    @property
    def ctx(self) -> C.c_void_p:
        return self._ctx

    def set_default_order(self, order) -> None:
        self.default_order = _order_code(order)

    def sync(self) -> None:
        call("rstsr_cuda_ctx_sync", self._ctx)

    def stream(self) -> int:
        return lib().rstsr_cuda_ctx_get_stream(self._ctx) or 0

    def set_stream(self, stream_ptr: int | None) -> None:
        call("rstsr_cuda_ctx_set_stream", self._ctx, C.c_void_p(stream_ptr or 0))

    def launch_count(self) -> int:
        return int(lib().rstsr_cuda_ctx_launch_count(self._ctx))

    def same_device(self, other: "DeviceCuda") -> bool:
        return self._ctx.value == other._ctx.value

    def close(self) -> None:
        if getattr(self, "_ctx", None) is not None and self._ctx.value:
            lib().rstsr_cuda_ctx_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass


class Storage:
    """A device allocation of ``nbytes`` owned by this object."""

    def __init__(self, device: DeviceCuda, nbytes: int, ptr: int | None = None):
        self.device = device
        self.nbytes = int(nbytes)
        if ptr is None:
            p = C.c_void_p()
            call("rstsr_cuda_malloc", device.ctx, C.c_size_t(self.nbytes), C.byref(p))
            ptr = p.value or 0
        self.ptr = int(ptr)

    def __del__(self):  # pragma: no cover
        try:
            if self.ptr and self.device.ctx.value:
                lib().rstsr_cuda_free(self.device.ctx, C.c_void_p(self.ptr))
        except Exception:
            pass
        self.ptr = 0


def _c_strides(shape) -> tuple:
    st, acc = [], 1
    for d in reversed(shape):
        st.append(acc)
        acc *= max(int(d), 1)
    return tuple(reversed(st))


def _f_strides(shape) -> tuple:
    st, acc = [], 1
    for d in shape:
        st.append(acc)
        acc *= max(int(d), 1)
    return tuple(st)


def _bounds(shape, stride, offset) -> tuple:
    if any(d == 0 for d in shape):
        return offset, offset
    lo = hi = offset
    for d, s in zip(shape, stride):
        if s > 0:
            hi += s * (d - 1)
        else:
            lo += s * (d - 1)
    return lo, hi + 1


class Tensor:
    """A strided view (shape, stride, offset in elements) into a device Storage."""

    def __init__(self, storage: Storage, shape, stride, offset: int, dtype: int):
        self.storage = storage
        self.shape = tuple(int(s) for s in shape)
        self.stride = tuple(int(s) for s in stride)
        self.offset = int(offset)
        self.dtype_code = int(dtype)

    # ------------------------------------------------------------ basics
    @property
    def device(self) -> DeviceCuda:
        return self.storage.device

    @property
    def ndim(self) -> int:
        return len(self.shape)

    @property
    def size(self) -> int:
        return int(np.prod(self.shape, dtype=np.int64)) if self.shape else 1

    @property
    def dtype(self):
        return "bf16" if self.dtype_code == _lib.BF16 else np_dtype(self.dtype_code)

    @property
    def itemsize(self) -> int:
        return 2 if self.dtype_code == _lib.BF16 else np_dtype(self.dtype_code).itemsize

    @property
    def ptr(self) -> int:
        return self.storage.ptr

    def layout(self) -> Layout:
        return Layout.make(self.shape, self.stride, self.offset)

    def _flags(self) -> int:
        return int(lib().rstsr_cuda_layout_flags(C.byref(self.layout())))

    def c_contig(self) -> bool:
        return bool(self._flags() & 1)

    def f_contig(self) -> bool:
        return bool(self._flags() & 2)

    def c_prefer(self) -> bool:
        return bool(self._flags() & 4)

    def f_prefer(self) -> bool:
        return bool(self._flags() & 8)

    def _view(self, shape, stride, offset) -> "Tensor":
        return Tensor(self.storage, shape, stride, offset, self.dtype_code)

    def __repr__(self) -> str:
        return f"Tensor(shape={self.shape}, stride={self.stride}, offset={self.offset}, dtype={self.dtype})"

    # -------------------------------------------------------- host moves
    def to_numpy(self) -> np.ndarray:
        """Copy to host (DeviceChangeAPI to a CPU device) keeping the layout's values."""
        lo, hi = _bounds(self.shape, self.stride, self.offset)
        isz = self.itemsize
        host_dt = np.dtype(np.uint16) if self.dtype_code == _lib.BF16 else np_dtype(self.dtype_code)
        if hi <= lo:
            return np.zeros(self.shape, dtype=host_dt)
        buf = np.empty(hi - lo, dtype=host_dt)
        call(
            "rstsr_cuda_memcpy_d2h",
            self.device.ctx,
            buf.ctypes.data_as(C.c_void_p),
            C.c_void_p(self.ptr + lo * isz),
            C.c_size_t((hi - lo) * isz),
        )
        view = np.lib.stride_tricks.as_strided(
            buf[self.offset - lo :], shape=self.shape, strides=tuple(s * isz for s in self.stride)
        )
        return np.array(view)

    def to_vec(self) -> list:
        return self.to_numpy().ravel(order="C").tolist()

    def to_scalar(self):
        if self.size != 1:
            raise RstsrError(1, "to_scalar needs exactly one element")
        return self.to_numpy().reshape(()).item()

    # -------------------------------------------------------------- views
    def permute_dims(self, *axes) -> "Tensor":
        if len(axes) == 1 and not isinstance(axes[0], numbers.Integral):
            axes = tuple(axes[0])
        axes = tuple(a + self.ndim if a < 0 else a for a in axes)
        if sorted(axes) != list(range(self.ndim)):
            raise RstsrError(1, f"invalid permutation {axes} for ndim {self.ndim}")
        return self._view([self.shape[a] for a in axes], [self.stride[a] for a in axes], self.offset)

    transpose = permute_dims

    def t(self) -> "Tensor":
        return self._view(self.shape[::-1], self.stride[::-1], self.offset)

    def reverse_axes(self) -> "Tensor":
        return self.t()

    def swapaxes(self, a1: int, a2: int) -> "Tensor":
        ax = list(range(self.ndim))
        ax[a1], ax[a2] = ax[a2], ax[a1]
        return self.permute_dims(ax)

    def flip(self, axis: int) -> "Tensor":
        axis = axis + self.ndim if axis < 0 else axis
        shape, stride = list(self.shape), list(self.stride)
        off = self.offset + (stride[axis] * (shape[axis] - 1) if shape[axis] > 0 else 0)
        stride[axis] = -stride[axis]
        return self._view(shape, stride, off)

    def i(self, key) -> "Tensor":
        """Basic indexing: ints select, slices narrow (any step), Ellipsis, None inserts."""
        if not isinstance(key, tuple):
            key = (key,)
        n_real = sum(1 for k in key if k is not None and k is not Ellipsis)
        if Ellipsis in key:
            i = key.index(Ellipsis)
            key = key[:i] + (slice(None),) * (self.ndim - n_real) + key[i + 1 :]
        key = key + (slice(None),) * (self.ndim - sum(1 for k in key if k is not None))
        shape, stride, off, ax = [], [], self.offset, 0
        for k in key:
            if k is None:
                shape.append(1)
                stride.append(0)
                continue
            d, s = self.shape[ax], self.stride[ax]
            if isinstance(k, numbers.Integral):
                kk = int(k) + d if k < 0 else int(k)
                if not 0 <= kk < d:
                    raise RstsrError(1, f"index {k} out of range for axis {ax} of extent {d}")
                off += kk * s
            else:
                start, stop, step = k.indices(d)
                cnt = len(range(start, stop, step))
                if cnt > 0:
                    off += start * s
                shape.append(cnt)
                stride.append(s * step)
            ax += 1
        return self._view(shape, stride, off)

    def broadcast_to(self, shape) -> "Tensor":
        shape = tuple(shape)
        n = len(shape)
        if n < self.ndim:
            raise RstsrError(1, "cannot broadcast to fewer dimensions")
        st = [0] * n
        for i in range(n):
            j = self.ndim - n + i
            if j < 0:
                continue
            if self.shape[j] == shape[i]:
                st[i] = self.stride[j]
            elif self.shape[j] == 1:
                st[i] = 0
            else:
                raise RstsrError(1, f"cannot broadcast {self.shape} to {shape}")
        return self._view(shape, st, self.offset)

    def reshape(self, shape, order=None) -> "Tensor":
        """View if the tensor is contiguous in the device order, else a copy (to_shape)."""
        shape = tuple(int(s) for s in shape)
        if -1 in shape:
            known = int(np.prod([s for s in shape if s != -1])) or 1
            shape = tuple(self.size // known if s == -1 else s for s in shape)
        if int(np.prod(shape, dtype=np.int64)) != self.size:
            raise RstsrError(1, f"cannot reshape {self.shape} into {shape}")
        order = self.device.default_order if order is None else _order_code(order)
        if order == ROW_MAJOR and self.c_contig():
            return self._view(shape, _c_strides(shape), self.offset)
        if order == COL_MAJOR and self.f_contig():
            return self._view(shape, _f_strides(shape), self.offset)
        out = empty(shape, self.dtype_code, self.device, order=order)
        call(
            "rstsr_cuda_assign_arbitrary", self.device.ctx, C.c_void_p(out.ptr), C.byref(out.layout()),
            out.dtype_code, C.c_void_p(self.ptr), C.byref(self.layout()), self.dtype_code, order,
        )
        return out

    into_shape = reshape

    # --------------------------------------------------------------- copies
    def to_layout(self, shape, stride, offset: int = 0) -> "Tensor":
        """change_layout_f (rstsr-core/src/tensor/manipulation/to_layout.rs:8-38)."""
        shape, stride = tuple(shape), tuple(stride)
        if shape == self.shape and stride == self.stride and offset == self.offset:
            return self
        _, hi = _bounds(shape, stride, offset)
        st = Storage(self.device, max(hi, 1) * self.itemsize)
        out = Tensor(st, shape, stride, offset, self.dtype_code)
        call(
            "rstsr_cuda_assign_arbitrary", self.device.ctx, C.c_void_p(out.ptr), C.byref(out.layout()),
            out.dtype_code, C.c_void_p(self.ptr), C.byref(self.layout()), self.dtype_code,
            self.device.default_order,
        )
        return out

    def to_contig(self, order="C") -> "Tensor":
        """A view when already contiguous in `order`, else a contiguous copy."""
        order = _order_code(order)
        if order == ROW_MAJOR:
            return self if self.c_contig() else self.to_layout(self.shape, _c_strides(self.shape), 0)
        return self if self.f_contig() else self.to_layout(self.shape, _f_strides(self.shape), 0)

    def copy(self) -> "Tensor":
        out = empty_like_k(self)
        assign(out, self)
        return out

    def astype(self, dtype) -> "Tensor":
        code = dtype_code(dtype)
        out = empty(self.shape, code, self.device, order="K", like=self)
        assign(out, self)
        return out

    # ----------------------------------------------------------- operators
    def _binary(self, other, op: str, reverse: bool = False) -> "Tensor":
        if isinstance(other, Tensor):
            a, b = (other, self) if reverse else (self, other)
            return binary(op, a, b)
        return binary_scalar(op, self, other, scalar_is_lhs=reverse)

    def __add__(self, o):
        return self._binary(o, "add")

    def __radd__(self, o):
        return self._binary(o, "add", True)

    def __sub__(self, o):
        return self._binary(o, "sub")

    def __rsub__(self, o):
        return self._binary(o, "sub", True)

    def __mul__(self, o):
        return self._binary(o, "mul")

    def __rmul__(self, o):
        return self._binary(o, "mul", True)

    def __truediv__(self, o):
        return self._binary(o, "div")

    def __rtruediv__(self, o):
        return self._binary(o, "div", True)

    def __and__(self, o):
        return self._binary(o, "bitand")

    def __or__(self, o):
        return self._binary(o, "bitor")

    def __xor__(self, o):
        return self._binary(o, "bitxor")

    def __lshift__(self, o):
        return self._binary(o, "shl")

    def __rshift__(self, o):
        return self._binary(o, "shr")

    def rem(self, o):
        """Element-wise remainder (rstsr's `rt::rem`; `%` is matmul)."""
        return self._binary(o, "rem")

    def __mod__(self, o):
        """`&a % &b` is matmul in rstsr (rstsr-core/src/tensor/linalg/matmul.rs:180-199)."""
        return matmul(self, o)

    def __matmul__(self, o):
        return matmul(self, o)

    def __neg__(self):
        return unary("neg", self)

    def __invert__(self):
        return unary("not_", self)

    def _inplace(self, other, op: str) -> "Tensor":
        if isinstance(other, Tensor):
            binary_inplace(op, self, other)
        else:
            s = _scalar_bytes(other, self.dtype_code)
            call(
                "rstsr_cuda_binary_scalar", self.device.ctx, _lib.OP[op], self.dtype_code, C.c_void_p(self.ptr),
                C.byref(self.layout()), C.c_void_p(self.ptr), C.byref(self.layout()), s, 0,
            )
        return self

    def __iadd__(self, o):
        return self._inplace(o, "add")

    def __isub__(self, o):
        return self._inplace(o, "sub")

    def __imul__(self, o):
        return self._inplace(o, "mul")

    def __itruediv__(self, o):
        return self._inplace(o, "div")

    # ---------------------------------------------------------- reductions
    def _red_all(self, op: str):
        return reduce_all(op, self)

    def _red_axes(self, op: str, axes) -> "Tensor":
        return reduce_axes(op, self, axes)

    def argmax_all(self) -> int:
        return argreduce_all(True, self)

    def argmin_all(self) -> int:
        return argreduce_all(False, self)

    def argmax_axes(self, axes) -> "Tensor":
        return argreduce_axes(True, self, axes)

    def argmin_axes(self, axes) -> "Tensor":
        return argreduce_axes(False, self, axes)


def _make_reduction_methods():
    for name in _lib.RED:
        def all_fn(self, _n=name):
            return reduce_all(_n, self)

        def axes_fn(self, axes=None, _n=name):
            if axes is None:
                return reduce_axes(_n, self, list(range(self.ndim)))
            return reduce_axes(_n, self, axes)

        setattr(Tensor, f"{name}_all", all_fn)
        setattr(Tensor, f"{name}_axes", axes_fn)
    for name in ["abs", "sqrt", "exp", "log", "sin", "cos", "tanh", "square", "floor", "ceil", "sign", "recip"]:
        setattr(Tensor, name, lambda self, _n=name: unary(_n, self))


_make_reduction_methods()


# ----------------------------------------------------------------- creation


def empty(shape, dtype, device: DeviceCuda, order="C", like: Tensor | None = None) -> Tensor:
    """Uninitialised tensor (uninit_impl); order 'K' copies `like`'s memory order."""
    code = dtype if isinstance(dtype, int) else dtype_code(dtype)
    shape = tuple(int(s) for s in shape)
    if order == "K" and like is not None:
        out_l = Layout()
        call("rstsr_cuda_layout_for_array_copy", C.byref(like.layout()), b"K", C.byref(out_l))
        stride = out_l.stride_t
    else:
        stride = _c_strides(shape) if _order_code(order) == ROW_MAJOR else _f_strides(shape)
    n = max(int(np.prod(shape, dtype=np.int64)) if shape else 1, 1)
    isz = 2 if code == _lib.BF16 else np_dtype(code).itemsize
    return Tensor(Storage(device, n * isz), shape, stride, 0, code)


def empty_like_k(t: Tensor) -> Tensor:
    return empty(t.shape, t.dtype_code, t.device, order="K", like=t)


def asarray(arr, device: DeviceCuda, dtype=None) -> Tensor:
    """Upload a host array (row-major copy) to the device."""
    a = np.ascontiguousarray(np.asarray(arr, dtype=dtype))
    code = dtype_code(a.dtype)
    out = empty(a.shape, code, device, order="C")
    if a.nbytes:
        call("rstsr_cuda_memcpy_h2d", device.ctx, C.c_void_p(out.ptr), a.ctypes.data_as(C.c_void_p), C.c_size_t(a.nbytes))
    return out


def from_host_layout(buf: np.ndarray, shape, stride, offset, device: DeviceCuda) -> Tensor:
    """Upload a flat host buffer and view it with an arbitrary layout (elements)."""
    buf = np.ascontiguousarray(buf).ravel()
    t = asarray(buf, device)
    return Tensor(t.storage, shape, stride, offset, t.dtype_code)


def zeros(shape, dtype, device: DeviceCuda, order="C") -> Tensor:
    return full(shape, 0, dtype, device, order)


def full(shape, value, dtype, device: DeviceCuda, order="C") -> Tensor:
    t = empty(shape, dtype, device, order)
    fill(t, value)
    return t


def fill(t: Tensor, value) -> None:
    s = _scalar_bytes(value, t.dtype_code)
    call("rstsr_cuda_fill", t.device.ctx, C.c_void_p(t.ptr), C.byref(t.layout()), t.dtype_code, s)


def arange(start, stop=None, step=1, *, dtype=None, device: DeviceCuda) -> Tensor:
    """arange_f (rstsr-core/src/tensor/creation.rs:55-110): `arange(stop)`,
    `arange(start, stop)` or `arange(start, stop, step)`, 1-D; the element type
    defaults to f64 when a bound is a float, else i64. The length is host
    arithmetic (rstsr_cuda_arange_len), the values one kernel."""
    if stop is None:
        start, stop = 0, start
    if dtype is None:
        dtype = np.float64 if any(isinstance(v, (float, np.floating)) for v in (start, stop, step)) else np.int64
    code = dtype if isinstance(dtype, int) else dtype_code(dtype)
    s, e, st = (_scalar_bytes(v, code) for v in (start, stop, step))
    n = C.c_int64()
    call("rstsr_cuda_arange_len", code, s, e, st, C.byref(n))
    out = empty((n.value,), code, device)
    if n.value:
        call("rstsr_cuda_arange", device.ctx, code, C.c_void_p(out.ptr), n.value, s, st)
    return out


def linspace(start, stop, num: int, *, endpoint: bool = True, dtype=np.float64, device: DeviceCuda) -> Tensor:
    """linspace_f (rstsr-core/src/tensor/creation.rs:760-800): `num` values from
    `start` to `stop` (f64 / f32), the last one `stop` when `endpoint`."""
    num = int(num)
    if num < 0:
        raise RstsrError(2, "linspace: num must not be negative")
    code = dtype if isinstance(dtype, int) else dtype_code(dtype)
    out = empty((num,), code, device)
    call("rstsr_cuda_linspace", device.ctx, code, C.c_void_p(out.ptr), num, _scalar_bytes(start, code),
         _scalar_bytes(stop, code), 1 if endpoint else 0)
    return out


def _tri_mask(t: Tensor, k: int, upper: bool, inplace: bool) -> Tensor:
    out = t
    if not inplace:
        out = empty(t.shape, t.dtype_code, t.device, order="C" if t.device.default_order == ROW_MAJOR else "F")
        assign(out, t)
    call("rstsr_cuda_tril", t.device.ctx, t.dtype_code, C.c_void_p(out.ptr), C.byref(out.layout()), int(k),
         1 if upper else 0)
    return out


def tril(t: Tensor, k: int = 0, inplace: bool = False) -> Tensor:
    """tril_f (rstsr-core/src/tensor/creation.rs:1451-1560): zeros above the k-th
    diagonal of the last two axes, in a contiguous copy (default order) or in
    place."""
    return _tri_mask(t, k, False, inplace)


def triu(t: Tensor, k: int = 0, inplace: bool = False) -> Tensor:
    """triu_f (rstsr-core/src/tensor/creation.rs:1640-1750): zeros below the k-th
    diagonal of the last two axes."""
    return _tri_mask(t, k, True, inplace)


def _scalar_bytes(value, code: int):
    if code == _lib.BF16:
        f = np.float32(value).view(np.uint32)
        bits = np.uint16((int(f) + 0x7FFF + ((int(f) >> 16) & 1)) >> 16)
        arr = np.array([bits], dtype=np.uint16)
    else:
        arr = np.array([value], dtype=np_dtype(code))
    buf = (C.c_uint8 * 8)()
    C.memmove(buf, arr.ctypes.data, arr.nbytes)
    return buf


# ---------------------------------------------------------------- operators


def _same_device(a: Tensor, b: Tensor) -> None:
    if not a.device.same_device(b.device):
        raise RstsrError(4, "tensors live on different devices")


def broadcast_layouts(a: Tensor, b: Tensor, order: int):
    oa, ob = Layout(), Layout()
    call("rstsr_cuda_layout_broadcast", C.byref(a.layout()), C.byref(b.layout()), order, C.byref(oa), C.byref(ob))
    return oa, ob


def binary(op: str, a: Tensor, b: Tensor) -> Tensor:
    """c = a (op) b with broadcasting and the K-order output layout of
    rstsr-core/src/tensor/operators/op_binary_arithmetic.rs:187-212."""
    _same_device(a, b)
    if a.dtype_code != b.dtype_code:
        raise RstsrError(2, f"dtype mismatch {a.dtype} vs {b.dtype}")
    order = a.device.default_order
    la, lb = broadcast_layouts(a, b, order)
    lc = Layout()
    call("rstsr_cuda_layout_binary_op", C.byref(la), C.byref(lb), order, C.byref(lc))
    _, hi = _bounds(lc.shape_t, lc.stride_t, lc.offset)
    out = Tensor(Storage(a.device, max(hi, 1) * a.itemsize), lc.shape_t, lc.stride_t, 0, a.dtype_code)
    call(
        "rstsr_cuda_binary", a.device.ctx, _lib.OP[op], a.dtype_code, C.c_void_p(out.ptr), C.byref(out.layout()),
        C.c_void_p(a.ptr), C.byref(la), C.c_void_p(b.ptr), C.byref(lb),
    )
    return out


def binary_scalar(op: str, a: Tensor, value, scalar_is_lhs: bool = False) -> Tensor:
    out = empty_like_k(a)
    s = _scalar_bytes(value, a.dtype_code)
    call(
        "rstsr_cuda_binary_scalar", a.device.ctx, _lib.OP[op], a.dtype_code, C.c_void_p(out.ptr),
        C.byref(out.layout()), C.c_void_p(a.ptr), C.byref(a.layout()), s, 1 if scalar_is_lhs else 0,
    )
    return out


def binary_inplace(op: str, a: Tensor, b: Tensor, reversed_: bool = False) -> Tensor:
    """a = a (op) b (OpAddAssignAPI / OpLConsume*API::op_muta_refb)."""
    _same_device(a, b)
    lb = b.broadcast_to(a.shape).layout()
    call(
        "rstsr_cuda_binary_inplace", a.device.ctx, _lib.OP[op], a.dtype_code, C.c_void_p(a.ptr),
        C.byref(a.layout()), C.c_void_p(b.ptr), C.byref(lb), 1 if reversed_ else 0,
    )
    return a


def unary(op: str, a: Tensor) -> Tensor:
    out = empty_like_k(a)
    call(
        "rstsr_cuda_unary", a.device.ctx, _lib.UOP[op], a.dtype_code, C.c_void_p(out.ptr), C.byref(out.layout()),
        C.c_void_p(a.ptr), C.byref(a.layout()),
    )
    return out


def fma(a: Tensor, b: Tensor, c: Tensor) -> Tensor:
    """d = a * b + c in one pass, with the layout `&a * &b + &c` gets in rstsr
    (binary-op layout of a*b, then c added in place)."""
    _same_device(a, b)
    _same_device(a, c)
    order = a.device.default_order
    la, lb = broadcast_layouts(a, b, order)
    lab = Layout()
    call("rstsr_cuda_layout_binary_op", C.byref(la), C.byref(lb), order, C.byref(lab))
    shape = lab.shape_t
    # c must broadcast into a*b's shape (the LConsume in-place path)
    cc = c.broadcast_to(shape)
    _, hi = _bounds(shape, lab.stride_t, 0)
    out = Tensor(Storage(a.device, max(hi, 1) * a.itemsize), shape, lab.stride_t, 0, a.dtype_code)
    call(
        "rstsr_cuda_fma", a.device.ctx, a.dtype_code, C.c_void_p(out.ptr), C.byref(out.layout()), C.c_void_p(a.ptr),
        C.byref(la), C.c_void_p(b.ptr), C.byref(lb), C.c_void_p(cc.ptr), C.byref(cc.layout()),
    )
    return out


def assign(dst: Tensor, src: Tensor) -> None:
    """OpAssignAPI::assign: same shape, values cast to dst's dtype."""
    _same_device(dst, src)
    lsrc = src.broadcast_to(dst.shape).layout()
    call(
        "rstsr_cuda_assign", dst.device.ctx, C.c_void_p(dst.ptr), C.byref(dst.layout()), dst.dtype_code,
        C.c_void_p(src.ptr), C.byref(lsrc), src.dtype_code,
    )


def to_contig(t: Tensor, order="C") -> Tensor:
    return t.to_contig(order)


# --------------------------------------------------------------- reductions


def _axes_arg(t: Tensor, axes):
    if isinstance(axes, numbers.Integral):
        axes = [int(axes)]
    axes = [int(a) for a in axes]
    arr = (C.c_int64 * max(len(axes), 1))(*axes)
    return arr, len(axes)


def reduce_all(op: str, t: Tensor):
    tout = C.c_int()
    call("rstsr_cuda_reduce_out_dtype", _lib.RED[op], t.dtype_code, C.byref(tout))
    out = np.zeros(1, dtype=np_dtype(tout.value) if tout.value != _lib.BF16 else np.uint16)
    call(
        "rstsr_cuda_reduce_all", t.device.ctx, _lib.RED[op], t.dtype_code, C.c_void_p(t.ptr), C.byref(t.layout()),
        out.ctypes.data_as(C.c_void_p),
    )
    v = out[0]
    return bool(v) if tout.value == _lib.BOOL else v.item()


def reduce_axes(op: str, t: Tensor, axes) -> Tensor:
    arr, n = _axes_arg(t, axes)
    tout = C.c_int()
    call("rstsr_cuda_reduce_out_dtype", _lib.RED[op], t.dtype_code, C.byref(tout))
    ptr = C.c_void_p()
    lout = Layout()
    call(
        "rstsr_cuda_reduce_axes", t.device.ctx, _lib.RED[op], t.dtype_code, C.c_void_p(t.ptr), C.byref(t.layout()),
        arr, n, C.byref(ptr), C.byref(lout),
    )
    isz = 2 if tout.value == _lib.BF16 else np_dtype(tout.value).itemsize
    st = Storage(t.device, max(int(np.prod(lout.shape_t, dtype=np.int64)) if lout.ndim else 1, 1) * isz, ptr.value or 0)
    return Tensor(st, lout.shape_t, lout.stride_t, lout.offset, tout.value)


def unravel_index(shape, index: int, order="C") -> tuple:
    """unravel_index_c / unravel_index_f (rstsr-common/src/layout/shape.rs:62-69)."""
    shape = tuple(int(s) for s in shape)
    sh = (C.c_int64 * max(len(shape), 1))(*shape)
    out = (C.c_int64 * max(len(shape), 1))()
    call("rstsr_cuda_unravel_index", sh, len(shape), int(index), _order_code(order), out)
    return tuple(int(out[i]) for i in range(len(shape)))


def unraveled_argmax_all(t: Tensor) -> tuple:
    """OpUnraveledArgMaxAPI::unraveled_argmax_all: the multi-index of the first
    maximum (C-order flat index unravelled over the shape)."""
    return unravel_index(t.shape, argreduce_all(True, t), "C")


def unraveled_argmin_all(t: Tensor) -> tuple:
    """OpUnraveledArgMinAPI::unraveled_argmin_all."""
    return unravel_index(t.shape, argreduce_all(False, t), "C")


def argreduce_all(is_max: bool, t: Tensor) -> int:
    out = C.c_uint64()
    call(
        "rstsr_cuda_argreduce_all", t.device.ctx, 1 if is_max else 0, t.dtype_code, C.c_void_p(t.ptr),
        C.byref(t.layout()), C.byref(out),
    )
    return int(out.value)


def argreduce_axes(is_max: bool, t: Tensor, axes) -> Tensor:
    arr, n = _axes_arg(t, axes)
    ptr = C.c_void_p()
    lout = Layout()
    call(
        "rstsr_cuda_argreduce_axes", t.device.ctx, 1 if is_max else 0, t.dtype_code, C.c_void_p(t.ptr),
        C.byref(t.layout()), arr, n, C.byref(ptr), C.byref(lout),
    )
    st = Storage(t.device, max(int(np.prod(lout.shape_t, dtype=np.int64)) if lout.ndim else 1, 1) * 8, ptr.value or 0)
    return Tensor(st, lout.shape_t, lout.stride_t, lout.offset, _lib.U64)


# ------------------------------------------------------------------- graphs


class Graph:
    """Capture the library calls made on a device into one CUDA graph.

    with Graph(dev) as g:
        ...calls on dev...
    g.launch()   # replays every captured kernel with one launch
    """

    def __init__(self, device: DeviceCuda):
        self.device = device
        self.handle = C.c_void_p()

    def __enter__(self) -> "Graph":
        call("rstsr_cuda_graph_begin", self.device.ctx)
        return self

    def __exit__(self, exc_type, exc, tb):
        h = C.c_void_p()
        rc = lib().rstsr_cuda_graph_end(self.device.ctx, C.byref(h))
        self.handle = h
        if exc_type is None:
            check(rc)

    def launch(self) -> None:
        call("rstsr_cuda_graph_launch", self.device.ctx, self.handle)

    def __del__(self):  # pragma: no cover
        try:
            if self.handle and self.handle.value:
                lib().rstsr_cuda_graph_destroy(self.handle)
        except Exception:
            pass


def reduce_axes_into(op: str, t: Tensor, axes, out: Tensor) -> Tensor:
    arr, n = _axes_arg(t, axes)
    call(
        "rstsr_cuda_reduce_axes_into", t.device.ctx, _lib.RED[op], t.dtype_code, C.c_void_p(t.ptr),
        C.byref(t.layout()), arr, n, C.c_void_p(out.ptr), C.byref(out.layout()),
    )
    return out


# ------------------------------------------------------------------- matmul


def matmul(a: Tensor, b: Tensor, precision: int = 0, slices: int = 0) -> Tensor:
    """`&a % &b` (DeviceMatMulAPI::matmul with the layout rules of
    rstsr-common/src/layout/matmul.rs)."""
    _same_device(a, b)
    order = a.device.default_order
    lc = Layout()
    call("rstsr_cuda_matmul_layout", C.byref(a.layout()), C.byref(b.layout()), order, C.byref(lc))
    out = Tensor(Storage(a.device, max(int(np.prod(lc.shape_t, dtype=np.int64)) if lc.ndim else 1, 1) * a.itemsize),
                 lc.shape_t, lc.stride_t, 0, a.dtype_code)
    matmul_into(out, a, b, 1.0, 0.0, precision, slices)
    return out


def matmul_into(c: Tensor, a: Tensor, b: Tensor, alpha: float = 1.0, beta: float = 0.0, precision: int = 0,
                slices: int = 0) -> Tensor:
    """c = alpha * a % b + beta * c (matmul_from)."""
    opts = _lib.GemmOpts()
    opts.precision = precision
    opts.ozaki_slices = slices
    call(
        "rstsr_cuda_matmul", a.device.ctx, a.dtype_code, C.c_void_p(c.ptr), C.byref(c.layout()), C.c_void_p(a.ptr),
        C.byref(a.layout()), C.c_void_p(b.ptr), C.byref(b.layout()), C.c_double(alpha), C.c_double(beta),
        a.device.default_order, C.byref(opts),
    )
    return c


def autotune_gemm(device: DeviceCuda, dtype, m: int, n: int, k: int, precision: int = 0, slices: int = 0) -> int:
    """Time the split-GEMM kernel configurations on an m x n x k problem of
    `dtype` (f64 Ozaki / f32 bf16 split) and keep the fastest for that shape
    class; returns its code kt | group << 8."""
    opts = _lib.GemmOpts()
    opts.precision = precision
    opts.ozaki_slices = slices
    best = C.c_int32(0)
    call("rstsr_cuda_autotune_gemm", device.ctx, dtype_code(dtype), C.c_int64(m), C.c_int64(n), C.c_int64(k),
         C.byref(opts), C.byref(best))
    return int(best.value)


def autotune_save(path: str) -> None:
    """Write the autotune table as text."""
    call("rstsr_cuda_autotune_save", str(path).encode())


def autotune_load(path: str) -> None:
    """Replace the autotune table by the one in `path`."""
    call("rstsr_cuda_autotune_load", str(path).encode())


# ------------------------------------------------- triangles and indexing

SYMM = {"Sy": 0, "He": 1, "Ay": 2, "Ah": 3, "N": 4}


def _uplo_byte(uplo) -> bytes:
    u = {"L": b"L", "l": b"L", "Lower": b"L", "U": b"U", "u": b"U", "Upper": b"U"}.get(uplo)
    if u is None:
        raise RstsrError(2, f"uplo must be 'L' or 'U', got {uplo!r}")
    return u


def _symm_code(symm) -> int:
    if isinstance(symm, int) and symm in SYMM.values():
        return symm
    if symm not in SYMM:
        raise RstsrError(2, f"unknown symmetry flag {symm!r}")
    return SYMM[symm]


def _tri_out_order(t: Tensor) -> int:
    # pack_tri_f / unpack_tri_f: C if the input prefers C only, F if F only,
    # else the device's default order (rstsr-core/src/tensor/operators/op_tri.rs:56-63)
    c, f = t.c_prefer(), t.f_prefer()
    if c and not f:
        return ROW_MAJOR
    if f and not c:
        return COL_MAJOR
    return t.device.default_order


def pack_tri(t: Tensor, uplo="L") -> Tensor:
    """pack_tri_f (rstsr-core/src/tensor/operators/op_tri.rs:13-71): the uplo
    triangle of the trailing (RowMajor) or leading (ColMajor) n x n axes,
    rows packed in order."""
    order = t.device.default_order
    if t.ndim < 2:
        raise RstsrError(1, "pack_tri needs at least two axes")
    if order == ROW_MAJOR:
        n, n2 = t.shape[-2], t.shape[-1]
        rest = t.shape[:-2]
    else:
        n, n2 = t.shape[0], t.shape[1]
        rest = t.shape[2:]
    if n != n2:
        raise RstsrError(1, "the two matrix dimensions should be the same for pack_tri")
    ntp = n * (n + 1) // 2
    out_shape = rest + (ntp,) if order == ROW_MAJOR else (ntp,) + rest
    out = empty(out_shape, t.dtype_code, t.device, order="C" if _tri_out_order(t) == ROW_MAJOR else "F")
    call("rstsr_cuda_pack_tri", t.device.ctx, t.dtype_code, C.c_void_p(out.ptr), C.byref(out.layout()),
         C.c_void_p(t.ptr), C.byref(t.layout()), _uplo_byte(uplo), order)
    return out


def unpack_tri(t: Tensor, uplo="L", symm="Sy") -> Tensor:
    """unpack_tri_f (op_tri.rs:105-162): the n x n matrices whose uplo
    triangle is packed along the trailing (RowMajor) / leading (ColMajor) axis,
    the other triangle filled by the symmetry. With symm "N" the other
    triangle is zero here (the reference leaves it uninitialised)."""
    order = t.device.default_order
    if t.ndim < 1:
        raise RstsrError(1, "unpack_tri needs at least one axis")
    ntp = t.shape[-1] if order == ROW_MAJOR else t.shape[0]
    n = int(np.floor(np.sqrt(float(2 * ntp))))
    if n * (n + 1) // 2 != ntp:
        raise RstsrError(1, "the packed dimension should be a triangular number for unpack_tri")
    code = _symm_code(symm)
    out_shape = t.shape[:-1] + (n, n) if order == ROW_MAJOR else (n, n) + t.shape[1:]
    out_order = "C" if _tri_out_order(t) == ROW_MAJOR else "F"
    out = zeros(out_shape, t.dtype_code, t.device, out_order) if code == SYMM["N"] else \
        empty(out_shape, t.dtype_code, t.device, order=out_order)
    call("rstsr_cuda_unpack_tri", t.device.ctx, t.dtype_code, C.c_void_p(out.ptr), C.byref(out.layout()),
         C.c_void_p(t.ptr), C.byref(t.layout()), _uplo_byte(uplo), code, order)
    return out


def index_select(t: Tensor, axis: int, indices) -> Tensor:
    """index_select_f (rstsr-core/src/tensor/adv_indexing.rs:10-46): gather
    along `axis`; negative indices count from the end. The output is
    contiguous in the device's default order."""
    ndim = t.ndim
    ax = int(axis)
    if ax < -ndim or ax >= ndim:
        raise RstsrError(10, f"axis {axis} out of range for ndim {ndim}")
    ax %= ndim if ndim else 1
    nshape = t.shape[ax]
    idx = np.asarray(list(indices) if not isinstance(indices, np.ndarray) else indices, dtype=np.int64).ravel()
    idx = np.where(idx < 0, idx + nshape, idx)
    if idx.size and (idx.min() < 0 or idx.max() >= nshape):
        raise RstsrError(9, f"invalid index that exceeds shape length at axis {ax}")
    out_shape = list(t.shape)
    out_shape[ax] = int(idx.size)
    out = empty(out_shape, t.dtype_code, t.device, order="C" if t.device.default_order == ROW_MAJOR else "F")
    host = np.ascontiguousarray(idx.astype(np.uint64))
    call("rstsr_cuda_index_select", t.device.ctx, t.dtype_code, C.c_void_p(out.ptr), C.byref(out.layout()),
         C.c_void_p(t.ptr), C.byref(t.layout()), ax, host.ctypes.data_as(C.POINTER(C.c_uint64)),
         C.c_int64(host.size))
    return out


def take(t: Tensor, indices, axis: int) -> Tensor:
    """take (adv_indexing.rs:66-78): index_select with the arguments swapped."""
    return index_select(t, axis, indices)


def bool_select(t: Tensor, axis: int, mask) -> Tensor:
    """bool_select_f (adv_indexing.rs:144-160): index_select of the positions
    where `mask` is true."""
    m = np.asarray(mask, dtype=bool).ravel()
    return index_select(t, axis, np.nonzero(m)[0])


Tensor.pack_tri = pack_tri
Tensor.pack_tril = lambda self: pack_tri(self, "L")
Tensor.pack_triu = lambda self: pack_tri(self, "U")
Tensor.unpack_tri = unpack_tri
Tensor.unpack_tril = lambda self, symm="Sy": unpack_tri(self, "L", symm)
Tensor.unpack_triu = lambda self, symm="Sy": unpack_tri(self, "U", symm)
Tensor.index_select = index_select
Tensor.take = lambda self, indices, axis: take(self, indices, axis)
Tensor.bool_select = bool_select


# ------------------------------------------------------------ contractions


def _gemm_opts(precision: int, slices: int):
    opts = _lib.GemmOpts()
    opts.precision = precision
    opts.ozaki_slices = slices
    return opts


def _contig_out(shape, dtype_code: int, device: DeviceCuda) -> Tensor:
    return empty(shape, dtype_code, device, order="C" if device.default_order == ROW_MAJOR else "F")


def einsum(subscripts: str, *operands: Tensor, precision: int = 0, slices: int = 0) -> Tensor:
    """einsum (crates-plugin/rstsr-tblis/src/einsum_impl.rs:146-199): the
    output is contiguous in the device's default order."""
    if not operands:
        raise RstsrError(2, "at least one operand is required")
    dev = operands[0].device
    for t in operands[1:]:
        if not t.device.same_device(dev):
            raise RstsrError(2, "all operands must be on the same device")
        if t.dtype_code != operands[0].dtype_code:
            raise RstsrError(2, "einsum operands must share one dtype")
    n = len(operands)
    lays = (Layout * n)(*[t.layout() for t in operands])
    nd = C.c_int32()
    shp = (C.c_int64 * _lib.MAX_NDIM)()
    sub = subscripts.encode("utf-8")
    call("rstsr_cuda_einsum_output_shape", sub, n, lays, C.byref(nd), shp)
    out = _contig_out(tuple(shp[i] for i in range(nd.value)), operands[0].dtype_code, dev)
    ptrs = (C.c_void_p * n)(*[t.ptr for t in operands])
    opts = _gemm_opts(precision, slices)
    call("rstsr_cuda_einsum", dev.ctx, operands[0].dtype_code, sub, n, ptrs, lays, C.c_void_p(out.ptr),
         C.byref(out.layout()), C.byref(opts))
    return out


def _axes_pair(axes, nda: int, ndb: int):
    if axes is None:
        axes = 2
    if isinstance(axes, numbers.Integral):
        n = int(axes)
        if n < 0:
            raise RstsrError(2, "n must be non-negative")
        if n > nda or n > ndb:
            raise RstsrError(1, "n must be less than or equal to the number of dimensions of both tensors")
        return list(range(nda - n, nda)), list(range(n))
    xa, xb = axes
    xa = [int(xa)] if isinstance(xa, numbers.Integral) else [int(x) for x in xa]
    xb = [int(xb)] if isinstance(xb, numbers.Integral) else [int(x) for x in xb]
    if len(xa) != len(xb):
        raise RstsrError(2, "axes_a and axes_b should have the same length")
    return xa, xb


def tensordot(a: Tensor, b: Tensor, axes=2, precision: int = 0, slices: int = 0) -> Tensor:
    """tensordot (crates-plugin/rstsr-tblis/src/tensordot_impl.rs:60-70):
    `axes` is n (last n axes of a with the first n of b) or (axes_a, axes_b)."""
    _same_device(a, b)
    xa, xb = _axes_pair(axes, a.ndim, b.ndim)
    na = [x % a.ndim if a.ndim else x for x in xa]
    nb = [x % b.ndim if b.ndim else x for x in xb]
    shape = tuple(a.shape[i] for i in range(a.ndim) if i not in na) + \
        tuple(b.shape[j] for j in range(b.ndim) if j not in nb)
    out = _contig_out(shape, a.dtype_code, a.device)
    ka = (C.c_int64 * max(len(xa), 1))(*xa)
    kb = (C.c_int64 * max(len(xb), 1))(*xb)
    opts = _gemm_opts(precision, slices)
    call("rstsr_cuda_tensordot", a.device.ctx, a.dtype_code, C.c_void_p(out.ptr), C.byref(out.layout()),
         C.c_void_p(a.ptr), C.byref(a.layout()), C.c_void_p(b.ptr), C.byref(b.layout()), ka, kb, len(xa),
         C.byref(opts))
    return out


def vecdot(a: Tensor, b: Tensor, axes=None) -> Tensor:
    """vecdot_f (rstsr-core/src/tensor/linalg/vecdot.rs:160-247): dot products
    along `axes` (default the last axis; an int counts from the end of each
    operand when negative), the remaining parts broadcast against each other."""
    _same_device(a, b)
    if axes is None:
        axes = -1
    if isinstance(axes, numbers.Integral):
        ax = int(axes)
        mn = min(a.ndim, b.ndim)
        if ax < 0:
            if not -mn <= ax <= -1:
                raise RstsrError(2, "axis should be [-N, -1] where N is min(a.ndim, b.ndim)")
            xa, xb = [ax + a.ndim], [ax + b.ndim]
        else:
            if not 0 <= ax < mn:
                raise RstsrError(2, "axis should be [0, N) where N is min(a.ndim, b.ndim)")
            xa, xb = [ax], [ax]
    else:
        xa, xb = _axes_pair(axes, a.ndim, b.ndim)
        xa = [x % a.ndim for x in xa]
        xb = [x % b.ndim for x in xb]
    order = a.device.default_order
    ra = a._view(tuple(a.shape[i] for i in range(a.ndim) if i not in xa),
                 tuple(a.stride[i] for i in range(a.ndim) if i not in xa), a.offset)
    rb = b._view(tuple(b.shape[i] for i in range(b.ndim) if i not in xb),
                 tuple(b.stride[i] for i in range(b.ndim) if i not in xb), b.offset)
    oa, ob = broadcast_layouts(ra, rb, order)
    lc = Layout()
    call("rstsr_cuda_layout_binary_op", C.byref(oa), C.byref(ob), order, C.byref(lc))
    _, hi = _bounds(lc.shape_t, lc.stride_t, lc.offset)
    out = Tensor(Storage(a.device, max(hi, 1) * a.itemsize), lc.shape_t, lc.stride_t, lc.offset, a.dtype_code)
    ka = (C.c_int64 * len(xa))(*xa)
    kb = (C.c_int64 * len(xb))(*xb)
    call("rstsr_cuda_vecdot", a.device.ctx, a.dtype_code, C.c_void_p(out.ptr), C.byref(out.layout()),
         C.c_void_p(a.ptr), C.byref(a.layout()), C.c_void_p(b.ptr), C.byref(b.layout()), ka, kb, len(xa), order)
    return out


# ----------------------------------------- predicates, comparisons, isclose


def _bool_out_like(lc: Layout, device: DeviceCuda) -> Tensor:
    _, hi = _bounds(lc.shape_t, lc.stride_t, lc.offset)
    return Tensor(Storage(device, max(hi, 1)), lc.shape_t, lc.stride_t, 0, _lib.BOOL)


def predicate(op: str, a: Tensor) -> Tensor:
    """isfinite / isinf / isnan / signbit (bool output, a's K-order layout).
    signbit is the reference's `is_positive()`: true for +0, +inf, +NaN."""
    lk = Layout()
    call("rstsr_cuda_layout_for_array_copy", C.byref(a.layout()), b"K", C.byref(lk))
    out = _bool_out_like(lk, a.device)
    call("rstsr_cuda_unary_predicate", a.device.ctx, _lib.PRED[op], a.dtype_code, C.c_void_p(out.ptr),
         C.byref(out.layout()), C.c_void_p(a.ptr), C.byref(a.layout()))
    return out


def compare(op: str, a, b) -> Tensor:
    """equal / not_equal / greater / greater_equal / less / less_equal with
    broadcasting (bool output); either side may be a Python scalar."""
    if not isinstance(a, Tensor):
        return _compare_scalar(op, b, a, True)
    if not isinstance(b, Tensor):
        return _compare_scalar(op, a, b, False)
    _same_device(a, b)
    if a.dtype_code != b.dtype_code:
        raise RstsrError(2, f"dtype mismatch {a.dtype} vs {b.dtype}")
    order = a.device.default_order
    la, lb = broadcast_layouts(a, b, order)
    lc = Layout()
    call("rstsr_cuda_layout_binary_op", C.byref(la), C.byref(lb), order, C.byref(lc))
    out = _bool_out_like(lc, a.device)
    call("rstsr_cuda_compare", a.device.ctx, _lib.CMP[op], a.dtype_code, C.c_void_p(out.ptr), C.byref(out.layout()),
         C.c_void_p(a.ptr), C.byref(la), C.c_void_p(b.ptr), C.byref(lb))
    return out


def _compare_scalar(op: str, t: Tensor, value, scalar_is_lhs: bool) -> Tensor:
    lk = Layout()
    call("rstsr_cuda_layout_for_array_copy", C.byref(t.layout()), b"K", C.byref(lk))
    out = _bool_out_like(lk, t.device)
    s = _scalar_bytes(value, t.dtype_code)
    call("rstsr_cuda_compare_scalar", t.device.ctx, _lib.CMP[op], t.dtype_code, C.c_void_p(out.ptr),
         C.byref(out.layout()), C.c_void_p(t.ptr), C.byref(t.layout()), s, 1 if scalar_is_lhs else 0)
    return out


def isclose(a: Tensor, b: Tensor, rtol: float = 1.0e-5, atol: float = 1.0e-8, equal_nan: bool = False) -> Tensor:
    """isclose (rstsr-dtype-traits/src/isclose.rs:92-105): |a - b| <= atol +
    rtol |b| (not symmetric), or both NaN with equal_nan; bool output."""
    _same_device(a, b)
    if a.dtype_code != b.dtype_code:
        raise RstsrError(2, f"dtype mismatch {a.dtype} vs {b.dtype}")
    order = a.device.default_order
    la, lb = broadcast_layouts(a, b, order)
    lc = Layout()
    call("rstsr_cuda_layout_binary_op", C.byref(la), C.byref(lb), order, C.byref(lc))
    out = _bool_out_like(lc, a.device)
    call("rstsr_cuda_isclose", a.device.ctx, a.dtype_code, C.c_void_p(out.ptr), C.byref(out.layout()),
         C.c_void_p(a.ptr), C.byref(la), C.c_void_p(b.ptr), C.byref(lb), float(rtol), float(atol),
         1 if equal_nan else 0)
    return out


def allclose(a: Tensor, b: Tensor, rtol: float = 1.0e-5, atol: float = 1.0e-8, equal_nan: bool = False) -> bool:
    """allclose (OpAllCloseAPI::allclose_all): every broadcast element pair
    isclose; a zero-size operand is an InvalidValue error, as in the reference."""
    _same_device(a, b)
    if a.dtype_code != b.dtype_code:
        raise RstsrError(2, f"dtype mismatch {a.dtype} vs {b.dtype}")
    la, lb = broadcast_layouts(a, b, a.device.default_order)
    out = C.c_uint8(0)
    call("rstsr_cuda_allclose_all", a.device.ctx, a.dtype_code, C.c_void_p(a.ptr), C.byref(la), C.c_void_p(b.ptr),
         C.byref(lb), float(rtol), float(atol), 1 if equal_nan else 0, C.byref(out))
    return bool(out.value)


# ---------------------------------------------------------- BLAS-3 drivers


def _blas_operand(t: Tensor):
    """(order, leading dimension) of a 2-D tensor with a unit stride."""
    if t.ndim != 2:
        raise RstsrError(1, "a BLAS operand is a 2-D tensor")
    r, c = t.shape
    if t.stride[1] == 1 and t.stride[0] >= max(c, 1):
        return ROW_MAJOR, t.stride[0]
    if t.stride[0] == 1 and t.stride[1] >= max(r, 1):
        return COL_MAJOR, t.stride[1]
    if r <= 1 or c <= 1:
        return ROW_MAJOR, max(c, 1)
    raise RstsrError(1, "a BLAS operand needs a unit stride along one axis")


def _same_order(*ts: Tensor):
    orders = {_blas_operand(t)[0] for t in ts}
    if len(orders) != 1:
        raise RstsrError(1, "BLAS operands must share one memory order")
    return orders.pop()


def _ptr(t: Tensor) -> C.c_void_p:
    return C.c_void_p(t.ptr + t.offset * t.itemsize)


def syrk(a: Tensor, c: Tensor, uplo="L", trans="N", alpha: float = 1.0, beta: float = 0.0,
         precision: int = 0, slices: int = 0) -> Tensor:
    """c's uplo triangle = alpha op(a) op(a)^T + beta c (the other triangle kept)."""
    order = _same_order(a, c)
    n = c.shape[0]
    k = a.shape[1] if trans in ("N", "n") else a.shape[0]
    call("rstsr_cuda_syrk", a.device.ctx, order, uplo.encode(), trans.encode(), n, k, float(alpha), _ptr(a),
         _blas_operand(a)[1], float(beta), _ptr(c), _blas_operand(c)[1], a.dtype_code,
         C.byref(_gemm_opts(precision, slices)))
    return c


def symm(a: Tensor, b: Tensor, c: Tensor, side="L", uplo="L", alpha: float = 1.0, beta: float = 0.0,
         precision: int = 0, slices: int = 0) -> Tensor:
    """c = alpha a b + beta c (side L) or alpha b a + beta c (side R), a read from its uplo triangle."""
    order = _same_order(a, b, c)
    m, n = c.shape
    call("rstsr_cuda_symm", a.device.ctx, order, side.encode(), uplo.encode(), m, n, float(alpha), _ptr(a),
         _blas_operand(a)[1], _ptr(b), _blas_operand(b)[1], float(beta), _ptr(c), _blas_operand(c)[1], a.dtype_code,
         C.byref(_gemm_opts(precision, slices)))
    return c


def trsm(a: Tensor, b: Tensor, side="L", uplo="L", transa="N", diag="N", alpha: float = 1.0,
         precision: int = 0, slices: int = 0) -> Tensor:
    """b := alpha op(a)^-1 b (side L) or alpha b op(a)^-1 (side R), in place."""
    order = _same_order(a, b)
    m, n = b.shape
    call("rstsr_cuda_trsm", a.device.ctx, order, side.encode(), uplo.encode(), transa.encode(), diag.encode(), m, n,
         float(alpha), _ptr(a), _blas_operand(a)[1], _ptr(b), _blas_operand(b)[1], a.dtype_code,
         C.byref(_gemm_opts(precision, slices)))
    return b
