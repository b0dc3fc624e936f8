"""Python restatement of rstsr-common's layout algebra (TEST INFRASTRUCTURE ONLY).

Written independently of the device library's C++ planner so the two can be
checked against each other and against the reference's own unit-test cases.
A layout is a tuple ``(shape, stride, offset)`` in elements.

  greedy_layout              rstsr-common/src/layout/rearrangement.rs:36-113
  layout_for_array_copy      rearrangement.rs:125-152
  get_axes_composition       rearrangement.rs:335-372
  get_layout_for_binary_op   rearrangement.rs:394-459
  broadcast_layout           rstsr-common/src/layout/broadcast.rs:21-245
  contiguity flags           rstsr-common/src/layout/layoutbase.rs:89-205
  matmul output layout       rstsr-common/src/layout/matmul.rs:70-460
"""

from __future__ import annotations

from functools import cmp_to_key


def c_stride(shape):
    st, acc = [], 1
    for d in reversed(shape):
        st.append(acc)
        acc *= max(d, 1)
    return tuple(reversed(st))


def f_stride(shape):
    st, acc = [], 1
    for d in shape:
        st.append(acc)
        acc *= max(d, 1)
    return tuple(st)


def size(shape):
    n = 1
    for d in shape:
        n *= d
    return n


def ndim_of_f_contig(shape, stride):
    if len(shape) == 0 or size(shape) == 0:
        return len(shape)
    acc = 1
    for i, (d, s) in enumerate(zip(shape, stride)):
        if d != 1 and s != acc:
            return i
        acc *= d
    return len(shape)


def ndim_of_c_contig(shape, stride):
    return ndim_of_f_contig(shape[::-1], stride[::-1])


def f_contig(shape, stride):
    return ndim_of_f_contig(shape, stride) == len(shape)


def c_contig(shape, stride):
    return ndim_of_c_contig(shape, stride) == len(shape)


def _prefer(shape, stride):
    if len(shape) == 0 or size(shape) == 0:
        return True
    last = 0
    for d, s in zip(shape, stride):
        if d != 1:
            if s < last:
                return False
            if last == 0 and s != 1:
                return False
            last = s
        elif last == 0:
            last = 1
    return True


def f_prefer(shape, stride):
    return _prefer(shape, stride)


def c_prefer(shape, stride):
    return _prefer(shape[::-1], stride[::-1])


def greedy_layout(layout, keep_shape):
    """Returns (layout, permutation)."""
    shape, stride, offset = list(layout[0]), list(layout[1]), layout[2]
    n = len(shape)
    if size(shape) == 0:
        return (tuple(shape), tuple(stride), offset), list(range(n))
    if keep_shape:
        for i in range(n):
            if stride[i] < 0:
                offset += stride[i] * (shape[i] - 1)
                stride[i] = -stride[i]

    def bc(i):
        return shape[i] == 1 or stride[i] == 0

    def cmp(i1, i2):
        b1, b2 = bc(i1), bc(i2)
        if b1 and b2:
            return (i1 > i2) - (i1 < i2)
        if b1 and not b2:
            return -1 if keep_shape else 1
        if b2 and not b1:
            return 1 if keep_shape else -1
        s1, s2 = abs(stride[i1]), abs(stride[i2])
        return (s1 > s2) - (s1 < s2)

    perm = sorted(range(n), key=cmp_to_key(cmp))  # Python's sort is stable
    nshape = [shape[p] for p in perm]
    nstride = [stride[p] for p in perm]
    if not keep_shape:
        for i in range(n):
            if nshape[i] == 1 or nstride[i] == 0:
                nshape[i], nstride[i] = 1, 0
    return (tuple(nshape), tuple(nstride), offset), perm


def layout_for_array_copy(layout, order="K"):
    shape = tuple(layout[0])
    if order == "C":
        return shape, c_stride(shape), 0
    if order == "F":
        return shape, f_stride(shape), 0
    (gshape, _, _), perm = greedy_layout(layout, True)
    fs = f_stride(gshape)
    inv = [0] * len(perm)
    for i, p in enumerate(perm):
        inv[p] = i
    return shape, tuple(fs[inv[i]] for i in range(len(shape))), 0


def axes_composition(layout):
    shape, stride = layout[0], layout[1]
    c1 = [i for i in range(len(shape)) if shape[i] == 1]
    c0 = [i for i in range(len(shape)) if shape[i] != 1 and stride[i] == 0]
    remain = sorted([i for i in range(len(shape)) if i not in c1 and i not in c0], key=lambda i: abs(stride[i]))
    cc, cur = [], 1
    for i in remain:
        if stride[i] == cur:
            cc.append(i)
            cur *= shape[i]
    cd = [i for i in remain if i not in cc]
    return c1, c0, cc, cd


def layout_for_binary_op(la, lb, order="C"):
    if tuple(la[0]) != tuple(lb[0]):
        raise ValueError("shapes differ")
    shape = tuple(la[0])
    n = len(shape)
    a1, a0a, aca, _ = axes_composition(la)
    _, a0b, acb, _ = axes_composition(lb)
    a0o = [i for i in a0a if i in a0b]
    aco = []
    for x, y in zip(aca, acb):
        if x == y:
            aco.append(x)
        else:
            break
    ado = [i for i in range(n) if i not in a0o and i not in aco and i not in a1]
    if order == "C":
        ado.reverse()
    stride = [0] * n
    cur = 1
    for i in aco + ado:
        stride[i] = cur
        cur *= shape[i]
    for i in a1:
        s = 1
        if order == "C":
            for x in stride[i:]:
                if x != 0:
                    s = x
                    break
        else:
            for x in reversed(stride[:i]):
                if x != 0:
                    s = x
                    break
        stride[i] = s
    return shape, tuple(stride), 0


def broadcast_layout(la, lb, order="C"):
    sa, sb = list(la[0]), list(lb[0])
    ta, tb = list(la[1]), list(lb[1])
    if order == "F":
        sa, sb, ta, tb = sa[::-1], sb[::-1], ta[::-1], tb[::-1]
    n = max(len(sa), len(sb))
    shape, oa, ob = [0] * n, [0] * n, [0] * n
    for i in range(n - 1, -1, -1):
        ia, ib = len(sa) + i - n, len(sb) + i - n
        da = sa[ia] if ia >= 0 else 1
        db = sb[ib] if ib >= 0 else 1
        xa = ta[ia] if ia >= 0 else 0
        xb = tb[ib] if ib >= 0 else 0
        if da == 1 and db == 1:
            d = 1
        elif db == 1:
            d, xb = da, 0
        elif da == 1:
            d, xa = db, 0
        else:
            if da != db:
                raise ValueError("Broadcasting failed.")
            d = da
        shape[i], oa[i], ob[i] = d, xa, xb
    if order == "F":
        shape, oa, ob = shape[::-1], oa[::-1], ob[::-1]
    return (tuple(shape), tuple(oa), la[2]), (tuple(shape), tuple(ob), lb[2])


def matmul_shape(sa, sb, order="C"):
    """Output shape of matmul (rules 1-7); col-major reverses axes and swaps operands."""
    if order == "F":
        return tuple(reversed(matmul_shape(tuple(reversed(sb)), tuple(reversed(sa)), "C")))
    na, nb = len(sa), len(sb)
    if na == 0 or nb == 0:
        raise ValueError("0-dim")
    if na == 1 and nb == 1:
        assert sa == sb
        return ()
    if na == 2 and nb == 2:
        assert sa[1] == sb[0]
        return (sa[0], sb[1])
    if na == 1:
        assert sa[0] == sb[-2]
        return tuple(sb[:-2]) + (sb[-1],)
    if nb == 1:
        assert sb[0] == sa[-1]
        return tuple(sa[:-2]) + (sa[-2],)
    if na == 2:
        return tuple(sb[:-2]) + (sa[0], sb[-1])
    if nb == 2:
        return tuple(sa[:-2]) + (sa[-2], sb[1])
    (bs, _, _), _ = broadcast_layout((tuple(sa[:-2]), (0,) * (na - 2), 0), (tuple(sb[:-2]), (0,) * (nb - 2), 0))
    return tuple(bs) + (sa[-2], sb[-1])


def reduce_output_layout(layout, axes):
    """layout_for_array_copy(kept, K) after dim_split_axes."""
    shape, stride, offset = layout
    n = len(shape)
    axes = [a + n if a < 0 else a for a in axes]
    kept = [i for i in range(n) if i not in axes]
    lm = (tuple(shape[i] for i in kept), tuple(stride[i] for i in kept), offset)
    return layout_for_array_copy(lm, "K")
