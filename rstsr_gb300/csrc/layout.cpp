// Host-side layout algebra; see layout.hpp for the reference files restated.
#include "layout.hpp"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <numeric>

namespace rstsr {

Layout Layout::from_abi(const rstsr_layout& l) {
    Layout r;
    r.ndim = l.ndim;
    r.offset = l.offset;
    for (int i = 0; i < l.ndim && i < RSTSR_MAX_NDIM; ++i) {
        r.shape[i] = l.shape[i];
        r.stride[i] = l.stride[i];
    }
    return r;
}

rstsr_layout Layout::to_abi() const {
    rstsr_layout r{};
    r.ndim = ndim;
    r.offset = offset;
    for (int i = 0; i < ndim; ++i) {
        r.shape[i] = shape[i];
        r.stride[i] = stride[i];
    }
    return r;
}

// stride_c_contig: last axis 1, each previous axis the product of later extents
// (a zero or one extent is treated as one, as rstsr's shape.c() does).
Layout Layout::c_contig(const int64_t* shp, int n, int64_t off) {
    Layout r;
    r.ndim = n;
    r.offset = off;
    int64_t acc = 1;
    for (int i = n - 1; i >= 0; --i) {
        r.shape[i] = shp[i];
        r.stride[i] = acc;
        acc *= std::max<int64_t>(shp[i], 1);
    }
    return r;
}

Layout Layout::f_contig(const int64_t* shp, int n, int64_t off) {
    Layout r;
    r.ndim = n;
    r.offset = off;
    int64_t acc = 1;
    for (int i = 0; i < n; ++i) {
        r.shape[i] = shp[i];
        r.stride[i] = acc;
        acc *= std::max<int64_t>(shp[i], 1);
    }
    return r;
}

int64_t Layout::size() const {
    int64_t s = 1;
    for (int i = 0; i < ndim; ++i) s *= shape[i];
    return s;
}

int Layout::ndim_of_f_contig() const {
    if (ndim == 0 || size() == 0) return ndim;
    int64_t acc = 1;
    for (int i = 0; i < ndim; ++i) {
        if (shape[i] != 1 && stride[i] != acc) return i;
        acc *= shape[i];
    }
    return ndim;
}

int Layout::ndim_of_c_contig() const {
    if (ndim == 0 || size() == 0) return ndim;
    int64_t acc = 1;
    for (int k = 0; k < ndim; ++k) {
        int i = ndim - 1 - k;
        if (shape[i] != 1 && stride[i] != acc) return k;
        acc *= shape[i];
    }
    return ndim;
}

bool Layout::f_prefer() const {
    if (ndim == 0 || size() == 0) return true;
    int64_t last = 0;
    for (int i = 0; i < ndim; ++i) {
        if (shape[i] != 1) {
            if (stride[i] < last) return false;
            if (last == 0 && stride[i] != 1) return false;
            last = stride[i];
        } else if (last == 0) {
            last = 1;
        }
    }
    return true;
}

bool Layout::c_prefer() const {
    if (ndim == 0 || size() == 0) return true;
    int64_t last = 0;
    for (int i = ndim - 1; i >= 0; --i) {
        if (shape[i] != 1) {
            if (stride[i] < last) return false;
            if (last == 0 && stride[i] != 1) return false;
            last = stride[i];
        } else if (last == 0) {
            last = 1;
        }
    }
    return true;
}

int64_t Layout::size_non_broadcast() const {
    if (size() == 0) return 0;
    int64_t s = 1;
    for (int i = 0; i < ndim; ++i)
        if (stride[i] != 0) s *= shape[i];
    return s;
}

bool Layout::bounds_index(int64_t* lo, int64_t* hi) const {
    if (ndim == 0) {
        *lo = offset;
        *hi = offset + 1;
        return offset >= 0;
    }
    int64_t mn = offset, mx = offset;
    for (int i = 0; i < ndim; ++i) {
        if (shape[i] == 0) {
            *lo = offset;
            *hi = offset;
            return true;
        }
        if (stride[i] > 0)
            mx += stride[i] * (shape[i] - 1);
        else
            mn += stride[i] * (shape[i] - 1);
    }
    *lo = mn;
    *hi = mx + 1;
    return mn >= 0;
}

bool Layout::check_strides(bool skip_zero) const {
    if (size() == 0 || ndim == 0) return true;
    std::vector<int> idx;
    for (int k = 0; k < ndim; ++k)
        if (shape[k] > 1) idx.push_back(k);
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int a, int b) { return std::llabs(stride[a]) < std::llabs(stride[b]); });
    int64_t elem_cum = 0;
    for (int k : idx) {
        int64_t s = std::llabs(stride[k]);
        if (s == 0 && skip_zero) continue;
        if (!(elem_cum < s)) return false;
        elem_cum += (shape[k] - 1) * s;
    }
    return true;
}

Layout Layout::transpose(const int* axes) const {
    Layout r;
    r.ndim = ndim;
    r.offset = offset;
    for (int i = 0; i < ndim; ++i) {
        r.shape[i] = shape[axes[i]];
        r.stride[i] = stride[axes[i]];
    }
    return r;
}

Layout Layout::reverse_axes() const {
    Layout r;
    r.ndim = ndim;
    r.offset = offset;
    for (int i = 0; i < ndim; ++i) {
        r.shape[i] = shape[ndim - 1 - i];
        r.stride[i] = stride[ndim - 1 - i];
    }
    return r;
}

Layout Layout::flip_axis(int n) const {
    Layout r = *this;
    if (shape[n] == 0) return r;
    r.offset = offset + stride[n] * (shape[n] - 1);
    r.stride[n] = -stride[n];
    return r;
}

bool Layout::same_as(const Layout& o) const {
    if (ndim != o.ndim || offset != o.offset) return false;
    for (int i = 0; i < ndim; ++i) {
        if (shape[i] != o.shape[i]) return false;
        if (shape[i] != 1 && shape[i] != 0 && stride[i] != o.stride[i]) return false;
    }
    return true;
}

std::string Layout::repr() const {
    std::string s = "shape=[";
    char buf[64];
    for (int i = 0; i < ndim; ++i) {
        snprintf(buf, sizeof buf, "%s%lld", i ? "," : "", (long long)shape[i]);
        s += buf;
    }
    s += "] stride=[";
    for (int i = 0; i < ndim; ++i) {
        snprintf(buf, sizeof buf, "%s%lld", i ? "," : "", (long long)stride[i]);
        s += buf;
    }
    snprintf(buf, sizeof buf, "] offset=%lld", (long long)offset);
    s += buf;
    return s;
}

Layout greedy_layout(const Layout& l0, bool keep_shape, int* perm) {
    Layout l = l0;
    int n = l.ndim;
    for (int i = 0; i < n; ++i) perm[i] = i;
    if (l.size() == 0) return l;
    if (keep_shape) {
        for (int i = 0; i < n; ++i)
            if (l.stride[i] < 0) l = l.flip_axis(i);
    }
    // Broadcast-like axes (extent 1 or stride 0) first when keeping the shape,
    // last otherwise, in their original order; the rest by ascending |stride|.
    // std::stable_sort mirrors Rust's stable sort_by.
    auto bcast = [&](int i) { return l.shape[i] == 1 || l.stride[i] == 0; };
    std::stable_sort(perm, perm + n, [&](int a, int b) {
        bool ba = bcast(a), bb = bcast(b);
        if (ba && bb) return a < b;
        if (ba != bb) return keep_shape ? ba : bb;
        return std::llabs(l.stride[a]) < std::llabs(l.stride[b]);
    });
    Layout r = l.transpose(perm);
    if (!keep_shape) {
        for (int i = 0; i < n; ++i) {
            if (r.shape[i] == 1 || r.stride[i] == 0) {
                r.shape[i] = 1;
                r.stride[i] = 0;
            }
        }
    }
    return r;
}

Layout layout_for_array_copy_k(const Layout& l) {
    int perm[RSTSR_MAX_NDIM];
    Layout g = greedy_layout(l, true, perm);
    Layout f = Layout::f_contig(g.shape, g.ndim, 0);
    // transpose by the reversed permutation puts each axis back in place
    int inv[RSTSR_MAX_NDIM];
    for (int i = 0; i < l.ndim; ++i) inv[perm[i]] = i;
    return f.transpose(inv);
}

Layout layout_for_array_copy(const Layout& l, char order) {
    switch (order) {
        case 'C': return Layout::c_contig(l.shape, l.ndim);
        case 'F': return Layout::f_contig(l.shape, l.ndim);
        default: return layout_for_array_copy_k(l);
    }
}

void axes_composition(const Layout& l, std::vector<int>& c1, std::vector<int>& c0,
                      std::vector<int>& cc, std::vector<int>& cd) {
    c1.clear();
    c0.clear();
    cc.clear();
    cd.clear();
    std::vector<int> remain;
    for (int i = 0; i < l.ndim; ++i) {
        if (l.shape[i] == 1)
            c1.push_back(i);
        else if (l.stride[i] == 0)
            c0.push_back(i);
        else
            remain.push_back(i);
    }
    std::stable_sort(remain.begin(), remain.end(), [&](int a, int b) {
        return std::llabs(l.stride[a]) < std::llabs(l.stride[b]);
    });
    int64_t cur = 1;
    for (int i : remain) {
        if (l.stride[i] == cur) {
            cc.push_back(i);
            cur *= l.shape[i];
        }
    }
    for (int i : remain)
        if (std::find(cc.begin(), cc.end(), i) == cc.end()) cd.push_back(i);
}

bool layout_for_binary_op(const Layout& la, const Layout& lb, rstsr_order order, Layout* out,
                          Error* err) {
    if (la.ndim != lb.ndim || !std::equal(la.shape, la.shape + la.ndim, lb.shape)) {
        *err = {RSTSR_ERR_INVALID_LAYOUT, "Shape of two layouts must be the same for this function."};
        return false;
    }
    int n = la.ndim;
    std::vector<int> a1, a0a, aca, ada, b1, a0b, acb, adb;
    axes_composition(la, a1, a0a, aca, ada);
    axes_composition(lb, b1, a0b, acb, adb);
    auto has = [](const std::vector<int>& v, int x) { return std::find(v.begin(), v.end(), x) != v.end(); };
    std::vector<int> a0o, aco, ado;
    for (int i : a0a)
        if (has(a0b, i)) a0o.push_back(i);
    for (size_t k = 0; k < std::min(aca.size(), acb.size()); ++k) {
        if (aca[k] == acb[k])
            aco.push_back(aca[k]);
        else
            break;
    }
    for (int i = 0; i < n; ++i)
        if (!has(a0o, i) && !has(aco, i) && !has(a1, i)) ado.push_back(i);
    if (order == RSTSR_ROW_MAJOR) std::reverse(ado.begin(), ado.end());
    Layout r;
    r.ndim = n;
    r.offset = 0;
    for (int i = 0; i < n; ++i) {
        r.shape[i] = la.shape[i];
        r.stride[i] = 0;
    }
    int64_t cur = 1;
    for (int i : aco) {
        r.stride[i] = cur;
        cur *= la.shape[i];
    }
    for (int i : ado) {
        r.stride[i] = cur;
        cur *= la.shape[i];
    }
    for (int i : a1) {
        int64_t s = 1;
        if (order == RSTSR_ROW_MAJOR) {
            for (int j = i; j < n; ++j)
                if (r.stride[j] != 0) {
                    s = r.stride[j];
                    break;
                }
        } else {
            for (int j = i - 1; j >= 0; --j)
                if (r.stride[j] != 0) {
                    s = r.stride[j];
                    break;
                }
        }
        r.stride[i] = s;
    }
    *out = r;
    return true;
}

bool split_axes(const Layout& l, const int64_t* axes, int naxes, Layout* ls, Layout* lm,
                std::vector<int>* axes_norm, Error* err) {
    std::vector<int> ax;
    for (int k = 0; k < naxes; ++k) {
        int64_t a = axes[k];
        if (a < 0) a += l.ndim;
        if (a < 0 || a >= l.ndim) {
            *err = {RSTSR_ERR_INVALID_LAYOUT, "axis " + std::to_string(axes[k]) +
                                                  " out of range for ndim " + std::to_string(l.ndim)};
            return false;
        }
        if (std::find(ax.begin(), ax.end(), (int)a) != ax.end()) {
            *err = {RSTSR_ERR_INVALID_LAYOUT, "duplicate axis " + std::to_string(axes[k])};
            return false;
        }
        ax.push_back((int)a);
    }
    Layout s, m;
    s.offset = m.offset = l.offset;
    for (int a : ax) {
        s.shape[s.ndim] = l.shape[a];
        s.stride[s.ndim] = l.stride[a];
        s.ndim++;
    }
    for (int i = 0; i < l.ndim; ++i) {
        if (std::find(ax.begin(), ax.end(), i) != ax.end()) continue;
        m.shape[m.ndim] = l.shape[i];
        m.stride[m.ndim] = l.stride[i];
        m.ndim++;
    }
    *ls = s;
    *lm = m;
    if (axes_norm) *axes_norm = ax;
    return true;
}

bool broadcast_layouts(const Layout& a0, const Layout& b0, rstsr_order order, Layout* oa,
                       Layout* ob, Error* err) {
    Layout a = order == RSTSR_COL_MAJOR ? a0.reverse_axes() : a0;
    Layout b = order == RSTSR_COL_MAJOR ? b0.reverse_axes() : b0;
    int n = std::max(a.ndim, b.ndim);
    if (n > RSTSR_MAX_NDIM) {
        *err = {RSTSR_ERR_INVALID_LAYOUT, "too many dimensions"};
        return false;
    }
    Layout ra, rb;
    ra.ndim = rb.ndim = n;
    ra.offset = a.offset;
    rb.offset = b.offset;
    for (int i = n - 1; i >= 0; --i) {
        int ia = a.ndim + i - n, ib = b.ndim + i - n;
        int64_t da = ia >= 0 ? a.shape[ia] : 1, db = ib >= 0 ? b.shape[ib] : 1;
        int64_t sa = ia >= 0 ? a.stride[ia] : 0, sb = ib >= 0 ? b.stride[ib] : 0;
        int64_t d;
        if (da == 1 && db == 1) {
            d = 1;
        } else if (db == 1) {
            d = da;
            sb = 0;
        } else if (da == 1) {
            d = db;
            sa = 0;
        } else {
            if (da != db) {
                *err = {RSTSR_ERR_INVALID_LAYOUT, "Broadcasting failed."};
                return false;
            }
            d = da;
        }
        if (ia < 0) sa = 0;
        if (ib < 0) sb = 0;
        ra.shape[i] = rb.shape[i] = d;
        ra.stride[i] = sa;
        rb.stride[i] = sb;
    }
    *oa = order == RSTSR_COL_MAJOR ? ra.reverse_axes() : ra;
    *ob = order == RSTSR_COL_MAJOR ? rb.reverse_axes() : rb;
    return true;
}

size_t dtype_size(rstsr_dtype t) {
    switch (t) {
        case RSTSR_F64: case RSTSR_I64: case RSTSR_U64: return 8;
        case RSTSR_F32: case RSTSR_I32: case RSTSR_U32: return 4;
        case RSTSR_F16: case RSTSR_BF16: case RSTSR_I16: case RSTSR_U16: return 2;
        case RSTSR_I8: case RSTSR_U8: case RSTSR_BOOL: return 1;
    }
    return 0;
}

bool dtype_valid(int t) { return t >= RSTSR_F64 && t <= RSTSR_BOOL; }

const char* dtype_name(rstsr_dtype t) {
    static const char* names[] = {"f64", "f32", "f16", "bf16", "i8", "i16", "i32",
                                  "i64", "u8",  "u16", "u32",  "u64", "bool"};
    return dtype_valid(t) ? names[t] : "?";
}

}  // namespace rstsr

namespace rstsr {

static bool matmul_row_major(const Layout& la, const Layout& lb, Layout* lc, Error* err) {
    const int na = la.ndim, nb = lb.ndim;
    auto bad = [&](const char* m) {
        *err = {RSTSR_ERR_INVALID_LAYOUT, std::string("matmul: ") + m + " (a " + la.repr() + ", b " + lb.repr() + ")"};
        return false;
    };
    if (na == 0 || nb == 0) return bad("0-dim operands are not allowed");
    int64_t sc[RSTSR_MAX_NDIM];
    int nc = 0;
    if (na == 1 && nb == 1) {  // rule 1: inner dot
        if (la.shape[0] != lb.shape[0]) return bad("inner-dot lengths differ");
    } else if (na == 2 && nb == 2) {  // rule 2
        if (la.shape[1] != lb.shape[0]) return bad("contracted extents differ");
        sc[nc++] = la.shape[0];
        sc[nc++] = lb.shape[1];
    } else if (na == 1) {  // rule 3: K @ (..., K, N) -> (..., N)
        if (la.shape[0] != lb.shape[nb - 2]) return bad("contracted extents differ");
        for (int i = 0; i < nb - 2; ++i) sc[nc++] = lb.shape[i];
        sc[nc++] = lb.shape[nb - 1];
    } else if (nb == 1) {  // rule 4: (..., M, K) @ K -> (..., M)
        if (lb.shape[0] != la.shape[na - 1]) return bad("contracted extents differ");
        for (int i = 0; i < na - 2; ++i) sc[nc++] = la.shape[i];
        sc[nc++] = la.shape[na - 2];
    } else if (na == 2) {  // rule 5
        if (la.shape[1] != lb.shape[nb - 2]) return bad("contracted extents differ");
        for (int i = 0; i < nb - 2; ++i) sc[nc++] = lb.shape[i];
        sc[nc++] = la.shape[0];
        sc[nc++] = lb.shape[nb - 1];
    } else if (nb == 2) {  // rule 6
        if (la.shape[na - 1] != lb.shape[0]) return bad("contracted extents differ");
        for (int i = 0; i < na - 2; ++i) sc[nc++] = la.shape[i];
        sc[nc++] = la.shape[na - 2];
        sc[nc++] = lb.shape[1];
    } else {  // rule 7: batch axes broadcast
        if (la.shape[na - 1] != lb.shape[nb - 2]) return bad("contracted extents differ");
        Layout ra, rb, oa, ob;
        ra.ndim = na - 2;
        rb.ndim = nb - 2;
        for (int i = 0; i < ra.ndim; ++i) {
            ra.shape[i] = la.shape[i];
            ra.stride[i] = la.stride[i];
        }
        for (int i = 0; i < rb.ndim; ++i) {
            rb.shape[i] = lb.shape[i];
            rb.stride[i] = lb.stride[i];
        }
        if (!broadcast_layouts(ra, rb, RSTSR_ROW_MAJOR, &oa, &ob, err)) return false;
        if (oa.ndim + 2 > RSTSR_MAX_NDIM) return bad("too many dimensions");
        for (int i = 0; i < oa.ndim; ++i) sc[nc++] = oa.shape[i];
        sc[nc++] = la.shape[na - 2];
        sc[nc++] = lb.shape[nb - 1];
    }
    *lc = Layout::c_contig(sc, nc);
    return true;
}

bool matmul_output_layout(const Layout& la, const Layout& lb, rstsr_order order, Layout* lc, Error* err) {
    if (order == RSTSR_ROW_MAJOR) return matmul_row_major(la, lb, lc, err);
    // col-major: C[n, m, t] = B[n, k, t] @ A[k, m, t] on reversed axes
    Layout r;
    if (!matmul_row_major(lb.reverse_axes(), la.reverse_axes(), &r, err)) return false;
    *lc = r.reverse_axes();
    return true;
}

}  // namespace rstsr
