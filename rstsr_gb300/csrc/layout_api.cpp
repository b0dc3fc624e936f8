// Host-only C ABI exports of the layout algebra (no GPU required).
#include <vector>

#include "layout.hpp"

using namespace rstsr;

static int check_abi_layout(const rstsr_layout* l, const char* name) {
    if (!l) return fail(RSTSR_ERR_INVALID_LAYOUT, std::string(name) + ": null layout");
    if (l->ndim < 0 || l->ndim > RSTSR_MAX_NDIM)
        return fail(RSTSR_ERR_INVALID_LAYOUT, std::string(name) + ": ndim outside [0, 8]");
    for (int i = 0; i < l->ndim; ++i)
        if (l->shape[i] < 0) return fail(RSTSR_ERR_INVALID_LAYOUT, std::string(name) + ": negative extent");
    return RSTSR_OK;
}

#define RSTSR_TRY_H(expr)              \
    do {                               \
        int _s = (expr);               \
        if (_s != RSTSR_OK) return _s; \
    } while (0)

extern "C" {

int rstsr_cuda_layout_broadcast(const rstsr_layout* la, const rstsr_layout* lb, rstsr_order order,
                                rstsr_layout* oa, rstsr_layout* ob) {
    clear_error();
    RSTSR_TRY_H(check_abi_layout(la, "a"));
    RSTSR_TRY_H(check_abi_layout(lb, "b"));
    if (!oa || !ob) return fail(RSTSR_ERR_INVALID_VALUE, "null output");
    Layout A, B;
    Error e;
    if (!broadcast_layouts(Layout::from_abi(*la), Layout::from_abi(*lb), order, &A, &B, &e)) return fail(e.code, e.msg);
    *oa = A.to_abi();
    *ob = B.to_abi();
    return RSTSR_OK;
}

int rstsr_cuda_layout_binary_op(const rstsr_layout* la, const rstsr_layout* lb, rstsr_order order,
                                rstsr_layout* out) {
    clear_error();
    RSTSR_TRY_H(check_abi_layout(la, "a"));
    RSTSR_TRY_H(check_abi_layout(lb, "b"));
    if (!out) return fail(RSTSR_ERR_INVALID_VALUE, "null output");
    Layout C;
    Error e;
    if (!layout_for_binary_op(Layout::from_abi(*la), Layout::from_abi(*lb), order, &C, &e)) return fail(e.code, e.msg);
    *out = C.to_abi();
    return RSTSR_OK;
}

int rstsr_cuda_layout_for_array_copy(const rstsr_layout* l, char order, rstsr_layout* out) {
    clear_error();
    RSTSR_TRY_H(check_abi_layout(l, "l"));
    if (!out) return fail(RSTSR_ERR_INVALID_VALUE, "null output");
    if (order != 'C' && order != 'F' && order != 'K')
        return fail(RSTSR_ERR_INVALID_VALUE, "Iter order for copy only accepts CFK.");
    *out = layout_for_array_copy(Layout::from_abi(*l), order).to_abi();
    return RSTSR_OK;
}

int rstsr_cuda_layout_greedy(const rstsr_layout* l, int32_t keep_shape, rstsr_layout* out, int32_t* perm) {
    clear_error();
    RSTSR_TRY_H(check_abi_layout(l, "l"));
    if (!out) return fail(RSTSR_ERR_INVALID_VALUE, "null output");
    int p[RSTSR_MAX_NDIM];
    *out = greedy_layout(Layout::from_abi(*l), keep_shape != 0, p).to_abi();
    if (perm)
        for (int i = 0; i < l->ndim; ++i) perm[i] = p[i];
    return RSTSR_OK;
}

int rstsr_cuda_unravel_index(const int64_t* shape, int32_t ndim, uint64_t index, rstsr_order order,
                             int64_t* out) {
    clear_error();
    if (ndim < 0 || ndim > RSTSR_MAX_NDIM) return fail(RSTSR_ERR_INVALID_VALUE, "unravel_index: ndim outside [0, 8]");
    if (ndim > 0 && (!shape || !out)) return fail(RSTSR_ERR_INVALID_VALUE, "unravel_index: null argument");
    uint64_t size = 1;
    for (int i = 0; i < ndim; ++i) {
        if (shape[i] < 0) return fail(RSTSR_ERR_INVALID_VALUE, "unravel_index: negative extent");
        size *= (uint64_t)shape[i];
    }
    if (index >= size) return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, "unravel_index: index outside the shape");
    // C order: the last axis varies fastest; F order: the first
    for (int k = 0; k < ndim; ++k) {
        const int i = order == RSTSR_ROW_MAJOR ? ndim - 1 - k : k;
        out[i] = (int64_t)(index % (uint64_t)shape[i]);
        index /= (uint64_t)shape[i];
    }
    return RSTSR_OK;
}

int32_t rstsr_cuda_layout_flags(const rstsr_layout* l) {
    if (!l || l->ndim < 0 || l->ndim > RSTSR_MAX_NDIM) return -1;
    Layout L = Layout::from_abi(*l);
    return (L.c_contig() ? 1 : 0) | (L.f_contig() ? 2 : 0) | (L.c_prefer() ? 4 : 0) | (L.f_prefer() ? 8 : 0);
}

int rstsr_cuda_reduce_axes_layout(const rstsr_layout* la, const int64_t* axes, int32_t naxes, rstsr_layout* lout) {
    clear_error();
    RSTSR_TRY_H(check_abi_layout(la, "a"));
    if (!lout) return fail(RSTSR_ERR_INVALID_VALUE, "null output");
    if (naxes > 0 && !axes) return fail(RSTSR_ERR_INVALID_VALUE, "null axes");
    Layout ls, lm;
    Error e;
    if (!split_axes(Layout::from_abi(*la), axes, naxes, &ls, &lm, nullptr, &e)) return fail(e.code, e.msg);
    *lout = layout_for_array_copy_k(lm).to_abi();
    return RSTSR_OK;
}

int rstsr_cuda_matmul_layout(const rstsr_layout* la, const rstsr_layout* lb, rstsr_order order, rstsr_layout* lc) {
    clear_error();
    RSTSR_TRY_H(check_abi_layout(la, "a"));
    RSTSR_TRY_H(check_abi_layout(lb, "b"));
    if (!lc) return fail(RSTSR_ERR_INVALID_VALUE, "null output");
    Layout C;
    Error e;
    if (!matmul_output_layout(Layout::from_abi(*la), Layout::from_abi(*lb), order, &C, &e)) return fail(e.code, e.msg);
    *lc = C.to_abi();
    return RSTSR_OK;
}

}  // extern "C"
