// Boolean-valued element-wise operators: the IsFinite / IsInf / IsNan /
// SignBit predicates (rstsr-core/src/feature_rayon/auto_impl/
// op_binary_common.rs:94-120), the comparisons OpEqualAPI ... OpLessEqualAPI
// and OpIsCloseAPI (rstsr-core/src/operators/ops/op_ternary_common.rs:3-100,
// rstsr-dtype-traits/src/isclose.rs:92-105). They run on the strided
// element-wise kernel with a bool (byte) output type. OpAllCloseAPI::allclose_all
// (rstsr-core/src/feature_rayon/auto_impl/reduction.rs:717-749) is isclose into
// scratch followed by the all-reduction.
#include "ew_kernel.cuh"

namespace rstsr {

namespace {

template <typename T>
__device__ __forceinline__ bool sign_bit_clear(T v) {
    if constexpr (std::is_same<T, double>::value) return !signbit(v);
    else if constexpr (std::is_same<T, float>::value) return !signbit(v);
    else if constexpr (std::is_same<T, __half>::value) return !(__half_as_ushort(v) & 0x8000);
    else return !(__bfloat16_as_ushort(v) & 0x8000);
}

template <typename T>
struct PredF {
    int op;
    __device__ __forceinline__ uint8_t operator()(const T* v) const {
        const T a = v[0];
        if constexpr (is_float_v<T>) {
            const auto x = widen(a);
            switch (op) {
                case RSTSR_PRED_ISFINITE: return (uint8_t)isfinite(x);
                case RSTSR_PRED_ISINF: return (uint8_t)isinf(x);
                case RSTSR_PRED_ISNAN: return (uint8_t)(x != x);
                default: return (uint8_t)sign_bit_clear(a);  // Signed::is_positive of a float
            }
        } else {
            return (uint8_t)(a > (T)0);  // Signed::is_positive of an integer
        }
    }
};

template <typename T>
struct CmpF {
    int op;
    __device__ __forceinline__ uint8_t operator()(const T* v) const {
        if constexpr (is_float_v<T>) {
            const auto x = widen(v[0]), y = widen(v[1]);
            switch (op) {
                case RSTSR_CMP_EQ: return x == y;
                case RSTSR_CMP_NE: return x != y;
                case RSTSR_CMP_GT: return x > y;
                case RSTSR_CMP_GE: return x >= y;
                case RSTSR_CMP_LT: return x < y;
                default: return x <= y;
            }
        } else {
            const T x = v[0], y = v[1];
            switch (op) {
                case RSTSR_CMP_EQ: return x == y;
                case RSTSR_CMP_NE: return x != y;
                case RSTSR_CMP_GT: return x > y;
                case RSTSR_CMP_GE: return x >= y;
                case RSTSR_CMP_LT: return x < y;
                default: return x <= y;
            }
        }
    }
};

// |a - b| (in T, wrapping for integers) <= atol + rtol |b| in f64, or both NaN
// with equal_nan. The f64 test keeps its two roundings (no fused multiply-add).
template <typename T>
struct IsCloseF {
    double rtol, atol;
    int equal_nan;
    __device__ __forceinline__ uint8_t operator()(const T* v) const {
        const T a = v[0], b = v[1];
        double diff, absb;
        bool both_nan = false;
        if constexpr (is_float_v<T>) {
            const T d = narrow<T>(widen(a) - widen(b));
            diff = fabs((double)widen(d));
            absb = fabs((double)widen(b));
            both_nan = widen(a) != widen(a) && widen(b) != widen(b);
        } else if constexpr (std::is_signed<T>::value) {
            using U = typename std::make_unsigned<T>::type;
            const T d = a >= b ? (T)((U)a - (U)b) : (T)((U)b - (U)a);
            diff = (double)d;
            absb = (double)(b < 0 ? (T)((U)0 - (U)b) : b);
        } else {
            diff = (double)(a >= b ? (T)(a - b) : (T)(b - a));
            absb = (double)b;
        }
        const bool comp = diff <= __dadd_rn(atol, __dmul_rn(rtol, absb));
        return (uint8_t)(comp || (equal_nan && both_nan));
    }
};

template <template <typename> class F, typename... Args>
int dispatch_bool_out(rstsr_ctx* ctx, rstsr_dtype t, const IterSpace& sp, void* c, const EwInput* ins, int nin,
                      Args... args) {
#define RSTSR_BOOL_OUT(T)                                                                                  \
    return nin == 1 ? launch_ew<uint8_t, T, 1>(ctx, sp, c, ins, F<T>{args...}, "bool_op")                 \
                    : launch_ew<uint8_t, T, 2>(ctx, sp, c, ins, F<T>{args...}, "bool_op")
    switch (t) {
        case RSTSR_F64: RSTSR_BOOL_OUT(double);
        case RSTSR_F32: RSTSR_BOOL_OUT(float);
        case RSTSR_F16: RSTSR_BOOL_OUT(__half);
        case RSTSR_BF16: RSTSR_BOOL_OUT(__nv_bfloat16);
        case RSTSR_I8: RSTSR_BOOL_OUT(int8_t);
        case RSTSR_I16: RSTSR_BOOL_OUT(int16_t);
        case RSTSR_I32: RSTSR_BOOL_OUT(int32_t);
        case RSTSR_I64: RSTSR_BOOL_OUT(int64_t);
        case RSTSR_U8: RSTSR_BOOL_OUT(uint8_t);
        case RSTSR_U16: RSTSR_BOOL_OUT(uint16_t);
        case RSTSR_U32: RSTSR_BOOL_OUT(uint32_t);
        case RSTSR_U64: RSTSR_BOOL_OUT(uint64_t);
        case RSTSR_BOOL: RSTSR_BOOL_OUT(uint8_t);
        default: return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    }
#undef RSTSR_BOOL_OUT
}

bool is_signed_dtype(rstsr_dtype t) {
    return t == RSTSR_I8 || t == RSTSR_I16 || t == RSTSR_I32 || t == RSTSR_I64;
}

// Shared checks of the two-operand forms; fills the iteration space.
int prepare2(rstsr_ctx* ctx, rstsr_dtype t, void* c, const rstsr_layout* lc, const void* a, const rstsr_layout* la,
             const void* b, const rstsr_layout* lb, const char* what, IterSpace* sp, bool* empty) {
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(lc, "c"));
    RSTSR_TRY(check_layout(la, "a"));
    if (lb) RSTSR_TRY(check_layout(lb, "b"));
    if (!dtype_valid(t)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    Layout Lc = Layout::from_abi(*lc), La = Layout::from_abi(*la);
    Layout Lb = lb ? Layout::from_abi(*lb) : La;
    if (!lb) {  // a scalar operand: all strides zero
        for (int i = 0; i < Lb.ndim; ++i) Lb.stride[i] = 0;
        Lb.offset = 0;
    }
    RSTSR_TRY(check_same_shape3(Lc, La, &Lb, what));
    RSTSR_TRY(check_write_layout(Lc, what));
    *empty = Lc.size() == 0;
    if (*empty) return RSTSR_OK;
    if (!c || !a || (lb && !b)) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    const Layout* ls[3] = {&Lc, &La, &Lb};
    *sp = make_iter_space(ls, 3);
    return RSTSR_OK;
}

}  // namespace

}  // namespace rstsr

using namespace rstsr;

extern "C" {

int rstsr_cuda_unary_predicate(rstsr_ctx* ctx, rstsr_predicate_op op, rstsr_dtype ta, void* c,
                               const rstsr_layout* lc, const void* a, const rstsr_layout* la) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(lc, "c"));
    RSTSR_TRY(check_layout(la, "a"));
    if (!dtype_valid(ta)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    if (op < RSTSR_PRED_ISFINITE || op > RSTSR_PRED_SIGNBIT) return fail(RSTSR_ERR_INVALID_VALUE, "unknown predicate");
    const bool ok = op == RSTSR_PRED_SIGNBIT ? (is_float_dtype(ta) || is_signed_dtype(ta)) : is_float_dtype(ta);
    if (!ok)
        return fail(RSTSR_ERR_INVALID_VALUE,
                    std::string("predicate ") + std::to_string(op) + " is not defined on " + dtype_name(ta));
    Layout Lc = Layout::from_abi(*lc), La = Layout::from_abi(*la);
    RSTSR_TRY(check_same_shape3(Lc, La, nullptr, "unary_predicate"));
    RSTSR_TRY(check_write_layout(Lc, "unary_predicate"));
    if (Lc.size() == 0) return RSTSR_OK;
    if (!c || !a) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    const Layout* ls[2] = {&Lc, &La};
    IterSpace sp = make_iter_space(ls, 2);
    EwInput ins[1] = {{a, nullptr}};
    return dispatch_bool_out<PredF>(ctx, ta, sp, c, ins, 1, (int)op);
}

int rstsr_cuda_compare(rstsr_ctx* ctx, rstsr_compare_op op, rstsr_dtype t, void* c, const rstsr_layout* lc,
                       const void* a, const rstsr_layout* la, const void* b, const rstsr_layout* lb) {
    clear_error();
    if (op < RSTSR_CMP_EQ || op > RSTSR_CMP_LE) return fail(RSTSR_ERR_INVALID_VALUE, "unknown comparison");
    IterSpace sp;
    bool empty;
    RSTSR_TRY(prepare2(ctx, t, c, lc, a, la, b, lb, "compare", &sp, &empty));
    if (empty) return RSTSR_OK;
    EwInput ins[2] = {{a, nullptr}, {b, nullptr}};
    return dispatch_bool_out<CmpF>(ctx, t, sp, c, ins, 2, (int)op);
}

int rstsr_cuda_compare_scalar(rstsr_ctx* ctx, rstsr_compare_op op, rstsr_dtype t, void* c, const rstsr_layout* lc,
                              const void* a, const rstsr_layout* la, const void* scalar, int32_t scalar_is_lhs) {
    clear_error();
    if (op < RSTSR_CMP_EQ || op > RSTSR_CMP_LE) return fail(RSTSR_ERR_INVALID_VALUE, "unknown comparison");
    if (!scalar) return fail(RSTSR_ERR_INVALID_VALUE, "null scalar");
    IterSpace sp;
    bool empty;
    RSTSR_TRY(prepare2(ctx, t, c, lc, a, la, nullptr, nullptr, "compare_scalar", &sp, &empty));
    if (empty) return RSTSR_OK;
    EwInput ins[2];
    if (scalar_is_lhs) {
        // the iteration space holds a's strides in operand 1: swap the operands' roles
        std::swap(sp.stride[1], sp.stride[2]);
        std::swap(sp.offset[1], sp.offset[2]);
        ins[0] = {nullptr, scalar};
        ins[1] = {a, nullptr};
    } else {
        ins[0] = {a, nullptr};
        ins[1] = {nullptr, scalar};
    }
    return dispatch_bool_out<CmpF>(ctx, t, sp, c, ins, 2, (int)op);
}

int rstsr_cuda_isclose(rstsr_ctx* ctx, rstsr_dtype t, void* c, const rstsr_layout* lc, const void* a,
                       const rstsr_layout* la, const void* b, const rstsr_layout* lb, double rtol, double atol,
                       int32_t equal_nan) {
    clear_error();
    if (t == RSTSR_BOOL) return fail(RSTSR_ERR_INVALID_VALUE, "isclose is not defined on bool");
    IterSpace sp;
    bool empty;
    RSTSR_TRY(prepare2(ctx, t, c, lc, a, la, b, lb, "isclose", &sp, &empty));
    if (empty) return RSTSR_OK;
    EwInput ins[2] = {{a, nullptr}, {b, nullptr}};
    return dispatch_bool_out<IsCloseF>(ctx, t, sp, c, ins, 2, rtol, atol, (int)(equal_nan != 0));
}

int rstsr_cuda_allclose_all(rstsr_ctx* ctx, rstsr_dtype t, const void* a, const rstsr_layout* la, const void* b,
                            const rstsr_layout* lb, double rtol, double atol, int32_t equal_nan, uint8_t* out_host) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(la, "a"));
    RSTSR_TRY(check_layout(lb, "b"));
    if (!out_host) return fail(RSTSR_ERR_INVALID_VALUE, "null output");
    const Layout A = Layout::from_abi(*la), B = Layout::from_abi(*lb);
    if (A.size() == 0 || B.size() == 0)
        return fail(RSTSR_ERR_INVALID_VALUE, "zero-size array is not supported for allclose");
    if (!same_shape(A, B))
        return fail(RSTSR_ERR_INVALID_LAYOUT, "allclose: a and b differ in shape (broadcast them first)");
    // the element-wise test into a C-contiguous bool scratch, then the all-reduction
    const Layout M = Layout::c_contig(A.shape, A.ndim);
    void* mask = nullptr;
    RSTSR_TRY(scratch_alloc(ctx, (size_t)M.size(), &mask));
    const rstsr_layout lm = M.to_abi();
    int rc = rstsr_cuda_isclose(ctx, t, mask, &lm, a, la, b, lb, rtol, atol, equal_nan);
    if (rc == RSTSR_OK) rc = rstsr_cuda_reduce_all(ctx, RSTSR_RED_ALL, RSTSR_BOOL, mask, &lm, out_host);
    scratch_free(ctx, mask);
    return rc;
}

}  // extern "C"
