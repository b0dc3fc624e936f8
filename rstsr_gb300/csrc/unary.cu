// Unary operators: OpNegAPI / OpNotAPI (rstsr-core/src/operators/ops/
// op_binary_arithmetic.rs:95-109) and the element-wise math family of
// rstsr-core/src/operators/ops/op_binary_common.rs:3-65. Transcendental
// functions call CUDA's own math library; they are not bit-identical to the
// host libm and are checked within a tolerance.
#include "ew_kernel.cuh"

namespace rstsr {

template <typename T>
using UnsignedOf = typename std::make_unsigned<T>::type;

template <typename T, int OP, bool IS_BOOL>
__device__ __forceinline__ T unop(T a) {
    if constexpr (IS_BOOL) {
        return (T)(a ^ 1);  // NOT
    } else {
        using U = UnsignedOf<T>;
        if constexpr (OP == RSTSR_UOP_NEG) return (T)((U)0 - (U)a);
        else if constexpr (OP == RSTSR_UOP_NOT) return (T)~a;
        else if constexpr (OP == RSTSR_UOP_ABS) {
            if constexpr (std::is_signed<T>::value) return a < 0 ? (T)((U)0 - (U)a) : a;
            else return a;
        } else if constexpr (OP == RSTSR_UOP_SQUARE) return (T)((U)a * (U)a);
        else {  // SIGN
            if constexpr (std::is_signed<T>::value) return (T)((a > 0) - (a < 0));
            else return (T)(a > 0);
        }
    }
}

static bool uop_valid(int op, rstsr_dtype t) {
    if (t == RSTSR_BOOL) return op == RSTSR_UOP_NOT;
    if (is_float_dtype(t)) return op != RSTSR_UOP_NOT;
    return op == RSTSR_UOP_NEG || op == RSTSR_UOP_NOT || op == RSTSR_UOP_ABS || op == RSTSR_UOP_SQUARE ||
           op == RSTSR_UOP_SIGN || op == RSTSR_UOP_CONJ || op == RSTSR_UOP_REAL || op == RSTSR_UOP_IMAG;
}

// Floating-point unary math in the compute type (float or double), kept out
// of line so the strided kernel's unrolled body stays small.
template <typename C>
__device__ __noinline__ C float_unary(int op, C x) {
    switch (op) {
        case RSTSR_UOP_NEG: return -x;
        case RSTSR_UOP_ABS: return fabs(x);
        case RSTSR_UOP_SQRT: return sqrt(x);
        case RSTSR_UOP_EXP: return exp(x);
        case RSTSR_UOP_LOG: return log(x);
        case RSTSR_UOP_SIN: return sin(x);
        case RSTSR_UOP_COS: return cos(x);
        case RSTSR_UOP_TANH: return tanh(x);
        case RSTSR_UOP_SQUARE: return x * x;
        case RSTSR_UOP_FLOOR: return floor(x);
        case RSTSR_UOP_CEIL: return ceil(x);
        // ExtNum::ext_sign (rstsr-dtype-traits/src/ext_num.rs:166-178): NaN stays, zeros give 0
        case RSTSR_UOP_SIGN: return (x != x) ? x : (x > (C)0 ? (C)1 : (x < (C)0 ? (C)-1 : (C)0));
        case RSTSR_UOP_ACOS: return acos(x);
        case RSTSR_UOP_ACOSH: return acosh(x);
        case RSTSR_UOP_ASIN: return asin(x);
        case RSTSR_UOP_ASINH: return asinh(x);
        case RSTSR_UOP_ATAN: return atan(x);
        case RSTSR_UOP_ATANH: return atanh(x);
        case RSTSR_UOP_COSH: return cosh(x);
        case RSTSR_UOP_EXPM1: return expm1(x);
        case RSTSR_UOP_LOG1P: return log1p(x);
        case RSTSR_UOP_LOG2: return log2(x);
        case RSTSR_UOP_LOG10: return log10(x);
        case RSTSR_UOP_ROUND: return round(x);  // half away from zero, as Rust's round
        case RSTSR_UOP_SINH: return sinh(x);
        case RSTSR_UOP_TAN: return tan(x);
        case RSTSR_UOP_TRUNC: return trunc(x);
        case RSTSR_UOP_CONJ:
        case RSTSR_UOP_REAL: return x;
        case RSTSR_UOP_IMAG: return (C)0;
        default: return (C)1 / x;  // RECIP, INV
    }
}

template <typename T, bool IS_BOOL>
struct UnRtF {
    int op;
    __device__ __forceinline__ T operator()(const T* v) const {
        const T a = v[0];
        if constexpr (IS_BOOL) {
            return unop<T, RSTSR_UOP_NOT, true>(a);
        } else if constexpr (is_float_v<T>) {
            return narrow<T>(float_unary(op, widen(a)));
        } else {
            switch (op) {
                case RSTSR_UOP_NEG: return unop<T, RSTSR_UOP_NEG, false>(a);
                case RSTSR_UOP_NOT: return unop<T, RSTSR_UOP_NOT, false>(a);
                case RSTSR_UOP_ABS: return unop<T, RSTSR_UOP_ABS, false>(a);
                case RSTSR_UOP_SQUARE: return unop<T, RSTSR_UOP_SQUARE, false>(a);
                case RSTSR_UOP_CONJ:
                case RSTSR_UOP_REAL: return a;
                case RSTSR_UOP_IMAG: return (T)0;
                default: return unop<T, RSTSR_UOP_SIGN, false>(a);
            }
        }
    }
};

// One runtime-dispatched kernel per dtype (the operator switch is uniform
// across a warp).
template <typename T, bool IS_BOOL>
static int unary_typed(rstsr_ctx* ctx, int op, const IterSpace& sp, void* c, const EwInput* ins) {
    return launch_ew<T, T, 1>(ctx, sp, c, ins, UnRtF<T, IS_BOOL>{op}, "unary");
}

}  // namespace rstsr

using namespace rstsr;

extern "C" int rstsr_cuda_unary(rstsr_ctx* ctx, rstsr_unary_op op, rstsr_dtype t, void* c, const rstsr_layout* lc,
                                const void* a, const rstsr_layout* la) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(lc, "c"));
    RSTSR_TRY(check_layout(la, "a"));
    if (!dtype_valid(t)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    if (op < RSTSR_UOP_NEG || op > RSTSR_UOP_IMAG) return fail(RSTSR_ERR_INVALID_VALUE, "unknown unary operator");
    if (!uop_valid(op, t))
        return fail(RSTSR_ERR_INVALID_VALUE,
                    std::string("unary operator ") + std::to_string(op) + " is not defined on " + dtype_name(t));
    Layout Lc = Layout::from_abi(*lc), La = Layout::from_abi(*la);
    RSTSR_TRY(check_same_shape3(Lc, La, nullptr, "unary"));
    RSTSR_TRY(check_write_layout(Lc, "unary"));
    if (Lc.size() == 0) return RSTSR_OK;
    if (!c || !a) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    const Layout* ls[2] = {&Lc, &La};
    IterSpace sp = make_iter_space(ls, 2);
    EwInput ins[1] = {{a, nullptr}};
    switch (t) {
        case RSTSR_F64: return unary_typed<double, false>(ctx, op, sp, c, ins);
        case RSTSR_F32: return unary_typed<float, false>(ctx, op, sp, c, ins);
        case RSTSR_F16: return unary_typed<__half, false>(ctx, op, sp, c, ins);
        case RSTSR_BF16: return unary_typed<__nv_bfloat16, false>(ctx, op, sp, c, ins);
        case RSTSR_I8: return unary_typed<int8_t, false>(ctx, op, sp, c, ins);
        case RSTSR_I16: return unary_typed<int16_t, false>(ctx, op, sp, c, ins);
        case RSTSR_I32: return unary_typed<int32_t, false>(ctx, op, sp, c, ins);
        case RSTSR_I64: return unary_typed<int64_t, false>(ctx, op, sp, c, ins);
        case RSTSR_U8: return unary_typed<uint8_t, false>(ctx, op, sp, c, ins);
        case RSTSR_U16: return unary_typed<uint16_t, false>(ctx, op, sp, c, ins);
        case RSTSR_U32: return unary_typed<uint32_t, false>(ctx, op, sp, c, ins);
        case RSTSR_U64: return unary_typed<uint64_t, false>(ctx, op, sp, c, ins);
        case RSTSR_BOOL: return unary_typed<uint8_t, true>(ctx, op, sp, c, ins);
        default: return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    }
}
