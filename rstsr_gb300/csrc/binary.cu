// Binary operators with broadcasting, their scalar and in-place (consuming)
// forms, and the fused d = a*b + c pass. Replaces
// rstsr-native-impl/src/cpu_rayon/op_with_func.rs (op_mutc_refa_refb :13-80,
// op_mutc_refa_numb / op_mutc_numa_refb :82-212, op_muta_refb :214-276,
// op_muta_numb :278-335) as driven by
// rstsr-core/src/feature_rayon/auto_impl/op_ternary_arithmetic.rs:16-56 and
// auto_impl/op_binary_arithmetic.rs:3-113.
//
// Integer arithmetic wraps (Rust release semantics); integer division or
// remainder by zero yields 0 instead of the reference's panic; shifts mask the
// shift amount to the bit width (wrapping_shl / wrapping_shr).
#include "ew_kernel.cuh"

namespace rstsr {

template <typename T>
using UnsignedOf = typename std::make_unsigned<T>::type;

// nextafter on the bit pattern of a 16-bit float (half or bfloat16): the
// neighbour of x toward y, y itself when equal, the smallest subnormal of y's
// sign from a zero, NaN when either is NaN.
template <typename T>
__device__ __forceinline__ uint16_t bits16(T v) {
    if constexpr (std::is_same<T, __half>::value) return __half_as_ushort(v);
    else return __bfloat16_as_ushort(v);
}
template <typename T>
__device__ __forceinline__ T from_bits16(uint16_t u) {
    if constexpr (std::is_same<T, __half>::value) return __ushort_as_half(u);
    else return __ushort_as_bfloat16(u);
}
template <typename T>
__device__ __forceinline__ T nextafter_t(T a, T b) {
    if constexpr (std::is_same<T, double>::value) {
        return nextafter(a, b);
    } else if constexpr (std::is_same<T, float>::value) {
        return nextafterf(a, b);
    } else {
        const float x = widen(a), y = widen(b);
        if (x != x || y != y) return narrow<T>(x + y);
        uint16_t ux = bits16(a);
        const uint16_t uy = bits16(b);
        if (ux == uy) return b;
        const uint16_t ax = ux & 0x7FFF, ay = uy & 0x7FFF;
        if (ax == 0) {
            if (ay == 0) return b;
            ux = (uint16_t)((uy & 0x8000) | 1);
        } else if (ax > ay || ((ux ^ uy) & 0x8000)) {
            ux = (uint16_t)(ux - 1);
        } else {
            ux = (uint16_t)(ux + 1);
        }
        return from_bits16<T>(ux);
    }
}

template <typename T, int OP, bool IS_BOOL>
__device__ __forceinline__ T binop(T a, T b) {
    if constexpr (is_float_v<T> && OP == RSTSR_OP_NEXTAFTER) {
        return nextafter_t<T>(a, b);
    } else if constexpr (is_float_v<T> && OP == RSTSR_OP_FLOOR_DIVIDE) {
        // Float::floor(a / b): the quotient rounded to T first (matters for 16-bit types)
        return narrow<T>(floor(widen(narrow<T>(widen(a) / widen(b)))));
    } else if constexpr (is_float_v<T> && OP == RSTSR_OP_LOGADDEXP) {
        // (a.exp() + b.exp()).ln(), each step rounded to T as the reference evaluates it
        using C = typename Compute<T>::type;
        const C ea = widen(narrow<T>(exp(widen(a)))), eb = widen(narrow<T>(exp(widen(b))));
        return narrow<T>(log(widen(narrow<T>(ea + eb))));
    } else if constexpr (is_float_v<T>) {
        using C = typename Compute<T>::type;
        C x = widen(a), y = widen(b);
        C r;
        if constexpr (OP == RSTSR_OP_ADD) r = x + y;
        else if constexpr (OP == RSTSR_OP_SUB) r = x - y;
        else if constexpr (OP == RSTSR_OP_MUL) r = x * y;
        else if constexpr (OP == RSTSR_OP_DIV) r = x / y;
        else if constexpr (OP == RSTSR_OP_REM) r = fmod(x, y);
        else if constexpr (OP == RSTSR_OP_MAXIMUM) r = fmax(x, y);
        else if constexpr (OP == RSTSR_OP_MINIMUM) r = fmin(x, y);
        else if constexpr (OP == RSTSR_OP_POW) r = pow(x, y);
        else if constexpr (OP == RSTSR_OP_ATAN2) r = atan2(x, y);
        else if constexpr (OP == RSTSR_OP_COPYSIGN) r = copysign(x, y);
        else if constexpr (OP == RSTSR_OP_HYPOT) r = hypot(x, y);
        else r = x;
        return narrow<T>(r);
    } else if constexpr (IS_BOOL) {
        if constexpr (OP == RSTSR_OP_BITAND) return a & b;
        else if constexpr (OP == RSTSR_OP_BITOR) return a | b;
        else return a ^ b;
    } else {
        using U = UnsignedOf<T>;
        constexpr int bits = 8 * sizeof(T);
        if constexpr (OP == RSTSR_OP_ADD) return (T)((U)a + (U)b);
        else if constexpr (OP == RSTSR_OP_SUB) return (T)((U)a - (U)b);
        else if constexpr (OP == RSTSR_OP_MUL) return (T)((U)a * (U)b);
        else if constexpr (OP == RSTSR_OP_DIV) {
            if (b == 0) return (T)0;
            if constexpr (std::is_signed<T>::value)
                if (b == (T)-1) return (T)((U)0 - (U)a);
            return (T)(a / b);
        } else if constexpr (OP == RSTSR_OP_REM) {
            if (b == 0) return (T)0;
            if constexpr (std::is_signed<T>::value)
                if (b == (T)-1) return (T)0;
            return (T)(a % b);
        } else if constexpr (OP == RSTSR_OP_BITAND) return (T)(a & b);
        else if constexpr (OP == RSTSR_OP_BITOR) return (T)(a | b);
        else if constexpr (OP == RSTSR_OP_BITXOR) return (T)(a ^ b);
        else if constexpr (OP == RSTSR_OP_SHL) return (T)((U)a << ((U)b & (bits - 1)));
        else if constexpr (OP == RSTSR_OP_SHR) return (T)(a >> ((U)b & (bits - 1)));
        else if constexpr (OP == RSTSR_OP_MAXIMUM) return a > b ? a : b;
        else if constexpr (OP == RSTSR_OP_MINIMUM) return a < b ? a : b;
        else if constexpr (OP == RSTSR_OP_FLOOR_DIVIDE) {
            // Integer::div_floor; x / 0 = 0 here (the reference panics); MIN / -1 wraps
            if (b == 0) return (T)0;
            if constexpr (std::is_signed<T>::value) {
                if (b == (T)-1) return (T)((U)0 - (U)a);
                const T q = (T)(a / b), r = (T)(a % b);
                return (r != 0 && ((r < 0) != (b < 0))) ? (T)(q - 1) : q;
            } else {
                return (T)(a / b);
            }
        } else {  // POW: wrapping power, exponent taken as unsigned
            U base = (U)a, e = (U)b, r = 1;
            while (e) {
                if (e & 1) r = (U)(r * base);
                base = (U)(base * base);
                e >>= 1;
            }
            return (T)r;
        }
    }
}

template <typename T, int OP, bool IS_BOOL>
struct BinF {
    __device__ __forceinline__ T operator()(const T* v) const { return binop<T, OP, IS_BOOL>(v[0], v[1]); }
};

// d = a * b + c as two rounded operations (mul, then add): the value the
// reference's two passes produce (a*b into a new tensor, then += c); no FMA
// contraction.
template <typename T>
struct FmaF {
    __device__ __forceinline__ T operator()(const T* v) const {
        if constexpr (std::is_same<T, double>::value) {
            return __dadd_rn(__dmul_rn(v[0], v[1]), v[2]);
        } else if constexpr (std::is_same<T, float>::value) {
            return __fadd_rn(__fmul_rn(v[0], v[1]), v[2]);
        } else if constexpr (is_half_like<T>::value) {
            T t = narrow<T>(__fmul_rn(widen(v[0]), widen(v[1])));
            return narrow<T>(__fadd_rn(widen(t), widen(v[2])));
        } else {
            using U = UnsignedOf<T>;
            return (T)((U)((U)v[0] * (U)v[1]) + (U)v[2]);
        }
    }
};

static bool op_valid(int op, rstsr_dtype t) {
    const bool bitop = op == RSTSR_OP_BITAND || op == RSTSR_OP_BITOR || op == RSTSR_OP_BITXOR ||
                       op == RSTSR_OP_SHL || op == RSTSR_OP_SHR;
    const bool float_only = op == RSTSR_OP_ATAN2 || op == RSTSR_OP_COPYSIGN || op == RSTSR_OP_HYPOT ||
                            op == RSTSR_OP_LOGADDEXP || op == RSTSR_OP_NEXTAFTER;
    if (is_float_dtype(t)) return !bitop;
    if (t == RSTSR_BOOL) return op == RSTSR_OP_BITAND || op == RSTSR_OP_BITOR || op == RSTSR_OP_BITXOR;
    return !float_only;
}

static int check_op_dtype(int op, rstsr_dtype t) {
    if (!dtype_valid(t)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    if (op < RSTSR_OP_ADD || op > RSTSR_OP_FLOOR_DIVIDE)
        return fail(RSTSR_ERR_INVALID_VALUE, "unknown binary operator");
    if (!op_valid(op, t))
        return fail(RSTSR_ERR_INVALID_VALUE,
                    std::string("operator ") + std::to_string(op) + " is not defined on " + dtype_name(t));
    return RSTSR_OK;
}

// Runtime operator selection: one kernel per dtype serves every operator
// (the switch is uniform across a warp). The arithmetic of the hot dtypes is
// additionally compiled per operator.
template <typename T, bool IS_BOOL>
__device__ __forceinline__ T binop_rt(int op, T a, T b) {
    if constexpr (IS_BOOL) {
        switch (op) {
            case RSTSR_OP_BITAND: return binop<T, RSTSR_OP_BITAND, true>(a, b);
            case RSTSR_OP_BITOR: return binop<T, RSTSR_OP_BITOR, true>(a, b);
            default: return binop<T, RSTSR_OP_BITXOR, true>(a, b);
        }
    } else {
        switch (op) {
            case RSTSR_OP_ADD: return binop<T, RSTSR_OP_ADD, false>(a, b);
            case RSTSR_OP_SUB: return binop<T, RSTSR_OP_SUB, false>(a, b);
            case RSTSR_OP_MUL: return binop<T, RSTSR_OP_MUL, false>(a, b);
            case RSTSR_OP_DIV: return binop<T, RSTSR_OP_DIV, false>(a, b);
            case RSTSR_OP_REM: return binop<T, RSTSR_OP_REM, false>(a, b);
            case RSTSR_OP_MAXIMUM: return binop<T, RSTSR_OP_MAXIMUM, false>(a, b);
            case RSTSR_OP_MINIMUM: return binop<T, RSTSR_OP_MINIMUM, false>(a, b);
            case RSTSR_OP_POW: return binop<T, RSTSR_OP_POW, false>(a, b);
            case RSTSR_OP_FLOOR_DIVIDE: return binop<T, RSTSR_OP_FLOOR_DIVIDE, false>(a, b);
            default: break;
        }
        if constexpr (is_float_v<T>) {
            switch (op) {
                case RSTSR_OP_ATAN2: return binop<T, RSTSR_OP_ATAN2, false>(a, b);
                case RSTSR_OP_COPYSIGN: return binop<T, RSTSR_OP_COPYSIGN, false>(a, b);
                case RSTSR_OP_HYPOT: return binop<T, RSTSR_OP_HYPOT, false>(a, b);
                case RSTSR_OP_LOGADDEXP: return binop<T, RSTSR_OP_LOGADDEXP, false>(a, b);
                case RSTSR_OP_NEXTAFTER: return binop<T, RSTSR_OP_NEXTAFTER, false>(a, b);
                default: break;
            }
        }
        if constexpr (!is_float_v<T>) {
            switch (op) {
                case RSTSR_OP_BITAND: return binop<T, RSTSR_OP_BITAND, false>(a, b);
                case RSTSR_OP_BITOR: return binop<T, RSTSR_OP_BITOR, false>(a, b);
                case RSTSR_OP_BITXOR: return binop<T, RSTSR_OP_BITXOR, false>(a, b);
                case RSTSR_OP_SHL: return binop<T, RSTSR_OP_SHL, false>(a, b);
                default: return binop<T, RSTSR_OP_SHR, false>(a, b);
            }
        }
        return a;
    }
}

template <typename T, bool IS_BOOL>
struct BinRtF {
    int op;
    __device__ __forceinline__ T operator()(const T* v) const { return binop_rt<T, IS_BOOL>(op, v[0], v[1]); }
};

template <typename T, bool IS_BOOL>
static int bin_typed(rstsr_ctx* ctx, int op, const IterSpace& sp, void* c, const EwInput* ins) {
    constexpr bool hot = std::is_same<T, double>::value || std::is_same<T, float>::value ||
                         std::is_same<T, int32_t>::value;
    if constexpr (hot && !IS_BOOL) {
        switch (op) {
            case RSTSR_OP_ADD: return launch_ew<T, T, 2>(ctx, sp, c, ins, BinF<T, RSTSR_OP_ADD, false>{}, "binary");
            case RSTSR_OP_SUB: return launch_ew<T, T, 2>(ctx, sp, c, ins, BinF<T, RSTSR_OP_SUB, false>{}, "binary");
            case RSTSR_OP_MUL: return launch_ew<T, T, 2>(ctx, sp, c, ins, BinF<T, RSTSR_OP_MUL, false>{}, "binary");
            case RSTSR_OP_DIV: return launch_ew<T, T, 2>(ctx, sp, c, ins, BinF<T, RSTSR_OP_DIV, false>{}, "binary");
            default: break;
        }
    }
    return launch_ew<T, T, 2>(ctx, sp, c, ins, BinRtF<T, IS_BOOL>{op}, "binary");
}

static int bin_dispatch(rstsr_ctx* ctx, int op, rstsr_dtype t, const IterSpace& sp, void* c, const EwInput* ins) {
    switch (t) {
        case RSTSR_F64: return bin_typed<double, false>(ctx, op, sp, c, ins);
        case RSTSR_F32: return bin_typed<float, false>(ctx, op, sp, c, ins);
        case RSTSR_F16: return bin_typed<__half, false>(ctx, op, sp, c, ins);
        case RSTSR_BF16: return bin_typed<__nv_bfloat16, false>(ctx, op, sp, c, ins);
        case RSTSR_I8: return bin_typed<int8_t, false>(ctx, op, sp, c, ins);
        case RSTSR_I16: return bin_typed<int16_t, false>(ctx, op, sp, c, ins);
        case RSTSR_I32: return bin_typed<int32_t, false>(ctx, op, sp, c, ins);
        case RSTSR_I64: return bin_typed<int64_t, false>(ctx, op, sp, c, ins);
        case RSTSR_U8: return bin_typed<uint8_t, false>(ctx, op, sp, c, ins);
        case RSTSR_U16: return bin_typed<uint16_t, false>(ctx, op, sp, c, ins);
        case RSTSR_U32: return bin_typed<uint32_t, false>(ctx, op, sp, c, ins);
        case RSTSR_U64: return bin_typed<uint64_t, false>(ctx, op, sp, c, ins);
        case RSTSR_BOOL: return bin_typed<uint8_t, true>(ctx, op, sp, c, ins);
        default: return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    }
}

}  // namespace rstsr

using namespace rstsr;

extern "C" {

int rstsr_cuda_binary(rstsr_ctx* ctx, rstsr_binary_op op, rstsr_dtype t, void* c, const rstsr_layout* lc,
                      const void* a, const rstsr_layout* la, const void* b, const rstsr_layout* lb) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(lc, "c"));
    RSTSR_TRY(check_layout(la, "a"));
    RSTSR_TRY(check_layout(lb, "b"));
    RSTSR_TRY(check_op_dtype(op, t));
    Layout Lc = Layout::from_abi(*lc), La = Layout::from_abi(*la), Lb = Layout::from_abi(*lb);
    RSTSR_TRY(check_same_shape3(Lc, La, &Lb, "binary"));
    RSTSR_TRY(check_write_layout(Lc, "binary"));
    if (Lc.size() == 0) return RSTSR_OK;
    if (!c || !a || !b) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    const Layout* ls[3] = {&Lc, &La, &Lb};
    IterSpace sp = make_iter_space(ls, 3);
    EwInput ins[2] = {{a, nullptr}, {b, nullptr}};
    return bin_dispatch(ctx, op, t, sp, c, ins);
}

int rstsr_cuda_binary_scalar(rstsr_ctx* ctx, rstsr_binary_op op, rstsr_dtype t, void* c, const rstsr_layout* lc,
                             const void* a, const rstsr_layout* la, const void* scalar, int32_t scalar_is_lhs) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(lc, "c"));
    RSTSR_TRY(check_layout(la, "a"));
    RSTSR_TRY(check_op_dtype(op, t));
    if (!scalar) return fail(RSTSR_ERR_INVALID_VALUE, "null scalar");
    Layout Lc = Layout::from_abi(*lc), La = Layout::from_abi(*la);
    RSTSR_TRY(check_same_shape3(Lc, La, nullptr, "binary_scalar"));
    RSTSR_TRY(check_write_layout(Lc, "binary_scalar"));
    if (Lc.size() == 0) return RSTSR_OK;
    if (!c || !a) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    // the scalar is an operand whose strides are all zero
    Layout Ls = La;
    for (int i = 0; i < Ls.ndim; ++i) Ls.stride[i] = 0;
    Ls.offset = 0;
    const Layout* ls[3] = {&Lc, scalar_is_lhs ? &Ls : &La, scalar_is_lhs ? &La : &Ls};
    IterSpace sp = make_iter_space(ls, 3);
    EwInput ins[2];
    if (scalar_is_lhs) {
        ins[0] = {nullptr, scalar};
        ins[1] = {a, nullptr};
    } else {
        ins[0] = {a, nullptr};
        ins[1] = {nullptr, scalar};
    }
    return bin_dispatch(ctx, op, t, sp, c, ins);
}

int rstsr_cuda_binary_inplace(rstsr_ctx* ctx, rstsr_binary_op op, rstsr_dtype t, void* a, const rstsr_layout* la,
                              const void* b, const rstsr_layout* lb, int32_t reversed) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(la, "a"));
    RSTSR_TRY(check_layout(lb, "b"));
    RSTSR_TRY(check_op_dtype(op, t));
    Layout La = Layout::from_abi(*la), Lb = Layout::from_abi(*lb);
    RSTSR_TRY(check_same_shape3(La, Lb, nullptr, "binary_inplace"));
    RSTSR_TRY(check_write_layout(La, "binary_inplace"));
    if (La.size() == 0) return RSTSR_OK;
    if (!a || !b) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    // the written operand is also read, with the same layout, by the same thread
    if (reversed) {
        const Layout* ls[3] = {&La, &Lb, &La};
        IterSpace sp = make_iter_space(ls, 3);
        EwInput ins[2] = {{b, nullptr}, {a, nullptr}};
        return bin_dispatch(ctx, op, t, sp, a, ins);
    }
    const Layout* ls[3] = {&La, &La, &Lb};
    IterSpace sp = make_iter_space(ls, 3);
    EwInput ins[2] = {{a, nullptr}, {b, nullptr}};
    return bin_dispatch(ctx, op, t, sp, a, ins);
}

int rstsr_cuda_fma(rstsr_ctx* ctx, rstsr_dtype t, void* d, const rstsr_layout* ld, const void* a,
                   const rstsr_layout* la, const void* b, const rstsr_layout* lb, const void* c,
                   const rstsr_layout* lc) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(ld, "d"));
    RSTSR_TRY(check_layout(la, "a"));
    RSTSR_TRY(check_layout(lb, "b"));
    RSTSR_TRY(check_layout(lc, "c"));
    if (!dtype_valid(t) || t == RSTSR_BOOL) return fail(RSTSR_ERR_INVALID_VALUE, "fma needs a numeric dtype");
    Layout Ld = Layout::from_abi(*ld), La = Layout::from_abi(*la), Lb = Layout::from_abi(*lb),
           Lc = Layout::from_abi(*lc);
    RSTSR_TRY(check_same_shape3(Ld, La, &Lb, "fma"));
    RSTSR_TRY(check_same_shape3(Ld, Lc, nullptr, "fma"));
    RSTSR_TRY(check_write_layout(Ld, "fma"));
    if (Ld.size() == 0) return RSTSR_OK;
    if (!d || !a || !b || !c) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    const Layout* ls[4] = {&Ld, &La, &Lb, &Lc};
    IterSpace sp = make_iter_space(ls, 4);
    EwInput ins[3] = {{a, nullptr}, {b, nullptr}, {c, nullptr}};
    switch (t) {
        case RSTSR_F64: return launch_ew<double, double, 3>(ctx, sp, d, ins, FmaF<double>{}, "fma");
        case RSTSR_F32: return launch_ew<float, float, 3>(ctx, sp, d, ins, FmaF<float>{}, "fma");
        case RSTSR_F16: return launch_ew<__half, __half, 3>(ctx, sp, d, ins, FmaF<__half>{}, "fma");
        case RSTSR_BF16:
            return launch_ew<__nv_bfloat16, __nv_bfloat16, 3>(ctx, sp, d, ins, FmaF<__nv_bfloat16>{}, "fma");
        case RSTSR_I8: return launch_ew<int8_t, int8_t, 3>(ctx, sp, d, ins, FmaF<int8_t>{}, "fma");
        case RSTSR_I16: return launch_ew<int16_t, int16_t, 3>(ctx, sp, d, ins, FmaF<int16_t>{}, "fma");
        case RSTSR_I32: return launch_ew<int32_t, int32_t, 3>(ctx, sp, d, ins, FmaF<int32_t>{}, "fma");
        case RSTSR_I64: return launch_ew<int64_t, int64_t, 3>(ctx, sp, d, ins, FmaF<int64_t>{}, "fma");
        case RSTSR_U8: return launch_ew<uint8_t, uint8_t, 3>(ctx, sp, d, ins, FmaF<uint8_t>{}, "fma");
        case RSTSR_U16: return launch_ew<uint16_t, uint16_t, 3>(ctx, sp, d, ins, FmaF<uint16_t>{}, "fma");
        case RSTSR_U32: return launch_ew<uint32_t, uint32_t, 3>(ctx, sp, d, ins, FmaF<uint32_t>{}, "fma");
        case RSTSR_U64: return launch_ew<uint64_t, uint64_t, 3>(ctx, sp, d, ins, FmaF<uint64_t>{}, "fma");
        default: return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    }
}

}  // extern "C"
