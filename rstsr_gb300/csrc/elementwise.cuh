// Element-wise value semantics shared by the strided kernels: Rust `as`
// casts, wrapping integer arithmetic and IEEE floating point exactly as the
// reference's closures compute them (rstsr-dtype-traits DTypeCastAPI;
// rstsr-core/src/feature_rayon/auto_impl/op_ternary_arithmetic.rs).
#pragma once

#include <cmath>
#include <type_traits>

#include "common.cuh"

namespace rstsr {

template <typename T> struct is_half_like : std::false_type {};
template <> struct is_half_like<__half> : std::true_type {};
template <> struct is_half_like<__nv_bfloat16> : std::true_type {};

template <typename T>
constexpr bool is_float_v = std::is_floating_point<T>::value || is_half_like<T>::value;

// widen half types to float for arithmetic
template <typename T> struct Compute { using type = T; };
template <> struct Compute<__half> { using type = float; };
template <> struct Compute<__nv_bfloat16> { using type = float; };

template <typename T>
__device__ __forceinline__ typename Compute<T>::type widen(T x) {
    if constexpr (is_half_like<T>::value)
        return static_cast<float>(x);
    else
        return x;
}
template <typename T>
__device__ __forceinline__ T narrow(typename Compute<T>::type x) {
    if constexpr (std::is_same<T, __half>::value)
        return __float2half_rn(x);
    else if constexpr (std::is_same<T, __nv_bfloat16>::value)
        return __float2bfloat16_rn(x);
    else
        return x;
}

// Rust `as` from a floating value to an integer type saturates at the target
// range and maps NaN to zero. lo/hi are the target's limits.
template <typename TI>
__device__ __forceinline__ TI float_to_int_sat(double d, double lo, double hi, TI tlo, TI thi) {
    if (d != d) return TI(0);
    if (d <= lo) return tlo;
    if (d >= hi) return thi;
    return (TI)d;
}

}  // namespace rstsr
