// The strided element-wise kernel shared by assign/fill, the binary and
// unary operators and the fused a*b+c pass.
//
// It replaces the closure-driven layout walkers of
// rstsr-native-impl/src/cpu_rayon/{assignment.rs, op_with_func.rs}: instead of
// an odometer per element, the host planner (make_iter_space) collapses the
// operands' layouts into one iteration space, dims merged wherever every
// operand is contiguous across them, and the kernel walks it with
//   * 16-byte vector loads/stores along the innermost dim when it is
//     contiguous and aligned; stride-0 (broadcast) operands are splatted,
//     other strides gathered element by element, scalars read from the
//     kernel parameters;
//   * invariant-divisor index decomposition of the outer dims (32-bit, or
//     plain 64-bit division above 2^31 elements).
#pragma once

#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "elementwise.cuh"

namespace rstsr {

constexpr int kThreads = 256;
constexpr int kUnroll = 4;

enum OperandMode : int {
    kSplat = 0,   // inner stride 0: one load per vector group
    kVector = 1,  // inner stride 1, aligned: one 16-byte load
    kGather = 2,  // any other inner stride: VEC scalar loads
    kScalar = 3   // value held in the kernel parameters
};

template <int NIN>
struct EwParams {
    DevDims dims;
    int64_t ngroups;
    int32_t big;  // 64-bit index decomposition
    int32_t mode[NIN > 0 ? NIN : 1];
    int64_t stride[NIN + 1][RSTSR_MAX_NDIM];
    int64_t offset[NIN + 1];
    const void* in[NIN > 0 ? NIN : 1];
    uint64_t scalar[NIN > 0 ? NIN : 1];
    void* out;
};

template <typename T, int VEC>
struct alignas(sizeof(T) * VEC) VecT {
    T v[VEC];
};

template <int NOPS>
__device__ __forceinline__ void decompose(const DevDims& d, const int64_t (*stride)[RSTSR_MAX_NDIM],
                                          const int64_t* offset, int64_t e, bool big, int64_t* off) {
#pragma unroll
    for (int k = 0; k < NOPS; ++k) off[k] = offset[k];
    if (big) {
        uint64_t rem = (uint64_t)e;
        for (int i = 0; i < d.ndim - 1; ++i) {
            uint64_t q = rem / d.shape[i];
            int64_t idx = (int64_t)(rem - q * d.shape[i]);
            rem = q;
#pragma unroll
            for (int k = 0; k < NOPS; ++k) off[k] += idx * stride[k][i];
        }
#pragma unroll
        for (int k = 0; k < NOPS; ++k) off[k] += (int64_t)rem * stride[k][d.ndim - 1];
    } else {
        uint32_t rem = (uint32_t)e;
        for (int i = 0; i < d.ndim - 1; ++i) {
            uint32_t q = d.div[i].div(rem);
            int64_t idx = (int64_t)(rem - q * d.shape[i]);
            rem = q;
#pragma unroll
            for (int k = 0; k < NOPS; ++k) off[k] += idx * stride[k][i];
        }
#pragma unroll
        for (int k = 0; k < NOPS; ++k) off[k] += (int64_t)rem * stride[k][d.ndim - 1];
    }
}

// Each thread handles kUnroll groups of VEC consecutive inner-dim elements;
// all loads of a thread are issued before its first store. The output
// (operand 0) is vector-stored when VEC > 1 (the host picks VEC > 1 only when
// the output is contiguous and aligned along dim 0). When the output aliases
// an input with the same layout (in-place forms) every element is read and
// written by the same thread, reads first.
template <typename TO, typename TI, int NIN, int VEC, typename F, int kUnroll = ::rstsr::kUnroll>
__global__ void __launch_bounds__(kThreads) ew_kernel(const EwParams<NIN> p, F f) {
    const int64_t base = (int64_t)blockIdx.x * (kThreads * kUnroll) + threadIdx.x;
    TI v[kUnroll][NIN > 0 ? NIN : 1][VEC];
    int64_t offo[kUnroll];
    bool live[kUnroll];
    const bool big = p.big != 0;
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
        const int64_t g = base + (int64_t)u * kThreads;
        live[u] = g < p.ngroups;
        if (!live[u]) continue;
        int64_t off[NIN + 1];
        decompose<NIN + 1>(p.dims, p.stride, p.offset, g * VEC, big, off);
        offo[u] = off[0];
#pragma unroll
        for (int k = 0; k < NIN; ++k) {
            const TI* src = reinterpret_cast<const TI*>(p.in[k]);
            const int mode = p.mode[k];
            if (mode == kScalar) {
                TI s;
                memcpy(&s, &p.scalar[k], sizeof(TI));
#pragma unroll
                for (int j = 0; j < VEC; ++j) v[u][k][j] = s;
            } else if (VEC > 1 && mode == kVector) {
                VecT<TI, VEC> t = *reinterpret_cast<const VecT<TI, VEC>*>(src + off[k + 1]);
#pragma unroll
                for (int j = 0; j < VEC; ++j) v[u][k][j] = t.v[j];
            } else if (VEC > 1 && mode == kSplat) {
                TI s = src[off[k + 1]];
#pragma unroll
                for (int j = 0; j < VEC; ++j) v[u][k][j] = s;
            } else {
                const int64_t s0 = p.stride[k + 1][0];
#pragma unroll
                for (int j = 0; j < VEC; ++j) v[u][k][j] = src[off[k + 1] + j * s0];
            }
        }
    }
    TO* dst = reinterpret_cast<TO*>(p.out);
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
        if (!live[u]) continue;
        VecT<TO, VEC> r;
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            TI args[NIN > 0 ? NIN : 1];
#pragma unroll
            for (int k = 0; k < NIN; ++k) args[k] = v[u][k][j];
            r.v[j] = f(args);
        }
        if constexpr (VEC > 1) {
            *reinterpret_cast<VecT<TO, VEC>*>(dst + offo[u]) = r;
        } else {
            dst[offo[u]] = r.v[0];
        }
    }
}

template <typename TO, typename TI, int NIN, int VEC, typename F, int U = kUnroll>
static int launch_ew_vec(rstsr_ctx* ctx, EwParams<NIN>& p, const IterSpace& sp, F f, const char* name) {
    p.ngroups = sp.size / VEC;
    int64_t blocks = (p.ngroups + kThreads * U - 1) / (kThreads * U);
    if (blocks > INT32_MAX) return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, "tensor too large for one launch");
    ew_kernel<TO, TI, NIN, VEC, F, U><<<(unsigned)blocks, kThreads, 0, ctx->stream>>>(p, f);
    return after_launch(ctx, name);
}

// Operand description for launch_ew: a device pointer, or a host scalar.
struct EwInput {
    const void* ptr;
    const void* host_scalar;  // non-null: the operand is this scalar
};

// Launch an element-wise kernel over `sp` (operand 0 = output of type TO;
// operands 1..NIN = inputs of type TI). Picks the widest legal vector.
template <typename TO, typename TI, int NIN, typename F>
static int launch_ew(rstsr_ctx* ctx, const IterSpace& sp, void* out, const EwInput* in, F f,
                     const char* name) {
    if (sp.size == 0) return RSTSR_OK;
    if (!inner_extents_fit_u32(sp))
        return fail(RSTSR_ERR_UNIMPLEMENTED, "element-wise kernel: an inner extent of 2^32 or more elements");
    EwParams<NIN> p;
    memset(&p, 0, sizeof(p));
    p.dims = make_dev_dims(sp);
    p.out = out;
    p.big = sp.size >= (int64_t(1) << 31) ? 1 : 0;
    for (int k = 0; k <= NIN; ++k) {
        for (int d = 0; d < RSTSR_MAX_NDIM; ++d) p.stride[k][d] = d < sp.ndim ? sp.stride[k][d] : 0;
        p.offset[k] = sp.offset[k];
    }
    constexpr int V = (16 / sizeof(TO)) < (16 / sizeof(TI)) ? (16 / sizeof(TO)) : (16 / sizeof(TI));
    // 4- and 8-byte elements: groups of 32 bytes (two groups per thread
    // instead of four) when the output is contiguous and aligned for them: an
    // index decomposition then serves twice the elements (f64 a*b+c on the
    // F-ordered workload: 228 -> 138 us). Inputs are loaded as 32-byte
    // vectors, splatted, or (8-byte types only: eight scalar gathers of 4-byte
    // elements per group were slower than four) gathered.
    if constexpr (sizeof(TO) == sizeof(TI) && (sizeof(TO) == 8 || sizeof(TO) == 4)) {
        constexpr int W = 32 / (int)sizeof(TO);
        bool wide = vec_aligned(sp, 0, out, sizeof(TO), W);
        for (int k = 0; wide && sizeof(TO) == 4 && k < NIN; ++k)
            if (!in[k].host_scalar && sp.stride[k + 1][0] != 0)
                wide = vec_aligned(sp, k + 1, in[k].ptr, sizeof(TI), W);
        if (wide) {
            for (int k = 0; k < NIN; ++k) {
                if (in[k].host_scalar) {
                    p.mode[k] = kScalar;
                    p.in[k] = nullptr;
                    memcpy(&p.scalar[k], in[k].host_scalar, sizeof(TI));
                    continue;
                }
                p.in[k] = in[k].ptr;
                const int64_t s0 = sp.stride[k + 1][0];
                p.mode[k] = s0 == 0 ? kSplat : vec_aligned(sp, k + 1, in[k].ptr, sizeof(TI), W) ? kVector : kGather;
            }
            return launch_ew_vec<TO, TI, NIN, W, F, 2>(ctx, p, sp, f, name);
        }
    }
    const bool vec_ok = V > 1 && vec_aligned(sp, 0, out, sizeof(TO), V);
    for (int k = 0; k < NIN; ++k) {
        if (in[k].host_scalar) {
            p.mode[k] = kScalar;
            p.in[k] = nullptr;
            memcpy(&p.scalar[k], in[k].host_scalar, sizeof(TI));
            continue;
        }
        p.in[k] = in[k].ptr;
        const int64_t s0 = sp.stride[k + 1][0];
        if (s0 == 0)
            p.mode[k] = kSplat;
        else if (vec_aligned(sp, k + 1, in[k].ptr, sizeof(TI), V))
            p.mode[k] = kVector;
        else
            p.mode[k] = kGather;
    }
    if (vec_ok) return launch_ew_vec<TO, TI, NIN, V>(ctx, p, sp, f, name);
    for (int k = 0; k < NIN; ++k)
        if (p.mode[k] != kScalar) p.mode[k] = kGather;
    return launch_ew_vec<TO, TI, NIN, 1>(ctx, p, sp, f, name);
}

inline bool same_shape(const Layout& a, const Layout& b) {
    if (a.ndim != b.ndim) return false;
    for (int i = 0; i < a.ndim; ++i)
        if (a.shape[i] != b.shape[i]) return false;
    return true;
}

// An output whose elements overlap (stride 0 on a non-trivial axis) would be
// written by several threads at once.
inline int check_write_layout(const Layout& lc, const char* name) {
    if (lc.size() > 1 && !lc.check_strides(false))
        return fail(RSTSR_ERR_INVALID_LAYOUT,
                    std::string(name) + ": output layout has overlapping elements (" + lc.repr() + ")");
    return RSTSR_OK;
}

inline int check_same_shape3(const Layout& c, const Layout& a, const Layout* b, const char* what) {
    if (!same_shape(c, a) || (b && !same_shape(c, *b)))
        return fail(RSTSR_ERR_INVALID_LAYOUT,
                    std::string(what) + ": operand shapes differ (broadcast them to the output first): c " +
                        c.repr() + ", a " + a.repr() + (b ? ", b " + b->repr() : std::string()));
    return RSTSR_OK;
}

inline bool is_float_dtype(rstsr_dtype t) {
    return t == RSTSR_F64 || t == RSTSR_F32 || t == RSTSR_F16 || t == RSTSR_BF16;
}

}  // namespace rstsr

#define RSTSR_TRY(expr)                \
    do {                               \
        int _s = (expr);               \
        if (_s != RSTSR_OK) return _s; \
    } while (0)
