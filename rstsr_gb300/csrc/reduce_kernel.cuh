// Axis reductions on the GPU. Replaces reduce_all_cpu_rayon /
// reduce_axes_cpu_rayon (rstsr-native-impl/src/cpu_rayon/reduction.rs:20-328)
// and the arg reductions (:440-631) with one group-reduction kernel:
//
//   * the reduced axes and the kept axes are each collapsed into a small
//     iteration space (inner-first, contiguous neighbours merged);
//   * a group of G threads (G = 1, 32 or 256) owns one output element and
//     strides over that element's reduced elements: G = 32/256 ("row" regime,
//     reduced axes innermost in memory) reads each output's run with 16-byte
//     vector loads and combines the group with warp shuffles and shared
//     memory; G = 1 ("column" regime, a kept axis innermost) lets neighbouring
//     threads own neighbouring outputs so every load is coalesced across the
//     warp;
//   * when there are too few outputs to fill the 152 SMs, the reduced range
//     is split into chunks over blockIdx.y; each chunk writes its accumulator
//     to scratch and a second kernel folds the chunks in chunk order.
//
// Every combination order is fixed by the launch shape, so results are
// deterministic run to run. Floating-point sums are tree-combined (they differ
// from the reference's 8-accumulator serial order only by rounding); integer
// arithmetic wraps as in Rust release builds and is exact.
#pragma once

#include <cfloat>
#include <climits>

#include "common.cuh"

namespace rstsr {

constexpr int kRedThreads = 256;

// Accumulator kinds (the init/f/f_sum algebra of
// rstsr-core/src/feature_rayon/auto_impl/reduction.rs).
enum RedKind : int {
    kRedSum = 0,      // acc + x                    (sum, mean)
    kRedMoments = 1,  // (acc + x, acc2 + x*x)      (var, std)
    kRedSumSq = 2,    // acc + x*x                  (l2_norm)
    kRedMin = 3,      // ext_min, init T::MAX
    kRedMax = 4,      // ext_max, init T::MIN
    kRedProd = 5,     // acc * x
    kRedCount = 6,    // acc + (x != 0)             (count_nonzero, bool sum)
    kRedAll = 7,      // acc && x
    kRedAny = 8,      // acc || x
    kRedArgMax = 9,
    kRedArgMin = 10
};

struct RedSpace {
    int nd;
    uint32_t shape[RSTSR_MAX_NDIM];
    FastDiv div[RSTSR_MAX_NDIM];
    int64_t stride[RSTSR_MAX_NDIM];   // input element stride
    int64_t lstride[RSTSR_MAX_NDIM];  // logical C-order stride (arg reductions)
};

struct KeptSpace {
    int nd;
    uint32_t shape[RSTSR_MAX_NDIM];
    FastDiv div[RSTSR_MAX_NDIM];
    int64_t in_stride[RSTSR_MAX_NDIM];
    int64_t out_stride[RSTSR_MAX_NDIM];
};

struct RedParams {
    RedSpace r;
    KeptSpace k;
    int64_t nred, nout;
    int64_t in_off, out_off;
    int32_t glog;    // log2 of the group size
    int32_t vec;     // reduced dim 0 is contiguous and aligned: VEC-wide loads
    int32_t nsplit;  // chunks of the reduced range (gridDim.y)
    int32_t op;      // rstsr_reduce_op (finalisation)
    int32_t ocol;    // column regime with vector loads: outputs per thread (1 = scalar)
    int64_t chunk;   // reduced elements per chunk
    void* partial;   // [nsplit][nout] accumulators, or null
    const void* in;
    void* out;
};

// ---------------------------------------------------------------- policies

template <typename T, int KIND>
struct Red;

template <typename T>
struct AccScalar {
    T a;
};
template <typename T>
struct AccPair {
    T a, b;
};
template <typename T>
struct AccArg {
    T v;
    int64_t idx;  // INT64_MAX: empty
    int32_t nan0; // the element at logical index 0 is NaN
};

template <typename T>
__device__ __forceinline__ bool is_nan_v(T x) {
    if constexpr (std::is_floating_point<T>::value)
        return x != x;
    else
        return false;
}

template <typename T>
__device__ __forceinline__ T lowest_v() {
    if constexpr (std::is_same<T, double>::value) return -DBL_MAX;
    else if constexpr (std::is_same<T, float>::value) return -FLT_MAX;
    else if constexpr (std::is_same<T, int32_t>::value) return INT32_MIN;
    else if constexpr (std::is_same<T, int64_t>::value) return INT64_MIN;
    else return (T)0;
}
template <typename T>
__device__ __forceinline__ T highest_v() {
    if constexpr (std::is_same<T, double>::value) return DBL_MAX;
    else if constexpr (std::is_same<T, float>::value) return FLT_MAX;
    else if constexpr (std::is_same<T, int32_t>::value) return INT32_MAX;
    else if constexpr (std::is_same<T, int64_t>::value) return INT64_MAX;
    else if constexpr (std::is_same<T, uint64_t>::value) return UINT64_MAX;
    else return (T)~(T)0;
}

template <typename T>
using UnsignedOfR = typename std::make_unsigned<T>::type;

template <typename T>
__device__ __forceinline__ T wrap_add(T a, T b) {
    if constexpr (std::is_integral<T>::value)
        return (T)((UnsignedOfR<T>)a + (UnsignedOfR<T>)b);
    else
        return a + b;
}
template <typename T>
__device__ __forceinline__ T wrap_mul(T a, T b) {
    if constexpr (std::is_integral<T>::value)
        return (T)((UnsignedOfR<T>)a * (UnsignedOfR<T>)b);
    else
        return a * b;
}

// Rust f64::max / f64::min ignore a NaN operand; integer Ord::max / min.
template <typename T>
__device__ __forceinline__ T ext_max(T a, T b) {
    if constexpr (std::is_floating_point<T>::value) return fmax(a, b);
    else return a > b ? a : b;
}
template <typename T>
__device__ __forceinline__ T ext_min(T a, T b) {
    if constexpr (std::is_floating_point<T>::value) return fmin(a, b);
    else return a < b ? a : b;
}

template <typename T>
struct Red<T, kRedSum> {
    using Acc = AccScalar<T>;
    using Out = T;
    __device__ static Acc init() { return {(T)0}; }
    __device__ static void fold(Acc& s, T x, int64_t) { s.a = wrap_add(s.a, x); }
    __device__ static void merge(Acc& s, const Acc& o) { s.a = wrap_add(s.a, o.a); }
    __device__ static Out fin(const Acc& s, int op, int64_t n) {
        if constexpr (std::is_floating_point<T>::value)
            if (op == RSTSR_RED_MEAN) return s.a / (T)n;
        return s.a;
    }
};

template <typename T>
struct Red<T, kRedMoments> {
    using Acc = AccPair<T>;
    using Out = T;
    __device__ static Acc init() { return {(T)0, (T)0}; }
    __device__ static void fold(Acc& s, T x, int64_t) {
        s.a += x;
        s.b += x * x;
    }
    __device__ static void merge(Acc& s, const Acc& o) {
        s.a += o.a;
        s.b += o.b;
    }
    // var = E[x^2] - E[x]^2 (one pass, auto_impl/reduction.rs:220-228)
    __device__ static Out fin(const Acc& s, int op, int64_t n) {
        T mean = s.a / (T)n;
        T var = s.b / (T)n - mean * mean;
        return op == RSTSR_RED_STD ? sqrt(var) : var;
    }
};

template <typename T>
struct Red<T, kRedSumSq> {
    using Acc = AccScalar<T>;
    using Out = T;
    __device__ static Acc init() { return {(T)0}; }
    __device__ static void fold(Acc& s, T x, int64_t) { s.a += x * x; }
    __device__ static void merge(Acc& s, const Acc& o) { s.a += o.a; }
    __device__ static Out fin(const Acc& s, int, int64_t) { return sqrt(s.a); }
};

template <typename T>
struct Red<T, kRedMin> {
    using Acc = AccScalar<T>;
    using Out = T;
    __device__ static Acc init() { return {highest_v<T>()}; }
    __device__ static void fold(Acc& s, T x, int64_t) { s.a = ext_min(s.a, x); }
    __device__ static void merge(Acc& s, const Acc& o) { s.a = ext_min(s.a, o.a); }
    __device__ static Out fin(const Acc& s, int, int64_t) { return s.a; }
};

template <typename T>
struct Red<T, kRedMax> {
    using Acc = AccScalar<T>;
    using Out = T;
    __device__ static Acc init() { return {lowest_v<T>()}; }
    __device__ static void fold(Acc& s, T x, int64_t) { s.a = ext_max(s.a, x); }
    __device__ static void merge(Acc& s, const Acc& o) { s.a = ext_max(s.a, o.a); }
    __device__ static Out fin(const Acc& s, int, int64_t) { return s.a; }
};

template <typename T>
struct Red<T, kRedProd> {
    using Acc = AccScalar<T>;
    using Out = T;
    __device__ static Acc init() { return {(T)1}; }
    __device__ static void fold(Acc& s, T x, int64_t) { s.a = wrap_mul(s.a, x); }
    __device__ static void merge(Acc& s, const Acc& o) { s.a = wrap_mul(s.a, o.a); }
    __device__ static Out fin(const Acc& s, int, int64_t) { return s.a; }
};

template <typename T>
struct Red<T, kRedCount> {
    using Acc = AccScalar<uint64_t>;
    using Out = uint64_t;
    __device__ static Acc init() { return {0}; }
    __device__ static void fold(Acc& s, T x, int64_t) { s.a += (x != (T)0) ? 1 : 0; }
    __device__ static void merge(Acc& s, const Acc& o) { s.a += o.a; }
    __device__ static Out fin(const Acc& s, int, int64_t) { return s.a; }
};

template <typename T>
struct Red<T, kRedAll> {
    using Acc = AccScalar<uint32_t>;  // 4-byte accumulator for the shuffles
    using Out = uint8_t;
    __device__ static Acc init() { return {1u}; }
    __device__ static void fold(Acc& s, T x, int64_t) { s.a = s.a & (x != 0 ? 1u : 0u); }
    __device__ static void merge(Acc& s, const Acc& o) { s.a = s.a & o.a; }
    __device__ static Out fin(const Acc& s, int, int64_t) { return (uint8_t)s.a; }
};

template <typename T>
struct Red<T, kRedAny> {
    using Acc = AccScalar<uint32_t>;
    using Out = uint8_t;
    __device__ static Acc init() { return {0u}; }
    __device__ static void fold(Acc& s, T x, int64_t) { s.a = s.a | (x != 0 ? 1u : 0u); }
    __device__ static void merge(Acc& s, const Acc& o) { s.a = s.a | o.a; }
    __device__ static Out fin(const Acc& s, int, int64_t) { return (uint8_t)s.a; }
};

// arg reductions: the smallest logical index among the extreme values; NaN is
// never accepted, except that a NaN at logical index 0 makes the answer 0 (the
// serial fold of cpu_serial/reduction.rs:425-477 starts from that element and
// no comparison against NaN succeeds afterwards).
//
// The empty accumulator holds the worst value (-inf / the type's minimum for
// argmax) at index INT64_MAX, so "strictly better, or equal at a smaller
// index" covers it without a separate test, and the fold selects without
// branches (the comparison-and-select chain bounded the argmax kernels).
template <typename T, bool IS_MAX>
struct RedArg {
    using Acc = AccArg<T>;
    using Out = uint64_t;
    __device__ static T start() {
        if constexpr (std::is_floating_point<T>::value) {
            return IS_MAX ? -(T)INFINITY : (T)INFINITY;
        } else if constexpr (std::is_signed<T>::value) {
            const T mn = (T)((UnsignedOfR<T>)1 << (sizeof(T) * 8 - 1));
            return IS_MAX ? mn : (T)~mn;
        } else {
            return IS_MAX ? (T)0 : (T)~(T)0;
        }
    }
    __device__ static Acc init() { return {start(), INT64_MAX, 0}; }
    __device__ static bool better(T x, int64_t ix, T v, int64_t iv) {
        return (IS_MAX ? (x > v) : (x < v)) | ((x == v) & (ix < iv));
    }
    __device__ static void fold(Acc& s, T x, int64_t lidx) {
        if (is_nan_v(x)) {
            if (lidx == 0) s.nan0 = 1;
            return;
        }
        const bool take = better(x, lidx, s.v, s.idx);
        s.v = take ? x : s.v;
        s.idx = take ? lidx : s.idx;
    }
    __device__ static void merge(Acc& s, const Acc& o) {
        s.nan0 |= o.nan0;
        if (o.idx != INT64_MAX && better(o.v, o.idx, s.v, s.idx)) {
            s.v = o.v;
            s.idx = o.idx;
        }
    }
    __device__ static Out fin(const Acc& s, int, int64_t) {
        if (s.nan0 || s.idx == INT64_MAX) return 0;
        return (uint64_t)s.idx;
    }
};
// f64 arg reductions compare order-preserving int64 keys instead of doubles:
// GB300's FP64 pipe runs at a small fraction of its integer rate, and a
// comparison per element made the f64 argmax FP64-bound. key(x) maps -0.0 to
// +0.0 (they compare equal) and flips the magnitude bits of negatives, so
// x < y  <=>  key(x) < key(y) and x == y <=> key(x) == key(y) for non-NaN x, y;
// NaN is recognised from its bits. Same results as RedArg<double>.
template <bool IS_MAX>
struct RedArgF64 {
    using Acc = AccArg<int64_t>;
    using Out = uint64_t;
    // keys of non-NaN doubles lie strictly inside (INT64_MIN, INT64_MAX)
    __device__ static Acc init() { return {IS_MAX ? INT64_MIN : INT64_MAX, INT64_MAX, 0}; }
    __device__ static bool better(int64_t x, int64_t ix, int64_t v, int64_t iv) {
        return (IS_MAX ? (x > v) : (x < v)) | ((x == v) & (ix < iv));
    }
    __device__ static void fold(Acc& s, double xd, int64_t lidx) {
        int64_t b = __double_as_longlong(xd);
        if ((b & INT64_MAX) > 0x7FF0000000000000LL) {  // NaN
            if (lidx == 0) s.nan0 = 1;
            return;
        }
        if (b == INT64_MIN) b = 0;  // -0.0 -> +0.0
        const int64_t key = b >= 0 ? b : (b ^ INT64_MAX);
        const bool take = better(key, lidx, s.v, s.idx);
        s.v = take ? key : s.v;
        s.idx = take ? lidx : s.idx;
    }
    __device__ static void merge(Acc& s, const Acc& o) {
        s.nan0 |= o.nan0;
        if (o.idx != INT64_MAX && better(o.v, o.idx, s.v, s.idx)) {
            s.v = o.v;
            s.idx = o.idx;
        }
    }
    __device__ static Out fin(const Acc& s, int, int64_t) {
        if (s.nan0 || s.idx == INT64_MAX) return 0;
        return (uint64_t)s.idx;
    }
};

template <typename T>
struct Red<T, kRedArgMax> : RedArg<T, true> {};
template <typename T>
struct Red<T, kRedArgMin> : RedArg<T, false> {};
template <>
struct Red<double, kRedArgMax> : RedArgF64<true> {};
template <>
struct Red<double, kRedArgMin> : RedArgF64<false> {};

// ---------------------------------------------------------------- shuffles

// Shuffle within segments of `width` lanes (a power of two <= 32).
template <typename A>
__device__ __forceinline__ A shfl_down_acc(const A& a, int delta, int width) {
    static_assert(sizeof(A) % 4 == 0, "accumulator must be a multiple of 4 bytes");
    A r;
    const int* src = reinterpret_cast<const int*>(&a);
    int* dst = reinterpret_cast<int*>(&r);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(A) / 4); ++i) dst[i] = __shfl_down_sync(0xffffffffu, src[i], delta, width);
    return r;
}

// loads in flight per thread in the reduction loops
constexpr int kRedUnroll = 4;

// ---------------------------------------------------------------- kernels

template <typename T, int VEC>
struct alignas(sizeof(T) * VEC) RVec {
    T v[VEC];
};

__device__ __forceinline__ int64_t red_offset(const RedSpace& r, uint32_t e, int64_t* lidx) {
    int64_t off = 0, li = 0;
    for (int i = 0; i < r.nd - 1; ++i) {
        uint32_t q = r.div[i].div(e);
        int64_t idx = (int64_t)(e - q * r.shape[i]);
        off += idx * r.stride[i];
        li += idx * r.lstride[i];
        e = q;
    }
    off += (int64_t)e * r.stride[r.nd - 1];
    li += (int64_t)e * r.lstride[r.nd - 1];
    *lidx = li;
    return off;
}

// Outputs per thread of the vectorised column regime: a 16-byte (f64: two,
// 4-byte types: four) or smaller load covers that many neighbouring outputs.
template <typename T>
constexpr int red_col_vec() {
    return 16 / sizeof(T) >= 4 ? 4 : (16 / sizeof(T) >= 2 ? 2 : 1);
}

// Column regime with vector loads (p.ocol = red_col_vec<T>()): the innermost
// kept dim is contiguous in the input, so OV neighbouring outputs read one
// OV-wide vector per reduced element; a warp reads 32 * OV * sizeof(T) bytes
// per step instead of 32 * sizeof(T), with OV accumulators per thread.
template <typename T, int KIND>
__device__ __forceinline__ void reduce_colvec(const RedParams& p) {
    using R = Red<T, KIND>;
    using Acc = typename R::Acc;
    constexpr int OV = red_col_vec<T>();
    const int64_t o0 = ((int64_t)blockIdx.x * kRedThreads + threadIdx.x) * OV;
    if (o0 >= p.nout) return;  // nout is a multiple of OV
    const T* __restrict__ in = reinterpret_cast<const T*>(p.in);
    int64_t base = p.in_off;
    {
        uint32_t e = (uint32_t)o0;
        for (int i = 0; i < p.k.nd - 1; ++i) {
            uint32_t q = p.k.div[i].div(e);
            base += (int64_t)(e - q * p.k.shape[i]) * p.k.in_stride[i];
            e = q;
        }
        if (p.k.nd > 0) base += (int64_t)e * p.k.in_stride[p.k.nd - 1];
    }
    Acc acc[OV];
#pragma unroll
    for (int j = 0; j < OV; ++j) acc[j] = R::init();
    const int64_t rb = (int64_t)blockIdx.y * p.chunk;
    const int64_t re = min(p.nred, rb + p.chunk);
    for (int64_t r0 = rb; r0 < re; r0 += kRedUnroll) {
        RVec<T, OV> v[kRedUnroll];
        int64_t li[kRedUnroll];
#pragma unroll
        for (int u = 0; u < kRedUnroll; ++u)
            if (r0 + u < re) {
                const int64_t off = red_offset(p.r, (uint32_t)(r0 + u), &li[u]);
                v[u] = *reinterpret_cast<const RVec<T, OV>*>(in + base + off);
            }
#pragma unroll
        for (int u = 0; u < kRedUnroll; ++u)
            if (r0 + u < re) {
#pragma unroll
                for (int j = 0; j < OV; ++j) R::fold(acc[j], v[u].v[j], li[u]);
            }
    }
    if (p.partial) {
        Acc* part = reinterpret_cast<Acc*>(p.partial) + (int64_t)blockIdx.y * p.nout + o0;
#pragma unroll
        for (int j = 0; j < OV; ++j) part[j] = acc[j];
        return;
    }
    int64_t oo = p.out_off;
    {
        uint32_t e = (uint32_t)o0;
        for (int i = 0; i < p.k.nd - 1; ++i) {
            uint32_t q = p.k.div[i].div(e);
            oo += (int64_t)(e - q * p.k.shape[i]) * p.k.out_stride[i];
            e = q;
        }
        if (p.k.nd > 0) oo += (int64_t)e * p.k.out_stride[p.k.nd - 1];
    }
    // the OV outputs are neighbours along kept dim 0
#pragma unroll
    for (int j = 0; j < OV; ++j)
        reinterpret_cast<typename R::Out*>(p.out)[oo + j * p.k.out_stride[0]] = R::fin(acc[j], p.op, p.nred);
}

// Outputs handled by one CTA.
__host__ __device__ inline int64_t red_outputs_per_cta(const RedParams& p) {
    return (int64_t)(kRedThreads >> p.glog) * (p.ocol > 1 ? p.ocol : 1);
}

template <typename T, int KIND>
__global__ void __launch_bounds__(kRedThreads) reduce_kernel(const RedParams p) {
    if (p.ocol > 1) {
        if constexpr (red_col_vec<T>() > 1) reduce_colvec<T, KIND>(p);
        return;
    }
    using R = Red<T, KIND>;
    using Acc = typename R::Acc;
    constexpr int VEC = 16 / sizeof(T) > 0 ? 16 / sizeof(T) : 1;
    const int G = 1 << p.glog;
    const int tid = threadIdx.x;
    const int lane = tid & (G - 1);
    const int64_t o = (int64_t)blockIdx.x * (kRedThreads >> p.glog) + (tid >> p.glog);
    const bool active = o < p.nout;
    const T* __restrict__ in = reinterpret_cast<const T*>(p.in);

    Acc acc = R::init();
    if (active) {
        // input base of this output element
        int64_t base = p.in_off;
        {
            uint32_t e = (uint32_t)o;
            for (int i = 0; i < p.k.nd - 1; ++i) {
                uint32_t q = p.k.div[i].div(e);
                base += (int64_t)(e - q * p.k.shape[i]) * p.k.in_stride[i];
                e = q;
            }
            if (p.k.nd > 0) base += (int64_t)e * p.k.in_stride[p.k.nd - 1];
        }
        const int64_t rb = (int64_t)blockIdx.y * p.chunk;
        const int64_t re = min(p.nred, rb + p.chunk);
        // kRedUnroll independent loads are issued before they are folded, so
        // each thread keeps several requests in flight
        if (VEC > 1 && p.vec) {
            const int64_t step = (int64_t)G * VEC;
            for (int64_t r0 = rb + (int64_t)lane * VEC; r0 < re; r0 += step * kRedUnroll) {
                RVec<T, VEC> v[kRedUnroll];
                int64_t li[kRedUnroll];
#pragma unroll
                for (int u = 0; u < kRedUnroll; ++u) {
                    const int64_t r = r0 + u * step;
                    if (r < re) {
                        const int64_t off = red_offset(p.r, (uint32_t)r, &li[u]);
                        v[u] = *reinterpret_cast<const RVec<T, VEC>*>(in + base + off);
                    }
                }
#pragma unroll
                for (int u = 0; u < kRedUnroll; ++u) {
                    if (r0 + u * step < re) {
#pragma unroll
                        for (int j = 0; j < VEC; ++j) R::fold(acc, v[u].v[j], li[u] + j * p.r.lstride[0]);
                    }
                }
            }
        } else {
            for (int64_t r0 = rb + lane; r0 < re; r0 += (int64_t)G * kRedUnroll) {
                T x[kRedUnroll];
                int64_t li[kRedUnroll];
#pragma unroll
                for (int u = 0; u < kRedUnroll; ++u) {
                    const int64_t r = r0 + (int64_t)u * G;
                    if (r < re) x[u] = in[base + red_offset(p.r, (uint32_t)r, &li[u])];
                }
#pragma unroll
                for (int u = 0; u < kRedUnroll; ++u)
                    if (r0 + (int64_t)u * G < re) R::fold(acc, x[u], li[u]);
            }
        }
    }
    // combine the group (fixed tree: deterministic)
    if (G > 1) {
        const int width = G < 32 ? G : 32;
        for (int d = width >> 1; d > 0; d >>= 1) {
            Acc other = shfl_down_acc(acc, d, width);
            R::merge(acc, other);
        }
        if (G > 32) {
            __shared__ Acc warp_acc[kRedThreads / 32];
            const int w = tid >> 5;
            if ((tid & 31) == 0) warp_acc[w] = acc;
            __syncthreads();
            if (tid == 0) {
                acc = warp_acc[0];
                for (int i = 1; i < kRedThreads / 32; ++i) R::merge(acc, warp_acc[i]);
            }
        }
    }
    if (!active || lane != 0) return;
    if (p.partial) {
        reinterpret_cast<Acc*>(p.partial)[(int64_t)blockIdx.y * p.nout + o] = acc;
        return;
    }
    int64_t oo = p.out_off;
    {
        uint32_t e = (uint32_t)o;
        for (int i = 0; i < p.k.nd - 1; ++i) {
            uint32_t q = p.k.div[i].div(e);
            oo += (int64_t)(e - q * p.k.shape[i]) * p.k.out_stride[i];
            e = q;
        }
        if (p.k.nd > 0) oo += (int64_t)e * p.k.out_stride[p.k.nd - 1];
    }
    reinterpret_cast<typename R::Out*>(p.out)[oo] = R::fin(acc, p.op, p.nred);
}

// Fold the per-chunk accumulators of every output in chunk order.
template <typename T, int KIND>
__global__ void __launch_bounds__(kRedThreads) reduce_combine_kernel(const RedParams p) {
    using R = Red<T, KIND>;
    using Acc = typename R::Acc;
    const int64_t o = (int64_t)blockIdx.x * kRedThreads + threadIdx.x;
    if (o >= p.nout) return;
    const Acc* part = reinterpret_cast<const Acc*>(p.partial);
    Acc acc = part[o];
    for (int s = 1; s < p.nsplit; ++s) R::merge(acc, part[(int64_t)s * p.nout + o]);
    int64_t oo = p.out_off;
    uint32_t e = (uint32_t)o;
    for (int i = 0; i < p.k.nd - 1; ++i) {
        uint32_t q = p.k.div[i].div(e);
        oo += (int64_t)(e - q * p.k.shape[i]) * p.k.out_stride[i];
        e = q;
    }
    if (p.k.nd > 0) oo += (int64_t)e * p.k.out_stride[p.k.nd - 1];
    reinterpret_cast<typename R::Out*>(p.out)[oo] = R::fin(acc, p.op, p.nred);
}

// Size of the accumulator of (T, KIND) in bytes (host side, for scratch).
template <typename T, int KIND>
constexpr size_t acc_size() {
    return sizeof(typename Red<T, KIND>::Acc);
}

// Host launcher for one (T, KIND); defined in the per-dtype translation units.
// `p` must be fully planned except for the scratch pointer.
template <typename T, int KIND>
int launch_reduce(rstsr_ctx* ctx, RedParams p) {
    const int64_t opc = red_outputs_per_cta(p);
    const int64_t gx = (p.nout + opc - 1) / opc;
    if (gx > INT32_MAX || p.nsplit > 65535) return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, "reduction too large");
    void* scratch = nullptr;
    if (p.nsplit > 1) {
        int s = scratch_alloc(ctx, (size_t)p.nsplit * (size_t)p.nout * acc_size<T, KIND>(), &scratch);
        if (s) return s;
        p.partial = scratch;
    } else {
        p.partial = nullptr;
    }
    reduce_kernel<T, KIND><<<dim3((unsigned)gx, (unsigned)p.nsplit), kRedThreads, 0, ctx->stream>>>(p);
    int s = after_launch(ctx, "reduce_kernel");
    if (s == RSTSR_OK && p.nsplit > 1) {
        const int64_t gc = (p.nout + kRedThreads - 1) / kRedThreads;
        reduce_combine_kernel<T, KIND><<<(unsigned)gc, kRedThreads, 0, ctx->stream>>>(p);
        s = after_launch(ctx, "reduce_combine_kernel");
    }
    if (scratch) scratch_free(ctx, scratch);
    return s;
}

// Dispatch entry of each per-dtype translation unit.
int reduce_launch_f64(rstsr_ctx* ctx, int kind, const RedParams& p);
int reduce_launch_f32(rstsr_ctx* ctx, int kind, const RedParams& p);
int reduce_launch_i32(rstsr_ctx* ctx, int kind, const RedParams& p);
int reduce_launch_i64(rstsr_ctx* ctx, int kind, const RedParams& p);
int reduce_launch_u64(rstsr_ctx* ctx, int kind, const RedParams& p);
int reduce_launch_bool(rstsr_ctx* ctx, int kind, const RedParams& p);

}  // namespace rstsr
