// Axis reductions on the GPU. Replaces reduce_all_cpu_rayon /
// reduce_axes_cpu_rayon (rstsr-native-impl/src/cpu_rayon/reduction.rs:20-328)
// and the arg reductions (:440-631) with one group-reduction kernel:
//
//   * the reduced axes and the kept axes are each collapsed into a small
//     iteration space (inner-first, contiguous neighbours merged);
//   * "row" regime (reduced axes innermost in memory, reduce_row_kernel): a
//     group of G threads (G = 1 ... 256) owns one output element and walks its
//     reduced elements with 16-byte vector loads, combining the group with
//     warp shuffles and shared memory; "column" regime (a kept axis
//     innermost, reduce_col_kernel): neighbouring threads own neighbouring
//     outputs (several per thread with vector loads) so every load is
//     coalesced across the warp; both walks advance a (row, column) position
//     instead of decomposing every index;
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
    // row regime: a group step of G * W reduced elements (W = the vector
    // width, or 1) moves the (row, column) position by adv_row rows and
    // adv_c columns of reduced dim 0 (step = adv_row * shape[0] + adv_c)
    uint32_t adv_row, adv_c;
    int32_t row;   // row regime (G threads per output, G may be 1)
    int32_t mono;  // the flattened reduced index is the logical index (walks visit it in order)
    int32_t s2;    // row regime, reduced dim 0 of stride 2: 16-byte loads serve VEC / 2 elements
    int64_t max_off;  // largest element offset of the input view (the s2 loads stay at or below it)
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

// f64 sum and mean without the FP64 pipe (GB300 issues about two FP64 adds
// per cycle and SM, which bounded the f64 sums below the memory rate). The
// accumulator is a signed 64-bit integer S in units of 2^(E - 1075), E being
// the largest biased exponent seen so far: a double x = +-M 2^(ex - 1075)
// (M the 53-bit significand, ex >= 1) adds +-(M >> (E - ex)), i.e. x
// truncated to that unit, an error below 2^-52 of the largest magnitude per
// term (an FP64 add rounds at 2^-53 of the running sum). A larger exponent
// shifts S right first. |S| is kept below 2^62 (one halving with E + 1 after
// each round of at most a few hundred terms; a term is below 2^53), so S never
// overflows. All steps are integer and deterministic. NaN and +-inf terms go
// to an FP64 side sum, added at the end with IEEE semantics (inf + -inf = NaN).
// The integer fold costs about 25 ALU instructions a term, so the walks hand
// every other term to the FP64 pipe instead (fold_fp, a plain FP64 add into
// d): the two pipes then share the work, and the result is the fixed-point
// sum plus d, still deterministic.
struct AccFix {
    long long s;   // the fixed-point sum
    int32_t e;     // biased exponent of its unit + 1075
    int32_t nonfinite;
    double spec;   // sum of the NaN / inf terms
    double d;      // FP64 sum of the terms given to the FP64 pipe
};
template <>
struct Red<double, kRedSum> {
    using Acc = AccFix;
    using Out = double;
    __device__ static Acc init() { return {0, 1, 0, 0.0, 0.0}; }
    __device__ static void fold_fp(Acc& a, double x) { a.d += x; }
    __device__ static void fix(Acc& a) {
        const long long lim = (long long)1 << 62;
        if (a.s >= lim || a.s <= -lim) {
            a.s >>= 1;
            a.e += 1;
        }
    }
    __device__ static void fold(Acc& a, double x, int64_t) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(x);
        const int ex = (int)((b >> 52) & 0x7FF);
        if (ex == 0x7FF) {
            a.nonfinite = 1;
            a.spec += x;
            return;
        }
        long long m = (long long)(b & 0xFFFFFFFFFFFFFULL) | (ex ? (1LL << 52) : 0LL);
        const int exe = ex > 1 ? ex : 1;
        if (exe > a.e) {
            const int up = exe - a.e;
            a.s = up > 63 ? (a.s < 0 ? -1 : 0) : (a.s >> up);
            a.e = exe;
        }
        const int d = a.e - exe;
        m = d > 63 ? 0 : (m >> d);
        a.s += (b >> 63) ? -m : m;
    }
    __device__ static void merge(Acc& a, const Acc& o) {
        if (o.nonfinite) {
            a.nonfinite = 1;
            a.spec += o.spec;
        }
        a.d += o.d;
        const int e = a.e > o.e ? a.e : o.e;
        const int da = e - a.e, db = e - o.e;
        const long long sa = da > 63 ? (a.s < 0 ? -1 : 0) : (a.s >> da);
        const long long sb = db > 63 ? (o.s < 0 ? -1 : 0) : (o.s >> db);
        a.s = sa + sb;
        a.e = e;
        fix(a);
    }
    __device__ static Out fin(const Acc& a, int op, int64_t n) {
        double r = ldexp((double)a.s, a.e - 1075) + a.d;
        if (a.nonfinite) r += a.spec;
        return op == RSTSR_RED_MEAN ? r / (double)n : r;
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

// Every policy folds into a thread-local accumulator `Local` first, with the
// element's logical index within the reduced set as a 32-bit value (the
// planner refuses 2^32 or more reduced elements per output), and turns it
// into its `Acc` for the shuffles, the partials and the finalisation. For the
// value reductions Local is Acc.
template <typename T, int KIND>
struct RedLocal : Red<T, KIND> {
    using R = Red<T, KIND>;
    using Local = typename R::Acc;
    __device__ static Local linit() { return R::init(); }
    __device__ static void lfold(Local& s, T x, uint32_t li) { R::fold(s, x, (int64_t)li); }
    __device__ static typename R::Acc to_acc(const Local& s) { return s; }
    // after every round of loads: keeps the fixed-point f64 sum in range
    __device__ static void lfix(Local& s) {
        if constexpr (KIND == kRedSum && std::is_same<T, double>::value) R::fix(s);
    }
    // the f64 sum gives every other term to the FP64 pipe
    static constexpr bool kSplitPipe = KIND == kRedSum && std::is_same<T, double>::value;
    __device__ static void lfold_fp(Local& s, T x) {
        if constexpr (kSplitPipe) R::fold_fp(s, x);
    }
    static constexpr bool kArg = false;

    // (the ordered-walk key interface of the arg reductions; unused here)
    using Key = int;
    __device__ static Key kstart() { return 0; }
    __device__ static Key key(T) { return 0; }
    __device__ static Key kbest(Key a, Key) { return a; }
    __device__ static bool kwins(Key, Key) { return false; }
};

// arg reductions: the smallest logical index among the extreme values; NaN is
// never accepted, except that a NaN at logical index 0 makes the answer 0 (the
// serial fold of cpu_serial/reduction.rs:425-477 starts from that element and
// no comparison against NaN succeeds afterwards).
//
// The empty accumulator holds the worst value (-inf / the type's minimum for
// argmax) at index "none", so "strictly better, or equal at a smaller index"
// covers it without a separate test, and the fold selects without branches.
// A floating-point NaN fails both comparisons and is never taken; the element
// at logical index 0 is tested for NaN once per output, outside the loop.
template <typename T, bool IS_MAX>
struct RedArg {
    using Acc = AccArg<T>;
    using Out = uint64_t;
    struct Local {
        T v;
        uint32_t idx;  // UINT32_MAX: empty
    };
    static constexpr bool kArg = true;
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
    __device__ static Local linit() { return {start(), UINT32_MAX}; }
    __device__ static void lfix(Local&) {}
    static constexpr bool kSplitPipe = false;
    __device__ static void lfold_fp(Local&, T) {}
    template <typename I>
    __device__ static bool better(T x, I ix, T v, I iv) {
        return (IS_MAX ? (x > v) : (x < v)) | ((x == v) & (ix < iv));
    }
    // Ordered walks (logical indices visited in increasing order): compare
    // keys; a later equal key never wins, NaN never wins (its key fails every
    // comparison, and fmax / fmin drop it).
    using Key = T;
    __device__ static Key kstart() { return start(); }
    __device__ static Key key(T x) { return x; }
    __device__ static Key kbest(Key a, Key b) {
        if constexpr (std::is_floating_point<T>::value) return IS_MAX ? fmax(a, b) : fmin(a, b);
        else return IS_MAX ? (a > b ? a : b) : (a < b ? a : b);
    }
    __device__ static bool kwins(Key a, Key b) { return IS_MAX ? (a > b) : (a < b); }
    __device__ static void lfold(Local& s, T x, uint32_t li) {
        const bool take = better(x, li, s.v, s.idx);
        s.v = take ? x : s.v;
        s.idx = take ? li : s.idx;
    }
    __device__ static Acc to_acc(const Local& s) {
        return {s.v, s.idx == UINT32_MAX ? INT64_MAX : (int64_t)s.idx, 0};
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
// NaN is recognised from its bits and skipped. Same results as RedArg<double>.
template <bool IS_MAX>
struct RedArgF64 {
    using Acc = AccArg<int64_t>;
    using Out = uint64_t;
    struct Local {
        int64_t v;
        uint32_t idx;
    };
    static constexpr bool kArg = true;
    // keys of non-NaN doubles lie strictly inside (INT64_MIN, INT64_MAX)
    __device__ static Acc init() { return {IS_MAX ? INT64_MIN : INT64_MAX, INT64_MAX, 0}; }
    __device__ static Local linit() { return {IS_MAX ? INT64_MIN : INT64_MAX, UINT32_MAX}; }
    __device__ static void lfix(Local&) {}
    static constexpr bool kSplitPipe = false;
    __device__ static void lfold_fp(Local&, double) {}
    template <typename I>
    __device__ static bool better(int64_t x, I ix, int64_t v, I iv) {
        return (IS_MAX ? (x > v) : (x < v)) | ((x == v) & (ix < iv));
    }
    // ordered walks: the key of a NaN is the start value, which never wins
    using Key = int64_t;
    __device__ static Key kstart() { return IS_MAX ? INT64_MIN : INT64_MAX; }
    __device__ static Key key(double xd) {
        int64_t b = __double_as_longlong(xd);
        const bool nan = (b & INT64_MAX) > 0x7FF0000000000000LL;
        if (b == INT64_MIN) b = 0;  // -0.0 -> +0.0
        const int64_t k = b >= 0 ? b : (b ^ INT64_MAX);
        return nan ? (IS_MAX ? INT64_MIN : INT64_MAX) : k;
    }
    __device__ static Key kbest(Key a, Key b) { return IS_MAX ? (a > b ? a : b) : (a < b ? a : b); }
    __device__ static bool kwins(Key a, Key b) { return IS_MAX ? (a > b) : (a < b); }
    __device__ static void lfold(Local& s, double xd, uint32_t li) {
        int64_t b = __double_as_longlong(xd);
        const bool nan = (b & INT64_MAX) > 0x7FF0000000000000LL;
        if (b == INT64_MIN) b = 0;  // -0.0 -> +0.0
        const int64_t key = b >= 0 ? b : (b ^ INT64_MAX);
        const bool take = !nan & better(key, li, s.v, s.idx);
        s.v = take ? key : s.v;
        s.idx = take ? li : s.idx;
    }
    __device__ static Acc to_acc(const Local& s) {
        return {s.v, s.idx == UINT32_MAX ? INT64_MAX : (int64_t)s.idx, 0};
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

template <typename T>
struct RedLocal<T, kRedArgMax> : Red<T, kRedArgMax> {};
template <typename T>
struct RedLocal<T, kRedArgMin> : Red<T, kRedArgMin> {};

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

// loads in flight per thread in the row walk and in the column walk (whose
// OV-wide loads and OV accumulators take more registers)
constexpr int kRedUnroll = 8;
constexpr int kRedUnrollCol = 4;
// the column walk with OV-wide vector loads: eight in flight (45-48 registers,
// five CTAs per SM); measured on GB300 against four and sixteen on the
// F-ordered [32,64,128,128] sums and argmax
constexpr int kRedUnrollColVec = 8;

// ---------------------------------------------------------------- kernels

template <typename T, int VEC>
struct alignas(sizeof(T) * VEC) RVec {
    T v[VEC];
};

// Input offset and logical index of row `row` of the reduced space: its dims
// 1 .. nd-1 (dim 1 fastest); dim 0 is the column inside the row. Reduced
// spaces of one or two dims (the common case after collapsing) read their one
// row stride at a fixed parameter offset; deeper ones loop.
__device__ __forceinline__ int64_t red_row_offset(const RedSpace& r, uint32_t row, uint32_t* lrow) {
    if (r.nd <= 1) {
        *lrow = 0;
        return 0;
    }
    if (r.nd == 2) {
        *lrow = row * (uint32_t)r.lstride[1];
        return (int64_t)row * r.stride[1];
    }
    int64_t off = 0;
    uint32_t li = 0;
    for (int i = 1; i < r.nd - 1; ++i) {
        const uint32_t q = r.div[i].div(row);
        const uint32_t idx = row - q * r.shape[i];
        off += (int64_t)idx * r.stride[i];
        li += idx * (uint32_t)r.lstride[i];
        row = q;
    }
    off += (int64_t)row * r.stride[r.nd - 1];
    li += row * (uint32_t)r.lstride[r.nd - 1];
    *lrow = li;
    return off;
}

__device__ __forceinline__ int64_t kept_offset(const KeptSpace& k, uint32_t e, bool out) {
    const int64_t* st = out ? k.out_stride : k.in_stride;
    if (k.nd <= 0) return 0;
    if (k.nd == 1) return (int64_t)e * st[0];
    int64_t off = 0;
    for (int i = 0; i < k.nd - 1; ++i) {
        const uint32_t q = k.div[i].div(e);
        off += (int64_t)(e - q * k.shape[i]) * st[i];
        e = q;
    }
    return off + (int64_t)e * st[k.nd - 1];
}

// Outputs per thread of the vectorised column regime: a 16-byte (f64: two,
// 4-byte types: four) or smaller load covers that many neighbouring outputs.
template <typename T>
constexpr int red_col_vec() {
    return 16 / sizeof(T) >= 4 ? 4 : (16 / sizeof(T) >= 2 ? 2 : 1);
}

// Outputs handled by one CTA.
__host__ __device__ inline int64_t red_outputs_per_cta(const RedParams& p) {
    return (int64_t)(kRedThreads >> p.glog) * (p.ocol > 1 ? p.ocol : 1);
}

// Row regime: a group of G = 2^glog threads owns one output and walks its
// reduced elements W at a time (W = VEC with p.vec: one vector load of
// neighbours along the contiguous reduced dim 0; else 1). Lane l starts at
// flattened reduced index rb + l W and steps by G W; its (row, column)
// position advances by the host-computed (adv_row, adv_c), so a step costs an
// add and a compare, plus the row's offset (one multiply for a 2-dim reduced
// space, a division chain beyond), instead of a full index decomposition.
// SS = 2: reduced dim 0 has stride 2 (a step-2 slice); a 16-byte load of 2W
// raw elements serves the W elements at its even positions, and a load that
// would reach past the view's last element (p.max_off) is replaced by W
// scalar loads: every access stays inside the view's span.
template <typename T, int W, int SS>
__device__ __forceinline__ RVec<T, W> red_load(const RedParams& p, const T* __restrict__ in, int64_t at) {
    if constexpr (SS == 1) {
        return *reinterpret_cast<const RVec<T, W>*>(in + at);
    } else {
        RVec<T, W> v;
        if (at + 2 * W - 1 <= p.max_off) {
            const RVec<T, 2 * W> raw = *reinterpret_cast<const RVec<T, 2 * W>*>(in + at);
#pragma unroll
            for (int j = 0; j < W; ++j) v.v[j] = raw.v[2 * j];
        } else {
#pragma unroll
            for (int j = 0; j < W; ++j) v.v[j] = in[at + 2 * j];
        }
        return v;
    }
}

template <typename T, int KIND, int W, bool MONO, int SS = 1>
__device__ __forceinline__ typename RedLocal<T, KIND>::Local red_rows(const RedParams& p, const T* __restrict__ in,
                                                                   int64_t base, int lane, int G) {
    using R = RedLocal<T, KIND>;
    // 8-byte elements: four loads in flight (their accumulators and keys take
    // twice the registers)
    constexpr int U = sizeof(T) >= 8 ? kRedUnroll / 2 : kRedUnroll;
    typename R::Local acc = R::linit();
    const int64_t rb = (int64_t)blockIdx.y * p.chunk;
    const int64_t re = min(p.nred, rb + p.chunk);
    int64_t r = rb + (int64_t)lane * W;
    if (r >= re) return acc;
    const uint32_t n0 = p.r.shape[0];
    const int64_t s0 = p.r.stride[0];
    const uint32_t l0 = (uint32_t)p.r.lstride[0];
    uint32_t row = p.r.div[0].div((uint32_t)r);
    uint32_t c = (uint32_t)r - row * n0;
    const int64_t step = (int64_t)G * W;
    // ordered arg reductions with vector loads: the best key of each vector
    // first, its position inside the vector located once at the end
    constexpr bool kFast = R::kArg && MONO && W > 1;
    [[maybe_unused]] typename R::Key best{};
    [[maybe_unused]] uint32_t best_r = UINT32_MAX;
    if constexpr (kFast) best = R::kstart();
    // logical indices of the loads are kept only where they cannot be
    // recomputed from the iteration's first flattened index (an arg reduction
    // over a reduced space whose flattened and logical orders differ)
    constexpr bool kKeepLi = R::kArg && !MONO;
    for (; r < re;) {
        const int64_t r0 = r;
        RVec<T, W> v[U];
        [[maybe_unused]] uint32_t li[kKeepLi ? U : 1];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (r0 + u * step < re) {
                uint32_t lrow;
                const int64_t off = red_row_offset(p.r, row, &lrow) + (int64_t)c * s0;
                if constexpr (kKeepLi) li[u] = lrow + c * l0;
                v[u] = red_load<T, W, SS>(p, in, base + off);
            }
            c += p.adv_c;
            row += p.adv_row;
            if (c >= n0) {
                c -= n0;
                ++row;
            }
        }
        r = r0 + U * step;
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (r0 + u * step < re) {
                const uint32_t lu = kKeepLi ? li[kKeepLi ? u : 0] : (uint32_t)(r0 + u * step);
                if constexpr (kFast) {
                    typename R::Key m = R::key(v[u].v[0]);
#pragma unroll
                    for (int j = 1; j < W; ++j) m = R::kbest(m, R::key(v[u].v[j]));
                    const bool take = R::kwins(m, best);
                    best = take ? m : best;
                    best_r = take ? lu : best_r;
                } else if constexpr (R::kSplitPipe) {
#pragma unroll
                    for (int j = 0; j < W; ++j) {
                        if ((W > 1 ? j : u) & 1)
                            R::lfold(acc, v[u].v[j], lu + (uint32_t)j * l0);
                        else
                            R::lfold_fp(acc, v[u].v[j]);
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < W; ++j) R::lfold(acc, v[u].v[j], lu + (uint32_t)j * l0);
                }
            }
        R::lfix(acc);
    }
    if constexpr (kFast) {
        if (best_r != UINT32_MAX) {
            // the first element of the winning vector that holds the best key
            // (best_r is its flattened index: a multiple of W inside a row)
            const uint32_t brow = p.r.div[0].div(best_r);
            uint32_t lrow;
            const int64_t boff = red_row_offset(p.r, brow, &lrow) + (int64_t)(best_r - brow * n0) * s0;
            const RVec<T, W> w = red_load<T, W, SS>(p, in, base + boff);
            int jj = W - 1;
#pragma unroll
            for (int j = W - 1; j >= 0; --j) jj = R::key(w.v[j]) == best ? j : jj;
            acc.v = best;
            acc.idx = best_r + (uint32_t)jj;
        }
    }
    return acc;
}

// Column regime: one thread owns OV neighbouring outputs (OV > 1: the kept
// dim 0 is contiguous and one OV-wide vector load per reduced element serves
// them all) and walks the reduced elements of its chunk in order, the
// (row, column) position advancing by one.
template <typename T, int KIND, int OV, bool MONO, int UC>
__device__ __forceinline__ void red_cols(const RedParams& p, const T* __restrict__ in, int64_t base,
                                         typename RedLocal<T, KIND>::Local (&acc)[OV]) {
    using R = RedLocal<T, KIND>;
    const int64_t rb = (int64_t)blockIdx.y * p.chunk;
    const int64_t re = min(p.nred, rb + p.chunk);
    if (rb >= re) return;
    const uint32_t n0 = p.r.shape[0];
    const int64_t s0 = p.r.stride[0];
    const uint32_t l0 = (uint32_t)p.r.lstride[0];
    uint32_t row = p.r.div[0].div((uint32_t)rb);
    uint32_t c = (uint32_t)rb - row * n0;
    uint32_t lrow;
    int64_t roff = red_row_offset(p.r, row, &lrow);
    for (int64_t r = rb; r < re; r += UC) {
        RVec<T, OV> v[UC];
        uint32_t li[UC];
#pragma unroll
        for (int u = 0; u < UC; ++u) {
            if (r + u < re) {
                li[u] = MONO ? (uint32_t)(r + u) : lrow + c * l0;
                v[u] = *reinterpret_cast<const RVec<T, OV>*>(in + base + roff + (int64_t)c * s0);
                if (++c == n0) {
                    c = 0;
                    ++row;
                    if (r + u + 1 < re) roff = red_row_offset(p.r, row, &lrow);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < UC; ++u)
            if (r + u < re) {
#pragma unroll
                for (int j = 0; j < OV; ++j) {
                    if constexpr (R::kArg && MONO) {
                        // logical indices increase along the walk: a later
                        // equal key never wins
                        const typename R::Key k = R::key(v[u].v[j]);
                        const bool take = R::kwins(k, acc[j].v);
                        acc[j].v = take ? k : acc[j].v;
                        acc[j].idx = take ? li[u] : acc[j].idx;
                    } else if constexpr (R::kSplitPipe) {
                        if (u & 1)
                            R::lfold(acc[j], v[u].v[j], li[u]);
                        else
                            R::lfold_fp(acc[j], v[u].v[j]);
                    } else {
                        R::lfold(acc[j], v[u].v[j], li[u]);
                    }
                }
            }
#pragma unroll
        for (int j = 0; j < OV; ++j) R::lfix(acc[j]);
    }
}

// Arg reductions: a NaN at logical index 0 (flattened reduced index 0, the
// element at the output's base offset) makes the answer 0; tested once per
// output by the thread that owns reduced index 0.
template <typename T, int KIND>
__device__ __forceinline__ void red_nan0(typename RedLocal<T, KIND>::Acc& acc, const T* __restrict__ in,
                                         int64_t base) {
    if constexpr (RedLocal<T, KIND>::kArg) {
        if (blockIdx.y == 0) {
            const T x = in[base];
            if (is_nan_v(x)) acc.nan0 = 1;
        }
    }
}

template <typename T, int KIND>
__device__ __forceinline__ void red_store(const RedParams& p, int64_t o, const typename Red<T, KIND>::Acc& acc) {
    using R = Red<T, KIND>;
    if (p.partial) {
        reinterpret_cast<typename R::Acc*>(p.partial)[(int64_t)blockIdx.y * p.nout + o] = acc;
        return;
    }
    reinterpret_cast<typename R::Out*>(p.out)[p.out_off + kept_offset(p.k, (uint32_t)o, true)] =
        R::fin(acc, p.op, p.nred);
}

// Column regime: one thread per output, or per OV neighbouring outputs.
template <typename T, int KIND, int OV, bool MONO, int UC = kRedUnrollCol>
__global__ void __launch_bounds__(kRedThreads) reduce_col_kernel(const RedParams p) {
    using R = RedLocal<T, KIND>;
    using Acc = typename R::Acc;
    const T* __restrict__ in = reinterpret_cast<const T*>(p.in);
    const int64_t o0 = ((int64_t)blockIdx.x * kRedThreads + threadIdx.x) * OV;
    if (o0 >= p.nout) return;  // with OV > 1, nout is a multiple of OV
    const int64_t base = p.in_off + kept_offset(p.k, (uint32_t)o0, false);
    typename R::Local acc[OV];
#pragma unroll
    for (int j = 0; j < OV; ++j) acc[j] = R::linit();
    red_cols<T, KIND, OV, MONO, UC>(p, in, base, acc);
#pragma unroll
    for (int j = 0; j < OV; ++j) {
        Acc a = R::to_acc(acc[j]);
        red_nan0<T, KIND>(a, in, base + (int64_t)j);  // kept dim 0 is contiguous when OV > 1
        red_store<T, KIND>(p, o0 + j, a);
    }
}

// Row regime: a group of G = 2^glog threads per output (G may be 1).
template <typename T, int KIND, int W, bool MONO, int SS = 1>
__global__ void __launch_bounds__(kRedThreads) reduce_row_kernel(const RedParams p) {
    using R = RedLocal<T, KIND>;
    using Acc = typename R::Acc;
    const T* __restrict__ in = reinterpret_cast<const T*>(p.in);
    const int G = 1 << p.glog;
    const int tid = threadIdx.x;
    const int lane = tid & (G - 1);
    const int64_t o = (int64_t)blockIdx.x * (kRedThreads >> p.glog) + (tid >> p.glog);
    const bool active = o < p.nout;
    int64_t base = 0;
    Acc acc = R::init();
    if (active) {
        base = p.in_off + kept_offset(p.k, (uint32_t)o, false);
        acc = R::to_acc(red_rows<T, KIND, W, MONO, SS>(p, in, base, lane, G));
    }
    // combine the group (fixed tree: deterministic)
    const int width = G < 32 ? G : 32;
    for (int d = width >> 1; d > 0; d >>= 1) {
        Acc other = shfl_down_acc(acc, d, width);
        R::merge(acc, other);
    }
    if (G > 32) {
        // a group spans G / 32 warps: its lane 0 folds those warps' partials
        __shared__ Acc warp_acc[kRedThreads / 32];
        const int w = tid >> 5;
        if ((tid & 31) == 0) warp_acc[w] = acc;
        __syncthreads();
        if (lane == 0) {
            const int nw = G >> 5;
            for (int i = 1; i < nw; ++i) R::merge(acc, warp_acc[w + i]);
        }
    }
    if (!active || lane != 0) return;
    red_nan0<T, KIND>(acc, in, base);
    red_store<T, KIND>(p, o, acc);
}

// Launch the main pass of a planned reduction (partials already assigned):
// the regime's kernel, with vector loads and the ordered fold where the plan
// allows them (the ordered fold matters only to the arg reductions).
template <typename T, int KIND>
cudaError_t launch_reduce_pass(const RedParams& p, dim3 grid, cudaStream_t stream) {
    constexpr int VEC = 16 / sizeof(T) > 0 ? 16 / sizeof(T) : 1;
    constexpr int OV = red_col_vec<T>();
    constexpr bool kArg = RedLocal<T, KIND>::kArg;
    const bool mono = kArg && p.mono;
    if (p.row) {
        if constexpr (VEC >= 4) {
            if (p.s2) {
                if (mono)
                    reduce_row_kernel<T, KIND, VEC / 2, kArg, 2><<<grid, kRedThreads, 0, stream>>>(p);
                else
                    reduce_row_kernel<T, KIND, VEC / 2, false, 2><<<grid, kRedThreads, 0, stream>>>(p);
                return cudaGetLastError();
            }
        }
        if (VEC > 1 && p.vec) {
            if (mono)
                reduce_row_kernel<T, KIND, VEC, kArg><<<grid, kRedThreads, 0, stream>>>(p);
            else
                reduce_row_kernel<T, KIND, VEC, false><<<grid, kRedThreads, 0, stream>>>(p);
        } else {
            if (mono)
                reduce_row_kernel<T, KIND, 1, kArg><<<grid, kRedThreads, 0, stream>>>(p);
            else
                reduce_row_kernel<T, KIND, 1, false><<<grid, kRedThreads, 0, stream>>>(p);
        }
    } else if (OV > 1 && p.ocol > 1) {
        if (mono)
            reduce_col_kernel<T, KIND, OV, kArg, kRedUnrollColVec><<<grid, kRedThreads, 0, stream>>>(p);
        else
            reduce_col_kernel<T, KIND, OV, false, kRedUnrollColVec><<<grid, kRedThreads, 0, stream>>>(p);
    } else {
        if (mono)
            reduce_col_kernel<T, KIND, 1, kArg><<<grid, kRedThreads, 0, stream>>>(p);
        else
            reduce_col_kernel<T, KIND, 1, false><<<grid, kRedThreads, 0, stream>>>(p);
    }
    return cudaGetLastError();
}

// Fold the per-chunk accumulators of every output: a CTA takes 32 outputs,
// its 8 warps each fold the chunks s = w, w + 8, ... of those outputs (loads
// coalesced across the outputs, four in flight), and the 8 partial folds are
// merged in warp order. The order is fixed by the launch shape, so results
// are deterministic. One thread per output folding every chunk in sequence
// was latency-bound: 16 us for the 152 chunks of 4096 outputs (an F-ordered
// f32 sum over two axes), 39 % of that reduction.
constexpr int kCombOuts = 32, kCombLanes = kRedThreads / kCombOuts;

template <typename T, int KIND>
__global__ void __launch_bounds__(kRedThreads) reduce_combine_kernel(const RedParams p) {
    using R = Red<T, KIND>;
    using Acc = typename R::Acc;
    __shared__ Acc part_acc[kCombLanes][kCombOuts];
    const int ol = threadIdx.x % kCombOuts, sl = threadIdx.x / kCombOuts;
    const int64_t o = (int64_t)blockIdx.x * kCombOuts + ol;
    const Acc* part = reinterpret_cast<const Acc*>(p.partial);
    Acc acc = R::init();
    if (o < p.nout) {
        int s = sl;
        for (; s + 3 * kCombLanes < p.nsplit; s += 4 * kCombLanes) {
            Acc v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = part[(int64_t)(s + u * kCombLanes) * p.nout + o];
#pragma unroll
            for (int u = 0; u < 4; ++u) R::merge(acc, v[u]);
        }
        for (; s < p.nsplit; s += kCombLanes) R::merge(acc, part[(int64_t)s * p.nout + o]);
    }
    part_acc[sl][ol] = acc;
    __syncthreads();
    if (sl != 0 || o >= p.nout) return;
#pragma unroll
    for (int i = 1; i < kCombLanes; ++i) R::merge(acc, part_acc[i][ol]);
    reinterpret_cast<typename R::Out*>(p.out)[p.out_off + kept_offset(p.k, (uint32_t)o, true)] =
        R::fin(acc, p.op, p.nred);
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
    cudaError_t e = launch_reduce_pass<T, KIND>(p, dim3((unsigned)gx, (unsigned)p.nsplit), ctx->stream);
    int s = e == cudaSuccess ? after_launch(ctx, "reduce pass") : cuda_fail(e, "reduce pass");
    if (s == RSTSR_OK && p.nsplit > 1) {
        const int64_t gc = (p.nout + kCombOuts - 1) / kCombOuts;
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
