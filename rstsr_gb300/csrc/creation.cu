// Creation entry points of the device (rstsr-core/src/storage/creation.rs:39-62):
// arange (DeviceCreationArangeAPI), linspace (DeviceCreationComplexFloatAPI)
// and the in-place triangle masks tril / triu (DeviceCreationTriAPI), with the
// results of the rayon device (rstsr-core/src/feature_rayon/auto_impl/creation.rs:74-119).
//
// arange's length is host arithmetic on three scalars (rstsr_cuda_arange_len,
// no GPU); its values come from one kernel over the flat index with the
// reference's formulas: f64 / f32 elements are start + i * step in f64 with a
// rounding after the product and one after the sum
// (rstsr-native-impl/src/cpu_rayon/creation.rs:36-55; the _rn intrinsics keep
// the compiler from fusing them), integers start + i * step in 64-bit wrapping
// arithmetic (:8-34). linspace is start + i * step in the element type
// (:108-128). tril / triu write zeros only where the mask applies, one CTA row
// at a time (rstsr-native-impl/src/cpu_serial/op_tri.rs:524-591).
#include <cmath>
#include <cstring>
#include <string>

#include "common.cuh"
#include "ew_kernel.cuh"

namespace rstsr {
namespace {

constexpr int kCrThreads = 256;
// Longest arange / linspace accepted (2^40 elements: more than the device holds).
constexpr uint64_t kMaxCreate = uint64_t(1) << 40;

// a + b * c with a rounding after the product and one after the sum on every
// host compiler (the product goes through memory, so it cannot be fused).
double add_mul_2r(double a, double b, double c) {
    volatile double p = b * c;
    return a + p;
}

double read_f(rstsr_dtype t, const void* p) {
    if (t == RSTSR_F64) {
        double v;
        std::memcpy(&v, p, 8);
        return v;
    }
    float v;
    std::memcpy(&v, p, 4);
    return v;
}

// Integer host element as (negative, magnitude bits): exact for every type.
struct IntVal {
    bool neg;
    uint64_t u;  // two's complement bits for signed types, the value for unsigned
};

IntVal read_i(rstsr_dtype t, const void* p) {
    IntVal r{false, 0};
    switch (t) {
        case RSTSR_I8: { int8_t v; std::memcpy(&v, p, 1); r = {v < 0, (uint64_t)(int64_t)v}; break; }
        case RSTSR_I16: { int16_t v; std::memcpy(&v, p, 2); r = {v < 0, (uint64_t)(int64_t)v}; break; }
        case RSTSR_I32: { int32_t v; std::memcpy(&v, p, 4); r = {v < 0, (uint64_t)(int64_t)v}; break; }
        case RSTSR_I64: { int64_t v; std::memcpy(&v, p, 8); r = {v < 0, (uint64_t)v}; break; }
        case RSTSR_U8: { uint8_t v; std::memcpy(&v, p, 1); r = {false, v}; break; }
        case RSTSR_U16: { uint16_t v; std::memcpy(&v, p, 2); r = {false, v}; break; }
        case RSTSR_U32: { uint32_t v; std::memcpy(&v, p, 4); r = {false, v}; break; }
        default: { uint64_t v; std::memcpy(&v, p, 8); r = {false, v}; break; }
    }
    return r;
}

void int_range(rstsr_dtype t, int64_t* lo, int64_t* hi) {
    switch (t) {
        case RSTSR_I8: *lo = INT8_MIN, *hi = INT8_MAX; break;
        case RSTSR_I16: *lo = INT16_MIN, *hi = INT16_MAX; break;
        case RSTSR_I32: *lo = INT32_MIN, *hi = INT32_MAX; break;
        case RSTSR_U8: *lo = 0, *hi = UINT8_MAX; break;
        case RSTSR_U16: *lo = 0, *hi = UINT16_MAX; break;
        case RSTSR_U32: *lo = 0, *hi = UINT32_MAX; break;
        case RSTSR_U64: *lo = 0, *hi = INT64_MAX; break;
        default: *lo = INT64_MIN, *hi = INT64_MAX; break;
    }
}

int no_end() {
    return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE,
                "arange: the reference's repeated addition (current = current + step while current < end) "
                "does not reach the end of this range");
}

int too_long(uint64_t n) {
    return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, "arange: " + std::to_string(n) + " elements is too many");
}

// f64 / f32: cpu_rayon/creation.rs:36-55, with cpu_serial/creation.rs:7-19
// where ceil((end - start) / step) is not a usize.
int arange_len_float(rstsr_dtype t, const void* ps, const void* pe, const void* pst, int64_t* n_out) {
    const double s = read_f(t, ps), e = read_f(t, pe), st = read_f(t, pst);
    if (st == 0.0) return fail(RSTSR_ERR_INVALID_VALUE, "arange: step must not be zero");
    if (std::isnan(st))
        return fail(RSTSR_ERR_UNIMPLEMENTED, "arange: a NaN step (the reference returns [start] when start < end)");
    const double q = (e - s) / st;
    double c = std::isfinite(q) ? std::ceil(q) : NAN;
    if (!(c > -1.0 && c < 18446744073709551616.0)) {
        // repeated addition: nothing when start < end fails; otherwise the sum
        // runs away from the end (step < 0) or stops changing (q infinite)
        if (!(s < e)) return *n_out = 0, RSTSR_OK;
        return no_end();
    }
    uint64_t n = (uint64_t)c;
    if (n > kMaxCreate) return too_long(n);
    if (n > 0) {
        const double v = add_mul_2r(s, (double)(n - 1), st);
        bool past;
        if (t == RSTSR_F32) {
            const float lf = (float)v, ef = (float)e;
            past = (st > 0.0 && lf >= ef) || (st < 0.0 && lf <= ef);
        } else {
            past = (st > 0.0 && v >= e) || (st < 0.0 && v <= e);
        }
        if (past) --n;
    }
    *n_out = (int64_t)n;
    return RSTSR_OK;
}

// Repeated addition in the element type (cpu_serial/creation.rs:7-19) for the
// integer types without the isize shortcut, and for u64 values above
// isize::MAX: exact while start + n * step stays inside the type.
int arange_len_loop(rstsr_dtype t, IntVal s, IntVal e, IntVal st, int64_t* n_out) {
    const bool is_signed = t == RSTSR_I8 || t == RSTSR_I16 || t == RSTSR_I32 || t == RSTSR_I64;
    auto less = [&](IntVal a, IntVal b) {
        if (is_signed) return (int64_t)a.u < (int64_t)b.u;
        return a.u < b.u;
    };
    if (!less(s, e)) return *n_out = 0, RSTSR_OK;
    if (is_signed && st.neg) return no_end();  // decreasing from below the end
    // unsigned distance and step
    const uint64_t d = e.u - s.u, stp = st.u;
    const uint64_t n = d / stp + (d % stp != 0);
    if (n > kMaxCreate) return too_long(n);
    // the value after the last one must still fit the type, or the addition wraps
    int64_t lo, hi;
    int_range(t, &lo, &hi);
    uint64_t span;
    if (__builtin_mul_overflow(n, stp, &span)) return no_end();
    if (is_signed) {
        const int64_t sv = (int64_t)s.u;
        int64_t next;
        if (span > (uint64_t)INT64_MAX || __builtin_add_overflow(sv, (int64_t)span, &next) || next > hi) return no_end();
    } else {
        uint64_t next;
        const uint64_t uhi = t == RSTSR_U64 ? UINT64_MAX : (uint64_t)hi;
        if (__builtin_add_overflow(s.u, span, &next) || next > uhi) return no_end();
    }
    *n_out = (int64_t)n;
    return RSTSR_OK;
}

// i32 / i64 / u32 / u64 through isize (cpu_rayon/creation.rs:8-34).
int arange_len_isize(rstsr_dtype t, IntVal s, IntVal e, IntVal st, int64_t* n_out) {
    const int64_t si = (int64_t)s.u, ei = (int64_t)e.u, sti = (int64_t)st.u;
    const int64_t diff = (int64_t)(e.u - s.u);  // isize subtraction, wrapping
    const double c = std::ceil((double)diff / (double)sti);
    if (!(c > -9223372036854777856.0 && c < 9223372036854775808.0)) return arange_len_loop(t, s, e, st, n_out);
    const int64_t ns = (int64_t)c;
    if (ns <= 0) return *n_out = 0, RSTSR_OK;
    uint64_t n = (uint64_t)ns;
    if (n > kMaxCreate) return too_long(n);
    int64_t span, last;
    if (__builtin_mul_overflow((int64_t)(n - 1), sti, &span) || __builtin_add_overflow(si, span, &last))
        return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, "arange: start + i * step overflows isize");
    int64_t lo, hi;
    int_range(t, &lo, &hi);
    if (last < lo || last > hi)
        return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, "arange: a value does not fit the element type");
    if ((sti > 0 && last >= ei) || (sti < 0 && last <= ei)) --n;
    *n_out = (int64_t)n;
    return RSTSR_OK;
}

template <typename T>
__global__ void __launch_bounds__(kCrThreads) arange_float_kernel(T* __restrict__ c, int64_t n, double s, double st) {
    for (int64_t i = (int64_t)blockIdx.x * kCrThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kCrThreads)
        c[i] = (T)__dadd_rn(s, __dmul_rn((double)i, st));
}

template <typename T>
__global__ void __launch_bounds__(kCrThreads) arange_int_kernel(T* __restrict__ c, int64_t n, uint64_t s, uint64_t st) {
    for (int64_t i = (int64_t)blockIdx.x * kCrThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kCrThreads)
        c[i] = (T)(s + (uint64_t)i * st);
}

__global__ void __launch_bounds__(kCrThreads) linspace_f64_kernel(double* __restrict__ c, int64_t n, double s, double st) {
    for (int64_t i = (int64_t)blockIdx.x * kCrThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kCrThreads)
        c[i] = n == 1 ? s : __dadd_rn(s, __dmul_rn((double)i, st));
}

__global__ void __launch_bounds__(kCrThreads) linspace_f32_kernel(float* __restrict__ c, int64_t n, float s, float st) {
    for (int64_t i = (int64_t)blockIdx.x * kCrThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kCrThreads)
        c[i] = n == 1 ? s : __fadd_rn(s, __fmul_rn((float)i, st));
}

unsigned flat_grid(const rstsr_ctx* ctx, int64_t n) {
    const int64_t blocks = (n + kCrThreads - 1) / kCrThreads;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)std::max(ctx->num_sms, 1) * 8));
}

struct TriMaskParams {
    int64_t nrow, ncol, rows;  // rows = batch * nrow
    int64_t si, sj;            // strides of the last two axes
    int64_t offset;
    int64_t k;
    int32_t nb, upper;
    int64_t bshape[RSTSR_MAX_NDIM], bstride[RSTSR_MAX_NDIM];  // batch axes, C order
};

// One row of one matrix per CTA iteration: the threads zero the row's masked
// column range (tril: j >= i + k + 1; triu: j < i + k, clipped to the row).
template <typename T>
__global__ void __launch_bounds__(kCrThreads) tri_mask_kernel(T* __restrict__ c, const TriMaskParams p) {
    for (int64_t r = blockIdx.x; r < p.rows; r += gridDim.x) {
        const int64_t i = r % p.nrow;
        int64_t b = r / p.nrow;
        int64_t off = p.offset + i * p.si;
        for (int d = p.nb - 1; d >= 0; --d) {
            const int64_t q = b / p.bshape[d];
            off += (b - q * p.bshape[d]) * p.bstride[d];
            b = q;
        }
        int64_t j0, j1;
        if (p.upper) {
            const int64_t d = i + p.k;
            j0 = 0;
            j1 = d < 0 ? 0 : (d > p.ncol ? p.ncol : d);
        } else {
            const int64_t d = i + p.k + 1;
            j0 = d < 0 ? 0 : d;
            j1 = p.ncol;
        }
        for (int64_t j = j0 + threadIdx.x; j < j1; j += kCrThreads) c[off + j * p.sj] = (T)0;
    }
}

}  // namespace
}  // namespace rstsr

using namespace rstsr;

extern "C" {

int rstsr_cuda_arange_len(rstsr_dtype t, const void* start, const void* end, const void* step, int64_t* n) {
    clear_error();
    if (!start || !end || !step || !n) return fail(RSTSR_ERR_INVALID_VALUE, "arange: null argument");
    *n = 0;
    if (!dtype_valid(t)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    if (t == RSTSR_F64 || t == RSTSR_F32) return arange_len_float(t, start, end, step, n);
    if (t == RSTSR_F16 || t == RSTSR_BF16 || t == RSTSR_BOOL)
        return fail(RSTSR_ERR_UNIMPLEMENTED, std::string("arange is not provided for ") + dtype_name(t));
    const IntVal s = read_i(t, start), e = read_i(t, end), st = read_i(t, step);
    if (st.u == 0) return fail(RSTSR_ERR_INVALID_VALUE, "arange: step must not be zero");
    const bool isize_path = t == RSTSR_I32 || t == RSTSR_I64 || t == RSTSR_U32 ||
                            (t == RSTSR_U64 && s.u <= (uint64_t)INT64_MAX && e.u <= (uint64_t)INT64_MAX &&
                             st.u <= (uint64_t)INT64_MAX);
    return isize_path ? arange_len_isize(t, s, e, st, n) : arange_len_loop(t, s, e, st, n);
}

int rstsr_cuda_arange(rstsr_ctx* ctx, rstsr_dtype t, void* c, int64_t n, const void* start, const void* step) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    if (!start || !step) return fail(RSTSR_ERR_INVALID_VALUE, "arange: null argument");
    if (!dtype_valid(t)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    if (t == RSTSR_F16 || t == RSTSR_BF16 || t == RSTSR_BOOL)
        return fail(RSTSR_ERR_UNIMPLEMENTED, std::string("arange is not provided for ") + dtype_name(t));
    if (n < 0 || (uint64_t)n > kMaxCreate) return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, "arange: bad length");
    if (n == 0) return RSTSR_OK;
    if (!c) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    const unsigned grid = flat_grid(ctx, n);
    if (t == RSTSR_F64 || t == RSTSR_F32) {
        const double s = read_f(t, start), st = read_f(t, step);
        if (t == RSTSR_F64)
            arange_float_kernel<double><<<grid, kCrThreads, 0, ctx->stream>>>((double*)c, n, s, st);
        else
            arange_float_kernel<float><<<grid, kCrThreads, 0, ctx->stream>>>((float*)c, n, s, st);
        return after_launch(ctx, "arange_float_kernel");
    }
    const uint64_t s = read_i(t, start).u, st = read_i(t, step).u;
    switch (dtype_size(t)) {
        case 8: arange_int_kernel<uint64_t><<<grid, kCrThreads, 0, ctx->stream>>>((uint64_t*)c, n, s, st); break;
        case 4: arange_int_kernel<uint32_t><<<grid, kCrThreads, 0, ctx->stream>>>((uint32_t*)c, n, s, st); break;
        case 2: arange_int_kernel<uint16_t><<<grid, kCrThreads, 0, ctx->stream>>>((uint16_t*)c, n, s, st); break;
        default: arange_int_kernel<uint8_t><<<grid, kCrThreads, 0, ctx->stream>>>((uint8_t*)c, n, s, st); break;
    }
    return after_launch(ctx, "arange_int_kernel");
}

int rstsr_cuda_linspace(rstsr_ctx* ctx, rstsr_dtype t, void* c, int64_t n, const void* start, const void* end,
                        int32_t endpoint) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    if (!start || !end) return fail(RSTSR_ERR_INVALID_VALUE, "linspace: null argument");
    if (t != RSTSR_F64 && t != RSTSR_F32)
        return fail(RSTSR_ERR_INVALID_VALUE, "linspace is defined for f64 and f32 (ComplexFloat) elements");
    if (n < 0 || (uint64_t)n > kMaxCreate) return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, "linspace: bad length");
    if (n == 0) return RSTSR_OK;
    if (!c) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    const unsigned grid = flat_grid(ctx, n);
    const uint64_t div = endpoint ? (uint64_t)n - 1 : (uint64_t)n;
    if (t == RSTSR_F64) {
        const double s = read_f(t, start), e = read_f(t, end);
        const double st = n == 1 ? 0.0 : (e - s) / (double)div;
        linspace_f64_kernel<<<grid, kCrThreads, 0, ctx->stream>>>((double*)c, n, s, st);
    } else {
        float s, e;
        std::memcpy(&s, start, 4);
        std::memcpy(&e, end, 4);
        const float diff = e - s, fdiv = (float)div;
        const float st = n == 1 ? 0.0f : diff / fdiv;
        linspace_f32_kernel<<<grid, kCrThreads, 0, ctx->stream>>>((float*)c, n, s, st);
    }
    return after_launch(ctx, "linspace_kernel");
}

int rstsr_cuda_tril(rstsr_ctx* ctx, rstsr_dtype t, void* c, const rstsr_layout* lc, int64_t k, int32_t upper) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(lc, "c"));
    if (!dtype_valid(t)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    Layout L = Layout::from_abi(*lc);
    if (L.ndim < 2) return fail(RSTSR_ERR_INVALID_LAYOUT, "tril / triu need at least two axes");
    RSTSR_TRY(check_write_layout(L, upper ? "triu" : "tril"));
    if (L.size() == 0) return RSTSR_OK;
    if (!c) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    TriMaskParams p;
    std::memset(&p, 0, sizeof(p));
    p.nrow = L.shape[L.ndim - 2];
    p.ncol = L.shape[L.ndim - 1];
    p.si = L.stride[L.ndim - 2];
    p.sj = L.stride[L.ndim - 1];
    p.offset = L.offset;
    // beyond +-(nrow + ncol) the mask is all or nothing: clamping keeps i + k in range
    const int64_t lim = p.nrow + p.ncol + 1;
    p.k = std::max(-lim, std::min(k, lim));
    p.upper = upper ? 1 : 0;
    p.nb = L.ndim - 2;
    int64_t batch = 1;
    for (int d = 0; d < p.nb; ++d) {
        p.bshape[d] = L.shape[d];
        p.bstride[d] = L.stride[d];
        batch *= L.shape[d];
    }
    p.rows = batch * p.nrow;
    const unsigned grid = (unsigned)std::max<int64_t>(
        1, std::min<int64_t>(p.rows, (int64_t)std::max(ctx->num_sms, 1) * 16));
    switch (dtype_size(t)) {
        case 8: tri_mask_kernel<uint64_t><<<grid, kCrThreads, 0, ctx->stream>>>((uint64_t*)c, p); break;
        case 4: tri_mask_kernel<uint32_t><<<grid, kCrThreads, 0, ctx->stream>>>((uint32_t*)c, p); break;
        case 2: tri_mask_kernel<uint16_t><<<grid, kCrThreads, 0, ctx->stream>>>((uint16_t*)c, p); break;
        default: tri_mask_kernel<uint8_t><<<grid, kCrThreads, 0, ctx->stream>>>((uint8_t*)c, p); break;
    }
    return after_launch(ctx, upper ? "triu_kernel" : "tril_kernel");
}

}  // extern "C"
