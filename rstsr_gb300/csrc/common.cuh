// Shared plumbing of the sm_103a device backend: the context object, error
// reporting across the C ABI, dtype dispatch, fast integer division and the
// dimension-collapsing planner used by every strided kernel.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include <atomic>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "layout.hpp"
#include "rstsr_cuda.h"

namespace rstsr {
struct StagingRing;  // page-locked buffers for pageable host transfers (transfer.cu)
}

struct rstsr_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    cudaMemPool_t pool = nullptr;
    std::atomic<uint64_t> launches{0};
    bool capturing = false;
    uint64_t launches_at_capture = 0;
    int* dev_err = nullptr;  // device word: non-zero after a kernel gave up a bounded wait
    std::mutex staging_mu;
    rstsr::StagingRing* staging = nullptr;  // created by the first pageable transfer
};

namespace rstsr {

// ---- error reporting (see layout.hpp) ----
int cuda_fail(cudaError_t e, const char* what);

#define RSTSR_CUDA_TRY(expr)                                   \
    do {                                                       \
        cudaError_t _e = (expr);                               \
        if (_e != cudaSuccess) return ::rstsr::cuda_fail(_e, #expr); \
    } while (0)

// After a launch: count it and surface launch-configuration errors.
int after_launch(rstsr_ctx* ctx, const char* name);

// Release the context's staging ring (transfer.cu); no-op without one.
void staging_destroy(rstsr_ctx* ctx);

// Validate a context pointer and make its device current.
int enter(rstsr_ctx* ctx);

// Loads the GEMM autotune table named by RSTSR_CUDA_AUTOTUNE_TABLE, once per
// process (no-op when unset); the status of that load on every call.
int load_env_table();

// Scratch memory from the context pool (stream-ordered).
int scratch_alloc(rstsr_ctx* ctx, size_t bytes, void** p);
void scratch_free(rstsr_ctx* ctx, void* p);

// ---- fast unsigned 32-bit division by an invariant divisor ----
// Granlund & Montgomery (PLDI 1994), "Division by invariant integers using
// multiplication": q = (mulhi(n, m) + n) >> s with s = ceil(log2 d) and
// m = floor(2^32 (2^s - d) / d) + 1; exact for every 0 <= n < 2^32.
struct FastDiv {
    uint32_t d = 1, m = 0, s = 0;
    FastDiv() = default;
    explicit FastDiv(uint32_t div) : d(div) {
        s = 0;
        while ((uint64_t(1) << s) < div) ++s;
        m = uint32_t(((uint64_t(1) << 32) * ((uint64_t(1) << s) - div)) / div + 1);
        if (div == 1) m = 0;
    }
    __host__ __device__ __forceinline__ uint32_t div(uint32_t n) const {
#ifdef __CUDA_ARCH__
        uint32_t hi = __umulhi(n, m);
#else
        uint32_t hi = uint32_t((uint64_t(n) * m) >> 32);
#endif
        return uint32_t((uint64_t(hi) + n) >> s);
    }
};

// ---- collapsed iteration space shared by N operands ----
// dims are ordered inner-first (dim 0 varies fastest); every operand has its
// own strides and offset (elements). Broadcast operands carry stride 0.
constexpr int kMaxOps = 4;
struct IterSpace {
    int ndim = 0;
    int nops = 0;
    int64_t size = 0;
    int64_t shape[RSTSR_MAX_NDIM];
    int64_t stride[kMaxOps][RSTSR_MAX_NDIM];
    int64_t offset[kMaxOps];
};

// Build the collapsed iteration space for same-shape layouts. Operand 0 is the
// one written (its memory order drives the iteration order, the device-side
// counterpart of translate_to_col_major(K) in rearrangement.rs:206-262):
// extent-1 axes are dropped, axes are sorted by operand 0's |stride| (ties by
// the next operands' strides) and neighbours that are contiguous in every
// operand are merged.
IterSpace make_iter_space(const Layout* const* ls, int nops);

// Kernel-side copy of an IterSpace with fast dividers (32-bit index domain).
struct DevDims {
    int ndim;
    uint32_t shape[RSTSR_MAX_NDIM];
    FastDiv div[RSTSR_MAX_NDIM];
};
DevDims make_dev_dims(const IterSpace& sp);

// DevDims holds 32-bit extents: the index decomposition (both the 32-bit and
// the 64-bit form) divides by every extent but the outermost, which is only
// multiplied, so each of those must be below 2^32. Always true below 2^31
// elements; false only for a non-collapsible inner extent of 2^32 or more.
inline bool inner_extents_fit_u32(const IterSpace& sp) {
    for (int i = 0; i + 1 < sp.ndim; ++i)
        if (sp.shape[i] > (int64_t)UINT32_MAX) return false;
    return true;
}

// ---- dtype helpers ----
template <typename T> struct DT;
template <> struct DT<double> { static constexpr rstsr_dtype v = RSTSR_F64; };
template <> struct DT<float> { static constexpr rstsr_dtype v = RSTSR_F32; };
template <> struct DT<__half> { static constexpr rstsr_dtype v = RSTSR_F16; };
template <> struct DT<__nv_bfloat16> { static constexpr rstsr_dtype v = RSTSR_BF16; };
template <> struct DT<int8_t> { static constexpr rstsr_dtype v = RSTSR_I8; };
template <> struct DT<int16_t> { static constexpr rstsr_dtype v = RSTSR_I16; };
template <> struct DT<int32_t> { static constexpr rstsr_dtype v = RSTSR_I32; };
template <> struct DT<int64_t> { static constexpr rstsr_dtype v = RSTSR_I64; };
template <> struct DT<uint8_t> { static constexpr rstsr_dtype v = RSTSR_U8; };
template <> struct DT<uint16_t> { static constexpr rstsr_dtype v = RSTSR_U16; };
template <> struct DT<uint32_t> { static constexpr rstsr_dtype v = RSTSR_U32; };
template <> struct DT<uint64_t> { static constexpr rstsr_dtype v = RSTSR_U64; };

struct Bool8 { uint8_t v; };

// Check that every element of layout l lies inside a buffer of `nelem`
// elements is not possible (the ABI passes no lengths); instead check the
// layout is well-formed: non-negative lower bound and consistent rank.
int check_layout(const rstsr_layout* l, const char* name);

// Every element-aligned base address in the iteration space is `align`-byte
// aligned for operand k when dims 1.. and the offset are multiples.
bool vec_aligned(const IterSpace& sp, int k, const void* base, size_t esize, int vec);

}  // namespace rstsr

// dtype switch helpers: call F<T>() for the runtime dtype.
#define RSTSR_DISPATCH_ALL(t, F, ...)                                  \
    switch (t) {                                                       \
        case RSTSR_F64: return F<double>(__VA_ARGS__);                 \
        case RSTSR_F32: return F<float>(__VA_ARGS__);                  \
        case RSTSR_F16: return F<__half>(__VA_ARGS__);                 \
        case RSTSR_BF16: return F<__nv_bfloat16>(__VA_ARGS__);         \
        case RSTSR_I8: return F<int8_t>(__VA_ARGS__);                  \
        case RSTSR_I16: return F<int16_t>(__VA_ARGS__);                \
        case RSTSR_I32: return F<int32_t>(__VA_ARGS__);                \
        case RSTSR_I64: return F<int64_t>(__VA_ARGS__);                \
        case RSTSR_U8: return F<uint8_t>(__VA_ARGS__);                 \
        case RSTSR_U16: return F<uint16_t>(__VA_ARGS__);               \
        case RSTSR_U32: return F<uint32_t>(__VA_ARGS__);               \
        case RSTSR_U64: return F<uint64_t>(__VA_ARGS__);               \
        case RSTSR_BOOL: return F<uint8_t>(__VA_ARGS__);               \
        default: return ::rstsr::fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype"); \
    }
