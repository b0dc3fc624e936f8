/*
 * rstsr_cuda.h — C ABI of the GB300 (sm_103a) device backend for RSTSR.
 *
 * Every entry point here replaces one method of rstsr-core's device-trait
 * family (the "plugin" boundary a device crate implements) or of
 * rstsr-blas-traits' GEMMDriverAPI. The citation above each declaration names
 * the reference trait method it stands in for (paths are relative to the
 * RESTGroup/rstsr workspace).
 *
 * Conventions
 *  - All calls return an rstsr_status (0 = OK). On error a message is kept in a
 *    thread-local buffer readable through rstsr_cuda_last_error(). Nothing
 *    panics, traps or aborts across the ABI.
 *  - Layouts are rstsr `Layout<IxD>` values: shape, stride and offset counted
 *    in ELEMENTS (not bytes); strides may be negative or zero (broadcast).
 *    A data pointer always points at element 0 of the storage buffer; the
 *    layout's offset selects the first element, exactly as rstsr does with
 *    `(&Raw, &Layout)` pairs.
 *  - Work is stream-ordered on the context's stream and asynchronous, except
 *    calls that return a host value (`*_all`, memcpy_d2h), which synchronise.
 *  - Device memory handed to the kernels must belong to the context's device.
 */
#ifndef RSTSR_CUDA_H
#define RSTSR_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The library is built with hidden visibility; everything declared here is
 * exported. */
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

#define RSTSR_MAX_NDIM 8

/* Error variants of rstsr_common::Error (rstsr-common/src/error.rs:15-48). */
typedef enum {
    RSTSR_OK = 0,
    RSTSR_ERR_INVALID_LAYOUT = 1,    /* RSTSRError::InvalidLayout */
    RSTSR_ERR_INVALID_VALUE = 2,     /* RSTSRError::InvalidValue */
    RSTSR_ERR_VALUE_OUT_OF_RANGE = 3,/* RSTSRError::ValueOutOfRange */
    RSTSR_ERR_DEVICE_MISMATCH = 4,   /* RSTSRError::DeviceMismatch */
    RSTSR_ERR_DEVICE = 5,            /* RSTSRError::DeviceError (CUDA error) */
    RSTSR_ERR_RUNTIME = 6,           /* RSTSRError::RuntimeError */
    RSTSR_ERR_UNIMPLEMENTED = 7,     /* RSTSRError::UnImplemented */
    RSTSR_ERR_TIMEOUT = 8,           /* a bounded device-side wait gave up */
    RSTSR_ERR_INDEX = 9,             /* RSTSRError::IndexError */
    RSTSR_ERR_AXIS = 10              /* RSTSRError::AxisError */
} rstsr_status;

/* Element types (the `T` of DeviceRawAPI<T>). U64 is Rust `usize`. */
typedef enum {
    RSTSR_F64 = 0,
    RSTSR_F32 = 1,
    RSTSR_F16 = 2,
    RSTSR_BF16 = 3,
    RSTSR_I8 = 4,
    RSTSR_I16 = 5,
    RSTSR_I32 = 6,
    RSTSR_I64 = 7,
    RSTSR_U8 = 8,
    RSTSR_U16 = 9,
    RSTSR_U32 = 10,
    RSTSR_U64 = 11,
    RSTSR_BOOL = 12
} rstsr_dtype;

/* FlagOrder (rstsr-common/src/flags.rs:62): RowMajor = C, ColMajor = F. */
typedef enum { RSTSR_ROW_MAJOR = 0, RSTSR_COL_MAJOR = 1 } rstsr_order;

/* Layout<IxD> (rstsr-common/src/layout/layoutbase.rs:15). */
typedef struct {
    int32_t ndim;
    int32_t _reserved;
    int64_t offset;
    int64_t shape[RSTSR_MAX_NDIM];
    int64_t stride[RSTSR_MAX_NDIM];
} rstsr_layout;

typedef struct rstsr_ctx rstsr_ctx;

/* ---------------------------------------------------------------- context */

/* Device construction (the DeviceCpuRayon/DeviceOpenBLAS `new` pattern,
 * rstsr-core/src/feature_rayon/device.rs:41-129): binds a CUDA device, an
 * owned non-blocking stream and a stream-ordered memory pool. The first call
 * in a process loads the GEMM autotune table named by the environment variable
 * RSTSR_CUDA_AUTOTUNE_TABLE (as rstsr_cuda_autotune_load) when it is set; a
 * missing or malformed file makes every context creation fail with that
 * load's error. */
int rstsr_cuda_ctx_create(int32_t device, rstsr_ctx** out);
int rstsr_cuda_ctx_destroy(rstsr_ctx* ctx);
/* Blocks until all work queued on the context's stream is done. The
 * reference's device calls are synchronous, so it has no counterpart; neither
 * have the stream, launch-count and version queries below. */
int rstsr_cuda_ctx_sync(rstsr_ctx* ctx);
/* Replace the stream work is queued on (NULL restores the owned stream). */
int rstsr_cuda_ctx_set_stream(rstsr_ctx* ctx, void* cuda_stream);
/* The cudaStream_t currently in use (for event timing by the caller). */
void* rstsr_cuda_ctx_get_stream(rstsr_ctx* ctx);
int32_t rstsr_cuda_ctx_device(const rstsr_ctx* ctx);
/* Number of kernels this library launched through the context so far. */
uint64_t rstsr_cuda_ctx_launch_count(const rstsr_ctx* ctx);
/* Message of the last failed call on this host thread ("" if none): the text of
 * the rstsr_common::Error the status code stands for (rstsr-common/src/error.rs:15-48). */
const char* rstsr_cuda_last_error(void);
/* Library version string. */
const char* rstsr_cuda_version(void);

/* ------------------------------------------------- host layout algebra */
/* Pure host functions (no GPU needed). They restate the rstsr-common layout
 * rules a device implementation needs so that output layouts match the CPU
 * devices'; the Rust side may call its own rstsr-common functions instead. */

/* broadcast_layout (rstsr-common/src/layout/broadcast.rs:166-245). */
int rstsr_cuda_layout_broadcast(const rstsr_layout* la, const rstsr_layout* lb, rstsr_order order,
                                rstsr_layout* oa, rstsr_layout* ob);
/* get_layout_for_binary_op (rstsr-common/src/layout/rearrangement.rs:394-459):
 * output layout of an element-wise op on two broadcast layouts. */
int rstsr_cuda_layout_binary_op(const rstsr_layout* la, const rstsr_layout* lb, rstsr_order order,
                                rstsr_layout* out);
/* layout_for_array_copy (rearrangement.rs:125-152); order 'C', 'F' or 'K'. */
int rstsr_cuda_layout_for_array_copy(const rstsr_layout* l, char order, rstsr_layout* out);
/* greedy_layout (rearrangement.rs:36-113); perm receives the transpose index. */
int rstsr_cuda_layout_greedy(const rstsr_layout* l, int32_t keep_shape, rstsr_layout* out,
                             int32_t* perm);
/* Contiguity flags of layoutbase.rs:89-205, bit 0 c_contig, 1 f_contig,
 * 2 c_prefer, 3 f_prefer. */
int32_t rstsr_cuda_layout_flags(const rstsr_layout* l);
/* unravel_index_c / unravel_index_f (rstsr-common/src/layout/shape.rs:62-69, tested
 * at layoutbase.rs:988-996): the multi-index of flat position `index` in `shape`,
 * last axis fastest (RSTSR_ROW_MAJOR) or first axis fastest. Turns the raveled
 * indices of rstsr_cuda_argreduce_* into the OpUnraveledArgMaxAPI /
 * OpUnraveledArgMinAPI results (operators/reduction.rs:35-70). */
int rstsr_cuda_unravel_index(const int64_t* shape, int32_t ndim, uint64_t index, rstsr_order order, int64_t* out);

/* ---------------------------------------------------------------- storage */

/* DeviceRawAPI / DeviceStorageAPI / uninit_impl
 * (rstsr-core/src/storage/device.rs:3-159, storage/creation.rs:3-62):
 * stream-ordered allocation from the context's pool. */
int rstsr_cuda_malloc(rstsr_ctx* ctx, size_t nbytes, void** out);
int rstsr_cuda_free(rstsr_ctx* ctx, void* ptr);
/* DeviceChangeAPI host<->device moves (rstsr-core/src/storage/conversion.rs:3-21;
 * to_cpu_vec / from_cpu_vec). d2h synchronises. */
int rstsr_cuda_memcpy_h2d(rstsr_ctx* ctx, void* dst, const void* src, size_t nbytes);
int rstsr_cuda_memcpy_d2h(rstsr_ctx* ctx, void* dst, const void* src, size_t nbytes);
/* Stream-ordered, asynchronous copy between any two addresses the device can
 * reach (device memory or pinned host memory); does not synchronise. */
int rstsr_cuda_memcpy_d2d(rstsr_ctx* ctx, void* dst, const void* src, size_t nbytes);
/* DeviceChangeAPI host<->device moves for any host memory
 * (rstsr-core/src/storage/conversion.rs:3-21; to_cpu_vec at storage/device.rs:33,
 * from_cpu_vec / outof_cpu_vec at storage/creation.rs:11-13, which move an
 * ordinary Vec<T> / &[T]).
 * Page-locked host memory (cudaHostAlloc, cudaHostRegister): one
 * stream-ordered copy; the call returns at once, the host buffer must stay
 * valid and untouched until the stream reaches the copy (rstsr_cuda_ctx_sync
 * or an event).
 * Pageable host memory: chunks of 8 MiB through the context's ring of
 * page-locked staging buffers (created by the first such call, freed with the
 * context), the host copies overlapping the transfers.
 *   h2d_async returns once every byte of src has been read: src may be reused
 *   at once; the device side completes in stream order.
 *   d2h_async returns once every byte has arrived in dst (it waits for the
 *   work queued before it on the context's stream).
 * A staged copy cannot be captured into a graph (RSTSR_ERR_RUNTIME). One
 * staged copy runs at a time per context. */
int rstsr_cuda_memcpy_h2d_async(rstsr_ctx* ctx, void* dst, const void* src, size_t nbytes);
int rstsr_cuda_memcpy_d2h_async(rstsr_ctx* ctx, void* dst, const void* src, size_t nbytes);

/* ------------------------------------------------------------- assignment */

/* OpAssignAPI::assign / assign_uninit (rstsr-core/src/operators/assignment.rs:30-53):
 * same-shape copy c[idx] = cast(a[idx]) for every multi-index idx. */
int rstsr_cuda_assign(rstsr_ctx* ctx, void* c, const rstsr_layout* lc, rstsr_dtype tc,
                      const void* a, const rstsr_layout* la, rstsr_dtype ta);

/* OpAssignArbitaryAPI::assign_arbitary / assign_arbitary_uninit
 * (rstsr-core/src/operators/assignment.rs:5-28): c and a have the same size but
 * possibly different shapes; the i-th element of c in `order` (C for RowMajor,
 * F for ColMajor) receives the i-th element of a in the same order. This is the
 * copy behind to_contig / to_layout / reshape. */
int rstsr_cuda_assign_arbitrary(rstsr_ctx* ctx, void* c, const rstsr_layout* lc, rstsr_dtype tc,
                                const void* a, const rstsr_layout* la, rstsr_dtype ta,
                                rstsr_order order);

/* OpAssignAPI::fill (rstsr-core/src/operators/assignment.rs:44-53). `value`
 * points at one HOST element of type tc. */
int rstsr_cuda_fill(rstsr_ctx* ctx, void* c, const rstsr_layout* lc, rstsr_dtype tc,
                    const void* value);

/* --------------------------------------------------------------- creation */

/* DeviceCreationArangeAPI::arange_impl (rstsr-core/src/storage/creation.rs:51-53;
 * rayon device rstsr-core/src/feature_rayon/auto_impl/creation.rs:74-86).
 * Host-only: the number of elements arange(start, end, step) has for element
 * type t (start, end, step point at one HOST element of type t each): f64 / f32
 * n = ceil((end - start) / step) in f64, i32 / i64 / u32 / u64 the same through
 * isize, each dropping a last element not strictly inside the interval
 * (rstsr-native-impl/src/cpu_rayon/creation.rs:8-55); i8 / i16 / u8 / u16 (and u64
 * values above isize::MAX) count the repeated addition `current < end`
 * (cpu_serial/creation.rs:7-19). A zero step is InvalidValue; ranges the
 * reference's repeated addition never finishes (it wraps, runs away from the
 * end or stops changing) are ValueOutOfRange; f16 / bf16 / bool and a NaN step
 * are UnImplemented. */
int rstsr_cuda_arange_len(rstsr_dtype t, const void* start, const void* end, const void* step, int64_t* n);
/* Writes the n values of that arange to c[0..n): start + i * step (f64 / f32 in
 * f64 with two roundings, integers in 64-bit wrapping arithmetic). */
int rstsr_cuda_arange(rstsr_ctx* ctx, rstsr_dtype t, void* c, int64_t n, const void* start, const void* step);
/* DeviceCreationComplexFloatAPI::linspace_impl (creation.rs:41-49; rayon device
 * rstsr-native-impl/src/cpu_rayon/creation.rs:108-128), f64 / f32: c[i] =
 * start + i * step in the element type, step = (end - start) / (n - 1), or / n
 * with endpoint = 0; c[0] = start when n = 1. */
int rstsr_cuda_linspace(rstsr_ctx* ctx, rstsr_dtype t, void* c, int64_t n, const void* start, const void* end,
                        int32_t endpoint);
/* DeviceCreationTriAPI::tril_impl / triu_impl (creation.rs:55-62;
 * rstsr-native-impl/src/cpu_serial/op_tri.rs:524-591), in place on the last two
 * axes of lc (ndim >= 2): upper = 0 zeroes j >= i + k + 1 (tril), upper = 1
 * zeroes j < i + k (triu, clipped to the row). */
int rstsr_cuda_tril(rstsr_ctx* ctx, rstsr_dtype t, void* c, const rstsr_layout* lc, int64_t k, int32_t upper);

/* ------------------------------------------------------------ elementwise */

/* Binary operators of rstsr-core/src/operators/ops/op_ternary_arithmetic.rs:3-56
 * (OpAdd ... OpShr) and the comparison/maximum/minimum/pow family of
 * operators/ops/op_ternary_common.rs. */
typedef enum {
    RSTSR_OP_ADD = 0,
    RSTSR_OP_SUB = 1,
    RSTSR_OP_MUL = 2,
    RSTSR_OP_DIV = 3,
    RSTSR_OP_REM = 4,
    RSTSR_OP_BITAND = 5,
    RSTSR_OP_BITOR = 6,
    RSTSR_OP_BITXOR = 7,
    RSTSR_OP_SHL = 8,
    RSTSR_OP_SHR = 9,
    RSTSR_OP_MAXIMUM = 10,
    RSTSR_OP_MINIMUM = 11,
    RSTSR_OP_POW = 12,
    /* op_ternary_common.rs:3-19 with the closures of
     * feature_rayon/auto_impl/op_ternary_common.rs:6-80 (floats only unless noted) */
    RSTSR_OP_ATAN2 = 13,        /* a.atan2(b) */
    RSTSR_OP_COPYSIGN = 14,     /* Float::copysign(a, b) */
    RSTSR_OP_HYPOT = 15,        /* a.hypot(b) */
    RSTSR_OP_LOGADDEXP = 16,    /* (a.exp() + b.exp()).ln(), as the reference writes it */
    RSTSR_OP_NEXTAFTER = 17,    /* nextafter(a, b) */
    RSTSR_OP_FLOOR_DIVIDE = 18  /* floats: floor(a / b); integers: floor division (x / 0 = 0 here) */
} rstsr_binary_op;

/* Op*API::op_mutc_refa_refb (op_ternary_arithmetic.rs:3-48; CPU impl
 * rstsr-core/src/feature_rayon/auto_impl/op_ternary_arithmetic.rs:16-56):
 * c = a (op) b. la and lb must already be broadcast to lc's shape (stride 0 on
 * broadcast axes), as the tensor layer does before calling the device. All
 * three tensors share dtype `t`. */
int rstsr_cuda_binary(rstsr_ctx* ctx, rstsr_binary_op op, rstsr_dtype t,
                      void* c, const rstsr_layout* lc,
                      const void* a, const rstsr_layout* la,
                      const void* b, const rstsr_layout* lb);

/* op_mutc_refa_numb / op_mutc_numa_refb (rstsr-core/src/operators/ops/
 * op_ternary_arithmetic.rs:3-48): one operand is a HOST scalar of type
 * t. scalar_is_lhs = 0 computes c = a (op) s, 1 computes c = s (op) a. */
int rstsr_cuda_binary_scalar(rstsr_ctx* ctx, rstsr_binary_op op, rstsr_dtype t,
                             void* c, const rstsr_layout* lc,
                             const void* a, const rstsr_layout* la,
                             const void* scalar, int32_t scalar_is_lhs);

/* In-place forms of rstsr-core/src/operators/ops/op_binary_arithmetic.rs:3-109:
 * OpAddAssignAPI / OpLConsume*API::op_muta_refb (reversed = 0): a = a (op) b;
 * OpRConsume*API (reversed = 1): a = b (op) a. lb is broadcast to la. */
int rstsr_cuda_binary_inplace(rstsr_ctx* ctx, rstsr_binary_op op, rstsr_dtype t,
                              void* a, const rstsr_layout* la,
                              const void* b, const rstsr_layout* lb, int32_t reversed);

/* Unary operators (OpNegAPI / OpNotAPI, op_binary_arithmetic.rs:95-109, and
 * the math family of rstsr-core/src/operators/ops/op_binary_common.rs:3-65). */
typedef enum {
    RSTSR_UOP_NEG = 0,
    RSTSR_UOP_NOT = 1,
    RSTSR_UOP_ABS = 2,
    RSTSR_UOP_SQRT = 3,
    RSTSR_UOP_EXP = 4,
    RSTSR_UOP_LOG = 5,
    RSTSR_UOP_SIN = 6,
    RSTSR_UOP_COS = 7,
    RSTSR_UOP_TANH = 8,
    RSTSR_UOP_SQUARE = 9,
    RSTSR_UOP_FLOOR = 10,
    RSTSR_UOP_CEIL = 11,
    RSTSR_UOP_SIGN = 12,        /* ExtNum::ext_sign: NaN -> NaN, +-0 -> 0, else +-1 */
    RSTSR_UOP_RECIP = 13,
    /* the rest of op_binary_common.rs:3-65 (auto_impl/op_binary_common.rs:10-40):
     * float element types; CONJ, REAL and IMAG on every numeric type */
    RSTSR_UOP_ACOS = 14,
    RSTSR_UOP_ACOSH = 15,
    RSTSR_UOP_ASIN = 16,
    RSTSR_UOP_ASINH = 17,
    RSTSR_UOP_ATAN = 18,
    RSTSR_UOP_ATANH = 19,
    RSTSR_UOP_COSH = 20,
    RSTSR_UOP_EXPM1 = 21,
    RSTSR_UOP_LOG1P = 22,
    RSTSR_UOP_LOG2 = 23,
    RSTSR_UOP_LOG10 = 24,
    RSTSR_UOP_ROUND = 25,       /* half away from zero (Rust round) */
    RSTSR_UOP_SINH = 26,
    RSTSR_UOP_TAN = 27,
    RSTSR_UOP_TRUNC = 28,
    RSTSR_UOP_INV = 29,         /* recip */
    RSTSR_UOP_CONJ = 30,        /* identity on real types */
    RSTSR_UOP_REAL = 31,        /* identity on real types */
    RSTSR_UOP_IMAG = 32         /* zero on real types */
} rstsr_unary_op;

/* c = op(a) (op_mutc_refa family); a in place when c == a with equal layouts. */
int rstsr_cuda_unary(rstsr_ctx* ctx, rstsr_unary_op op, rstsr_dtype t,
                     void* c, const rstsr_layout* lc, const void* a, const rstsr_layout* la);

/* Boolean-valued unary operators (auto_impl/op_binary_common.rs:94-120):
 * IsFinite / IsInf / IsNan on float types; SignBit writes the reference's
 * `is_positive()` (floats: sign bit clear, so +0, +inf and +NaN give true;
 * signed integers: x > 0). c is BOOL. */
typedef enum {
    RSTSR_PRED_ISFINITE = 0,
    RSTSR_PRED_ISINF = 1,
    RSTSR_PRED_ISNAN = 2,
    RSTSR_PRED_SIGNBIT = 3
} rstsr_predicate_op;
int rstsr_cuda_unary_predicate(rstsr_ctx* ctx, rstsr_predicate_op op, rstsr_dtype ta, void* c,
                               const rstsr_layout* lc, const void* a, const rstsr_layout* la);

/* Comparisons (OpEqualAPI ... OpLessEqualAPI, op_ternary_common.rs:3-19):
 * c (BOOL) = a (op) b with PartialEq / PartialOrd (any comparison with NaN is
 * false, != is true). la and lb are broadcast to lc. */
typedef enum {
    RSTSR_CMP_EQ = 0,
    RSTSR_CMP_NE = 1,
    RSTSR_CMP_GT = 2,
    RSTSR_CMP_GE = 3,
    RSTSR_CMP_LT = 4,
    RSTSR_CMP_LE = 5
} rstsr_compare_op;
int rstsr_cuda_compare(rstsr_ctx* ctx, rstsr_compare_op op, rstsr_dtype t, void* c, const rstsr_layout* lc,
                       const void* a, const rstsr_layout* la, const void* b, const rstsr_layout* lb);
/* One operand a HOST scalar of type t (op_mutc_refa_numb / op_mutc_numa_refb of
 * op_ternary_common.rs; scalar_is_lhs as in rstsr_cuda_binary_scalar). */
int rstsr_cuda_compare_scalar(rstsr_ctx* ctx, rstsr_compare_op op, rstsr_dtype t, void* c,
                              const rstsr_layout* lc, const void* a, const rstsr_layout* la,
                              const void* scalar, int32_t scalar_is_lhs);

/* OpIsCloseAPI (op_ternary_common.rs:65-100; rstsr-dtype-traits/src/isclose.rs:92-105):
 * c (BOOL) = |a - b| <= atol + rtol |b| (the difference in the operands' type,
 * the test in f64) or (equal_nan and both NaN). */
int rstsr_cuda_isclose(rstsr_ctx* ctx, rstsr_dtype t, void* c, const rstsr_layout* lc,
                       const void* a, const rstsr_layout* la, const void* b, const rstsr_layout* lb,
                       double rtol, double atol, int32_t equal_nan);
/* OpAllCloseAPI::allclose_all (rstsr-core/src/operators/reduction.rs:73-85; rayon
 * device rstsr-core/src/feature_rayon/auto_impl/reduction.rs:717-749): every
 * element of a and b (same shape) isclose; the bool is written to HOST memory at
 * out_host (synchronises). A zero-size operand is InvalidValue, as in the
 * reference. */
int rstsr_cuda_allclose_all(rstsr_ctx* ctx, rstsr_dtype t, const void* a, const rstsr_layout* la, const void* b,
                            const rstsr_layout* lb, double rtol, double atol, int32_t equal_nan, uint8_t* out_host);

/* Fused d = a * b + c (one pass). The reference evaluates `&a * &b + &c` as
 * OpMulAPI::op_mutc_refa_refb (tensor/operators/op_binary_arithmetic.rs:170-213)
 * followed by OpLConsumeAddAPI::op_muta_refb (:261-305); this entry point
 * produces the same values in the same output layout in a single pass.
 * la, lb, lc are broadcast to ld's shape. */
int rstsr_cuda_fma(rstsr_ctx* ctx, rstsr_dtype t, void* d, const rstsr_layout* ld,
                   const void* a, const rstsr_layout* la,
                   const void* b, const rstsr_layout* lb,
                   const void* c, const rstsr_layout* lc);

/* ------------------------------------------------------------- reductions */

/* Reductions of rstsr-core/src/operators/reduction.rs:3-33 with the
 * init/f/f_sum/f_out algebra of rstsr-core/src/feature_rayon/auto_impl/reduction.rs. */
typedef enum {
    RSTSR_RED_SUM = 0,          /* OpSumAPI            (auto_impl/reduction.rs:7)   */
    RSTSR_RED_MEAN = 1,         /* OpMeanAPI           (:167)                       */
    RSTSR_RED_VAR = 2,          /* OpVarAPI            (:207) one-pass E[x^2]-E[x]^2*/
    RSTSR_RED_STD = 3,          /* OpStdAPI            (:267)                       */
    RSTSR_RED_MIN = 4,          /* OpMinAPI            (:43)  init = T::MAX         */
    RSTSR_RED_MAX = 5,          /* OpMaxAPI            (:87)  init = T::MIN         */
    RSTSR_RED_PROD = 6,         /* OpProdAPI                                        */
    RSTSR_RED_L2NORM = 7,       /* OpL2NormAPI         (:327)                       */
    RSTSR_RED_ALL = 8,          /* OpAllAPI  (bool)    (:466)                       */
    RSTSR_RED_ANY = 9,          /* OpAnyAPI  (bool)    (:494)                       */
    RSTSR_RED_COUNT_NONZERO = 10/* OpCountNonZeroAPI   (:522) -> usize              */
} rstsr_reduce_op;

/* Output dtype of a reduction over input dtype ta (T, T::Real, bool or usize). */
int rstsr_cuda_reduce_out_dtype(rstsr_reduce_op op, rstsr_dtype ta, rstsr_dtype* tout);

/* Op*API::*_all (rstsr-core/src/operators/reduction.rs:3-33; rayon device
 * feature_rayon/auto_impl/reduction.rs:7-716): reduce every element; the scalar is written to HOST memory at
 * out_host (one element of the output dtype). Synchronises. Zero-size input
 * is an InvalidValue error for min/max, as in the reference. */
int rstsr_cuda_reduce_all(rstsr_ctx* ctx, rstsr_reduce_op op, rstsr_dtype ta,
                          const void* a, const rstsr_layout* la, void* out_host);

/* Output layout the device picks for *_axes: layout_for_array_copy(lm, K) of
 * the kept axes (rstsr-native-impl/src/cpu_serial/reduction.rs:210-215,
 * rstsr-common/src/layout/rearrangement.rs:125-152). Pure host function. */
int rstsr_cuda_reduce_axes_layout(const rstsr_layout* la, const int64_t* axes, int32_t naxes,
                                  rstsr_layout* lout);

/* Op*API::*_axes (rstsr-core/src/operators/reduction.rs:27-31): the DEVICE
 * allocates the output (from the context pool) and returns it with its layout,
 * as the reference returns (Storage, Layout<IxD>). Free *out with
 * rstsr_cuda_free. */
int rstsr_cuda_reduce_axes(rstsr_ctx* ctx, rstsr_reduce_op op, rstsr_dtype ta,
                           const void* a, const rstsr_layout* la,
                           const int64_t* axes, int32_t naxes,
                           void** out, rstsr_layout* lout);

/* Same reduction into caller-provided storage (no reference counterpart: the
 * reference's *_axes always allocate): lout must have the kept-axes
 * shape (any strides). */
int rstsr_cuda_reduce_axes_into(rstsr_ctx* ctx, rstsr_reduce_op op, rstsr_dtype ta,
                                const void* a, const rstsr_layout* la,
                                const int64_t* axes, int32_t naxes,
                                void* out, const rstsr_layout* lout);

/* OpArgMaxAPI / OpArgMinAPI::arg*_all (auto_impl/reduction.rs:356-464):
 * the C-order (row-major) flat index of the first extreme element; ties keep
 * the smaller index. Writes one uint64 (usize) to HOST memory. Zero-size input
 * is an InvalidLayout error. */
int rstsr_cuda_argreduce_all(rstsr_ctx* ctx, int32_t is_max, rstsr_dtype ta,
                             const void* a, const rstsr_layout* la, uint64_t* out_host);

/* OpArgMaxAPI / OpArgMinAPI::arg*_axes (feature_rayon/auto_impl/reduction.rs:356-464,
 * rstsr-native-impl/src/cpu_serial/reduction.rs:425-580): per kept element, the C-order index within the reduced-axes shape
 * (axes in the order given) of the first extreme element. Output dtype U64. */
int rstsr_cuda_argreduce_axes(rstsr_ctx* ctx, int32_t is_max, rstsr_dtype ta,
                              const void* a, const rstsr_layout* la,
                              const int64_t* axes, int32_t naxes,
                              void** out, rstsr_layout* lout);
int rstsr_cuda_argreduce_axes_into(rstsr_ctx* ctx, int32_t is_max, rstsr_dtype ta,
                                   const void* a, const rstsr_layout* la,
                                   const int64_t* axes, int32_t naxes,
                                   void* out, const rstsr_layout* lout);

/* Allocation-free sum over axes. No counterpart in the reference: it exists
 * for callers that must not have the library allocate device memory -- a
 * host that hands out all GPU memory from its own arena, a latency-critical
 * loop that cannot afford the synchronisation of cudaMalloc/cudaFree, or a
 * plugin host that forbids allocations outside its own allocator. It takes a
 * CUDA stream instead of a context (creating a context allocates) and the
 * caller provides input and output, the output laid out over the kept axes
 * (any strides). The split reduction's partial sums live in one fixed static
 * device array of RSTSR_NOALLOC_SCRATCH_BYTES that every GPU loading this
 * library holds until the process exits; a reduction whose default split
 * would need more scratch runs with fewer chunks of the reduced range (down
 * to one unsplit pass, which needs none), so no valid input is rejected for
 * its size. The stream must belong to the current device
 * (RSTSR_ERR_DEVICE_MISMATCH otherwise). The first call on a device looks up
 * that array's device address (cudaGetSymbolAddress), so make the first call
 * on each device before any stream capture. All calls share the array: calls
 * that can overlap on the GPU (different streams, or different host threads)
 * race on it and must be serialised by the caller. Supported dtypes: f64,
 * f32, i32, i64. Never calls cudaMalloc or cudaFree. */
#define RSTSR_NOALLOC_SCRATCH_BYTES (1u << 20)
int rstsr_cuda_sum_axes_noalloc(void* cuda_stream, rstsr_dtype ta, const void* a, const rstsr_layout* la,
                                const int64_t* axes, int32_t naxes, void* out, const rstsr_layout* lout);

/* ---------------------------------------------- triangles and indexing */

/* FlagSymm (rstsr-common/src/flags.rs:220-240). For the real element types
 * of this library He behaves as Sy and Ah as Ay. */
typedef enum {
    RSTSR_SYMM_SY = 0,  /* symmetric: mirror = value */
    RSTSR_SYMM_HE = 1,  /* Hermitian: mirror = conj(value) */
    RSTSR_SYMM_AY = 2,  /* anti-symmetric: mirror = -value, diagonal 0 */
    RSTSR_SYMM_AH = 3,  /* anti-Hermitian: mirror = -conj(value), diagonal 0 */
    RSTSR_SYMM_N = 4    /* no symmetry: only the packed triangle is written */
} rstsr_symm;

/* OpPackTriAPI::pack_tri (rstsr-core/src/operators/ops/op_tri.rs:3-15; CPU
 * impl rstsr-native-impl/src/cpu_serial/op_tri.rs:73-144): a (.., n(n+1)/2)
 * receives the uplo ('L' | 'U') triangle of b (.., n, n), rows packed in
 * order (for RowMajor; ColMajor reverses all axes and flips uplo first,
 * feature_rayon/auto_impl/op_tri.rs:7-30). Any dtype. */
int rstsr_cuda_pack_tri(rstsr_ctx* ctx, rstsr_dtype t, void* a, const rstsr_layout* la,
                        const void* b, const rstsr_layout* lb, char uplo, rstsr_order order);

/* OpUnpackTriAPI::unpack_tri (op_tri.rs:17-30; cpu_serial/op_tri.rs:148-410):
 * a (.., n, n) from the packed triangle b (.., n(n+1)/2) and its mirror by
 * symm. With RSTSR_SYMM_N the other triangle of a is left as it was (the
 * reference leaves it uninitialised). Float dtypes (F64, F32, F16, BF16), as
 * the reference's `T: ComplexFloat`. */
int rstsr_cuda_unpack_tri(rstsr_ctx* ctx, rstsr_dtype t, void* a, const rstsr_layout* la,
                          const void* b, const rstsr_layout* lb, char uplo, rstsr_symm symm,
                          rstsr_order order);

/* DeviceIndexSelectAPI::index_select (rstsr-core/src/operators/adv_indexing.rs:8-23;
 * CPU impl rstsr-native-impl/src/cpu_serial/adv_indexing.rs:3-69):
 * c[.., k, ..] = a[.., indices[k], ..] along `axis`. `indices` is HOST memory
 * (the reference's &[usize]); each must be below a's extent on the axis
 * (RSTSR_ERR_INDEX otherwise); lc's extent on the axis is nindices and its
 * other extents equal la's. Any dtype. At most 512 indices inside a graph
 * capture (they are baked into the captured launch). */
int rstsr_cuda_index_select(rstsr_ctx* ctx, rstsr_dtype t, void* c, const rstsr_layout* lc,
                            const void* a, const rstsr_layout* la, int32_t axis,
                            const uint64_t* indices, int64_t nindices);

/* ---------------------------------------------------------------- matmul */

/* How a floating-point GEMM is evaluated on the tensor cores. */
typedef enum {
    RSTSR_PREC_AUTO = 0,    /* f64 -> OZAKI, f32 -> BF16X3 (6-product split), others native */
    RSTSR_PREC_NATIVE = 1,  /* CUDA-core FMA in the operand type (reference for checking) */
    RSTSR_PREC_OZAKI = 2,   /* f64: error-free split into integer slices on the tensor cores */
    RSTSR_PREC_BF16X3 = 3   /* f32: three-term bf16 split, FP32 accumulate */
} rstsr_precision;

/* Tuning knobs shared by the GEMM entry points. Zero-initialise for defaults. */
typedef struct {
    int32_t precision;      /* rstsr_precision */
    int32_t ozaki_slices;   /* 0 = choose from the operands' exponent spread (8 for calls of
                               at most 2^30 multiply-adds, without measuring it) */
    int32_t reserved[6];
} rstsr_gemm_opts;

/* GEMMDriverAPI::driver_gemm (rstsr-blas-traits/src/blas3/gemm.rs:4-21):
 * BLAS-style GEMM by raw (device) pointers. order = RowMajor/ColMajor as in
 * CBLAS; trans* = 'N' | 'T' | 'C' (C == T for real types).
 * c = alpha * op(a) op(b) + beta * c. dtype is F64 or F32. */
int rstsr_cuda_gemm(rstsr_ctx* ctx, rstsr_order order, char transa, char transb,
                    int64_t m, int64_t n, int64_t k, double alpha,
                    const void* a, int64_t lda, const void* b, int64_t ldb,
                    double beta, void* c, int64_t ldc, rstsr_dtype t,
                    const rstsr_gemm_opts* opts);

/* DeviceMatMulAPI::matmul (rstsr-core/src/operators/matmul.rs:7-25; CPU impl
 * rstsr-core/src/device_faer/matmul.rs:83-239): c = alpha * a @ b + beta * c
 * under the matmul broadcasting rules 1-7 of rstsr-common/src/layout/matmul.rs
 * for the given order. Batched (broadcast) products run as one grouped launch.
 * When b is the transpose view of a's own buffer and beta == 0 the SYRK
 * shortcut of device_faer/matmul.rs:38-48 is taken (lower triangle computed,
 * then mirrored). */
int rstsr_cuda_matmul(rstsr_ctx* ctx, rstsr_dtype t,
                      void* c, const rstsr_layout* lc,
                      const void* a, const rstsr_layout* la,
                      const void* b, const rstsr_layout* lb,
                      double alpha, double beta, rstsr_order order,
                      const rstsr_gemm_opts* opts);

/* Output layout of matmul for the given operand layouts and order
 * (LayoutMatMulConfig::layout_matmul, rstsr-common/src/layout/matmul.rs:70-460). */
int rstsr_cuda_matmul_layout(const rstsr_layout* la, const rstsr_layout* lb,
                             rstsr_order order, rstsr_layout* lc);

/* One problem of a grouped GEMM: row-major, c[m,n] = alpha a[m,k] b[k,n] + beta c. */
typedef struct {
    int64_t m, n, k;
    int64_t lda, ldb, ldc;
    const void* a;
    const void* b;
    void* c;
    double alpha, beta;
} rstsr_gemm_problem;

/* Uneven grouped GEMM in one persistent launch (the batched `rest` loop of
 * device_faer/matmul.rs:151-199 as one grid). `problems` is HOST memory. */
int rstsr_cuda_gemm_grouped(rstsr_ctx* ctx, rstsr_dtype t, const rstsr_gemm_problem* problems,
                            int32_t nproblems, const rstsr_gemm_opts* opts);

/* Ozaki split statistics of the last f64 GEMM on this thread: slices used (no
 * reference counterpart). */
int32_t rstsr_cuda_last_ozaki_slices(void);

/* ------------------------------------------------------ contractions */

/* einsum (crates-plugin/rstsr-tblis/src/einsum_impl.rs:146-199, there through
 * TBLIS): out = the contraction `subscripts` ("ij,jk->ik"; labels are any
 * Unicode characters, whitespace ignored, "->" optional with numpy's implicit
 * output) of the nops operands. Every pairwise contraction runs as one
 * batched matmul (Ozaki split for F64, bf16 split for F32 unless opts says
 * otherwise); diagonals are views, single-operand sums use the reduction
 * kernels. Dtypes F64, F32, I32, I64. lout has the output labels' extents,
 * any strides. Ellipsis is not supported (RSTSR_ERR_UNIMPLEMENTED). */
int rstsr_cuda_einsum(rstsr_ctx* ctx, rstsr_dtype t, const char* subscripts, int32_t nops,
                      const void* const* ops, const rstsr_layout* lops, void* out,
                      const rstsr_layout* lout, const rstsr_gemm_opts* opts);
/* Output extents of an einsum (host only; the output labels and extents of
 * crates-plugin/rstsr-tblis/src/einsum_impl.rs:146-199). shape_out holds RSTSR_MAX_NDIM. */
int rstsr_cuda_einsum_output_shape(const char* subscripts, int32_t nops, const rstsr_layout* lops,
                                   int32_t* ndim_out, int64_t* shape_out);

/* tensordot (crates-plugin/rstsr-tblis/src/tensordot_impl.rs:33-70 with the
 * labels of rstsr-common/src/tensordot_to_einsum.rs:18-112): c's axes are a's
 * remaining axes then b's; axes_a[q] of a contracts with axes_b[q] of b
 * (negative axes count from the end). */
int rstsr_cuda_tensordot(rstsr_ctx* ctx, rstsr_dtype t, void* c, const rstsr_layout* lc,
                         const void* a, const rstsr_layout* la, const void* b, const rstsr_layout* lb,
                         const int64_t* axes_a, const int64_t* axes_b, int32_t naxes,
                         const rstsr_gemm_opts* opts);

/* DeviceVecdotAPI::vecdot (rstsr-core/src/operators/linalg.rs:3-20; CPU impl
 * rstsr-native-impl/src/cpu_serial/vecdot.rs): c[m] = sum over the contracted
 * axes of a[m, s] * b[m, s], the remaining parts of a and b broadcast to c
 * (for `order`). Real types (no conjugation needed). */
int rstsr_cuda_vecdot(rstsr_ctx* ctx, rstsr_dtype t, void* c, const rstsr_layout* lc,
                      const void* a, const rstsr_layout* la, const void* b, const rstsr_layout* lb,
                      const int64_t* axes_a, const int64_t* axes_b, int32_t naxes, rstsr_order order);

/* BLAS-3 drivers beyond GEMM (CBLAS conventions; F64 or F32; alpha / beta as
 * doubles; opts as for rstsr_cuda_gemm). */

/* SYRK (DeviceSYRKAPI::syrk, rstsr-core/src/operators/matmul.rs:64-78): the
 * uplo ('L' | 'U') triangle of C (n x n) = alpha op(A) op(A)^T + beta C, op(A)
 * = A (trans 'N', A n x k) or A^T ('T', A k x n); the other triangle of C is not
 * touched, and C is not read when beta = 0. */
int rstsr_cuda_syrk(rstsr_ctx* ctx, rstsr_order order, char uplo, char trans, int64_t n, int64_t k,
                    double alpha, const void* a, int64_t lda, double beta, void* c, int64_t ldc,
                    rstsr_dtype t, const rstsr_gemm_opts* opts);

/* SYMM (driver_syhemm, rstsr-blas-traits/src/blas3/syhemm.rs:5-19): C (m x n) =
 * alpha A B + beta C (side 'L', A m x m) or alpha B A + beta C ('R', A n x n),
 * A symmetric and read from its uplo triangle only. */
int rstsr_cuda_symm(rstsr_ctx* ctx, rstsr_order order, char side, char uplo, int64_t m, int64_t n,
                    double alpha, const void* a, int64_t lda, const void* b, int64_t ldb, double beta,
                    void* c, int64_t ldc, rstsr_dtype t, const rstsr_gemm_opts* opts);

/* TRSM (driver_trsm, rstsr-blas-traits/src/blas3/trsm.rs:5-18): B (m x n) :=
 * alpha op(A)^-1 B (side 'L', A m x m) or alpha B op(A)^-1 ('R', A n x n), A
 * triangular in its uplo triangle, diag 'U' (unit, not read) or 'N'. */
int rstsr_cuda_trsm(rstsr_ctx* ctx, rstsr_order order, char side, char uplo, char transa, char diag,
                    int64_t m, int64_t n, double alpha, const void* a, int64_t lda, void* b, int64_t ldb,
                    rstsr_dtype t, const rstsr_gemm_opts* opts);

/* ---------------------------------------------------------------- graphs */

/* Capture every call made on the context between begin and end into a CUDA
 * graph, then replay it with one launch (no reference counterpart). */
typedef struct rstsr_graph rstsr_graph;
int rstsr_cuda_graph_begin(rstsr_ctx* ctx);
int rstsr_cuda_graph_end(rstsr_ctx* ctx, rstsr_graph** out);
int rstsr_cuda_graph_launch(rstsr_ctx* ctx, rstsr_graph* g);
int rstsr_cuda_graph_destroy(rstsr_graph* g);

/* --------------------------------------------------------------- autotune */

/* Time the GEMM tile configurations for one problem shape and remember the
 * fastest for that (m, n, k, dtype, precision) class. The table can be saved
 * and loaded as text (no reference counterpart: rstsr's CPU GEMMs take their
 * blocking from faer or the BLAS library). */
int rstsr_cuda_autotune_gemm(rstsr_ctx* ctx, rstsr_dtype t, int64_t m, int64_t n, int64_t k,
                             const rstsr_gemm_opts* opts, int32_t* best_config);
int rstsr_cuda_autotune_save(const char* path);
int rstsr_cuda_autotune_load(const char* path);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif

#endif /* RSTSR_CUDA_H */
