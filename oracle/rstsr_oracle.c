/*
 * rstsr_oracle.c -- CPU restatement of the reference's hot-path semantics.
 *
 * TEST INFRASTRUCTURE ONLY. This file gives the results the CUDA backend is
 * compared with and the timed CPU baseline of the benchmark; the product never links or calls
 * it. It restates, in plain C over explicit (shape, stride, offset) layouts:
 *
 *   assign            rstsr-native-impl/src/cpu_serial/assignment.rs:95-153
 *   assign_arbitrary  rstsr-native-impl/src/cpu_serial/assignment.rs:28-67
 *   binary / fma      rstsr-native-impl/src/cpu_serial/op_with_func.rs:10-199
 *                     with the closures of rstsr-core/src/feature_rayon/
 *                     auto_impl/op_ternary_arithmetic.rs:16-56
 *   reduce_axes       rstsr-native-impl/src/cpu_serial/reduction.rs:180-368
 *                     (unrolled_reduce :44-83 with its 8 accumulators) and the
 *                     init/f/f_sum/f_out of auto_impl/reduction.rs:7-716
 *   argreduce_axes    rstsr-native-impl/src/cpu_serial/reduction.rs:425-580
 *                     (row-major fold, ties keep the smaller index)
 *   pack_tri          rstsr-native-impl/src/cpu_serial/op_tri.rs:26-71
 *                     (inner_pack_tri{l,u}_general, row loop i, column j)
 *   unpack_tri        rstsr-native-impl/src/cpu_serial/op_tri.rs:217-410
 *                     (inner_unpack_tri{l,u}_general for Sy/He/Ay/Ah/N)
 *   index_select      rstsr-native-impl/src/cpu_serial/adv_indexing.rs:3-69
 *   einsum            the definition of an Einstein summation (the reference
 *                     calls TBLIS 0.2 through crates-plugin/rstsr-tblis/src/
 *                     einsum_impl.rs:146-199): every output element is the
 *                     sum, over all values of the labels not in the output,
 *                     of the product of the operands' elements; f64 with
 *                     Neumaier-compensated sums, i64 with wrapping arithmetic
 *
 * Every function takes `nthreads`: 1 runs the serial semantics; more threads
 * run the same per-output / per-row algorithm split across OpenMP threads the
 * way the rstsr-native-impl/src/cpu_rayon modules split it across rayon workers
 * (outer offsets of contiguous runs for element-wise work, output elements or
 * output chunks for reductions). Results of exact (integer, copy, arg) work
 * do not depend on the thread count; float sums regroup like rayon's.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXD 8

typedef struct {
    int32_t ndim;
    int32_t reserved;
    int64_t offset;
    int64_t shape[MAXD];
    int64_t stride[MAXD];
} olayout;

enum { T_F64 = 0, T_F32 = 1, T_I32 = 6, T_I64 = 7, T_U64 = 11, T_BOOL = 12 };
enum { OP_ADD = 0, OP_SUB = 1, OP_MUL = 2, OP_DIV = 3 };
enum {
    R_SUM = 0, R_MEAN = 1, R_VAR = 2, R_STD = 3, R_MIN = 4, R_MAX = 5, R_PROD = 6, R_L2 = 7,
    R_ALL = 8, R_ANY = 9, R_COUNT = 10
};

static int64_t lsize(const olayout* l) {
    int64_t s = 1;
    for (int i = 0; i < l->ndim; ++i) s *= l->shape[i];
    return s;
}

/* ----------------------------------------------------------- iteration */

/* A collapsed iteration space over up to 4 same-shape operands: dims sorted
 * inner-first by operand 0's |stride| (the K order of
 * rstsr-common/src/layout/rearrangement.rs:206-262 for the written operand),
 * neighbours merged where contiguous in every operand
 * (translate_to_col_major_with_contig, rearrangement.rs:297-322). */
typedef struct {
    int nd, nops;
    int64_t size;
    int64_t shape[MAXD];
    int64_t stride[4][MAXD];
    int64_t offset[4];
} ospace;

static void make_space(const olayout* const* ls, int nops, ospace* sp) {
    const olayout* l0 = ls[0];
    int axes[MAXD], na = 0;
    sp->nops = nops;
    sp->size = lsize(l0);
    for (int k = 0; k < nops; ++k) sp->offset[k] = ls[k]->offset;
    for (int i = 0; i < l0->ndim; ++i)
        if (l0->shape[i] != 1) axes[na++] = i;
    /* stable insertion sort by |stride| of operand 0, then 1, ... */
    for (int i = 1; i < na; ++i) {
        int x = axes[i], j = i - 1;
        while (j >= 0) {
            int y = axes[j], less = 0, decided = 0;
            for (int k = 0; k < nops && !decided; ++k) {
                int64_t sx = llabs(ls[k]->stride[x]), sy = llabs(ls[k]->stride[y]);
                if (sx != sy) {
                    less = sx < sy;
                    decided = 1;
                }
            }
            if (!less) break;
            axes[j + 1] = axes[j];
            --j;
        }
        axes[j + 1] = x;
    }
    int nd = 0;
    for (int t = 0; t < na; ++t) {
        int a = axes[t], merge = nd > 0;
        for (int k = 0; merge && k < nops; ++k)
            if (ls[k]->stride[a] != sp->stride[k][nd - 1] * sp->shape[nd - 1]) merge = 0;
        if (merge) {
            sp->shape[nd - 1] *= l0->shape[a];
        } else {
            sp->shape[nd] = l0->shape[a];
            for (int k = 0; k < nops; ++k) sp->stride[k][nd] = ls[k]->stride[a];
            nd++;
        }
    }
    if (nd == 0) {
        sp->shape[0] = 1;
        for (int k = 0; k < nops; ++k) sp->stride[k][0] = 0;
        nd = 1;
    }
    sp->nd = nd;
}

/* offsets of outer index q (dims 1..nd-1, inner-first) */
static void outer_offsets(const ospace* sp, int64_t q, int64_t* off) {
    for (int k = 0; k < sp->nops; ++k) off[k] = sp->offset[k];
    for (int d = 1; d < sp->nd; ++d) {
        int64_t i = q % sp->shape[d];
        q /= sp->shape[d];
        for (int k = 0; k < sp->nops; ++k) off[k] += i * sp->stride[k][d];
    }
}

static int64_t outer_count(const ospace* sp) {
    int64_t n = 1;
    for (int d = 1; d < sp->nd; ++d) n *= sp->shape[d];
    return n;
}

static void set_threads(int nthreads) {
#ifdef _OPENMP
    omp_set_num_threads(nthreads > 0 ? nthreads : 1);
#else
    (void)nthreads;
#endif
}

/* ----------------------------------------------------------- assign */

int oracle_assign(void* c, const olayout* lc, const void* a, const olayout* la, int esize, int nthreads) {
    const olayout* ls[2] = {lc, la};
    ospace sp;
    if (lsize(lc) == 0) return 0;
    make_space(ls, 2, &sp);
    const int64_t nq = outer_count(&sp), n0 = sp.shape[0];
    const int64_t s0c = sp.stride[0][0], s0a = sp.stride[1][0];
    set_threads(nthreads);
#pragma omp parallel for schedule(static) if (nthreads > 1)
    for (int64_t q = 0; q < nq; ++q) {
        int64_t off[4];
        outer_offsets(&sp, q, off);
        char* pc = (char*)c;
        const char* pa = (const char*)a;
        if (s0c == 1 && s0a == 1) {
            memcpy(pc + off[0] * esize, pa + off[1] * esize, (size_t)(n0 * esize));
        } else {
            for (int64_t i = 0; i < n0; ++i)
                memcpy(pc + (off[0] + i * s0c) * esize, pa + (off[1] + i * s0a) * esize, (size_t)esize);
        }
    }
    return 0;
}

/* Walk both layouts in logical C (order 0) or F (order 1) order; the i-th
 * elements correspond (cpu_serial/assignment.rs:28-67). */
static void unravel_offset(const olayout* l, int64_t e, int order, int64_t* off) {
    int64_t o = l->offset;
    if (order == 0) {
        for (int d = l->ndim - 1; d >= 0; --d) {
            int64_t i = e % l->shape[d];
            e /= l->shape[d];
            o += i * l->stride[d];
        }
    } else {
        for (int d = 0; d < l->ndim; ++d) {
            int64_t i = e % l->shape[d];
            e /= l->shape[d];
            o += i * l->stride[d];
        }
    }
    *off = o;
}

int oracle_assign_arbitrary(void* c, const olayout* lc, const void* a, const olayout* la, int esize, int order,
                            int nthreads) {
    const int64_t n = lsize(lc);
    if (n != lsize(la)) return 1;
    set_threads(nthreads);
#pragma omp parallel for schedule(static) if (nthreads > 1)
    for (int64_t e = 0; e < n; ++e) {
        int64_t oc, oa;
        unravel_offset(lc, e, order, &oc);
        unravel_offset(la, e, order, &oa);
        memcpy((char*)c + oc * esize, (const char*)a + oa * esize, (size_t)esize);
    }
    return 0;
}

/* ----------------------------------------------------------- binary */

#define BIN_LOOP(T, EXPR)                                                              \
    do {                                                                               \
        T* pc = (T*)c;                                                                 \
        const T* pa = (const T*)a;                                                     \
        const T* pb = (const T*)b;                                                     \
        _Pragma("omp parallel for schedule(static) if (nthreads > 1)")                 \
        for (int64_t q = 0; q < nq; ++q) {                                             \
            int64_t off[4];                                                            \
            outer_offsets(&sp, q, off);                                                \
            for (int64_t i = 0; i < n0; ++i) {                                         \
                T x = pa[off[1] + i * sp.stride[1][0]];                                \
                T y = pb[off[2] + i * sp.stride[2][0]];                                \
                pc[off[0] + i * sp.stride[0][0]] = (EXPR);                             \
            }                                                                          \
        }                                                                              \
    } while (0)

/* wrapping integer arithmetic through unsigned types */
#define WADD(T, U, x, y) ((T)((U)(x) + (U)(y)))
#define WSUB(T, U, x, y) ((T)((U)(x) - (U)(y)))
#define WMUL(T, U, x, y) ((T)((U)(x) * (U)(y)))

int oracle_binary(int op, int dtype, void* c, const olayout* lc, const void* a, const olayout* la, const void* b,
                  const olayout* lb, int nthreads) {
    const olayout* ls[3] = {lc, la, lb};
    ospace sp;
    if (lsize(lc) == 0) return 0;
    make_space(ls, 3, &sp);
    const int64_t nq = outer_count(&sp), n0 = sp.shape[0];
    set_threads(nthreads);
    switch (dtype) {
        case T_F64:
            if (op == OP_ADD) BIN_LOOP(double, x + y);
            else if (op == OP_SUB) BIN_LOOP(double, x - y);
            else if (op == OP_MUL) BIN_LOOP(double, x * y);
            else if (op == OP_DIV) BIN_LOOP(double, x / y);
            else return 2;
            return 0;
        case T_F32:
            if (op == OP_ADD) BIN_LOOP(float, x + y);
            else if (op == OP_SUB) BIN_LOOP(float, x - y);
            else if (op == OP_MUL) BIN_LOOP(float, x * y);
            else if (op == OP_DIV) BIN_LOOP(float, x / y);
            else return 2;
            return 0;
        case T_I32:
            if (op == OP_ADD) BIN_LOOP(int32_t, WADD(int32_t, uint32_t, x, y));
            else if (op == OP_SUB) BIN_LOOP(int32_t, WSUB(int32_t, uint32_t, x, y));
            else if (op == OP_MUL) BIN_LOOP(int32_t, WMUL(int32_t, uint32_t, x, y));
            else if (op == OP_DIV) BIN_LOOP(int32_t, y == 0 ? 0 : (y == -1 ? WSUB(int32_t, uint32_t, 0, x) : x / y));
            else return 2;
            return 0;
        case T_I64:
            if (op == OP_ADD) BIN_LOOP(int64_t, WADD(int64_t, uint64_t, x, y));
            else if (op == OP_SUB) BIN_LOOP(int64_t, WSUB(int64_t, uint64_t, x, y));
            else if (op == OP_MUL) BIN_LOOP(int64_t, WMUL(int64_t, uint64_t, x, y));
            else if (op == OP_DIV) BIN_LOOP(int64_t, y == 0 ? 0 : (y == -1 ? WSUB(int64_t, uint64_t, 0, x) : x / y));
            else return 2;
            return 0;
        default:
            return 2;
    }
}

/* d = a * b + c, the reference's two passes: tmp = a * b (rounded), then
 * tmp + c (rounded). volatile keeps the compiler from contracting to FMA. */
#define FMA_LOOP(T, EXPR)                                                              \
    do {                                                                               \
        T* pd = (T*)d;                                                                 \
        const T* pa = (const T*)a;                                                     \
        const T* pb = (const T*)b;                                                     \
        const T* pc = (const T*)c;                                                     \
        _Pragma("omp parallel for schedule(static) if (nthreads > 1)")                 \
        for (int64_t q = 0; q < nq; ++q) {                                             \
            int64_t off[4];                                                            \
            outer_offsets(&sp, q, off);                                                \
            for (int64_t i = 0; i < n0; ++i) {                                         \
                T x = pa[off[1] + i * sp.stride[1][0]];                                \
                T y = pb[off[2] + i * sp.stride[2][0]];                                \
                T z = pc[off[3] + i * sp.stride[3][0]];                                \
                pd[off[0] + i * sp.stride[0][0]] = (EXPR);                             \
            }                                                                          \
        }                                                                              \
    } while (0)

static inline double mul_d(double x, double y) {
    volatile double t = x * y;
    return t;
}
static inline float mul_f(float x, float y) {
    volatile float t = x * y;
    return t;
}

int oracle_fma(int dtype, void* d, const olayout* ld, const void* a, const olayout* la, const void* b,
               const olayout* lb, const void* c, const olayout* lc, int nthreads) {
    const olayout* ls[4] = {ld, la, lb, lc};
    ospace sp;
    if (lsize(ld) == 0) return 0;
    make_space(ls, 4, &sp);
    const int64_t nq = outer_count(&sp), n0 = sp.shape[0];
    set_threads(nthreads);
    switch (dtype) {
        case T_F64: FMA_LOOP(double, mul_d(x, y) + z); return 0;
        case T_F32: FMA_LOOP(float, mul_f(x, y) + z); return 0;
        case T_I32: FMA_LOOP(int32_t, WADD(int32_t, uint32_t, WMUL(int32_t, uint32_t, x, y), z)); return 0;
        case T_I64: FMA_LOOP(int64_t, WADD(int64_t, uint64_t, WMUL(int64_t, uint64_t, x, y), z)); return 0;
        default: return 2;
    }
}

/* ----------------------------------------------------------- reductions */

/* reduced / kept split (dim_split_axes, rstsr-common/src/layout/indexer.rs:453) */
static int split_axes(const olayout* la, const int64_t* axes, int naxes, olayout* ls, olayout* lm) {
    int used[MAXD] = {0};
    memset(ls, 0, sizeof(*ls));
    memset(lm, 0, sizeof(*lm));
    ls->offset = lm->offset = la->offset;
    for (int k = 0; k < naxes; ++k) {
        int64_t x = axes[k] < 0 ? axes[k] + la->ndim : axes[k];
        if (x < 0 || x >= la->ndim || used[x]) return 1;
        used[x] = 1;
        ls->shape[ls->ndim] = la->shape[x];
        ls->stride[ls->ndim] = la->stride[x];
        ls->ndim++;
    }
    for (int i = 0; i < la->ndim; ++i) {
        if (used[i]) continue;
        lm->shape[lm->ndim] = la->shape[i];
        lm->stride[lm->ndim] = la->stride[i];
        lm->ndim++;
    }
    return 0;
}

/* kept multi-index in C order of lm for output element e */
static void kept_offsets(const olayout* lm, const olayout* lo, int64_t e, int64_t* oin, int64_t* oout) {
    int64_t a = 0, b = lo->offset;
    for (int d = lm->ndim - 1; d >= 0; --d) {
        int64_t i = e % lm->shape[d];
        e /= lm->shape[d];
        a += i * lm->stride[d];
        b += i * lo->stride[d];
    }
    *oin = a;
    *oout = b;
}

/* Fold the reduced elements of one output in logical C order; when the
 * innermost reduced axis is contiguous with >= 32 elements, each run goes
 * through unrolled_reduce's 8 accumulators (cpu_serial/reduction.rs:44-83):
 * p_j accumulates elements j, j+8, ...; then acc = f_sum(acc, f_sum(p0,p4)),
 * ... f_sum(p3,p7); then the tail (< 8 elements) is folded into acc. */
#define RED_FOLD(T, A, INIT, F, FSUM)                                                          \
    static A fold_##T##_##A##_##F(const T* p, const olayout* ls, int64_t base) {              \
        A acc = INIT;                                                                          \
        const int nd = ls->ndim;                                                               \
        int64_t ninner = nd ? ls->shape[nd - 1] : 1, sinner = nd ? ls->stride[nd - 1] : 0;    \
        int64_t nouter = 1;                                                                    \
        for (int d = 0; d < nd - 1; ++d) nouter *= ls->shape[d];                               \
        for (int64_t q = 0; q < nouter; ++q) {                                                 \
            int64_t off = base, r = q;                                                         \
            for (int d = nd - 2; d >= 0; --d) {                                                \
                off += (r % ls->shape[d]) * ls->stride[d];                                     \
                r /= ls->shape[d];                                                             \
            }                                                                                  \
            if (sinner == 1 && ninner >= 32) {                                                 \
                A pp[8], in = INIT;                                                            \
                for (int j = 0; j < 8; ++j) pp[j] = INIT;                                      \
                int64_t i = 0;                                                                 \
                for (; i + 8 <= ninner; i += 8)                                                \
                    for (int j = 0; j < 8; ++j) pp[j] = F(pp[j], p[off + i + j]);              \
                for (int j = 0; j < 4; ++j) in = FSUM(in, FSUM(pp[j], pp[j + 4]));             \
                for (; i < ninner; ++i) in = F(in, p[off + i]);                                \
                acc = FSUM(acc, in);                                                           \
            } else {                                                                           \
                for (int64_t i = 0; i < ninner; ++i) acc = F(acc, p[off + i * sinner]);        \
            }                                                                                  \
        }                                                                                      \
        return acc;                                                                            \
    }

typedef struct {
    double s, q;
} dpair;
typedef struct {
    float s, q;
} fpair;

#define F_ADD(a, x) ((a) + (x))
#define F_SQ(a, x) ((a) + (x) * (x))
#define F_MUL(a, x) ((a) * (x))
#define F_MINF(a, x) fmin((a), (x))
#define F_MAXF(a, x) fmax((a), (x))
#define F_MINI(a, x) ((x) < (a) ? (x) : (a))
#define F_MAXI(a, x) ((x) > (a) ? (x) : (a))
#define F_CNT(a, x) ((a) + ((x) != 0))
#define S_ADD(a, b) ((a) + (b))
#define S_MUL(a, b) ((a) * (b))

static inline dpair dp_f(dpair a, double x) { a.s += x; a.q += x * x; return a; }
static inline dpair dp_s(dpair a, dpair b) { a.s += b.s; a.q += b.q; return a; }
static inline fpair fp_f(fpair a, float x) { a.s += x; a.q += x * x; return a; }
static inline fpair fp_s(fpair a, fpair b) { a.s += b.s; a.q += b.q; return a; }
static inline int32_t i32_add(int32_t a, int32_t x) { return (int32_t)((uint32_t)a + (uint32_t)x); }
static inline int32_t i32_mul(int32_t a, int32_t x) { return (int32_t)((uint32_t)a * (uint32_t)x); }
static inline int64_t i64_add(int64_t a, int64_t x) { return (int64_t)((uint64_t)a + (uint64_t)x); }
static inline int64_t i64_mul(int64_t a, int64_t x) { return (int64_t)((uint64_t)a * (uint64_t)x); }
static const dpair DP0 = {0, 0};
static const fpair FP0 = {0, 0};

RED_FOLD(double, double, 0.0, F_ADD, S_ADD)
RED_FOLD(double, dpair, DP0, dp_f, dp_s)
RED_FOLD(double, double, 0.0, F_SQ, S_ADD)
RED_FOLD(double, double, 1.0, F_MUL, S_MUL)
RED_FOLD(double, double, DBL_MAX, F_MINF, F_MINF)
RED_FOLD(double, double, -DBL_MAX, F_MAXF, F_MAXF)
RED_FOLD(double, uint64_t, 0, F_CNT, S_ADD)
RED_FOLD(float, float, 0.0f, F_ADD, S_ADD)
RED_FOLD(float, fpair, FP0, fp_f, fp_s)
RED_FOLD(float, float, 0.0f, F_SQ, S_ADD)
RED_FOLD(float, float, 1.0f, F_MUL, S_MUL)
RED_FOLD(float, float, FLT_MAX, F_MINF, F_MINF)
RED_FOLD(float, float, -FLT_MAX, F_MAXF, F_MAXF)
RED_FOLD(float, uint64_t, 0, F_CNT, S_ADD)
RED_FOLD(int32_t, int32_t, 0, i32_add, i32_add)
RED_FOLD(int32_t, int32_t, 1, i32_mul, i32_mul)
RED_FOLD(int32_t, int32_t, INT32_MAX, F_MINI, F_MINI)
RED_FOLD(int32_t, int32_t, INT32_MIN, F_MAXI, F_MAXI)
RED_FOLD(int32_t, uint64_t, 0, F_CNT, S_ADD)
RED_FOLD(int64_t, int64_t, 0, i64_add, i64_add)
RED_FOLD(int64_t, int64_t, 1, i64_mul, i64_mul)
RED_FOLD(int64_t, int64_t, INT64_MAX, F_MINI, F_MINI)
RED_FOLD(int64_t, int64_t, INT64_MIN, F_MAXI, F_MAXI)
RED_FOLD(int64_t, uint64_t, 0, F_CNT, S_ADD)

static inline uint8_t b_and(uint8_t a, uint8_t x) { return a & (x != 0); }
static inline uint8_t b_or(uint8_t a, uint8_t x) { return a | (x != 0); }
RED_FOLD(uint8_t, uint8_t, 1, b_and, b_and)
RED_FOLD(uint8_t, uint8_t, 0, b_or, b_or)
RED_FOLD(uint8_t, uint64_t, 0, F_CNT, S_ADD)

/* One reduction over axes; `out` receives the f_out values at layout lo. */
int oracle_reduce_axes(int op, int dtype, const void* a, const olayout* la, const int64_t* axes, int naxes, void* out,
                       const olayout* lo, int nthreads) {
    olayout ls, lm;
    if (split_axes(la, axes, naxes, &ls, &lm)) return 1;
    const int64_t nout = lsize(&lm), nred = lsize(&ls);
    set_threads(nthreads);
#define RED_CASE(T, A, F, OUTT, OUTEXPR)                                                       \
    {                                                                                          \
        const T* p = (const T*)a;                                                              \
        OUTT* o = (OUTT*)out;                                                                  \
        _Pragma("omp parallel for schedule(static) if (nthreads > 1)")                         \
        for (int64_t e = 0; e < nout; ++e) {                                                   \
            int64_t oin, oout;                                                                 \
            kept_offsets(&lm, lo, e, &oin, &oout);                                             \
            A acc = fold_##T##_##A##_##F(p, &ls, la->offset + oin);                            \
            o[oout] = (OUTEXPR);                                                               \
        }                                                                                      \
        return 0;                                                                              \
    }
    const double nd_ = (double)nred;
    const float nf_ = (float)nred;
    switch (dtype) {
        case T_F64:
            switch (op) {
                case R_SUM: RED_CASE(double, double, F_ADD, double, acc)
                case R_MEAN: RED_CASE(double, double, F_ADD, double, acc / nd_)
                case R_VAR: RED_CASE(double, dpair, dp_f, double, acc.q / nd_ - (acc.s / nd_) * (acc.s / nd_))
                case R_STD: RED_CASE(double, dpair, dp_f, double, sqrt(acc.q / nd_ - (acc.s / nd_) * (acc.s / nd_)))
                case R_L2: RED_CASE(double, double, F_SQ, double, sqrt(acc))
                case R_PROD: RED_CASE(double, double, F_MUL, double, acc)
                case R_MIN: RED_CASE(double, double, F_MINF, double, acc)
                case R_MAX: RED_CASE(double, double, F_MAXF, double, acc)
                case R_COUNT: RED_CASE(double, uint64_t, F_CNT, uint64_t, acc)
                default: return 2;
            }
        case T_F32:
            switch (op) {
                case R_SUM: RED_CASE(float, float, F_ADD, float, acc)
                case R_MEAN: RED_CASE(float, float, F_ADD, float, acc / nf_)
                case R_VAR: RED_CASE(float, fpair, fp_f, float, acc.q / nf_ - (acc.s / nf_) * (acc.s / nf_))
                case R_STD: RED_CASE(float, fpair, fp_f, float, sqrtf(acc.q / nf_ - (acc.s / nf_) * (acc.s / nf_)))
                case R_L2: RED_CASE(float, float, F_SQ, float, sqrtf(acc))
                case R_PROD: RED_CASE(float, float, F_MUL, float, acc)
                case R_MIN: RED_CASE(float, float, F_MINF, float, acc)
                case R_MAX: RED_CASE(float, float, F_MAXF, float, acc)
                case R_COUNT: RED_CASE(float, uint64_t, F_CNT, uint64_t, acc)
                default: return 2;
            }
        case T_I32:
            switch (op) {
                case R_SUM: RED_CASE(int32_t, int32_t, i32_add, int32_t, acc)
                case R_PROD: RED_CASE(int32_t, int32_t, i32_mul, int32_t, acc)
                case R_MIN: RED_CASE(int32_t, int32_t, F_MINI, int32_t, acc)
                case R_MAX: RED_CASE(int32_t, int32_t, F_MAXI, int32_t, acc)
                case R_COUNT: RED_CASE(int32_t, uint64_t, F_CNT, uint64_t, acc)
                default: return 2;
            }
        case T_I64:
            switch (op) {
                case R_SUM: RED_CASE(int64_t, int64_t, i64_add, int64_t, acc)
                case R_PROD: RED_CASE(int64_t, int64_t, i64_mul, int64_t, acc)
                case R_MIN: RED_CASE(int64_t, int64_t, F_MINI, int64_t, acc)
                case R_MAX: RED_CASE(int64_t, int64_t, F_MAXI, int64_t, acc)
                case R_COUNT: RED_CASE(int64_t, uint64_t, F_CNT, uint64_t, acc)
                default: return 2;
            }
        case T_BOOL:
            switch (op) {
                case R_ALL: RED_CASE(uint8_t, uint8_t, b_and, uint8_t, acc)
                case R_ANY: RED_CASE(uint8_t, uint8_t, b_or, uint8_t, acc)
                case R_SUM:
                case R_COUNT: RED_CASE(uint8_t, uint64_t, F_CNT, uint64_t, acc)
                default: return 2;
            }
        default:
            return 2;
    }
#undef RED_CASE
}

/* Arg reduction: per output, fold the reduced elements in row-major order of
 * the reduced axes (as given), starting from the first element; accept y
 * when y > acc (max) or y < acc (min); ties keep the earlier (smaller) index.
 * A NaN first element is never replaced (no comparison with NaN succeeds). */
#define ARG_CASE(T)                                                                            \
    {                                                                                          \
        const T* p = (const T*)a;                                                              \
        _Pragma("omp parallel for schedule(static) if (nthreads > 1)")                         \
        for (int64_t e = 0; e < nout; ++e) {                                                   \
            int64_t oin, oout;                                                                 \
            kept_offsets(&lm, lo, e, &oin, &oout);                                             \
            const int64_t base = la->offset + oin;                                             \
            int64_t best = 0;                                                                  \
            T bv = 0;                                                                          \
            for (int64_t r = 0; r < nred; ++r) {                                               \
                int64_t off = base, rr = r;                                                    \
                for (int d = ls.ndim - 1; d >= 0; --d) {                                       \
                    off += (rr % ls.shape[d]) * ls.stride[d];                                  \
                    rr /= ls.shape[d];                                                         \
                }                                                                              \
                T y = p[off];                                                                  \
                if (r == 0 || (is_max ? (y > bv) : (y < bv))) {                                \
                    bv = y;                                                                    \
                    best = r;                                                                  \
                }                                                                              \
            }                                                                                  \
            out[oout] = (uint64_t)best;                                                        \
        }                                                                                      \
        return 0;                                                                              \
    }

int oracle_argreduce_axes(int is_max, int dtype, const void* a, const olayout* la, const int64_t* axes, int naxes,
                          uint64_t* out, const olayout* lo, int nthreads) {
    olayout ls, lm;
    if (split_axes(la, axes, naxes, &ls, &lm)) return 1;
    const int64_t nout = lsize(&lm), nred = lsize(&ls);
    if (nred == 0) return 3;
    set_threads(nthreads);
    switch (dtype) {
        case T_F64: ARG_CASE(double)
        case T_F32: ARG_CASE(float)
        case T_I32: ARG_CASE(int32_t)
        case T_I64: ARG_CASE(int64_t)
        default: return 2;
    }
}

/* ------------------------------------------------------ triangles */

/* Row-major view of a (matrix or packed) layout pair: ColMajor reverses the
 * axes and flips uplo (feature_rayon/auto_impl/op_tri.rs:20-26). */
static void reverse_layout(olayout* l) {
    for (int i = 0, j = l->ndim - 1; i < j; ++i, --j) {
        int64_t t = l->shape[i];
        l->shape[i] = l->shape[j];
        l->shape[j] = t;
        t = l->stride[i];
        l->stride[i] = l->stride[j];
        l->stride[j] = t;
    }
}

/* Offset of batch element e (C order over the first nb axes). */
static int64_t batch_offset(const olayout* l, int nb, int64_t e) {
    int64_t o = l->offset;
    for (int d = nb - 1; d >= 0; --d) {
        int64_t i = e % l->shape[d];
        e /= l->shape[d];
        o += i * l->stride[d];
    }
    return o;
}

/* a (.., n(n+1)/2) <- triangle of b (.., n, n). */
int oracle_pack_tri(void* a, const olayout* la0, const void* b, const olayout* lb0, int esize, int lower, int order) {
    olayout la = *la0, lb = *lb0;
    if (order == 1) {
        reverse_layout(&la);
        reverse_layout(&lb);
        lower = !lower;
    }
    if (lb.ndim < 2 || la.ndim != lb.ndim - 1) return 1;
    const int nb = la.ndim - 1;
    const int64_t n = lb.shape[lb.ndim - 1];
    const int64_t si = lb.stride[lb.ndim - 2], sj = lb.stride[lb.ndim - 1], sp = la.stride[nb];
    int64_t nbatch = 1;
    for (int d = 0; d < nb; ++d) nbatch *= la.shape[d];
    for (int64_t e = 0; e < nbatch; ++e) {
        const int64_t oa = batch_offset(&la, nb, e), ob = batch_offset(&lb, nb, e);
        int64_t idx = 0;
        for (int64_t i = 0; i < n; ++i) {
            const int64_t j0 = lower ? 0 : i, j1 = lower ? i + 1 : n;
            for (int64_t j = j0; j < j1; ++j, ++idx)
                memcpy((char*)a + (oa + idx * sp) * esize, (const char*)b + (ob + i * si + j * sj) * esize,
                       (size_t)esize);
        }
    }
    return 0;
}

/* Negation of a float element of `esize` bytes: arithmetic for f64 / f32,
 * the sign bit for the 16-bit formats (IEEE negation). */
static void neg_elem(void* dst, const void* src, int esize) {
    if (esize == 8) {
        double x;
        memcpy(&x, src, 8);
        x = -x;
        memcpy(dst, &x, 8);
    } else if (esize == 4) {
        float x;
        memcpy(&x, src, 4);
        x = -x;
        memcpy(dst, &x, 4);
    } else {
        uint16_t x;
        memcpy(&x, src, 2);
        x ^= 0x8000u;
        memcpy(dst, &x, 2);
    }
}

/* a (.., n, n) <- packed triangle b (.., n(n+1)/2) and its mirror.
 * symm: 0 Sy, 1 He, 2 Ay, 3 Ah, 4 N (real types: He = Sy, Ah = Ay). */
int oracle_unpack_tri(void* a, const olayout* la0, const void* b, const olayout* lb0, int esize, int lower,
                      int symm, int order) {
    olayout la = *la0, lb = *lb0;
    if (order == 1) {
        reverse_layout(&la);
        reverse_layout(&lb);
        lower = !lower;
    }
    if (la.ndim < 2 || lb.ndim != la.ndim - 1) return 1;
    const int nb = lb.ndim - 1;
    const int64_t n = la.shape[la.ndim - 1];
    const int64_t si = la.stride[la.ndim - 2], sj = la.stride[la.ndim - 1], sp = lb.stride[nb];
    const int anti = symm == 2 || symm == 3, mirror = symm != 4;
    int64_t nbatch = 1;
    for (int d = 0; d < nb; ++d) nbatch *= lb.shape[d];
    for (int64_t e = 0; e < nbatch; ++e) {
        const int64_t oa = batch_offset(&la, nb, e), ob = batch_offset(&lb, nb, e);
        int64_t idx = 0;
        for (int64_t i = 0; i < n; ++i) {
            const int64_t j0 = lower ? 0 : i, j1 = lower ? i + 1 : n;
            for (int64_t j = j0; j < j1; ++j, ++idx) {
                const char* v = (const char*)b + (ob + idx * sp) * esize;
                char* aij = (char*)a + (oa + i * si + j * sj) * esize;
                char* aji = (char*)a + (oa + j * si + i * sj) * esize;
                if (anti && i == j) {
                    memset(aij, 0, (size_t)esize);
                    continue;
                }
                memcpy(aij, v, (size_t)esize);
                if (!mirror) continue;
                if (anti)
                    neg_elem(aji, v, esize);
                else
                    memcpy(aji, v, (size_t)esize);
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------ index_select */

/* c[.., k, ..] = a[.., idx[k], ..] along `axis` (every c element, C order). */
int oracle_index_select(void* c, const olayout* lc, const void* a, const olayout* la, int axis,
                        const uint64_t* idx, int64_t nidx, int esize) {
    if (lc->ndim != la->ndim || axis < 0 || axis >= lc->ndim || lc->shape[axis] != nidx) return 1;
    for (int64_t k = 0; k < nidx; ++k)
        if (idx[k] >= (uint64_t)la->shape[axis]) return 2;
    const int64_t n = lsize(lc);
    for (int64_t e = 0; e < n; ++e) {
        int64_t r = e, oc = lc->offset, oa = la->offset;
        for (int d = lc->ndim - 1; d >= 0; --d) {
            const int64_t i = r % lc->shape[d];
            r /= lc->shape[d];
            oc += i * lc->stride[d];
            oa += (d == axis ? (int64_t)idx[i] : i) * la->stride[d];
        }
        memcpy((char*)c + oc * esize, (const char*)a + oa * esize, (size_t)esize);
    }
    return 0;
}

/* ----------------------------------------------------------- einsum */

/* Labels are ids 0..nlab-1 with extents ext[]; labs holds each operand's
 * label per axis (ls[k].ndim entries for operand k, concatenated); olabs the
 * output's. dtype T_F64 or T_I64. */
int oracle_einsum(int dtype, int nops, const void* const* ops, const olayout* ls, const int32_t* labs, void* out,
                  const olayout* lo, const int32_t* olabs, int nlab, const int64_t* ext) {
    if (nlab > 64 || nops > 16) return 1;
    int is_out[64] = {0};
    for (int a = 0; a < lo->ndim; ++a) is_out[olabs[a]] = 1;
    int sum_labs[64], nsum = 0;
    for (int c = 0; c < nlab; ++c)
        if (!is_out[c]) sum_labs[nsum++] = c;
    const int32_t* lab_of[16];
    int off = 0;
    for (int k = 0; k < nops; ++k) {
        lab_of[k] = labs + off;
        off += ls[k].ndim;
    }
    int64_t nsumtot = 1;
    for (int q = 0; q < nsum; ++q) nsumtot *= ext[sum_labs[q]];
    const int64_t nout = lsize(lo);
    int64_t idx[64];
    for (int64_t e = 0; e < nout; ++e) {
        /* output label values (C order over the output axes) */
        int64_t r = e, oo = lo->offset;
        for (int a = lo->ndim - 1; a >= 0; --a) {
            idx[olabs[a]] = r % lo->shape[a];
            r /= lo->shape[a];
            oo += idx[olabs[a]] * lo->stride[a];
        }
        double s = 0.0, comp = 0.0;
        uint64_t si = 0;
        for (int64_t q = 0; q < nsumtot; ++q) {
            int64_t rr = q;
            for (int t = nsum - 1; t >= 0; --t) {
                idx[sum_labs[t]] = rr % ext[sum_labs[t]];
                rr /= ext[sum_labs[t]];
            }
            double p = 1.0;
            uint64_t pi = 1;
            for (int k = 0; k < nops; ++k) {
                int64_t o = ls[k].offset;
                for (int a = 0; a < ls[k].ndim; ++a) o += idx[lab_of[k][a]] * ls[k].stride[a];
                if (dtype == T_F64)
                    p *= ((const double*)ops[k])[o];
                else
                    pi *= (uint64_t)((const int64_t*)ops[k])[o];
            }
            if (dtype == T_F64) { /* Neumaier */
                const double t2 = s + p;
                if (fabs(s) >= fabs(p))
                    comp += (s - t2) + p;
                else
                    comp += (p - t2) + s;
                s = t2;
            } else {
                si += pi;
            }
        }
        if (dtype == T_F64)
            ((double*)out)[oo] = s + comp;
        else
            ((int64_t*)out)[oo] = (int64_t)si;
    }
    return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_num_procs();
#else
    return 1;
#endif
}
