// GEMM entry points: GEMMDriverAPI::driver_gemm
// (rstsr-blas-traits/src/blas3/gemm.rs:4-21), DeviceMatMulAPI::matmul with the
// broadcasting rules 1-7 (rstsr-core/src/device_faer/matmul.rs:83-239,
// rstsr-common/src/layout/matmul.rs:287-460) including the SYRK shortcut of
// device_faer/matmul.rs:38-48, and the grouped GEMM.
//
// f64 runs through the Ozaki split, f32 through the three-term bf16 split
// (ozaki.cu), both on the tcgen05 tensor cores. Other dtypes (integers, with
// wrapping arithmetic like the reference's naive kernel,
// rstsr-native-impl/src/cpu_rayon/matmul_naive.rs:13-54) and the NATIVE
// precision mode use a CUDA-core tiled kernel.
#include <algorithm>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "ew_kernel.cuh"
#include "split_gemm.hpp"
#include "tc_gemm.cuh"

namespace rstsr {

int ozaki_dgemm(rstsr_ctx* ctx, int64_t M, int64_t N, int64_t K, double alpha, Operand A, Operand Bt, double beta,
                double* C, int64_t ldc, int slices, bool symmetric);
int split_sgemm(rstsr_ctx* ctx, int64_t M, int64_t N, int64_t K, double alpha, Operand A, Operand Bt, double beta,
                float* C, int64_t ldc, int terms, bool symmetric);
int last_ozaki_slices();

// ---------------------------------------------------------- native kernel

// C[i,j] = alpha * sum_k A[i,k] B[k,j] + beta * C[i,j] with arbitrary element
// strides, 64x64 output tile per CTA (256 threads, 4x4 per thread), K staged
// through shared memory 16 at a time. Integers wrap; floats use FMA in T.
template <typename T, bool F = std::is_floating_point<T>::value>
struct AccTrait {
    using type = T;
};
template <typename T>
struct AccTrait<T, false> {
    using type = typename std::make_unsigned<T>::type;
};
template <typename T>
using AccOf = typename AccTrait<T>::type;

struct NativeParams {
    int64_t M, N, K;
    int64_t a_si, a_sk, b_sk, b_sj, c_si, c_sj;
    double alpha, beta;
};

template <typename T>
__global__ void __launch_bounds__(256) native_gemm_kernel(const T* __restrict__ A, const T* __restrict__ B,
                                                          T* __restrict__ C, const NativeParams p) {
    using Acc = AccOf<T>;
    __shared__ T As[16][65];
    __shared__ T Bs[16][65];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int64_t i0 = (int64_t)blockIdx.y * 64, j0 = (int64_t)blockIdx.x * 64;
    Acc acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = (Acc)0;
    for (int64_t k0 = 0; k0 < p.K; k0 += 16) {
        for (int t = threadIdx.x; t < 16 * 64; t += 256) {
            const int kk = t & 15, ii = t >> 4;
            const int64_t gi = i0 + ii, gk = k0 + kk;
            As[kk][ii] = (gi < p.M && gk < p.K) ? A[gi * p.a_si + gk * p.a_sk] : (T)0;
            const int jj = t & 63, kb = t >> 6;
            const int64_t gj = j0 + jj, gkb = k0 + kb;
            Bs[kb][jj] = (gj < p.N && gkb < p.K) ? B[gkb * p.b_sk + gj * p.b_sj] : (T)0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            Acc av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) av[a] = (Acc)As[kk][ty * 4 + a];
#pragma unroll
            for (int b = 0; b < 4; ++b) bv[b] = (Acc)Bs[kk][tx * 4 + b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] += av[a] * bv[b];
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int64_t i = i0 + ty * 4 + a, j = j0 + tx * 4 + b;
            if (i >= p.M || j >= p.N) continue;
            T* dst = C + i * p.c_si + j * p.c_sj;
            if constexpr (std::is_floating_point<T>::value) {
                T r = (T)p.alpha * acc[a][b];
                if (p.beta != 0.0) r += (T)p.beta * *dst;
                *dst = r;
            } else {
                // integer matmul: alpha, beta are taken as integers (wrapping)
                Acc r = (Acc)(int64_t)p.alpha * acc[a][b];
                if (p.beta != 0.0) r += (Acc)(int64_t)p.beta * (Acc)*dst;
                *dst = (T)r;
            }
        }
}

template <typename T>
static int launch_native(rstsr_ctx* ctx, const T* A, const T* B, T* C, const NativeParams& p) {
    dim3 grid((unsigned)((p.N + 63) / 64), (unsigned)((p.M + 63) / 64));
    if (grid.y > 65535) return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, "matrix too tall for the native kernel");
    native_gemm_kernel<T><<<grid, 256, 0, ctx->stream>>>(A, B, C, p);
    return after_launch(ctx, "native_gemm_kernel");
}

static int native_dispatch(rstsr_ctx* ctx, rstsr_dtype t, const void* A, const void* B, void* C,
                           const NativeParams& p) {
    switch (t) {
        case RSTSR_F64: return launch_native<double>(ctx, (const double*)A, (const double*)B, (double*)C, p);
        case RSTSR_F32: return launch_native<float>(ctx, (const float*)A, (const float*)B, (float*)C, p);
        case RSTSR_I8: return launch_native<int8_t>(ctx, (const int8_t*)A, (const int8_t*)B, (int8_t*)C, p);
        case RSTSR_I16: return launch_native<int16_t>(ctx, (const int16_t*)A, (const int16_t*)B, (int16_t*)C, p);
        case RSTSR_I32: return launch_native<int32_t>(ctx, (const int32_t*)A, (const int32_t*)B, (int32_t*)C, p);
        case RSTSR_I64: return launch_native<int64_t>(ctx, (const int64_t*)A, (const int64_t*)B, (int64_t*)C, p);
        case RSTSR_U8: return launch_native<uint8_t>(ctx, (const uint8_t*)A, (const uint8_t*)B, (uint8_t*)C, p);
        case RSTSR_U16: return launch_native<uint16_t>(ctx, (const uint16_t*)A, (const uint16_t*)B, (uint16_t*)C, p);
        case RSTSR_U32: return launch_native<uint32_t>(ctx, (const uint32_t*)A, (const uint32_t*)B, (uint32_t*)C, p);
        case RSTSR_U64: return launch_native<uint64_t>(ctx, (const uint64_t*)A, (const uint64_t*)B, (uint64_t*)C, p);
        default: return fail(RSTSR_ERR_UNIMPLEMENTED, std::string("matmul is not implemented for ") + dtype_name(t));
    }
}

// ------------------------------------------------------------ one GEMM

// A strided matrix product problem: C[i,j] = alpha sum_k A[i,k] B[k,j] + beta C.
struct GemmProblem {
    int64_t M, N, K;
    const void* A;
    int64_t a_si, a_sk;
    const void* B;
    int64_t b_sk, b_sj;
    void* C;
    int64_t c_si, c_sj;
    double alpha, beta;
    bool symmetric;  // B is A^T of the same buffer, beta == 0
};

static int gemm_one(rstsr_ctx* ctx, rstsr_dtype t, const GemmProblem& q, const rstsr_gemm_opts* opts) {
    if (q.M == 0 || q.N == 0) return RSTSR_OK;
    int prec = opts ? opts->precision : RSTSR_PREC_AUTO;
    const bool is_f = t == RSTSR_F64 || t == RSTSR_F32;
    if (!is_f && prec != RSTSR_PREC_AUTO && prec != RSTSR_PREC_NATIVE)
        return fail(RSTSR_ERR_INVALID_VALUE, "split precisions apply to f64 / f32 only");
    if (prec == RSTSR_PREC_OZAKI && t != RSTSR_F64) return fail(RSTSR_ERR_INVALID_VALUE, "the Ozaki split is for f64");
    if (prec == RSTSR_PREC_BF16X3 && t != RSTSR_F32) return fail(RSTSR_ERR_INVALID_VALUE, "the bf16 split is for f32");
    const bool native = !is_f || prec == RSTSR_PREC_NATIVE;
    if (q.K == 0) {
        // alpha * (empty sum) + beta * C
        Layout Lc;
        Lc.ndim = 2;
        Lc.shape[0] = q.M;
        Lc.shape[1] = q.N;
        Lc.stride[0] = q.c_si;
        Lc.stride[1] = q.c_sj;
        rstsr_layout lc = Lc.to_abi();
        if (q.beta == 0.0) {
            uint64_t zero = 0;
            return rstsr_cuda_fill(ctx, q.C, &lc, t, &zero);
        }
        if (t == RSTSR_F64) {
            double b = q.beta;
            return rstsr_cuda_binary_scalar(ctx, RSTSR_OP_MUL, t, q.C, &lc, q.C, &lc, &b, 0);
        }
        if (t == RSTSR_F32) {
            float b = (float)q.beta;
            return rstsr_cuda_binary_scalar(ctx, RSTSR_OP_MUL, t, q.C, &lc, q.C, &lc, &b, 0);
        }
        int64_t bi = (int64_t)q.beta;
        uint64_t buf = 0;
        memcpy(&buf, &bi, dtype_size(t));
        return rstsr_cuda_binary_scalar(ctx, RSTSR_OP_MUL, t, q.C, &lc, q.C, &lc, &buf, 0);
    }
    if (native) {
        NativeParams p{q.M, q.N, q.K, q.a_si, q.a_sk, q.b_sk, q.b_sj, q.c_si, q.c_sj, q.alpha, q.beta};
        return native_dispatch(ctx, t, q.A, q.B, q.C, p);
    }
    // tensor-core split paths write C row-major with unit column stride; a
    // column-major C is the row-major C^T = B^T A^T
    GemmProblem r = q;
    if (r.c_sj != 1 && r.c_si == 1) {
        r.M = q.N;
        r.N = q.M;
        r.A = q.B;
        r.a_si = q.b_sj;
        r.a_sk = q.b_sk;
        r.B = q.A;
        r.b_sk = q.a_sk;
        r.b_sj = q.a_si;
        r.c_si = q.c_sj;
        r.c_sj = 1;
    }
    if (r.c_sj != 1 || r.c_si < r.N) {
        // arbitrary output strides: compute into a row-major temporary
        void* tmp = nullptr;
        const size_t es = dtype_size(t);
        int s = scratch_alloc(ctx, (size_t)q.M * q.N * es, &tmp);
        if (s) return s;
        GemmProblem w = q;
        w.C = tmp;
        w.c_si = q.N;
        w.c_sj = 1;
        w.beta = 0.0;
        s = gemm_one(ctx, t, w, opts);
        if (!s) {
            // C = tmp + beta * C through the element-wise kernels
            Layout Lc, Lt;
            Lc.ndim = Lt.ndim = 2;
            Lc.shape[0] = Lt.shape[0] = q.M;
            Lc.shape[1] = Lt.shape[1] = q.N;
            Lc.stride[0] = q.c_si;
            Lc.stride[1] = q.c_sj;
            Lt.stride[0] = q.N;
            Lt.stride[1] = 1;
            rstsr_layout lc = Lc.to_abi(), lt = Lt.to_abi();
            if (q.beta == 0.0) {
                s = rstsr_cuda_assign(ctx, q.C, &lc, t, tmp, &lt, t);
            } else {
                if (t == RSTSR_F64) {
                    double b = q.beta;
                    s = rstsr_cuda_binary_scalar(ctx, RSTSR_OP_MUL, t, q.C, &lc, q.C, &lc, &b, 0);
                } else {
                    float b = (float)q.beta;
                    s = rstsr_cuda_binary_scalar(ctx, RSTSR_OP_MUL, t, q.C, &lc, q.C, &lc, &b, 0);
                }
                if (!s) s = rstsr_cuda_binary_inplace(ctx, RSTSR_OP_ADD, t, q.C, &lc, tmp, &lt, 0);
            }
        }
        scratch_free(ctx, tmp);
        return s;
    }
    Operand A{r.A, r.a_si, r.a_sk};
    Operand Bt{r.B, r.b_sj, r.b_sk};  // [N, K] view of B
    if (t == RSTSR_F64)
        return ozaki_dgemm(ctx, r.M, r.N, r.K, r.alpha, A, Bt, r.beta, (double*)r.C, r.c_si,
                           opts ? opts->ozaki_slices : 0, r.symmetric);
    const int terms = opts && opts->reserved[0] > 0 ? opts->reserved[0] : 3;
    return split_sgemm(ctx, r.M, r.N, r.K, r.alpha, A, Bt, r.beta, (float*)r.C, r.c_si, terms, r.symmetric);
}

// ------------------------------------------------------------ a batch

// Several products at once. f64 / f32 with a split precision run as one
// grouped split GEMM (one statistics, one split and one tensor-core launch
// for the whole batch, operands shared between problems split once) when
// every output is row- or column-major; anything else runs problem by problem.
static int gemm_batch(rstsr_ctx* ctx, rstsr_dtype t, const std::vector<GemmProblem>& batch,
                      const rstsr_gemm_opts* opts) {
    if (batch.size() == 1) return gemm_one(ctx, t, batch[0], opts);
    const int prec = opts ? opts->precision : RSTSR_PREC_AUTO;
    const bool ozaki = t == RSTSR_F64 && (prec == RSTSR_PREC_AUTO || prec == RSTSR_PREC_OZAKI);
    const bool bf16 = t == RSTSR_F32 && (prec == RSTSR_PREC_AUTO || prec == RSTSR_PREC_BF16X3);
    bool grouped = ozaki || bf16;
    std::vector<GemmProblem> rm;  // problems in row-major-output form
    for (const GemmProblem& q : batch) {
        if (!grouped) break;
        if (q.M == 0 || q.N == 0) continue;
        if (q.K == 0) {
            grouped = false;
            break;
        }
        GemmProblem r = q;
        if (r.c_sj != 1 && r.c_si == 1) {  // column-major C: C^T = B^T A^T
            r.M = q.N;
            r.N = q.M;
            r.A = q.B;
            r.a_si = q.b_sj;
            r.a_sk = q.b_sk;
            r.B = q.A;
            r.b_sk = q.a_sk;
            r.b_sj = q.a_si;
            r.c_si = q.c_sj;
            r.c_sj = 1;
        }
        if (r.c_sj != 1 || r.c_si < r.N) {
            grouped = false;
            break;
        }
        rm.push_back(r);
    }
    if (!grouped) {
        for (const GemmProblem& q : batch) {
            int s = gemm_one(ctx, t, q, opts);
            if (s) return s;
        }
        return RSTSR_OK;
    }
    if (rm.empty()) return RSTSR_OK;
    // distinct operand matrices: a broadcast batch reuses them
    std::vector<SplitItem> ai, bi;
    std::map<std::tuple<const void*, int64_t, int64_t, int64_t, int64_t>, int> amap, bmap;
    int rows_a = 0, rows_b = 0;
    // items start on the tile layouts' row units: 8-row groups (A), 64-row blocks (B)
    auto item = [](std::vector<SplitItem>& v, decltype(amap)& m, int& rows, int unit, const void* p, int64_t sr,
                   int64_t sk, int64_t R, int64_t K) {
        auto key = std::make_tuple(p, sr, sk, R, K);
        auto it = m.find(key);
        if (it != m.end()) return it->second;
        const int idx = (int)v.size();
        v.push_back(SplitItem{p, sr, sk, (int32_t)R, (int32_t)K, rows});
        rows += (int)((R + unit - 1) / unit * unit);
        m.emplace(key, idx);
        return idx;
    };
    std::vector<SplitProblem> probs;
    for (const GemmProblem& r : rm) {
        if (r.M > INT32_MAX / 8 || r.N > INT32_MAX / 8 || r.K > INT32_MAX / 2)
            return fail(RSTSR_ERR_UNIMPLEMENTED, "matrix too large for the split GEMM");
        SplitProblem sp;
        sp.ia = item(ai, amap, rows_a, 8, r.A, r.a_si, r.a_sk, r.M, r.K);
        sp.ib = item(bi, bmap, rows_b, 64, r.B, r.b_sj, r.b_sk, r.N, r.K);  // B^T view [N, K]
        sp.M = r.M;
        sp.N = r.N;
        sp.K = r.K;
        sp.C = r.C;
        sp.ldc = r.c_si;
        sp.alpha = r.alpha;
        sp.beta = r.beta;
        probs.push_back(sp);
    }
    const int slices = ozaki ? (opts ? opts->ozaki_slices : 0) : (opts && opts->reserved[0] > 0 ? opts->reserved[0] : 3);
    return split_gemm_run(ctx, ozaki ? SplitMode::Ozaki : SplitMode::Bf16x3, ai, bi, probs, slices, false);
}

// -------------------------------------------------------------- matmul

static void split_at(const Layout& l, int at, Layout* rest, Layout* mat) {
    *rest = Layout();
    *mat = Layout();
    rest->offset = mat->offset = l.offset;
    for (int i = 0; i < l.ndim; ++i) {
        Layout* d = i < at ? rest : mat;
        d->shape[d->ndim] = l.shape[i];
        d->stride[d->ndim] = l.stride[i];
        d->ndim++;
    }
}

// Row-major matmul over (la, lb, lc) following rules 1-7. Each problem of the
// batch is one GemmProblem.
static int matmul_row_major(rstsr_ctx* ctx, rstsr_dtype t, void* c, const Layout& lc, const void* a, const Layout& la,
                            const void* b, const Layout& lb, double alpha, double beta, const rstsr_gemm_opts* opts) {
    const size_t es = dtype_size(t);
    const int na = la.ndim, nb = lb.ndim, nc = lc.ndim;
    auto bad = [&](const char* m) {
        return fail(RSTSR_ERR_INVALID_LAYOUT, std::string("matmul: ") + m + " (a " + la.repr() + ", b " + lb.repr() +
                                                  ", c " + lc.repr() + ")");
    };
    if (na == 0 || nb == 0) return bad("0-dim operands are not allowed");
    // matrix views (rows x cols) and batch ("rest") layouts
    Layout ar, am, br, bm, cr, cm;
    if (na == 1 && nb == 1) {
        if (nc != 0 || la.shape[0] != lb.shape[0]) return bad("inner dot shapes");
        am.ndim = 2;
        am.shape[0] = 1;
        am.shape[1] = la.shape[0];
        am.stride[0] = 0;
        am.stride[1] = la.stride[0];
        am.offset = la.offset;
        bm.ndim = 2;
        bm.shape[0] = lb.shape[0];
        bm.shape[1] = 1;
        bm.stride[0] = lb.stride[0];
        bm.stride[1] = 0;
        bm.offset = lb.offset;
        cm.ndim = 2;
        cm.shape[0] = cm.shape[1] = 1;
        cm.stride[0] = cm.stride[1] = 1;
        cm.offset = lc.offset;
    } else {
        if (na == 1) {
            split_at(lb, nb - 2, &br, &bm);
            am.ndim = 2;
            am.shape[0] = 1;
            am.shape[1] = la.shape[0];
            am.stride[0] = 0;
            am.stride[1] = la.stride[0];
            am.offset = la.offset;
            if (nc != nb - 1) return bad("output rank");
            Layout cv;
            split_at(lc, nc - 1, &cr, &cv);
            cm.ndim = 2;
            cm.shape[0] = 1;
            cm.shape[1] = cv.shape[0];
            cm.stride[0] = 0;
            cm.stride[1] = cv.stride[0];
            cm.offset = lc.offset;
            ar = cr;
            for (int i = 0; i < ar.ndim; ++i) ar.stride[i] = 0;
        } else if (nb == 1) {
            split_at(la, na - 2, &ar, &am);
            bm.ndim = 2;
            bm.shape[0] = lb.shape[0];
            bm.shape[1] = 1;
            bm.stride[0] = lb.stride[0];
            bm.stride[1] = 0;
            bm.offset = lb.offset;
            if (nc != na - 1) return bad("output rank");
            Layout cv;
            split_at(lc, nc - 1, &cr, &cv);
            cm.ndim = 2;
            cm.shape[0] = cv.shape[0];
            cm.shape[1] = 1;
            cm.stride[0] = cv.stride[0];
            cm.stride[1] = 0;
            cm.offset = lc.offset;
            br = cr;
            for (int i = 0; i < br.ndim; ++i) br.stride[i] = 0;
        } else {
            split_at(la, na - 2, &ar, &am);
            split_at(lb, nb - 2, &br, &bm);
            if (nc < 2) return bad("output rank");
            split_at(lc, nc - 2, &cr, &cm);
        }
        // broadcast the batch layouts of a and b to c's batch shape (rule 3-7)
        Error e;
        Layout ar2, br2, tmp;
        if (!broadcast_layouts(cr, ar, RSTSR_ROW_MAJOR, &tmp, &ar2, &e)) return fail(e.code, e.msg);
        if (!broadcast_layouts(cr, br, RSTSR_ROW_MAJOR, &tmp, &br2, &e)) return fail(e.code, e.msg);
        if (tmp.ndim != cr.ndim || !std::equal(cr.shape, cr.shape + cr.ndim, tmp.shape))
            return bad("batch shapes do not broadcast to the output");
        ar = ar2;
        br = br2;
        ar.offset = la.offset;
        br.offset = lb.offset;
    }
    const int64_t M = am.shape[0], K = am.shape[1], N = bm.shape[1];
    if (bm.shape[0] != K || cm.shape[0] != M || cm.shape[1] != N) return bad("matrix shapes do not conform");
    // SYRK shortcut (device_faer/matmul.rs:38-48): same buffer, B = A^T, beta 0
    const bool syrk = (t == RSTSR_F64 || t == RSTSR_F32) && beta == 0.0 && a == b && M == N && am.offset == bm.offset &&
                      am.stride[0] == bm.stride[1] && am.stride[1] == bm.stride[0] && cr.ndim == 0;
    // enumerate the batch
    const int64_t nbatch = cr.size();
    const char* pa = (const char*)a;
    const char* pb = (const char*)b;
    char* pc = (char*)c;
    std::vector<GemmProblem> batch;
    batch.reserve((size_t)nbatch);
    for (int64_t bi = 0; bi < nbatch; ++bi) {
        int64_t oa = am.offset, ob = bm.offset, oc = cm.offset;
        if (cr.ndim > 0) {
            int64_t rem = bi;
            for (int d = cr.ndim - 1; d >= 0; --d) {
                const int64_t i = rem % cr.shape[d];
                rem /= cr.shape[d];
                oa += i * ar.stride[d];
                ob += i * br.stride[d];
                oc += i * cr.stride[d];
            }
            oa += 0 * 0;
        }
        GemmProblem q;
        q.M = M;
        q.N = N;
        q.K = K;
        q.A = pa + oa * (int64_t)es;
        q.a_si = am.stride[0];
        q.a_sk = am.stride[1];
        q.B = pb + ob * (int64_t)es;
        q.b_sk = bm.stride[0];
        q.b_sj = bm.stride[1];
        q.C = pc + oc * (int64_t)es;
        q.c_si = cm.stride[0];
        q.c_sj = cm.stride[1];
        q.alpha = alpha;
        q.beta = beta;
        q.symmetric = syrk;
        if (M == 1 && q.c_si == 0) q.c_si = N;  // single-row views
        if (N == 1 && q.c_sj == 0) q.c_sj = 1;
        batch.push_back(q);
    }
    return gemm_batch(ctx, t, batch, opts);
}

}  // namespace rstsr

using namespace rstsr;

extern "C" {

int rstsr_cuda_gemm(rstsr_ctx* ctx, rstsr_order order, char transa, char transb, int64_t m, int64_t n, int64_t k,
                    double alpha, const void* a, int64_t lda, const void* b, int64_t ldb, double beta, void* c,
                    int64_t ldc, rstsr_dtype t, const rstsr_gemm_opts* opts) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    if (!dtype_valid(t)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    if (m < 0 || n < 0 || k < 0) return fail(RSTSR_ERR_INVALID_VALUE, "negative GEMM extent");
    auto tr = [](char x) { return x == 'T' || x == 't' || x == 'C' || x == 'c'; };
    auto ok = [](char x) { return x == 'N' || x == 'n' || x == 'T' || x == 't' || x == 'C' || x == 'c'; };
    if (!ok(transa) || !ok(transb)) return fail(RSTSR_ERR_INVALID_VALUE, "trans must be N, T or C");
    const bool ta = tr(transa), tb = tr(transb);
    if (m == 0 || n == 0) return RSTSR_OK;
    if (!a || !b || !c) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    GemmProblem q;
    q.M = m;
    q.N = n;
    q.K = k;
    q.A = a;
    q.B = b;
    q.C = c;
    q.alpha = alpha;
    q.beta = beta;
    q.symmetric = false;
    if (order == RSTSR_ROW_MAJOR) {
        // A row-major [m,k] (or [k,m] if transposed) with leading dim lda
        q.a_si = ta ? 1 : lda;
        q.a_sk = ta ? lda : 1;
        q.b_sk = tb ? 1 : ldb;
        q.b_sj = tb ? ldb : 1;
        q.c_si = ldc;
        q.c_sj = 1;
    } else {
        q.a_si = ta ? lda : 1;
        q.a_sk = ta ? 1 : lda;
        q.b_sk = tb ? ldb : 1;
        q.b_sj = tb ? 1 : ldb;
        q.c_si = 1;
        q.c_sj = ldc;
    }
    return gemm_one(ctx, t, q, opts);
}

int rstsr_cuda_matmul(rstsr_ctx* ctx, rstsr_dtype t, void* c, const rstsr_layout* lc, const void* a,
                      const rstsr_layout* la, const void* b, const rstsr_layout* lb, double alpha, double beta,
                      rstsr_order order, const rstsr_gemm_opts* opts) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(lc, "c"));
    RSTSR_TRY(check_layout(la, "a"));
    RSTSR_TRY(check_layout(lb, "b"));
    if (!dtype_valid(t) || t == RSTSR_BOOL || t == RSTSR_F16 || t == RSTSR_BF16)
        return fail(RSTSR_ERR_UNIMPLEMENTED, std::string("matmul is not implemented for ") + dtype_name(t));
    Layout Lc = Layout::from_abi(*lc), La = Layout::from_abi(*la), Lb = Layout::from_abi(*lb);
    if (Lc.size() == 0) return RSTSR_OK;
    if (!a || !b || !c) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    if (order == RSTSR_COL_MAJOR) {
        // C[n,m,t] = B[n,k,t] @ A[k,m,t]: reverse every axis and swap operands
        return matmul_row_major(ctx, t, c, Lc.reverse_axes(), b, Lb.reverse_axes(), a, La.reverse_axes(), alpha, beta,
                                opts);
    }
    return matmul_row_major(ctx, t, c, Lc, a, La, b, Lb, alpha, beta, opts);
}

int rstsr_cuda_gemm_grouped(rstsr_ctx* ctx, rstsr_dtype t, const rstsr_gemm_problem* problems, int32_t nproblems,
                            const rstsr_gemm_opts* opts) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    if (nproblems < 0 || (nproblems > 0 && !problems)) return fail(RSTSR_ERR_INVALID_VALUE, "bad problem list");
    if (!dtype_valid(t) || t == RSTSR_BOOL || t == RSTSR_F16 || t == RSTSR_BF16)
        return fail(RSTSR_ERR_UNIMPLEMENTED, std::string("grouped GEMM is not implemented for ") + dtype_name(t));
    std::vector<GemmProblem> batch;
    for (int i = 0; i < nproblems; ++i) {
        const rstsr_gemm_problem& g = problems[i];
        if (g.m < 0 || g.n < 0 || g.k < 0) return fail(RSTSR_ERR_INVALID_VALUE, "negative GEMM extent");
        if ((g.m > 0 && g.n > 0) && (!g.c || (g.k > 0 && (!g.a || !g.b))))
            return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer in problem " + std::to_string(i));
        GemmProblem q;
        q.M = g.m;
        q.N = g.n;
        q.K = g.k;
        q.A = g.a;
        q.a_si = g.lda;
        q.a_sk = 1;
        q.B = g.b;
        q.b_sk = g.ldb;
        q.b_sj = 1;
        q.C = g.c;
        q.c_si = g.ldc;
        q.c_sj = 1;
        q.alpha = g.alpha;
        q.beta = g.beta;
        q.symmetric = false;
        batch.push_back(q);
    }
    return gemm_batch(ctx, t, batch, opts);
}

int32_t rstsr_cuda_last_ozaki_slices(void) { return last_ozaki_slices(); }

}  // extern "C"
