// Floating-point GEMM on the BF16 tensor cores by error-free splitting.
//
// f64 (Ozaki scheme): Ozaki, Ogita, Oishi & Rump, "Error-free transformations
// of matrix multiplication by using fast routines of matrix multiplication and
// its applications", Numer. Algorithms 59 (2012); the integer-slice form of
// Ootomo, Ozaki & Yokota, "DGEMM on integer matrix multiplication unit",
// IJHPCA (2024). Each row i of A is scaled by 2^-e_i so that |a| < 1 and cut
// into S slices d_s of 7 bits plus sign, a = 2^-7 sum_s d_s 2^(-7s) with
// integers |d_s| <= 128; the same for the columns of B. Integers of at most
// 8 significant bits are exact in bf16, so on GB300 -- whose INT8 tensor
// rate is far below its BF16 rate -- the slice products run on the BF16
// tensor cores with FP32 accumulation: a slice product summed over a K chunk
// of at most 1024 is an integer below 2^24 for levels 0 and 1 and is therefore
// exact. Products of the same level s+t accumulate in one TMEM accumulator
// (levels 0 to 3 separately, every higher level in a fifth one). The tensor
// cores accumulate FP32 by truncation, so the merged accumulator errs by one
// unit of its last place per step; starting it at level 4 keeps that below
// 2^-51 of the result per step. Only levels s + t < L are formed.
// The epilogue adds the accumulators in double and rescales by
// 2^(e_i + f_j - 14).
//
// f32 (three-term bf16 split): Henry, Tang & Heinecke, "Leveraging the
// bfloat16 artificial intelligence datatype for higher-precision computations",
// ARITH 2019. x = hi + mid + lo exactly (8 bits each); the six products with
// term order <= 2 (hi*hi | hi*mid + mid*hi | hi*lo + mid*mid + lo*hi)
// accumulate in three FP32 accumulators and are summed in double.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "tc_gemm.cuh"

namespace rstsr {

static thread_local int g_last_slices = 0;

// ------------------------------------------------------------- statistics

// Per-row max |x| (as ordered uint64 bits of the non-negative double) and
// sum |x| of a logical [R, K] operand X[r*sr + k*sk].
template <typename T>
__global__ void __launch_bounds__(256) row_stats_kernel(const T* __restrict__ X, int64_t sr, int64_t sk, int R, int K,
                                                        unsigned long long* __restrict__ maxbits,
                                                        double* __restrict__ sumabs) {
    __shared__ double smax[8][33];
    __shared__ double ssum[8][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
    const bool kfast = sk == 1 || (sr != 1 && llabs(sk) <= llabs(sr));
    // thread owns row (r0 + rr) where rr = kfast ? ty + 8j : tx
    double m[4] = {0, 0, 0, 0}, s[4] = {0, 0, 0, 0};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int rr = kfast ? ty + 8 * j : tx;
        const int kk = kfast ? tx : ty + 8 * j;
        const int r = r0 + rr, k = k0 + kk;
        if (r < R && k < K) {
            const double v = fabs((double)X[(int64_t)r * sr + (int64_t)k * sk]);
            m[j] = v;
            s[j] = v;
        }
    }
    if (kfast) {
        // reduce over tx (k) within the warp: rows ty + 8j
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            double mm = m[j], ss = s[j];
            for (int d = 16; d > 0; d >>= 1) {
                mm = fmax(mm, __shfl_down_sync(0xffffffffu, mm, d));
                ss += __shfl_down_sync(0xffffffffu, ss, d);
            }
            const int r = r0 + ty + 8 * j;
            if (tx == 0 && r < R) {
                atomicMax(&maxbits[r], (unsigned long long)__double_as_longlong(mm));
                atomicAdd(&sumabs[r], ss);
            }
        }
    } else {
        // row = tx; reduce the 4 k's per thread, then across ty through smem
        double mm = fmax(fmax(m[0], m[1]), fmax(m[2], m[3]));
        double ss = s[0] + s[1] + s[2] + s[3];
        smax[ty][tx] = mm;
        ssum[ty][tx] = ss;
        __syncthreads();
        if (ty == 0) {
            for (int i = 1; i < 8; ++i) {
                mm = fmax(mm, smax[i][tx]);
                ss += ssum[i][tx];
            }
            const int r = r0 + tx;
            if (r < R) {
                atomicMax(&maxbits[r], (unsigned long long)__double_as_longlong(mm));
                atomicAdd(&sumabs[r], ss);
            }
        }
    }
}

// e_r such that max_r < 2^e_r (0 for an all-zero row)
__global__ void exps_kernel(const unsigned long long* __restrict__ maxbits, int R, int32_t* __restrict__ exps) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    const double m = __longlong_as_double((long long)maxbits[r]);
    int e = 0;
    if (m > 0) frexp(m, &e);
    exps[r] = e;
}

// ------------------------------------------------------------------ split

// Cut a logical [R, K] operand into slices, written K-major as
// out[s * R * kp + r * kp + k] (bf16), zero in the K padding [K, kp).
// MODE 0: Ozaki integer slices of x * 2^-e_r, slice s stored as d_s 2^(-7s).
// MODE 1: f32 three-term split hi / mid / lo.
template <typename T, int MODE>
__global__ void __launch_bounds__(256) split_kernel(const T* __restrict__ X, int64_t sr, int64_t sk, int R, int K,
                                                    int kp, int S, const int32_t* __restrict__ exps,
                                                    __nv_bfloat16* __restrict__ out) {
    __shared__ T tile[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
    const bool kfast = sk == 1 || (sr != 1 && llabs(sk) <= llabs(sr));
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int rr = kfast ? ty + 8 * j : tx;
        const int kk = kfast ? tx : ty + 8 * j;
        const int r = r0 + rr, k = k0 + kk;
        T v = (T)0;
        if (r < R && k < K) v = X[(int64_t)r * sr + (int64_t)k * sk];
        tile[rr][kk] = v;
    }
    __syncthreads();
    const size_t plane = (size_t)R * kp;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int rr = ty + 8 * j;
        const int r = r0 + rr, k = k0 + tx;
        if (r >= R || k >= kp) continue;
        const size_t o = (size_t)r * kp + k;
        if (k >= K) {
            for (int s = 0; s < S; ++s) out[s * plane + o] = __float2bfloat16_rn(0.f);
            continue;
        }
        if constexpr (MODE == 0) {
            double y = ldexp((double)tile[rr][tx], -exps[r]);
            for (int s = 0; s < S; ++s) {
                const double t = y * 128.0;      // exact
                const double d = rint(t);        // |d| <= 128
                out[s * plane + o] = __double2bfloat16(ldexp(d, -7 * s));  // exact: 8-bit integer
                y = t - d;                       // exact
            }
        } else {
            const float x = (float)tile[rr][tx];
            const __nv_bfloat16 hi = __float2bfloat16_rn(x);
            const float r1 = x - __bfloat162float(hi);
            const __nv_bfloat16 mid = __float2bfloat16_rn(r1);
            const float r2 = r1 - __bfloat162float(mid);
            const __nv_bfloat16 lo = __float2bfloat16_rn(r2);
            out[o] = hi;
            if (S > 1) out[plane + o] = mid;
            if (S > 2) out[2 * plane + o] = lo;
        }
    }
}

// ------------------------------------------------------------------ driver


static int kt_for_slices(int s) { return s <= 7 ? (s <= 3 ? 64 : 32) : 16; }

// Slices needed for <= 1e-12 relative error given the spread (log2 of row
// max over row mean |x|) of both operands: 7 L >= 44 + spreadA + spreadB.
static int auto_levels(double spread_a, double spread_b) {
    const double need = 44.0 + std::max(0.0, spread_a) + std::max(0.0, spread_b);
    int L = (int)std::ceil(need / 7.0);
    return std::min(std::max(L, 4), 8);
}

template <typename T>
static void launch_stats(rstsr_ctx* ctx, const Operand& op, int R, int K, unsigned long long* maxbits, double* sumabs) {
    dim3 grid((K + 31) / 32, (R + 31) / 32);
    row_stats_kernel<T><<<grid, 256, 0, ctx->stream>>>((const T*)op.ptr, op.s_row, op.s_k, R, K, maxbits, sumabs);
}

// C[M,N] (row-major, ldc) = alpha * A[M,K] B[K,N] + beta * C by the Ozaki
// split. B is described as its transpose view [N, K]. symmetric: B^T is A
// itself (same data), beta == 0, only the lower triangle is computed.
int ozaki_dgemm(rstsr_ctx* ctx, int64_t M, int64_t N, int64_t K, double alpha, Operand A, Operand Bt, double beta,
                double* C, int64_t ldc, int slices, bool symmetric) {
    if (M == 0 || N == 0) return RSTSR_OK;
    if (M > INT32_MAX / 8 || N > INT32_MAX / 8 || K > INT32_MAX)
        return fail(RSTSR_ERR_UNIMPLEMENTED, "matrix too large for the split GEMM");
    const int kp = (int)((K + 7) / 8 * 8);
    const int rows_a = (int)M, rows_b = (int)N;
    // statistics
    void* stats = nullptr;
    const size_t nst = (size_t)(rows_a + rows_b);
    int s = scratch_alloc(ctx, nst * (8 + 8 + 4), &stats);
    if (s) return s;
    auto* maxbits = (unsigned long long*)stats;
    auto* sumabs = (double*)(maxbits + nst);
    auto* exps = (int32_t*)(sumabs + nst);
    cudaMemsetAsync(stats, 0, nst * 16, ctx->stream);
    launch_stats<double>(ctx, A, rows_a, (int)K, maxbits, sumabs);
    s = after_launch(ctx, "row_stats_kernel");
    if (!s && !symmetric) {
        launch_stats<double>(ctx, Bt, rows_b, (int)K, maxbits + rows_a, sumabs + rows_a);
        s = after_launch(ctx, "row_stats_kernel");
    }
    if (!s) {
        exps_kernel<<<(unsigned)((nst + 255) / 256), 256, 0, ctx->stream>>>(maxbits, (int)nst, exps);
        s = after_launch(ctx, "exps_kernel");
    }
    if (s) {
        scratch_free(ctx, stats);
        return s;
    }
    int L = slices;
    if (L <= 0) {
        // choose the slice count from the operands' exponent spread (needs the
        // statistics on the host: one synchronisation)
        std::vector<unsigned long long> hm(nst);
        std::vector<double> hs(nst);
        cudaMemcpyAsync(hm.data(), maxbits, nst * 8, cudaMemcpyDeviceToHost, ctx->stream);
        cudaMemcpyAsync(hs.data(), sumabs, nst * 8, cudaMemcpyDeviceToHost, ctx->stream);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) {
            scratch_free(ctx, stats);
            return cuda_fail(e, "ozaki statistics");
        }
        auto spread = [&](int lo, int hi) {
            double sp = 0;
            for (int i = lo; i < hi; ++i) {
                double mx;
                memcpy(&mx, &hm[i], 8);
                const double mean = hs[i] / (double)std::max<int64_t>(K, 1);
                if (mx > 0 && mean > 0) sp = std::max(sp, std::log2(mx / mean));
            }
            return sp;
        };
        const double sa = spread(0, rows_a);
        const double sb = symmetric ? sa : spread(rows_a, rows_a + rows_b);
        L = auto_levels(sa, sb);
    }
    L = std::min(std::max(L, 1), 8);
    g_last_slices = L;
    const int S = L;
    // slices
    void* sl = nullptr;
    const size_t a_elems = (size_t)S * rows_a * kp, b_elems = symmetric ? 0 : (size_t)S * rows_b * kp;
    s = scratch_alloc(ctx, (a_elems + b_elems) * 2, &sl);
    if (s) {
        scratch_free(ctx, stats);
        return s;
    }
    auto* as = (__nv_bfloat16*)sl;
    auto* bs = symmetric ? as : as + a_elems;
    {
        dim3 grid((kp + 31) / 32, (rows_a + 31) / 32);
        split_kernel<double, 0><<<grid, 256, 0, ctx->stream>>>((const double*)A.ptr, A.s_row, A.s_k, rows_a, (int)K,
                                                               kp, S, exps, as);
        s = after_launch(ctx, "split_kernel");
    }
    if (!s && !symmetric) {
        dim3 grid((kp + 31) / 32, (rows_b + 31) / 32);
        split_kernel<double, 0><<<grid, 256, 0, ctx->stream>>>((const double*)Bt.ptr, Bt.s_row, Bt.s_k, rows_b, (int)K,
                                                               kp, S, exps + rows_a, bs);
        s = after_launch(ctx, "split_kernel");
    }
    if (!s) {
        TcGemmParams p;
        memset(&p, 0, sizeof(p));
        p.M = (int)M;
        p.N = (int)N;
        p.sa = S;
        p.sb = S;
        p.a_rows = rows_a;
        p.b_rows = rows_b;
        int np = 0;
        for (int l = 0; l < L; ++l)
            for (int a = 0; a <= l; ++a) {
                const int b = l - a;
                if (a >= S || b >= S) continue;
                p.prod_a[np] = (uint8_t)a;
                p.prod_b[np] = (uint8_t)b;
                p.prod_acc[np] = (uint8_t)std::min(l, 4);
                ++np;
            }
        p.nprod = np;
        p.nacc = std::min(L, 5);
        p.C = C;
        p.ldc = ldc;
        p.out_f64 = 1;
        p.alpha = alpha;
        p.beta = beta;
        p.row_exp = exps;
        p.col_exp = symmetric ? exps : exps + rows_a;
        p.exp_bias = -14;
        p.symmetric = symmetric ? 1 : 0;
        p.err = ctx->dev_err;
        const int kt = kt_for_slices(S);
        const int k_tiles = (int)((K + kt - 1) / kt);
        // <= 1024 per chunk keeps levels 0 and 1 exact in FP32
        const int chunk = std::max(1, 1024 / kt);
        s = launch_tc_gemm(ctx, kt, as, bs, (uint64_t)kp, p, k_tiles, chunk);
    }
    scratch_free(ctx, sl);
    scratch_free(ctx, stats);
    return s;
}

// C[M,N] (f32, row-major) = alpha * A B + beta * C with the three-term bf16
// split (terms = 3: six products; terms = 2: three products).
int split_sgemm(rstsr_ctx* ctx, int64_t M, int64_t N, int64_t K, double alpha, Operand A, Operand Bt, double beta,
                float* C, int64_t ldc, int terms, bool symmetric) {
    if (M == 0 || N == 0) return RSTSR_OK;
    if (M > INT32_MAX / 4 || N > INT32_MAX / 4 || K > INT32_MAX)
        return fail(RSTSR_ERR_UNIMPLEMENTED, "matrix too large for the split GEMM");
    const int S = std::min(std::max(terms, 1), 3);
    const int kp = (int)((K + 7) / 8 * 8);
    void* sl = nullptr;
    const size_t a_elems = (size_t)S * M * kp, b_elems = symmetric ? 0 : (size_t)S * N * kp;
    int s = scratch_alloc(ctx, (a_elems + b_elems) * 2, &sl);
    if (s) return s;
    auto* as = (__nv_bfloat16*)sl;
    auto* bs = symmetric ? as : as + a_elems;
    {
        dim3 grid((kp + 31) / 32, (unsigned)((M + 31) / 32));
        split_kernel<float, 1><<<grid, 256, 0, ctx->stream>>>((const float*)A.ptr, A.s_row, A.s_k, (int)M, (int)K, kp,
                                                              S, nullptr, as);
        s = after_launch(ctx, "split_kernel");
    }
    if (!s && !symmetric) {
        dim3 grid((kp + 31) / 32, (unsigned)((N + 31) / 32));
        split_kernel<float, 1><<<grid, 256, 0, ctx->stream>>>((const float*)Bt.ptr, Bt.s_row, Bt.s_k, (int)N, (int)K,
                                                              kp, S, nullptr, bs);
        s = after_launch(ctx, "split_kernel");
    }
    if (!s) {
        TcGemmParams p;
        memset(&p, 0, sizeof(p));
        p.M = (int)M;
        p.N = (int)N;
        p.sa = S;
        p.sb = S;
        p.a_rows = (int)M;
        p.b_rows = (int)N;
        int np = 0;
        for (int l = 0; l < S; ++l)
            for (int a = 0; a <= l; ++a) {
                p.prod_a[np] = (uint8_t)a;
                p.prod_b[np] = (uint8_t)(l - a);
                p.prod_acc[np] = (uint8_t)l;
                ++np;
            }
        p.nprod = np;
        p.nacc = S;
        p.C = C;
        p.ldc = ldc;
        p.out_f64 = 0;
        p.alpha = alpha;
        p.beta = beta;
        p.symmetric = symmetric ? 1 : 0;
        p.err = ctx->dev_err;
        const int kt = 64;
        const int k_tiles = (int)((K + kt - 1) / kt);
        // K chunks of 512: the FP32 accumulators truncate, so their error
        // grows with the number of accumulation steps; chunk results are
        // summed in C
        s = launch_tc_gemm(ctx, kt, as, bs, (uint64_t)kp, p, k_tiles, 512 / kt);
    }
    scratch_free(ctx, sl);
    return s;
}

int last_ozaki_slices() { return g_last_slices; }

}  // namespace rstsr
