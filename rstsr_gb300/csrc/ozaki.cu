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
//
// Work is described as a list of problems over a list of distinct operand
// matrices ("items"): one matrix product, a broadcast batch (rule 7 of the
// matmul rules, where one A item meets many B items) or an uneven grouped
// GEMM all run as one statistics launch, one split launch and one tensor-core
// launch.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "split_gemm.hpp"
#include "tc_gemm.cuh"

namespace rstsr {

static thread_local int g_last_slices = 0;

// Operand items: matrix i is the logical [R, K] view X[r*s_row + k*s_k]; its
// rows start at `row0` of the item stack (slices, exponents, statistics).
struct SegArg {
    int32_t n;
    SplitItem inl[2];
    const SplitItem* dev;
};

__device__ __forceinline__ SplitItem seg_at(const SegArg& a, int i) { return a.n <= 2 ? a.inl[i] : a.dev[i]; }

// ------------------------------------------------------------- statistics

// Per-row max |x| (ordered uint64 bits of a non-negative double) and sum |x|.
template <typename T>
__global__ void __launch_bounds__(256) row_stats_kernel(const SegArg segs, unsigned long long* __restrict__ maxbits,
                                                        double* __restrict__ sumabs) {
    const SplitItem it = seg_at(segs, blockIdx.z);
    const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
    if (r0 >= it.R || k0 >= it.K) return;  // uniform per block
    __shared__ double smax[8][33];
    __shared__ double ssum[8][33];
    const T* X = (const T*)it.ptr;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const bool kfast = it.s_k == 1 || (it.s_row != 1 && llabs(it.s_k) <= llabs(it.s_row));
    double m[4] = {0, 0, 0, 0}, s[4] = {0, 0, 0, 0};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int rr = kfast ? ty + 8 * j : tx;
        const int kk = kfast ? tx : ty + 8 * j;
        const int r = r0 + rr, k = k0 + kk;
        if (r < it.R && k < it.K) {
            const double v = fabs((double)X[(int64_t)r * it.s_row + (int64_t)k * it.s_k]);
            m[j] = v;
            s[j] = v;
        }
    }
    if (kfast) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            double mm = m[j], ss = s[j];
            for (int d = 16; d > 0; d >>= 1) {
                mm = fmax(mm, __shfl_down_sync(0xffffffffu, mm, d));
                ss += __shfl_down_sync(0xffffffffu, ss, d);
            }
            const int r = r0 + ty + 8 * j;
            if (tx == 0 && r < it.R) {
                atomicMax(&maxbits[it.row0 + r], (unsigned long long)__double_as_longlong(mm));
                atomicAdd(&sumabs[it.row0 + r], ss);
            }
        }
    } else {
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
            if (r < it.R) {
                atomicMax(&maxbits[it.row0 + r], (unsigned long long)__double_as_longlong(mm));
                atomicAdd(&sumabs[it.row0 + r], ss);
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

// Cut every item into slices, written K-major into the stack as
// out[s * plane + (row0 + r) * pitch + k] (bf16), zero in [K, pitch).
// MODE 0: Ozaki integer slices of x * 2^-e_r, slice s stored as d_s 2^(-7s).
// MODE 1: f32 three-term split hi / mid / lo.
template <typename T, int MODE>
__global__ void __launch_bounds__(256) split_kernel(const SegArg segs, int pitch, int S, size_t plane,
                                                    const int32_t* __restrict__ exps, __nv_bfloat16* __restrict__ out) {
    const SplitItem it = seg_at(segs, blockIdx.z);
    const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
    if (r0 >= it.R || k0 >= pitch) return;  // uniform per block
    __shared__ T tile[32][33];
    const T* X = (const T*)it.ptr;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const bool kfast = it.s_k == 1 || (it.s_row != 1 && llabs(it.s_k) <= llabs(it.s_row));
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int rr = kfast ? ty + 8 * j : tx;
        const int kk = kfast ? tx : ty + 8 * j;
        const int r = r0 + rr, k = k0 + kk;
        T v = (T)0;
        if (r < it.R && k < it.K) v = X[(int64_t)r * it.s_row + (int64_t)k * it.s_k];
        tile[rr][kk] = v;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int rr = ty + 8 * j;
        const int r = r0 + rr, k = k0 + tx;
        if (r >= it.R || k >= pitch) continue;
        const size_t o = (size_t)(it.row0 + r) * pitch + k;
        if (k >= it.K) {
            for (int s = 0; s < S; ++s) out[s * plane + o] = __float2bfloat16_rn(0.f);
            continue;
        }
        if constexpr (MODE == 0) {
            double y = ldexp((double)tile[rr][tx], -exps[it.row0 + r]);
            for (int s = 0; s < S; ++s) {
                const double t = y * 128.0;  // exact
                const double d = rint(t);    // |d| <= 128
                out[s * plane + o] = __double2bfloat16(ldexp(d, -7 * s));  // exact: 8-bit integer
                y = t - d;                   // exact
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
// max over row mean |x|) of both operands. Dropping the levels >= L leaves an
// error near 2^(-7L + spreadA + spreadB - 6) of the result (measured on GB300:
// 2.5e-12 at L = 6 and 2.8e-13 at L = 7 for spreads 4.9 + 4.9); keeping it
// below 2^-43 gives 7 L >= 37 + spreadA + spreadB.
static int auto_levels(double spread_a, double spread_b) {
    const double need = 37.0 + std::max(0.0, spread_a) + std::max(0.0, spread_b);
    int L = (int)std::ceil(need / 7.0);
    return std::min(std::max(L, 4), 8);
}

// Upload a host vector to stream-ordered scratch (pageable copy: the source
// may be released as soon as the call returns).
template <typename V>
static int upload(rstsr_ctx* ctx, const std::vector<V>& v, void** out) {
    *out = nullptr;
    if (v.empty()) return RSTSR_OK;
    int s = scratch_alloc(ctx, v.size() * sizeof(V), out);
    if (s) return s;
    RSTSR_CUDA_TRY(cudaMemcpyAsync(*out, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice, ctx->stream));
    return RSTSR_OK;
}

static int make_segs(rstsr_ctx* ctx, const std::vector<SplitItem>& items, SegArg* sa, void** dev) {
    memset(sa, 0, sizeof(*sa));
    sa->n = (int32_t)items.size();
    *dev = nullptr;
    if (items.size() <= 2) {
        for (size_t i = 0; i < items.size(); ++i) sa->inl[i] = items[i];
        return RSTSR_OK;
    }
    bool capturing = false;
    cudaStreamCaptureStatus cs;
    if (cudaStreamIsCapturing(ctx->stream, &cs) == cudaSuccess) capturing = cs != cudaStreamCaptureStatusNone;
    if (capturing) return fail(RSTSR_ERR_UNIMPLEMENTED, "batched split GEMMs cannot be captured into a CUDA graph");
    int s = upload(ctx, items, dev);
    sa->dev = (const SplitItem*)*dev;
    return s;
}

static void grid_for(const std::vector<SplitItem>& items, int pitch, dim3* g) {
    int maxr = 1;
    for (const auto& it : items) maxr = std::max(maxr, it.R);
    *g = dim3((unsigned)((pitch + 31) / 32), (unsigned)((maxr + 31) / 32), (unsigned)items.size());
}

int split_gemm_run(rstsr_ctx* ctx, SplitMode mode, const std::vector<SplitItem>& a_items,
                   const std::vector<SplitItem>& b_items, const std::vector<SplitProblem>& probs, int slices,
                   bool symmetric) {
    if (probs.empty()) return RSTSR_OK;
    const bool f64 = mode == SplitMode::Ozaki;
    int rows_a = 0, rows_b = 0, maxk = 0;
    for (const auto& it : a_items) rows_a = std::max(rows_a, it.row0 + it.R), maxk = std::max(maxk, it.K);
    for (const auto& it : b_items) rows_b = std::max(rows_b, it.row0 + it.R), maxk = std::max(maxk, it.K);
    if (items_too_large(rows_a, rows_b, maxk)) return fail(RSTSR_ERR_UNIMPLEMENTED, "operands too large for the split GEMM");
    const int pitch = (maxk + 7) / 8 * 8;
    if (symmetric && (probs.size() != 1 || !b_items.empty()))
        return fail(RSTSR_ERR_RUNTIME, "symmetric split GEMM takes one problem and the A operand only");
    std::vector<void*> owned;
    auto cleanup = [&]() {
        for (void* p : owned) scratch_free(ctx, p);
    };
    int s = RSTSR_OK;
    SegArg sa_arg, sb_arg;
    void* dseg = nullptr;
    if ((s = make_segs(ctx, a_items, &sa_arg, &dseg))) return cleanup(), s;
    if (dseg) owned.push_back(dseg);
    if ((s = make_segs(ctx, b_items, &sb_arg, &dseg))) return cleanup(), s;
    if (dseg) owned.push_back(dseg);
    // per-row statistics and exponents (Ozaki only)
    const size_t nst = (size_t)rows_a + rows_b;
    int32_t* exps = nullptr;
    int L;
    if (f64) {
        void* stats = nullptr;
        if ((s = scratch_alloc(ctx, nst * (8 + 8 + 4), &stats))) return cleanup(), s;
        owned.push_back(stats);
        auto* maxbits = (unsigned long long*)stats;
        auto* sumabs = (double*)(maxbits + nst);
        exps = (int32_t*)(sumabs + nst);
        cudaMemsetAsync(stats, 0, nst * 16, ctx->stream);
        dim3 g;
        grid_for(a_items, maxk, &g);
        row_stats_kernel<double><<<g, 256, 0, ctx->stream>>>(sa_arg, maxbits, sumabs);
        if ((s = after_launch(ctx, "row_stats_kernel"))) return cleanup(), s;
        if (!b_items.empty()) {
            grid_for(b_items, maxk, &g);
            // B rows follow A rows in the statistics arrays
            row_stats_kernel<double><<<g, 256, 0, ctx->stream>>>(sb_arg, maxbits + rows_a, sumabs + rows_a);
            if ((s = after_launch(ctx, "row_stats_kernel"))) return cleanup(), s;
        }
        exps_kernel<<<(unsigned)((nst + 255) / 256), 256, 0, ctx->stream>>>(maxbits, (int)nst, exps);
        if ((s = after_launch(ctx, "exps_kernel"))) return cleanup(), s;
        L = slices;
        bool capturing = false;
        cudaStreamCaptureStatus cs;
        if (cudaStreamIsCapturing(ctx->stream, &cs) == cudaSuccess) capturing = cs != cudaStreamCaptureStatusNone;
        if (L <= 0 && capturing) L = 7;  // no host round trip inside a graph capture
        if (L <= 0) {
            // choose the slice count from the exponent spread (one synchronisation)
            std::vector<unsigned long long> hm(nst);
            std::vector<double> hs(nst);
            cudaMemcpyAsync(hm.data(), maxbits, nst * 8, cudaMemcpyDeviceToHost, ctx->stream);
            cudaMemcpyAsync(hs.data(), sumabs, nst * 8, cudaMemcpyDeviceToHost, ctx->stream);
            cudaError_t e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) return cleanup(), cuda_fail(e, "split GEMM statistics");
            auto spread = [&](const std::vector<SplitItem>& items, int base) {
                double sp = 0;
                for (const auto& it : items)
                    for (int i = 0; i < it.R; ++i) {
                        double mx;
                        memcpy(&mx, &hm[base + it.row0 + i], 8);
                        const double mean = hs[base + it.row0 + i] / (double)std::max(it.K, 1);
                        if (mx > 0 && mean > 0) sp = std::max(sp, std::log2(mx / mean));
                    }
                return sp;
            };
            const double sA = spread(a_items, 0);
            const double sB = b_items.empty() ? sA : spread(b_items, rows_a);
            L = auto_levels(sA, sB);
        }
        L = std::min(std::max(L, 1), 8);
    } else {
        L = std::min(std::max(slices, 1), 3);
    }
    g_last_slices = f64 ? L : 0;
    const int S = L;
    // slices
    void* sl = nullptr;
    const size_t plane_a = (size_t)rows_a * pitch, plane_b = (size_t)rows_b * pitch;
    if ((s = scratch_alloc(ctx, ((size_t)S * (plane_a + plane_b)) * 2, &sl))) return cleanup(), s;
    owned.push_back(sl);
    auto* as = (__nv_bfloat16*)sl;
    auto* bs = b_items.empty() ? as : as + (size_t)S * plane_a;
    {
        dim3 g;
        grid_for(a_items, pitch, &g);
        if (f64)
            split_kernel<double, 0><<<g, 256, 0, ctx->stream>>>(sa_arg, pitch, S, plane_a, exps, as);
        else
            split_kernel<float, 1><<<g, 256, 0, ctx->stream>>>(sa_arg, pitch, S, plane_a, nullptr, as);
        if ((s = after_launch(ctx, "split_kernel"))) return cleanup(), s;
        if (!b_items.empty()) {
            grid_for(b_items, pitch, &g);
            if (f64)
                split_kernel<double, 0><<<g, 256, 0, ctx->stream>>>(sb_arg, pitch, S, plane_b, exps + rows_a, bs);
            else
                split_kernel<float, 1><<<g, 256, 0, ctx->stream>>>(sb_arg, pitch, S, plane_b, nullptr, bs);
            if ((s = after_launch(ctx, "split_kernel"))) return cleanup(), s;
        }
    }
    // products and accumulators
    TcGemmParams p;
    memset(&p, 0, sizeof(p));
    p.sa = S;
    p.sb = S;
    p.a_rows = rows_a;
    p.b_rows = b_items.empty() ? rows_a : rows_b;
    int np = 0;
    for (int l = 0; l < L; ++l)
        for (int a = 0; a <= l; ++a) {
            const int b = l - a;
            if (a >= S || b >= S) continue;
            p.prod_a[np] = (uint8_t)a;
            p.prod_b[np] = (uint8_t)b;
            p.prod_acc[np] = (uint8_t)(f64 ? std::min(l, 4) : l);
            ++np;
        }
    p.nprod = np;
    p.nacc = f64 ? std::min(L, 5) : S;
    p.out_f64 = f64 ? 1 : 0;
    p.exp_bias = -14;
    p.row_exp = exps;
    p.col_exp = exps ? (b_items.empty() ? exps : exps + rows_a) : nullptr;
    p.err = ctx->dev_err;
    const int kt = f64 ? kt_for_slices(S) : 64;
    // FP32 accumulation truncates: Ozaki chunks of <= 1024 keep levels 0 and 1
    // exact; the f32 split sums chunks of 512 in C
    const int chunk = f64 ? std::max(1, 1024 / kt) : 512 / kt;
    const int BN = p.nacc > 4 ? 96 : 128;
    int k_tiles_max = 0;
    for (const auto& q : probs) k_tiles_max = std::max<int>(k_tiles_max, (int)((q.K + kt - 1) / kt));
    if (probs.size() == 1) {
        const SplitProblem& q = probs[0];
        p.M = (int)q.M;
        p.N = (int)q.N;
        p.C = q.C;
        p.ldc = q.ldc;
        p.alpha = q.alpha;
        p.beta = q.beta;
        p.symmetric = symmetric ? 1 : 0;
        const auto& ia = a_items[q.ia];
        const auto& ib = b_items.empty() ? a_items[q.ib] : b_items[q.ib];
        if (ia.row0 != 0 || ib.row0 != 0) {
            // one problem inside a larger stack: use the grouped form
        } else {
            s = launch_tc_gemm(ctx, kt, as, bs, (uint64_t)pitch, p, k_tiles_max, chunk);
            return cleanup(), s;
        }
    }
    // grouped: problem descriptors and the tile list
    std::vector<TcProblem> tp(probs.size());
    std::vector<int4> tiles;
    for (size_t i = 0; i < probs.size(); ++i) {
        const SplitProblem& q = probs[i];
        const auto& ia = a_items[q.ia];
        const auto& ib = b_items.empty() ? a_items[q.ib] : b_items[q.ib];
        TcProblem& t = tp[i];
        t.M = (int32_t)q.M;
        t.N = (int32_t)q.N;
        t.k_tiles = (int32_t)((q.K + kt - 1) / kt);
        t.a_row0 = ia.row0;
        t.b_row0 = ib.row0;
        t.row_exp0 = ia.row0;
        t.col_exp0 = ib.row0;
        t.symmetric = 0;
        t.C = q.C;
        t.ldc = q.ldc;
        t.alpha = q.alpha;
        t.beta = q.beta;
        const int tm = (int)((q.M + kTcBM - 1) / kTcBM), tn = (int)((q.N + BN - 1) / BN);
        for (int x = 0; x < tm; ++x)
            for (int y = 0; y < tn; ++y) tiles.push_back(make_int4((int)i, x, y, 0));
    }
    void* dprob = nullptr;
    void* dtiles = nullptr;
    if ((s = upload(ctx, tp, &dprob))) return cleanup(), s;
    owned.push_back(dprob);
    if ((s = upload(ctx, tiles, &dtiles))) return cleanup(), s;
    owned.push_back(dtiles);
    p.problems = (const TcProblem*)dprob;
    p.tiles = (const int4*)dtiles;
    p.kt_count = chunk;
    s = launch_tc_gemm(ctx, kt, as, bs, (uint64_t)pitch, p, k_tiles_max, chunk, (int64_t)tiles.size());
    return cleanup(), s;
}

int ozaki_dgemm(rstsr_ctx* ctx, int64_t M, int64_t N, int64_t K, double alpha, Operand A, Operand Bt, double beta,
                double* C, int64_t ldc, int slices, bool symmetric) {
    if (M == 0 || N == 0) return RSTSR_OK;
    if (M > INT32_MAX / 8 || N > INT32_MAX / 8 || K > INT32_MAX)
        return fail(RSTSR_ERR_UNIMPLEMENTED, "matrix too large for the split GEMM");
    std::vector<SplitItem> ai{{A.ptr, A.s_row, A.s_k, (int32_t)M, (int32_t)K, 0}};
    std::vector<SplitItem> bi;
    if (!symmetric) bi.push_back({Bt.ptr, Bt.s_row, Bt.s_k, (int32_t)N, (int32_t)K, 0});
    std::vector<SplitProblem> pr{{0, 0, M, N, K, C, ldc, alpha, beta}};
    return split_gemm_run(ctx, SplitMode::Ozaki, ai, bi, pr, slices, symmetric);
}

int split_sgemm(rstsr_ctx* ctx, int64_t M, int64_t N, int64_t K, double alpha, Operand A, Operand Bt, double beta,
                float* C, int64_t ldc, int terms, bool symmetric) {
    if (M == 0 || N == 0) return RSTSR_OK;
    if (M > INT32_MAX / 4 || N > INT32_MAX / 4 || K > INT32_MAX)
        return fail(RSTSR_ERR_UNIMPLEMENTED, "matrix too large for the split GEMM");
    std::vector<SplitItem> ai{{A.ptr, A.s_row, A.s_k, (int32_t)M, (int32_t)K, 0}};
    std::vector<SplitItem> bi;
    if (!symmetric) bi.push_back({Bt.ptr, Bt.s_row, Bt.s_k, (int32_t)N, (int32_t)K, 0});
    std::vector<SplitProblem> pr{{0, 0, M, N, K, C, ldc, alpha, beta}};
    return split_gemm_run(ctx, SplitMode::Bf16x3, ai, bi, pr, terms, symmetric);
}

int last_ozaki_slices() { return g_last_slices; }

}  // namespace rstsr
