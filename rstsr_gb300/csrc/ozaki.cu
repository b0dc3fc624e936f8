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
// The epilogue adds the accumulators in 64-bit fixed point and rescales by
// 2^(e_i + f_j - 14). Statistics, slicing and epilogue use integer arithmetic
// on the doubles' bits: GB300's FP64 rate is a small fraction of its integer
// rate, and FP64 instructions per element bounded every stage before.
//
// f32 (three-term bf16 split): Henry, Tang & Heinecke, "Leveraging the
// bfloat16 artificial intelligence datatype for higher-precision computations",
// ARITH 2019. x = hi + mid + lo exactly (8 bits each); the six products with
// term order <= 2 (hi*hi | hi*mid + mid*hi | hi*lo + mid*mid + lo*hi)
// accumulate in three FP32 accumulators, summed in FP32 with a two-sum.
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
    int32_t ublk;  // blocks of every item when all items of the side have one shape (else 0)
    SplitItem inl[2];
    const SplitItem* dev;
};

__device__ __forceinline__ SplitItem seg_at(const SegArg& a, int i) { return a.n <= 2 ? a.inl[i] : a.dev[i]; }

// ------------------------------------------------------------- statistics

// The A items and the B items of one call are handled by the same launches:
// items are numbered A first, then B; B rows follow the A rows (rows_a of
// them) in the statistics arrays. The grid is flat: item i owns blocks
// [blk0, blk0 + ceil(R / 32) * kblk) of 32 rows x 64 columns, so a grouped
// call of many small items launches only the blocks that have work (a grid
// sized for the largest item over every item left most blocks idle: 1 ms of
// a 512-problem call on GB300).
struct SegPair {
    SegArg a, b;
    int32_t rows_a;
    int64_t a_blocks;  // flat blocks of the A items (the B items' blocks follow)
};

__device__ __forceinline__ int pair_blk0(const SegPair& sp, int i) {
    return i < sp.a.n ? (sp.a.n <= 2 ? sp.a.inl[i].blk0 : sp.a.dev[i].blk0)
                      : (sp.b.n <= 2 ? sp.b.inl[i - sp.a.n].blk0 : sp.b.dev[i - sp.a.n].blk0);
}

// The item of flat block `b` and the block's first row and column in it.
// Items of one shape (a batch) find theirs by one division; mixed shapes by a
// binary search over the items' first blocks.
__device__ __forceinline__ SplitItem pair_block(const SegPair& sp, int64_t b, bool& is_b, int& r0, int& k0) {
    int lo = 0;
    if (b < sp.a_blocks && sp.a.ublk) {
        lo = (int)(b / sp.a.ublk);
    } else if (b >= sp.a_blocks && sp.b.ublk) {
        lo = sp.a.n + (int)((b - sp.a_blocks) / sp.b.ublk);
    } else {
        int hi = sp.a.n + sp.b.n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (pair_blk0(sp, mid) <= b) lo = mid;
            else hi = mid - 1;
        }
    }
    is_b = lo >= sp.a.n;
    const SplitItem it = is_b ? seg_at(sp.b, lo - sp.a.n) : seg_at(sp.a, lo);
    const int64_t local = b - it.blk0;
    r0 = (int)(local / it.kblk) * 32;
    k0 = (int)(local % it.kblk) * 64;
    return it;
}

// GB300 executes FP64 arithmetic at a small fraction of its integer and FP32
// rates, so the statistics, the split and the GEMM epilogue work on the bit
// patterns of the doubles wherever they can: |x| is the value's bits with the
// sign cleared, whose integer order is the order of the values.

// e such that m < 2^e for the row maximum m given as |x| bits (0 for zero).
__device__ __forceinline__ int exp_above(unsigned long long b) {
    const int E = (int)(b >> 52);
    if (E != 0) return E - 1022;
    if (b == 0) return 0;
    return -1010 - __clzll((long long)b);  // subnormal: highest set bit p, m < 2^(p - 1073)
}

// Shared-tile column of element k of a row: each 8-element chunk j is rotated
// by 2 (j / 2) so that the 8 threads reading chunks 0..7 of one row at the same
// step hit 8 different 8-byte bank pairs (without the rotation, chunks 64
// bytes apart collide 4 ways).
__device__ __forceinline__ int tile_col(int k) { return (k & ~7) | ((k + 2 * ((k >> 4) & 3)) & 7); }

// Load the block's 32 x 64 tile of an item into shared memory (zeros outside
// the item), coalesced along whichever of rows / K is contiguous in memory;
// element (r, k) lands at tile[r][tile_col(k)].
template <typename T>
__device__ __forceinline__ void load_tile(const SplitItem& it, int r0, int k0, T (*tile)[65]) {
    const T* X = (const T*)it.ptr;
    const int t = threadIdx.x;
    const bool kfast = it.s_k == 1 || (it.s_row != 1 && llabs(it.s_k) <= llabs(it.s_row));
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int rr = kfast ? (t >> 6) + 4 * j : (t & 31);
        const int kk = kfast ? (t & 63) : (t >> 5) + 8 * j;
        const int r = r0 + rr, k = k0 + kk;
        tile[rr][tile_col(kk)] = (r < it.R && k < it.K) ? X[(int64_t)r * it.s_row + (int64_t)k * it.s_k] : (T)0;
    }
}

// Per-row max |x| (as |x| bits) and sum |x|: thread t takes row t / 8 of the
// tile and its 8 consecutive columns, the 8 threads of a row combine by
// shuffles, one atomic pair per row and block.
template <typename T>
__global__ void __launch_bounds__(256) row_stats_kernel(const SegPair segs, unsigned long long* __restrict__ maxbits,
                                                        double* __restrict__ sumabs) {
    bool is_b;
    int r0, k0;
    const SplitItem it = pair_block(segs, blockIdx.x, is_b, r0, k0);
    if (r0 >= it.R || k0 >= it.K) return;  // uniform per block
    __shared__ T tile[32][65];
    load_tile<T>(it, r0, k0, tile);
    __syncthreads();
    const int rr = threadIdx.x >> 3, kq = (threadIdx.x & 7) * 8;
    unsigned long long mm = 0, bv[8];
#pragma unroll
    for (int v = 0; v < 8; ++v) {
        bv[v] = (unsigned long long)__double_as_longlong((double)tile[rr][tile_col(kq + v)]) & 0x7FFFFFFFFFFFFFFFull;
        mm = bv[v] > mm ? bv[v] : mm;
    }
    // The sum of |x| only feeds the exponent-spread estimate: add the 8 values
    // in FP32 on the scale of their largest binade (floats assembled from the
    // doubles' bits; values below 2^-125 of it dropped) and rescale once, so
    // that the FP64 pipe (a small fraction of GB300's FP32 rate) sees one
    // multiply per 8 elements instead of 8 adds.
    double ss = 0.0;
    const int em = (int)(mm >> 52);
    if (em > 0) {
        float fs = 0.f;
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            const int e = (int)(bv[v] >> 52), d = e - em;
            if (e > 0 && d > -126)
                fs += __uint_as_float(((uint32_t)(127 + d) << 23) | (uint32_t)((bv[v] >> 29) & 0x7FFFFFu));
        }
        ss = (double)fs * __longlong_as_double((long long)((unsigned long long)em << 52));
    } else {  // zeros and subnormals only
#pragma unroll
        for (int v = 0; v < 8; ++v) ss += __longlong_as_double((long long)bv[v]);
    }
#pragma unroll
    for (int d = 4; d > 0; d >>= 1) {
        const unsigned long long o = __shfl_down_sync(0xffffffffu, mm, d, 8);
        mm = o > mm ? o : mm;
        ss += __shfl_down_sync(0xffffffffu, ss, d, 8);
    }
    const int r = r0 + rr;
    if ((threadIdx.x & 7) == 0 && r < it.R) {
        const int row = (is_b ? segs.rows_a : 0) + it.row0 + r;
        atomicMax(&maxbits[row], mm);
        atomicAdd(&sumabs[row], ss);
    }
}

// The exponent spread of each side: max over rows of log2(row max / row mean
// |x|) for the A rows (out[0]) and the B rows (out[1]), as the bits of
// non-negative floats (ordered like the values). Grid: row blocks x items.
__global__ void __launch_bounds__(256) spread_kernel(const SegPair segs, const unsigned long long* __restrict__ maxbits,
                                                     const double* __restrict__ sumabs, unsigned int* __restrict__ out) {
    const int z = blockIdx.y;
    const bool is_b = z >= segs.a.n;
    const SplitItem it = is_b ? seg_at(segs.b, z - segs.a.n) : seg_at(segs.a, z);
    const int r = blockIdx.x * 256 + threadIdx.x;
    if (r >= it.R) return;
    const int row = (is_b ? segs.rows_a : 0) + it.row0 + r;
    const double mx = __longlong_as_double((long long)maxbits[row]);
    const double mean = sumabs[row] / (double)(it.K > 1 ? it.K : 1);
    if (mx > 0 && mean > 0) {
        const float sp = (float)log2(mx / mean);
        if (sp > 0.f) atomicMax(&out[is_b ? 1 : 0], __float_as_uint(sp));
    }
}

// ------------------------------------------------------------------ split

// Cut every item into slices, written into the stack of its side in the
// tensor-core tile layouts (KT = 2^lkt): A items as tc_offset_a (groups_a row
// groups, slice stride 8 KT), B items as tc_offset_b (blocks_b 64-row blocks,
// slice stride 64 KT); with `dual` (a symmetric product, B = A) the A items
// are written in both layouts. Zero in [K, pitch).
// Thread t takes row t / 8 of the block's 32 x 64 tile and 8 consecutive
// columns, i.e. one core-matrix row per slice: each slice is one 16-byte
// store.
// MODE 0: Ozaki slices of each double x of a row with exponent e_r: y = x 2^-e_r
//         as the fixed-point integer Y = y 2^63 (|Y| < 2^63; bits below 2^-63
//         of the row maximum are dropped), then balanced base-128 digits from
//         the top, the kept value being Y rounded to the nearest multiple of
//         2^(56 - 7 (S-1)), ties up: |d_0| <= 128 and -64 <= d_s < 64 after it.
//         Slice s is d_s 2^(-7s), exact in bf16; a non-finite x puts itself in
//         slice 0 and zeros after it. The column-0 threads also store the row
//         exponents e_r.
// MODE 1: f32 three-term split hi / mid / lo.
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(lo)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(hi)) << 16);
}

template <typename T, int MODE>
__global__ void __launch_bounds__(256) split_kernel(const SegPair segs, int pitch, int S, int lkt, int groups_a,
                                                    int blocks_b, int dual,
                                                    const unsigned long long* __restrict__ maxbits,
                                                    int32_t* __restrict__ exps, __nv_bfloat16* __restrict__ out_a,
                                                    __nv_bfloat16* __restrict__ out_b) {
    bool is_b;
    int r0, k0;
    const SplitItem it = pair_block(segs, blockIdx.x, is_b, r0, k0);
    if (r0 >= it.R || k0 >= pitch) return;  // uniform per block
    __shared__ T tile[32][65];
    load_tile<T>(it, r0, k0, tile);
    __syncthreads();
    const int rr = threadIdx.x >> 3, kq = (threadIdx.x & 7) * 8;
    const int r = r0 + rr, kb = k0 + kq;
    if (r >= it.R || kb >= pitch) return;  // pitch is a multiple of 16: whole runs
    const int row = it.row0 + r;
    const int KT = 1 << lkt;
    const size_t kt = (size_t)(kb >> lkt);
    const size_t inner = (size_t)((((kb & (KT - 1)) >> 3) << 6) + ((row & 7) << 3));
    uint4* oa = is_b ? nullptr
                     : reinterpret_cast<uint4*>(out_a + (((kt * groups_a + (size_t)(row >> 3)) * S) << (3 + lkt)) + inner);
    uint4* ob = (is_b || dual)
                    ? reinterpret_cast<uint4*>(out_b +
                                               ((((kt * blocks_b + (size_t)(row >> 6)) * S) * 8 +
                                                 (size_t)((row >> 3) & 7))
                                                << (3 + lkt)) +
                                               inner)
                    : nullptr;
    // slice strides in 16-byte units: 8 KT elements (A), 64 KT elements (B)
    const size_t sa = (size_t)1 << (lkt - 0), sb = (size_t)8 << lkt;
    if constexpr (MODE == 0) {
        const int e_r = exp_above(maxbits[(is_b ? segs.rows_a : 0) + row]);
        if (kb == 0) exps[(is_b ? segs.rows_a : 0) + row] = e_r;
        // the values as fixed-point integers Y = x 2^(63 - e_r)
        long long Y[8];
        uint32_t special = 0;    // bit v: value v is inf / NaN
        float spv[8];            // its bf16-exact float (slice 0)
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            const unsigned long long u = (unsigned long long)__double_as_longlong((double)tile[rr][tile_col(kq + v)]);
            const int E = (int)((u >> 52) & 0x7FF);
            const long long mant =
                (long long)(E ? (u & 0xFFFFFFFFFFFFFull) | (1ull << 52) : (u & 0xFFFFFFFFFFFFFull));
            const int sh = (E ? E : 1) - 1012 - e_r;
            long long y = sh >= 0 ? mant << (sh < 63 ? sh : 63) : (sh > -63 ? mant >> -sh : 0);
            if (u >> 63) y = -y;
            Y[v] = y;
            spv[v] = 0.f;
            if (E == 0x7FF) {
                special |= 1u << v;
                Y[v] = 0;
                const uint32_t nan = (u & 0xFFFFFFFFFFFFFull) ? 0x7FC00000u : 0x7F800000u;
                spv[v] = __uint_as_float(((uint32_t)(u >> 32) & 0x80000000u) | nan);
            }
        }
        // Balanced base-128 digits without a per-digit rounding chain: with
        // C = 64 (2^49 + 2^42 + ... + 2^(56 - 7 (S-1))) + 2^(55 - 7 (S-1)), the
        // sum lo = (Y mod 2^56) + C (< 2^57) holds digit j + 64 (j >= 1) in bits
        // [56 - 7j, 63 - 7j) and its carry out of bit 56 completes the top digit
        // d_0 = (Y >> 56) + carry in [-128, 128]; the kept value is Y rounded to
        // the nearest multiple of 2^(56 - 7 (S-1)), ties up, as a digit by digit
        // round-half-up recurrence gives.
        unsigned long long C = 1ull << (55 - 7 * (S - 1));
        for (int sl = 1; sl < S; ++sl) C += 64ull << (56 - 7 * sl);
        unsigned long long lo[8];
        int top[8];
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            const unsigned long long l = ((unsigned long long)Y[v] & ((1ull << 56) - 1)) + C;
            top[v] = (int)(Y[v] >> 56) + (int)(l >> 56);
            lo[v] = l;
        }
        for (int sl = 0; sl < S; ++sl) {
            const int k = 56 - 7 * sl;
            const float scale = __int_as_float((127 - 7 * sl) << 23);
            // 0x4B400000 | f is the float 12582912 + f (f < 2^22): (f - off) 2^(-7 sl) by
            // one exact FFMA, no integer-to-float conversion
            const float off = sl == 0 ? 12583040.0f : 12582976.0f;  // 12582912 + 128 / + 64
            uint32_t bits[8];
#pragma unroll
            for (int v = 0; v < 8; ++v) {
                const uint32_t f = sl == 0 ? (uint32_t)(top[v] + 128) : (uint32_t)(lo[v] >> k) & 0x7Fu;
                const float d = __fmaf_rn(__uint_as_float(0x4B400000u | f), scale, -off * scale);
                bits[v] = __float_as_uint(d);
                if (sl == 0 && (special >> v) & 1u) bits[v] = __float_as_uint(spv[v]);
            }
            // at most 8 significant bits: the bf16 is the float's upper half
            const uint4 w = make_uint4(__byte_perm(bits[0], bits[1], 0x7632), __byte_perm(bits[2], bits[3], 0x7632),
                                       __byte_perm(bits[4], bits[5], 0x7632), __byte_perm(bits[6], bits[7], 0x7632));
            if (oa) oa[sl * sa] = w;
            if (ob) ob[sl * sb] = w;
        }
    } else {
        float h[8], m[8], l[8];
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            const float x = (float)tile[rr][tile_col(kq + v)];
            h[v] = __bfloat162float(__float2bfloat16_rn(x));
            const float r1 = x - h[v];
            m[v] = __bfloat162float(__float2bfloat16_rn(r1));
            l[v] = r1 - m[v];
        }
        const uint4 wh = make_uint4(pack_bf16(h[0], h[1]), pack_bf16(h[2], h[3]), pack_bf16(h[4], h[5]),
                                    pack_bf16(h[6], h[7]));
        const uint4 wm = make_uint4(pack_bf16(m[0], m[1]), pack_bf16(m[2], m[3]), pack_bf16(m[4], m[5]),
                                    pack_bf16(m[6], m[7]));
        const uint4 wl = make_uint4(pack_bf16(l[0], l[1]), pack_bf16(l[2], l[3]), pack_bf16(l[4], l[5]),
                                    pack_bf16(l[6], l[7]));
        if (oa) {
            oa[0] = wh;
            if (S > 1) oa[sa] = wm;
            if (S > 2) oa[2 * sa] = wl;
        }
        if (ob) {
            ob[0] = wh;
            if (S > 1) ob[sb] = wm;
            if (S > 2) ob[2 * sb] = wl;
        }
    }
}

// ------------------------------------------------------------------ driver

// K tile width: the widest of 64 / 32 / 16 whose pipeline stage (every slice
// of a 128-row A tile and a BN-row B tile) leaves room for four stages, so
// that the bulk-copy latency stays hidden behind the products of the other
// stages.
static int kt_for_stages(int slices, int bn) {
    const size_t budget = kTcSmemMax - 1024 - kTcSmemTail;
    for (int kt : {64, 32}) {
        const size_t stage = (size_t)slices * (kTcBM + bn) * kt * 2;
        if (budget / stage >= 4) return kt;
    }
    return 16;
}

// Calls of at most this many multiply-adds skip the spread measurement and
// run with the largest slice count (8): measured on GB300 the synchronisation
// that brings the spread to the host costs 10-25 us, more than the extra
// products below about 2^30 multiply-adds.
constexpr double kNoSpreadMacs = 1073741824.0;

// Slices needed for <= 1e-12 relative error given the spread (log2 of row
// max over row mean |x|) of both operands. Dropping the levels >= L leaves an
// error near 2^(-7L + spreadA + spreadB - 6) of the result (measured on GB300:
// 2.5e-12 at L = 6 and 2.8e-13 at L = 7 for spreads 4.9 + 4.9); keeping it
// below 2^-43 gives 7 L >= 37 + spreadA + spreadB. Products whose results
// cancel exceed that estimate (uniform(-1, 1) operands, K = 128: 2.0e-13 at
// L = 6). Calls of at most 2^24 multiply-adds are bound by launch latency, not
// by the tensor cores: they take one slice more (seven more bits, for
// <= 1e-13 on such operands), which costs no time there.
static int auto_levels(double spread_a, double spread_b, bool small) {
    const double need = (small ? 44.0 : 37.0) + std::max(0.0, spread_a) + std::max(0.0, spread_b);
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

// Number the flat-grid blocks of the items (A items first): 32 x 64 blocks
// over each item's rows and its K rounded up to 64 (the widest K tile, so
// the split also zero-fills the K padding any tile width reads). Returns the
// total block count.
static int64_t number_blocks(std::vector<SplitItem>& a, std::vector<SplitItem>& b) {
    int64_t n = 0;
    for (auto* v : {&a, &b})
        for (auto& it : *v) {
            it.blk0 = (int32_t)n;
            it.kblk = std::max(1, (it.K + 63) / 64);
            n += (int64_t)((it.R + 31) / 32) * it.kblk;
        }
    return n;
}

int split_gemm_run(rstsr_ctx* ctx, SplitMode mode, const std::vector<SplitItem>& a_items_in,
                   const std::vector<SplitItem>& b_items_in, const std::vector<SplitProblem>& probs, int slices,
                   bool symmetric) {
    if (probs.empty()) return RSTSR_OK;
    std::vector<SplitItem> a_items = a_items_in, b_items = b_items_in;
    const int64_t nblocks = number_blocks(a_items, b_items);
    if (nblocks > INT32_MAX) return fail(RSTSR_ERR_UNIMPLEMENTED, "operands too large for the split GEMM");
    const bool f64 = mode == SplitMode::Ozaki;
    int rows_a = 0, rows_b = 0, maxk = 0;
    for (const auto& it : a_items) rows_a = std::max(rows_a, it.row0 + it.R), maxk = std::max(maxk, it.K);
    for (const auto& it : b_items) rows_b = std::max(rows_b, it.row0 + it.R), maxk = std::max(maxk, it.K);
    if (items_too_large(rows_a, rows_b, maxk)) return fail(RSTSR_ERR_UNIMPLEMENTED, "operands too large for the split GEMM");
    if (symmetric && (probs.size() != 1 || !b_items.empty()))
        return fail(RSTSR_ERR_RUNTIME, "symmetric split GEMM takes one problem and the A operand only");
    std::vector<void*> owned;
    auto cleanup = [&]() {
        for (void* p : owned) scratch_free(ctx, p);
    };
    int s = RSTSR_OK;
    SegPair segs;
    memset(&segs, 0, sizeof(segs));
    segs.rows_a = rows_a;
    void* dseg = nullptr;
    if ((s = make_segs(ctx, a_items, &segs.a, &dseg))) return cleanup(), s;
    if (dseg) owned.push_back(dseg);
    if ((s = make_segs(ctx, b_items, &segs.b, &dseg))) return cleanup(), s;
    // one block count for every item of a side: the item of a block is a division
    auto uniform_blocks = [](const std::vector<SplitItem>& v, int64_t* total) {
        *total = 0;
        int64_t first = -1;
        bool same = true;
        for (const SplitItem& it : v) {
            const int64_t nb = (int64_t)((it.R + 31) / 32) * it.kblk;
            *total += nb;
            if (first < 0) first = nb;
            same = same && nb == first;
        }
        return same && first > 0 && first <= INT32_MAX ? (int32_t)first : 0;
    };
    int64_t b_total = 0;
    segs.a.ublk = uniform_blocks(a_items, &segs.a_blocks);
    segs.b.ublk = uniform_blocks(b_items, &b_total);
    if (dseg) owned.push_back(dseg);
    // per-row statistics (Ozaki only); B rows follow A rows
    const size_t nst = (size_t)rows_a + rows_b;
    int32_t* exps = nullptr;
    unsigned long long* maxbits = nullptr;
    int L;
    if (f64) {
        void* stats = nullptr;
        if ((s = scratch_alloc(ctx, nst * (8 + 8 + 4), &stats))) return cleanup(), s;
        owned.push_back(stats);
        maxbits = (unsigned long long*)stats;
        auto* sumabs = (double*)(maxbits + nst);
        exps = (int32_t*)(sumabs + nst);
        RSTSR_CUDA_TRY(cudaMemsetAsync(stats, 0, nst * 16, ctx->stream));
        row_stats_kernel<double><<<(unsigned)nblocks, 256, 0, ctx->stream>>>(segs, maxbits, sumabs);
        if ((s = after_launch(ctx, "row_stats_kernel"))) return cleanup(), s;
        L = slices;
        bool capturing = false;
        cudaStreamCaptureStatus cs;
        if (cudaStreamIsCapturing(ctx->stream, &cs) == cudaSuccess) capturing = cs != cudaStreamCaptureStatusNone;
        if (L <= 0 && capturing) L = 7;  // no host round trip inside a graph capture
        // up to 2^30 multiply-adds the spread's host round trip (a stream
        // synchronisation, 10-25 us) costs more than the products of the
        // largest slice count: take 8, which no automatic choice exceeds
        double macs = 0;
        for (const auto& q : probs) macs += (double)q.M * (double)q.N * (double)q.K;
        if (L <= 0 && macs <= kNoSpreadMacs) L = 8;
        if (L <= 0) {
            // choose the slice count from the exponent spread of each side,
            // reduced on the device: one synchronisation, 8 bytes back
            void* dsp = nullptr;
            if ((s = scratch_alloc(ctx, 8, &dsp))) return cleanup(), s;
            owned.push_back(dsp);
            RSTSR_CUDA_TRY(cudaMemsetAsync(dsp, 0, 8, ctx->stream));
            int maxr = 1;
            for (const auto* v : {&a_items, &b_items})
                for (const auto& it : *v) maxr = std::max(maxr, it.R);
            spread_kernel<<<dim3((unsigned)((maxr + 255) / 256), (unsigned)(a_items.size() + b_items.size())), 256, 0,
                            ctx->stream>>>(segs, maxbits, sumabs, (unsigned int*)dsp);
            if ((s = after_launch(ctx, "spread_kernel"))) return cleanup(), s;
            unsigned int hsp[2] = {0, 0};
            RSTSR_CUDA_TRY(cudaMemcpyAsync(hsp, dsp, 8, cudaMemcpyDeviceToHost, ctx->stream));
            cudaError_t e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) return cleanup(), cuda_fail(e, "split GEMM statistics");
            float fa, fb;
            memcpy(&fa, &hsp[0], 4);
            memcpy(&fb, &hsp[1], 4);
            L = auto_levels(fa, b_items.empty() ? fa : fb, macs <= 16777216.0);
        }
        L = std::min(std::max(L, 1), 8);
    } else {
        L = std::min(std::max(slices, 1), 3);
    }
    g_last_slices = f64 ? L : 0;
    const int S = L;
    constexpr int BN = kTcBN;
    // kernel configuration: the autotuned one for this shape class, if any
    int64_t maxm = 0, maxn = 0;
    for (const auto& q : probs) maxm = std::max(maxm, q.M), maxn = std::max(maxn, q.N);
    const TuneConfig tune = tune_config(mode, S, maxm, maxn, maxk);
    int kt = kt_for_stages(S, BN);
    if (tune.kt && (kTcSmemMax - 1024 - kTcSmemTail) / ((size_t)S * (kTcBM + BN) * tune.kt * 2) >= 2) kt = tune.kt;
    const int lkt = kt == 64 ? 6 : kt == 32 ? 5 : 4;
    const int pitch = (maxk + kt - 1) / kt * kt;
    // slice stacks in the tile layouts; the row groups / blocks past the last
    // row cover what a 128-row A tile or 64-row B tile reads beyond it. A
    // symmetric product (B = A) keeps its A items in both layouts.
    const bool dual = b_items.empty();
    const int rows_bl = dual ? rows_a : rows_b;
    const int groups_a = (rows_a + 7) / 8 + kTcBM / 8, blocks_b = (rows_bl + 63) / 64 + 1;
    const size_t stack_a = (size_t)S * pitch * groups_a * 8, stack_b = (size_t)S * pitch * blocks_b * 64;
    void* sl = nullptr;
    if ((s = scratch_alloc(ctx, (stack_a + stack_b) * 2, &sl))) return cleanup(), s;
    owned.push_back(sl);
    auto* as = (__nv_bfloat16*)sl;
    auto* bs = as + stack_a;
    {
        const unsigned g = (unsigned)nblocks;
        if (f64)
            split_kernel<double, 0><<<g, 256, 0, ctx->stream>>>(segs, pitch, S, lkt, groups_a, blocks_b, dual ? 1 : 0,
                                                                maxbits, exps, as, bs);
        else
            split_kernel<float, 1><<<g, 256, 0, ctx->stream>>>(segs, pitch, S, lkt, groups_a, blocks_b, dual ? 1 : 0,
                                                               nullptr, nullptr, as, bs);
        if ((s = after_launch(ctx, "split_kernel"))) return cleanup(), s;
    }
    // products and accumulators
    TcGemmParams p;
    memset(&p, 0, sizeof(p));
    p.sa = S;
    p.sb = S;
    p.a_stack = as;
    p.b_stack = bs;
    p.a_groups = groups_a;
    p.b_blocks = blocks_b;
    // products A_a B_b with a + b < L, level a + b in TMEM slot a + b: for each
    // A slice, its B slices 0 .. L-1-a in runs of up to four per MMA
    int nm = 0;
    for (int a = 0; a < S && a < L; ++a) {
        const int nb = std::min(S, L - a);
        for (int b0 = 0; b0 < nb; b0 += kTcMaxStack) {
            if (nm >= kTcMaxMma) return cleanup(), fail(RSTSR_ERR_UNIMPLEMENTED, "too many slices");
            p.mma_a[nm] = (uint8_t)a;
            p.mma_b0[nm] = (uint8_t)b0;
            p.mma_n[nm] = (uint8_t)std::min(kTcMaxStack, nb - b0);
            ++nm;
        }
    }
    p.nmma = nm;
    p.nslots = L;
    p.out_f64 = f64 ? 1 : 0;
    p.exp_bias = -14;
    p.row_exp = exps;
    p.col_exp = exps ? (b_items.empty() ? exps : exps + rows_a) : nullptr;
    p.err = ctx->dev_err;
    p.group_m = tune.group;
    // FP32 accumulation truncates: Ozaki chunks of <= 1024 keep levels 0 to 3
    // exact; the f32 split sums chunks of 512 in C
    const int chunk = f64 ? std::max(1, 1024 / kt) : 512 / kt;
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
            s = launch_tc_gemm(ctx, kt, p, k_tiles_max, chunk);
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
    s = launch_tc_gemm(ctx, kt, p, k_tiles_max, chunk, (int64_t)tiles.size());
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
