// Multi-product tensor-core GEMM for sm_103a (tcgen05 + TMA + TMEM).
//
// Work unit: a 128 x 64 output tile and one K chunk of it. The operands are
// stacks of bf16 "slices" written by the split kernel directly in the tensor
// cores' shared-memory image (tc_tiled_offset): K tiles of width KT, each
// holding per slice the 8-row groups of all rows as core matrices (8 rows x
// 16 bytes, K-major, no swizzle). The rows of one tile of one slice are then a
// single contiguous block of 128 x KT (A) or 64 x KT (B) elements, fetched by
// one bulk copy: large sequential L2 requests instead of one 2 KT-byte
// request per row. Per K tile, one pipeline stage holds every slice of the A
// and B tiles, the B slices stacked along N. The products A_a * B_b accumulate in FP32 TMEM
// "level slots": slot l (columns 64 l .. 64 l + 63) sums every product with
// a + b = l. Since slot a + b follows slot a + b - 1, the products of one A
// slice with B slices b0 .. b0 + n - 1 are a single tcgen05.mma with N = 64 n
// (n <= 4) whose accumulator starts at slot a + b0: one MMA instruction per
// (A slice, run of up to four B slices) instead of one per product, each
// reading its A operand once. Measured on GB300: a 128 x N x 16 MMA takes
// max(N / 2, (4 KB + 32 N bytes) / 128 B per cycle) cycles, so N = 256 runs at
// the full 4096 MAC per cycle and SM, N = 64 at two thirds.
//
// The epilogue adds the slots (f64 output: exactly, in 64-bit fixed point;
// f32 output: in FP32 with a two-sum), applies per-row / per-column
// power-of-two scales, alpha and beta, and adds the K chunks after the first
// into C.
//
// This one kernel serves
//   * the Ozaki split for f64 (L integer slices, L level slots),
//   * the three-term bf16 split for f32 (hi/mid/lo, three level slots),
// for a single problem or for a list of problems (batched and grouped
// matmul) whose slices share one pair of TMA maps, read from a device tile
// list {problem, tile row, tile column}.
//
// Persistent: one CTA per SM walks tiles blockIdx.x, + gridDim.x, ... Roles
// (320 threads): warp 0 streams TMA loads through a ring of stages, warp 1
// owns TMEM and issues tcgen05.mma from one thread (descriptors precomputed in
// registers: an MMA loop that reads its product list from memory issued one
// MMA per ~90 cycles on GB300, slower than the MMAs), warps 2-9 are the
// epilogue (warp w reads TMEM lanes 32*(w%4)..+31, columns of half (w-2)/4).
// The epilogue copies a unit's slots into registers, zeroes them (the MMAs
// always accumulate: a stacked MMA cannot start some of its slots and add to
// others) and releases TMEM, so that the next unit's MMAs run while it
// converts and stores. All waits are bounded (tc_ptx.cuh); on a timeout the
// CTA records an error code in p.err and unwinds.
#pragma once

#include "common.cuh"
#include "tc_ptx.cuh"

namespace rstsr {

constexpr int kTcBM = 128;
// Tile width = level slot width: eight slots of 64 columns fill the 512 TMEM
// columns, and 32 columns per epilogue warp fit its registers (three warps per
// scheduler leave 168 registers a thread).
constexpr int kTcBN = 64;
constexpr int kTcEpiWarps = 8;
constexpr int kTcThreads = 64 + 32 * kTcEpiWarps;
constexpr int kTcMaxStages = 8;
constexpr int kTcMaxSlots = 8;
constexpr int kTcMaxMma = 16;      // MMA instructions per 16-wide K step
constexpr int kTcMaxStack = 4;     // B slices stacked in one MMA (N <= 256)
constexpr uint32_t kTcTmemCols = 512;

// error codes written to p.err
constexpr int kTcErrProducerWait = 1;
constexpr int kTcErrMmaWait = 2;
constexpr int kTcErrEpilogueWait = 3;
constexpr int kTcErrTmemWait = 4;

// One problem of a grouped launch (device memory).
struct TcProblem {
    int32_t M, N;
    int32_t k_tiles;          // K tiles of this problem
    int32_t a_row0, b_row0;   // first row of this problem in every slice of A / B
    int32_t row_exp0, col_exp0;
    int32_t symmetric;
    void* C;
    int64_t ldc;
    double alpha, beta;
};

// Element (slice s, row, k) of an operand stack of S slices whose rows are
// padded to 8 * G: K tile kt = k / KT holds, per slice, G row groups of KT / 8
// core matrices of 8 x 8 elements.
__host__ __device__ __forceinline__ size_t tc_tiled_offset(int S, int G, int KT, int s, int row, int k) {
    const int kt = k / KT, kk = k % KT;
    return (((size_t)kt * S + s) * G + (size_t)(row >> 3)) * (size_t)(8 * KT) + (size_t)((kk >> 3) * 64) +
           (size_t)((row & 7) * 8 + (k & 7));
}

struct TcGemmParams {
    const __nv_bfloat16* a_stack;  // operand stacks (tc_tiled_offset layout)
    const __nv_bfloat16* b_stack;
    int32_t a_groups, b_groups;  // G of each stack
    int32_t M, N;                // single-problem mode: output extent
    int32_t k_tiles;             // single-problem mode: K tiles
    int32_t chunk_tiles;         // K tiles summed in TMEM before the epilogue adds them to C
    int32_t ntiles;              // output tiles
    int32_t sa, sb;              // slices of A and B
    int32_t nslots;              // level slots in TMEM
    int32_t nmma;                // MMA instructions per 16-wide K step:
    uint8_t mma_a[kTcMaxMma];    //   A slice,
    uint8_t mma_b0[kTcMaxMma];   //   first B slice (slot mma_a + mma_b0),
    uint8_t mma_n[kTcMaxMma];    //   B slices stacked (N = 64 n)
    int32_t stages;
    uint32_t a_tile_bytes;       // 128 x KT bf16
    uint32_t b_tile_bytes;       // BN x KT bf16
    uint32_t stage_bytes;        // sa A tiles + sb B tiles
    // epilogue
    void* C;
    int64_t ldc;                 // row-major leading dimension of C (elements)
    int32_t out_f64;             // 1: C is f64, 0: C is f32
    double alpha, beta;
    const int32_t* row_exp;      // per-row power-of-two exponent (or null)
    const int32_t* col_exp;      // per-column exponent (or null)
    int32_t exp_bias;
    int32_t symmetric;           // lower triangle only (row >= col), mirrored
    int32_t tiles_m, tiles_n;
    int32_t group_m;             // raster swizzle: tiles grouped along M
    // grouped mode (tiles != null): tile t is tiles[t] = {problem, tm, tn, 0}
    const int4* tiles;
    const TcProblem* problems;
    int* err;
};

// Tile of a single-problem launch. Symmetric problems enumerate, column tile
// by column tile, the tiles that hold at least one element with row >= col.
template <int BN>
__device__ __forceinline__ void tc_tile_coords(const TcGemmParams& p, int bid, int& tm, int& tn) {
    if (p.symmetric) {
        int rem = bid;
        for (int j = 0; j < p.tiles_n; ++j) {
            const int first = (j * BN) / kTcBM;
            const int cnt = p.tiles_m - first;
            if (rem < cnt) {
                tm = first + rem;
                tn = j;
                return;
            }
            rem -= cnt;
        }
        tm = tn = 0;
        return;
    }
    // grouped raster: consecutive tiles share B tiles within a group of rows
    const int per_group = p.group_m * p.tiles_n;
    const int g = bid / per_group;
    const int first_m = g * p.group_m;
    const int gm = min(p.tiles_m - first_m, p.group_m);
    const int in_g = bid - g * per_group;
    tm = first_m + in_g % gm;
    tn = in_g / gm;
}

// One output tile with its problem's parameters.
struct TcUnit {
    int32_t tm, tn, M, N, a_row0, b_row0, k_tiles, symmetric;
    void* C;
    int64_t ldc;
    double alpha, beta;
    const int32_t* row_exp;
    const int32_t* col_exp;
};

template <int BN>
__device__ __forceinline__ void tc_resolve(const TcGemmParams& p, int t, TcUnit& u) {
    if (p.tiles) {
        const int4 e = p.tiles[t];
        const TcProblem q = p.problems[e.x];
        u.tm = e.y;
        u.tn = e.z;
        u.M = q.M;
        u.N = q.N;
        u.a_row0 = q.a_row0;
        u.b_row0 = q.b_row0;
        u.k_tiles = q.k_tiles;
        u.symmetric = q.symmetric;
        u.C = q.C;
        u.ldc = q.ldc;
        u.alpha = q.alpha;
        u.beta = q.beta;
        u.row_exp = p.row_exp ? p.row_exp + q.row_exp0 : nullptr;
        u.col_exp = p.col_exp ? p.col_exp + q.col_exp0 : nullptr;
    } else {
        tc_tile_coords<BN>(p, t, u.tm, u.tn);
        u.M = p.M;
        u.N = p.N;
        u.a_row0 = 0;
        u.b_row0 = 0;
        u.k_tiles = p.k_tiles;
        u.symmetric = p.symmetric;
        u.C = p.C;
        u.ldc = p.ldc;
        u.alpha = p.alpha;
        u.beta = p.beta;
        u.row_exp = p.row_exp;
        u.col_exp = p.col_exp;
    }
}

// ---- epilogue arithmetic. GB300 runs FP64 instructions at a small fraction
// of its FP32 and integer rates, so the f64 epilogue adds the FP32
// accumulators as 64-bit fixed-point integers and builds the double from its
// bits; the f32 epilogue stays in FP32 with an error-free two-sum.

// trunc(f 2^37) for an accumulator f given as bits. The accumulators of one K
// chunk of at most 1024 stay below 2^24.1 in magnitude, so the sum of all of
// them stays below 2^62; the truncation error is below 2^-37 per accumulator.
__device__ __forceinline__ long long acc_fixed37(uint32_t u) {
    const int e = (int)((u >> 23) & 0xFF);
    const long long m = (long long)((u & 0x7FFFFFu) | 0x800000u);
    const int sh = e - 113;  // f 2^37 = m 2^(e - 150 + 37)
    long long v = sh >= 0 ? m << min(sh, 39) : m >> min(-sh, 63);
    if (e == 0) v = 0;
    return (u >> 31) ? -v : v;
}

// v 2^e rounded to the nearest double (ties to even) into *out; false when the
// result is subnormal or overflows (left to epilogue_rare).
__device__ __forceinline__ bool fixed_to_double(long long v, int e, double* out) {
    const unsigned long long sgn = v < 0 ? (1ull << 63) : 0ull;
    const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
    const int lz = __clzll((long long)a);
    const unsigned long long n = a << lz;  // leading one at bit 63
    unsigned long long mant = n >> 11;     // 53 bits with the leading one
    const unsigned long long rem = n & 0x7FFull;
    mant += (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) ? 1ull : 0ull;
    const int be = 63 - lz + e + 1023;  // biased exponent
    // the leading one of mant adds 1 to (be - 1); a rounding carry to 2^53 adds one more
    *out = __longlong_as_double(
        (long long)(a == 0 ? 0ull : sgn | (((unsigned long long)(be - 1) << 52) + mant)));
    return a == 0 || (be >= 1 && be <= 2046);
}

// Out-of-line so that its FP64 instructions stay off the common path.
// special: 2 NaN, 1 +inf, -1 -inf (non-finite accumulators, from inf/NaN
// inputs, summed as IEEE would), 0: v 2^e outside the normal range of double.
static __device__ __noinline__ double epilogue_rare(long long v, int e, int special) {
    if (special == 2) return __longlong_as_double(0x7FF8000000000000ll);
    if (special == 1) return __longlong_as_double(0x7FF0000000000000ll);
    if (special == -1) return __longlong_as_double((long long)0xFFF0000000000000ull);
    return ldexp((double)v, e);
}

// Zero this warp's columns of every level slot, then tell the MMA thread that
// TMEM is free for the next unit.
template <int BN>
__device__ __forceinline__ void tc_zero_release(const TcGemmParams& p, uint32_t tbase, uint64_t* tmem_empty,
                                                int lane) {
    for (int a = 0; a < p.nslots; ++a) {
#pragma unroll
        for (int j0 = 0; j0 < BN / 2; j0 += 16) tc::tmem_st_zero_x16(tbase + (uint32_t)(a * BN + j0));
    }
    tc::tmem_st_wait();
    tc::tc_fence_before();
    __syncwarp();
    if (lane == 0) tc::mbar_arrive(tmem_empty);
}

// Load this warp's EC (= 32) columns of level slot a.
template <int BN, int EC>
__device__ __forceinline__ void tc_load_slot(uint32_t tbase, int a, uint32_t (&r)[EC]) {
    static_assert(EC == 32, "two 16-column loads per slot");
    tc::tmem_ld_32x32b_x16(tbase + (uint32_t)(a * BN), r);
    tc::tmem_ld_32x32b_x16(tbase + (uint32_t)(a * BN + 16), r + 16);
    tc::tmem_ld_wait();
}

// f64 epilogue of one unit for this thread's row and EC columns from col0.
template <int BN, int EC>
__device__ __forceinline__ void tc_epilogue_f64(const TcGemmParams& p, const TcUnit& u, uint32_t tbase,
                                                uint64_t* tmem_empty, int64_t row, int64_t col0, int mode,
                                                int lane, int* colexp) {
    long long fx[EC];
    unsigned long long m_nan = 0, m_pinf = 0, m_ninf = 0;
#pragma unroll
    for (int i = 0; i < EC; ++i) fx[i] = 0;
    for (int a = 0; a < p.nslots; ++a) {
        uint32_t r[EC];
        tc_load_slot<BN, EC>(tbase, a, r);
#pragma unroll
        for (int i = 0; i < EC; ++i) {
            const uint32_t x = r[i];
            fx[i] += acc_fixed37(x);
            if ((x & 0x7F800000u) == 0x7F800000u) {
                const unsigned long long bit = 1ull << i;
                if (x & 0x7FFFFFu) m_nan |= bit;
                else if (x >> 31) m_ninf |= bit;
                else m_pinf |= bit;
            }
        }
    }
    // the slots are in registers: zero them for the next unit's MMAs
    tc_zero_release<BN>(p, tbase, tmem_empty, lane);
    // column exponents of this warp's columns, staged in its shared-memory slot
    for (int j = lane; j < EC; j += 32) {
        const int64_t col = col0 + j;
        colexp[j] = (u.col_exp && col < u.N) ? u.col_exp[col] : 0;
    }
    __syncwarp();
    if (row >= u.M) return;
    const int rexp = (u.row_exp ? u.row_exp[row] : 0) + p.exp_bias - 37;
    const bool scale = u.alpha != 1.0;
    double* Cd = reinterpret_cast<double*>(u.C);
    const unsigned long long m_any = m_nan | m_pinf | m_ninf;
#pragma unroll
    for (int i = 0; i < EC; ++i) {
        const int64_t col = col0 + i;
        if (col >= u.N) break;
        if (u.symmetric && col > row) continue;  // upper triangle: written by the mirror
        const int e = rexp + colexp[i];
        double x;
        const unsigned long long bit = 1ull << i;
        if (!fixed_to_double(fx[i], e, &x) || (m_any & bit)) {
            const int special = (m_nan & bit) || ((m_pinf & bit) && (m_ninf & bit)) ? 2
                                : (m_pinf & bit)                                    ? 1
                                : (m_ninf & bit)                                    ? -1
                                                                                    : 0;
            x = epilogue_rare(fx[i], e, special);
        }
        if (scale) x *= u.alpha;
        double* dst = Cd + row * u.ldc + col;
        if (mode == 1) x += *dst;
        else if (mode == 2) x = fma(u.beta, *dst, x);
        *dst = x;
        if (u.symmetric && col != row) Cd[col * u.ldc + row] = x;
    }
}

// f32 epilogue: alpha (acc_0 + sum_{a>0} acc_a) + c with c = beta C (first K
// chunk) or C (later chunks); alpha acc_0 + c is added by an exact two-sum.
template <int BN, int EC>
__device__ __forceinline__ void tc_epilogue_f32(const TcGemmParams& p, const TcUnit& u, uint32_t tbase,
                                                uint64_t* tmem_empty, int64_t row, int64_t col0, int mode,
                                                int lane) {
    float s0[EC], t[EC];
    for (int a = 0; a < p.nslots; ++a) {
        uint32_t r[EC];
        tc_load_slot<BN, EC>(tbase, a, r);
#pragma unroll
        for (int i = 0; i < EC; ++i) {
            const float x = __uint_as_float(r[i]);
            if (a == 0) s0[i] = x, t[i] = 0.f;
            else t[i] += x;
        }
    }
    tc_zero_release<BN>(p, tbase, tmem_empty, lane);
    if (row >= u.M) return;
    const float af = (float)u.alpha, bf = (float)u.beta;
    float* Cf = reinterpret_cast<float*>(u.C);
#pragma unroll
    for (int i = 0; i < EC; ++i) {
        const int64_t col = col0 + i;
        if (col >= u.N) break;
        if (u.symmetric && col > row) continue;
        float* dst = Cf + row * u.ldc + col;
        const float ph = af * s0[i], pl = fmaf(af, s0[i], -ph);
        float ch = 0.f, cl = 0.f;
        if (mode == 1) {
            ch = *dst;
        } else if (mode == 2) {
            const float c = *dst;
            ch = bf * c;
            cl = fmaf(bf, c, -ch);
        }
        const float sh = ph + ch, bb = sh - ph;
        const float se = (ph - (sh - bb)) + (ch - bb);
        const float y = sh + (se + pl + cl + af * t[i]);
        *dst = y;
        if (u.symmetric && col != row) Cf[col * u.ldc + row] = y;
    }
}

// Dynamic shared memory: the stages, then kTcSmemTail bytes of barriers,
// TMEM slot, abort flag (256 bytes) and the epilogue warps' column-exponent
// slots (64 ints each), plus 1024 bytes of alignment slack in front.
constexpr size_t kTcSmemTail = 256 + kTcEpiWarps * 64 * 4;
constexpr size_t kTcSmemMax = 232448;

template <int KT, int BN, bool F64>
__global__ void __launch_bounds__(kTcThreads, 1) tc_gemm_kernel(const TcGemmParams p) {
    constexpr int EC = BN / 2;  // columns per epilogue warp
    static_assert(EC <= 64, "column masks and exponent slots hold 64 columns");
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)p.stages * p.stage_bytes);
    uint64_t* empty = full + kTcMaxStages;
    uint64_t* accum_full = empty + kTcMaxStages;
    uint64_t* tmem_empty = accum_full + 1;
    uint64_t* mma_done = tmem_empty + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    int* colexp_all = reinterpret_cast<int*>(reinterpret_cast<uint8_t*>(full) + 256);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t stages = (uint32_t)p.stages;

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < stages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(accum_full, 1);
        tc::mbar_init(tmem_empty, kTcEpiWarps);
        tc::mbar_init(mma_done, 1);
        *abort_flag = 0;
        tc::fence_barrier_init();
    }
    if (warp == 1) tc::tmem_alloc(tmem_slot, kTcTmemCols);
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t it = 0, issued = 0;
            bool stop = false;
            for (int t = blockIdx.x; t < p.ntiles && !stop; t += gridDim.x) {
                TcUnit u;
                tc_resolve<BN>(p, t, u);
                for (int kt = 0; kt < u.k_tiles; ++kt, ++it) {
                    const uint32_t s = it % stages;
                    const uint32_t ph = (it / stages) & 1u;
                    if (it >= stages && !tc::mbar_wait(&empty[s], ph ^ 1u)) {
                        atomicExch(p.err, kTcErrProducerWait);
                        *abort_flag = 1;
                    }
                    if (*abort_flag) {
                        stop = true;
                        break;
                    }
                    uint8_t* st = smem + (size_t)s * p.stage_bytes;
                    tc::mbar_arrive_expect_tx(&full[s], p.stage_bytes);
                    const int ga = (u.a_row0 + u.tm * kTcBM) >> 3, gb = (u.b_row0 + u.tn * BN) >> 3;
                    for (int a = 0; a < p.sa; ++a)
                        tc::bulk_load(st + (size_t)a * p.a_tile_bytes,
                                      p.a_stack + (((size_t)kt * p.sa + a) * p.a_groups + ga) * (8 * KT),
                                      p.a_tile_bytes, &full[s]);
                    uint8_t* sb = st + (size_t)p.sa * p.a_tile_bytes;
                    for (int b = 0; b < p.sb; ++b)
                        tc::bulk_load(sb + (size_t)b * p.b_tile_bytes,
                                      p.b_stack + (((size_t)kt * p.sb + b) * p.b_groups + gb) * (8 * KT),
                                      p.b_tile_bytes, &full[s]);
                    issued = it + 1;
                }
            }
            // never leave the CTA with copies in flight: wait (bounded) for the
            // last use of every stage that was issued
            for (uint32_t s = 0; s < stages && s < issued; ++s) {
                const uint32_t last = s + ((issued - 1 - s) / stages) * stages;
                tc::mbar_wait(&full[s], (last / stages) & 1u);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            // the MMA list of one 16-wide K step as descriptor offsets (16-byte
            // units, relative to the stage), instruction descriptors and TMEM
            // addresses, kept in registers
            uint32_t a_off[kTcMaxMma], b_off[kTcMaxMma], idesc[kTcMaxMma], dcol[kTcMaxMma];
            const int nmma = min(p.nmma, kTcMaxMma);
#pragma unroll
            for (int q = 0; q < kTcMaxMma; ++q) {
                const int qq = q < nmma ? q : 0;
                a_off[q] = ((uint32_t)p.mma_a[qq] * p.a_tile_bytes) >> 4;
                b_off[q] = ((uint32_t)p.sa * p.a_tile_bytes + (uint32_t)p.mma_b0[qq] * p.b_tile_bytes) >> 4;
                idesc[q] = tc::idesc_bf16_f32(kTcBM, (uint32_t)BN * p.mma_n[qq]);
                dcol[q] = tmem_base + (uint32_t)(p.mma_a[qq] + p.mma_b0[qq]) * BN;
            }
            // core matrices: 128 bytes apart along K, 16 KT bytes apart along M/N
            const uint64_t desc_hi = tc::smem_desc_noswizzle(128, 16 * KT);
            uint32_t it = 0, unit = 0;
            bool stop = false;
            for (int t = blockIdx.x; t < p.ntiles && !stop; t += gridDim.x) {
                TcUnit u;
                tc_resolve<BN>(p, t, u);
                for (int c0 = 0; c0 < u.k_tiles && !stop; c0 += p.chunk_tiles, ++unit) {
                    // the epilogue has copied out and zeroed the previous unit's slots
                    if (!tc::mbar_wait(tmem_empty, unit & 1u)) {
                        atomicExch(p.err, kTcErrTmemWait);
                        *abort_flag = 1;
                    }
                    if (*abort_flag) {
                        stop = true;
                        break;
                    }
                    tc::tc_fence_after();
                    const int c1 = min(c0 + p.chunk_tiles, u.k_tiles);
                    for (int kt = c0; kt < c1; ++kt, ++it) {
                        const uint32_t s = it % stages;
                        const uint32_t ph = (it / stages) & 1u;
                        if (!tc::mbar_wait(&full[s], ph)) {
                            atomicExch(p.err, kTcErrMmaWait);
                            *abort_flag = 1;
                        }
                        if (*abort_flag) {
                            stop = true;
                            break;
                        }
                        tc::tc_fence_after();
                        const uint32_t st4 = tc::smem_u32(smem + (size_t)s * p.stage_bytes) >> 4;
#pragma unroll
                        for (int j = 0; j < KT / 16; ++j) {
#pragma unroll
                            for (int q = 0; q < kTcMaxMma; ++q) {
                                if (q >= nmma) break;
                                // the j-th 16-wide K step starts two core matrices (256 bytes) later
                                const uint64_t ad = desc_hi | (uint64_t)((st4 + a_off[q] + 16 * j) & 0x3FFF);
                                const uint64_t bd = desc_hi | (uint64_t)((st4 + b_off[q] + 16 * j) & 0x3FFF);
                                tc::mma_f16(dcol[q], ad, bd, idesc[q], 1u);
                            }
                        }
                        tc::mma_commit(&empty[s]);
                    }
                    if (!stop) tc::mma_commit(accum_full);
                }
            }
            // every MMA issued by this thread completes before TMEM is released
            tc::mma_commit(mma_done);
            tc::mbar_wait(mma_done, 0);
        }
        __syncwarp();
    } else {
        const int quad = warp & 3, half = (warp - 2) >> 2;
        const uint32_t tbase = tmem_base + ((uint32_t)(quad * 32) << 16) + (uint32_t)(half * EC);
        tc_zero_release<BN>(p, tbase, tmem_empty, lane);  // the slots start at zero
        uint32_t unit = 0;
        bool stop = false;
        for (int t = blockIdx.x; t < p.ntiles && !stop; t += gridDim.x) {
            TcUnit u;
            tc_resolve<BN>(p, t, u);
            const int64_t row = (int64_t)u.tm * kTcBM + quad * 32 + lane;
            const int64_t col0 = (int64_t)u.tn * BN + half * EC;
            for (int c0 = 0; c0 < u.k_tiles; c0 += p.chunk_tiles, ++unit) {
                // converged warp, warp-uniform outcome: the TMEM loads below are
                // warp-collective (lanes past the last row leave the previous
                // unit's stores early)
                __syncwarp();
                const bool waited = tc::mbar_wait(accum_full, unit & 1u);
                if (!__all_sync(0xffffffffu, waited && !*abort_flag)) {
                    if (!waited) atomicExch(p.err, kTcErrEpilogueWait);
                    *abort_flag = 1;
                    stop = true;
                    break;
                }
                tc::tc_fence_after();
                const int mode = c0 > 0 ? 1 : (u.beta != 0.0 ? 2 : 0);
                if constexpr (F64)
                    tc_epilogue_f64<BN, EC>(p, u, tbase, tmem_empty, row, col0, mode, lane,
                                            colexp_all + (warp - 2) * 64);
                else
                    tc_epilogue_f32<BN, EC>(p, u, tbase, tmem_empty, row, col0, mode, lane);
            }
        }
    }
    // every warp reconverges before the CTA barrier (a warp that reaches an
    // aligned barrier diverged can release it early)
    __syncwarp();
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem_base, kTcTmemCols);
    }
}

// A strided operand viewed as [rows, K]: element (r, k) at ptr[r*s_row + k*s_k].
struct Operand {
    const void* ptr;
    int64_t s_row, s_k;
};

// Launch tc_gemm_kernel<KT, kTcBN, f64 output> once over
// all tiles and K chunks described by p: single-problem mode (p.tiles null,
// k_tiles_total K tiles) or grouped mode (p.tiles / p.problems set,
// `ntiles_grouped` tiles). k_chunk_tiles: K tiles per TMEM accumulation.
// p.a_stack / b_stack / a_groups / b_groups describe the operand stacks.
int launch_tc_gemm(rstsr_ctx* ctx, int kt, TcGemmParams p, int k_tiles_total, int k_chunk_tiles,
                   int64_t ntiles_grouped = 0);

}  // namespace rstsr
