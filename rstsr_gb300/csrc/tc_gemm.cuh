// Multi-product tensor-core GEMM for sm_103a (tcgen05 + bulk copies + TMEM).
//
// Work unit: a 128 x 64 output tile and one K chunk of it. The operands are
// stacks of bf16 "slices" written by the split kernel directly in the tensor
// cores' shared-memory image: core matrices of 8 rows x 16 bytes (K-major, no
// swizzle), ordered so that every slice of one operand tile in one K tile of
// width KT is a single contiguous block (tc_offset_a: row group, then slice;
// tc_offset_b: 64-row block, then slice, then row group). A pipeline stage is
// then two bulk copies. Measured on GB300: the copy count, not the bytes,
// bounds a SM's intake (16 B per cycle with 2 KB copies, 50 with one 43 KB
// copy), and a stage of this kernel needs about 46 B per cycle to keep the
// tensor cores busy. In shared memory the B slices are stacked along N. The
// products A_a * B_b accumulate in FP32 TMEM
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
// matmul) whose slices share one pair of operand stacks, read from a device
// tile list {problem, tile row, tile column}.
//
// Persistent: one CTA per SM walks tiles blockIdx.x, + gridDim.x, ... Roles
// (576 threads): warp 0 streams bulk copies through a ring of stages, warp 1
// owns TMEM and issues tcgen05.mma from one thread, warps 2-17 are the
// epilogue (warp w reads TMEM lanes 32*(w%4)..+31 and 16 columns of part
// (w-2)/4). Measured
// on GB300 for 7 slices: the MMAs of a 16-wide K step take 921 cycles alone;
// behind the stage barrier wait of one issuing thread they take about 1150
// (the MMA queue is shallower than the wait).
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
// columns.
constexpr int kTcBN = 64;
// Sixteen epilogue warps, four per TMEM lane quadrant with 16 columns each:
// draining TMEM is latency-bound, and the MMAs wait for it at every unit of a
// single-buffered problem (five warps per scheduler leave 96 registers a
// thread).
constexpr int kTcEpiWarps = 16;
constexpr int kTcEpiCols = kTcBN * 4 / kTcEpiWarps;
constexpr int kTcEpiWarp0 = 2;    // first epilogue warp
constexpr int kTcThreads = 32 * (kTcEpiWarp0 + kTcEpiWarps);
constexpr int kTcMaxStages = 8;
constexpr int kTcMaxSlots = 8;
constexpr int kTcMaxMma = 12;      // MMA instructions per 16-wide K step (11 for 8 slices)
constexpr int kTcMaxStack = 4;     // B slices stacked in one MMA (N <= 256)
constexpr uint32_t kTcTmemCols = 512;
constexpr int kTcMaxBands = 64;    // row bands of the symmetric tile order
constexpr uint32_t kTcBufCols = 256;  // second accumulator buffer (when the slots fit twice)

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

// Element (slice s, row, k) of the A operand stack (S slices, G row groups):
// K tile kt = k / KT holds, per row group, the S slices' KT / 8 core matrices
// of 8 x 8 elements. Slice s + 1 lies 8 KT elements after slice s; a 128-row
// tile is 16 consecutive row groups.
__host__ __device__ __forceinline__ size_t tc_offset_a(int S, int G, int KT, int s, int row, int k) {
    const int kt = k / KT, kk = k % KT;
    return (((size_t)kt * G + (size_t)(row >> 3)) * S + s) * (size_t)(8 * KT) + (size_t)((kk >> 3) * 64) +
           (size_t)((row & 7) * 8 + (k & 7));
}

// Element (slice s, row, k) of the B operand stack (S slices, NB blocks of 64
// rows): K tile kt holds, per 64-row block, the S slices' 8 row groups. Slice
// s + 1 lies 64 KT elements after slice s.
__host__ __device__ __forceinline__ size_t tc_offset_b(int S, int NB, int KT, int s, int row, int k) {
    const int kt = k / KT, kk = k % KT;
    return ((((size_t)kt * NB + (size_t)(row >> 6)) * S + s) * 8 + (size_t)((row >> 3) & 7)) * (size_t)(8 * KT) +
           (size_t)((kk >> 3) * 64) + (size_t)((row & 7) * 8 + (k & 7));
}

struct TcGemmParams {
    const __nv_bfloat16* a_stack;  // operand stacks (tc_offset_a / tc_offset_b layouts)
    const __nv_bfloat16* b_stack;
    int32_t a_groups;            // G: 8-row groups of the A stack
    int32_t b_blocks;            // NB: 64-row blocks of the B stack
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
    int32_t nbuf;                // TMEM accumulator buffers (2 when 2 * nslots * BN <= 512)
    // symmetric order: bands of band_rows row tiles; band g's first tile
    int32_t band_rows, nbands;
    int32_t band_first[kTcMaxBands + 1];
    // grouped mode (tiles != null): tile t is tiles[t] = {problem, tm, tn, 0}
    const int4* tiles;
    const TcProblem* problems;
    int* err;
};

// Tile of a single-problem launch. Symmetric problems enumerate the tiles that
// hold an element with row >= col (row tile tm, column tile j with j / 2 <=
// tm) band by band: band g is row tiles [g R, g R + R) (R = band_rows), its
// columns left to right, each column's rows top to bottom. A band's A rows
// stay in L2 while its columns stream by; a plain column-by-column order
// re-reads all of A from HBM once per column. Other problems use a grouped
// raster: group_m row tiles share each B tile.
template <int BN>
__device__ __forceinline__ void tc_tile_coords(const TcGemmParams& p, int bid, int& tm, int& tn) {
    static_assert(2 * BN == kTcBM, "column tile j first meets the lower triangle at row tile j / 2");
    if (p.symmetric) {
        int g = 0;
        while (g + 1 < p.nbands && p.band_first[g + 1] <= bid) ++g;
        const int bs = g * p.band_rows, be = min(bs + p.band_rows, p.tiles_m), h = be - bs;
        const int jmax = min(2 * be, p.tiles_n), nf = min(2 * bs + 2, jmax);
        int t = bid - p.band_first[g];
        if (t < nf * h) {
            tn = t / h;
            tm = bs + t % h;
            return;
        }
        t -= nf * h;
        for (int j = nf; j < jmax; ++j) {
            const int first = j >> 1, cnt = be - first;
            if (t < cnt) {
                tm = first + t;
                tn = j;
                return;
            }
            t -= cnt;
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
// of its FP32 and integer rates, so the f64 epilogue adds the FP32 level slots
// as 64-bit fixed-point integers (2^-37 units) and builds the double from its
// bits; the f32 epilogue stays in FP32 with an error-free two-sum.

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
template <int BN, int EC>
__device__ __forceinline__ void tc_zero_release(const TcGemmParams& p, uint32_t tbase, uint64_t* tmem_empty,
                                                int lane) {
    static_assert(EC == 16, "one 16-column store per slot");
    for (int a = 0; a < p.nslots; ++a) tc::tmem_st_zero_x16(tbase + (uint32_t)(a * BN));
    tc::tmem_st_wait();
    tc::tc_fence_before();
    __syncwarp();
    if (lane == 0) tc::mbar_arrive(tmem_empty);
}

// Load this warp's EC (= 16) columns of level slot a.
template <int BN, int EC>
__device__ __forceinline__ void tc_load_slot(uint32_t tbase, int a, uint32_t (&r)[EC]) {
    static_assert(EC == 16, "one 16-column load per slot");
    tc::tmem_ld_32x32b_x16(tbase + (uint32_t)(a * BN), r);
    tc::tmem_ld_wait();
}

// Per-warp staging tile for C: each lane holds one row of the warp's 32 x EC
// block, so direct stores from registers touch 32 rows per instruction (the
// L1 then serialises 32 wavefronts). Through the tile, an instruction covers
// 32 / W rows of W neighbouring columns (W = 8 for 8-byte, 16 for 4-byte
// elements). Measured on GB300 before: the f32 split's epilogue spent ~25k
// cycles per K chunk on the read-modify-write of C.
constexpr int kTcStageBytes = 32 * 9 * 8;  // 32 rows x (8 + 1) doubles or (16 + 1) floats

template <typename T, int EC>
__device__ __forceinline__ void warp_store_block(T* C, int64_t ldc, int64_t r0, int64_t c0, int64_t M, int64_t N,
                                                 bool symmetric, const T (&v)[EC], T* stg, int lane) {
    constexpr int W = sizeof(T) == 8 ? 8 : 16;  // columns per pass
    constexpr int P = W + 1;                    // padded row pitch
    constexpr int RPI = 32 / W;                 // rows per instruction
#pragma unroll
    for (int h = 0; h < EC / W; ++h) {
        __syncwarp();
#pragma unroll
        for (int i = 0; i < W; ++i) stg[lane * P + i] = v[h * W + i];
        __syncwarp();
#pragma unroll
        for (int it = 0; it < 32 / RPI; ++it) {
            const int rr = it * RPI + lane / W, cc = lane % W;
            const int64_t row = r0 + rr, col = c0 + h * W + cc;
            if (row < M && col < N && !(symmetric && col > row)) C[row * ldc + col] = stg[rr * P + cc];
        }
    }
}

template <typename T, int EC>
__device__ __forceinline__ void warp_load_block(const T* C, int64_t ldc, int64_t r0, int64_t c0, int64_t M,
                                                int64_t N, T (&v)[EC], T* stg, int lane) {
    constexpr int W = sizeof(T) == 8 ? 8 : 16;
    constexpr int P = W + 1;
    constexpr int RPI = 32 / W;
#pragma unroll
    for (int h = 0; h < EC / W; ++h) {
        __syncwarp();
#pragma unroll
        for (int it = 0; it < 32 / RPI; ++it) {
            const int rr = it * RPI + lane / W, cc = lane % W;
            const int64_t row = r0 + rr, col = c0 + h * W + cc;
            stg[rr * P + cc] = (row < M && col < N) ? C[row * ldc + col] : (T)0;
        }
        __syncwarp();
#pragma unroll
        for (int i = 0; i < W; ++i) v[h * W + i] = stg[lane * P + i];
    }
}

// f64 epilogue of one unit for this thread's row and EC columns from col0.
template <int BN, int EC>
__device__ __forceinline__ void tc_epilogue_f64(const TcGemmParams& p, const TcUnit& u, uint32_t tbase,
                                                uint64_t* tmem_empty, int64_t row, int64_t col0, int mode,
                                                int lane, int* colexp, double* stg) {
    long long fx[EC];
    float fs[EC];  // FP32 sum of the slots: non-finite iff a slot is (inf / NaN inputs)
#pragma unroll
    for (int i = 0; i < EC; ++i) fx[i] = 0, fs[i] = 0.f;
    for (int a = 0; a < p.nslots; ++a) {
        uint32_t r[EC];
        tc_load_slot<BN, EC>(tbase, a, r);
        // slot a as fixed point at 2^-37: levels 0-3 hold integers times
        // 2^(-7a) below 2^24.7 (K chunk <= 1024, digits |d_0| <= 128, |d_s| <=
        // 64), converted exactly; higher levels are below 2^-3, converted at
        // 2^-34 (error below 2^-35 a slot)
        const float sc = __int_as_float((127 + (a < 4 ? 7 * a : 34)) << 23);
        const int sh = a < 4 ? 37 - 7 * a : 3;
#pragma unroll
        for (int i = 0; i < EC; ++i) {
            const float v = __uint_as_float(r[i]);
            fx[i] += (long long)__float2int_rn(v * sc) << sh;
            fs[i] += v;
        }
    }
    // the slots are in registers: zero them for the next unit's MMAs
    tc_zero_release<BN, EC>(p, tbase, tmem_empty, lane);
    // column exponents of this warp's columns, staged in its shared-memory slot
    for (int j = lane; j < EC; j += 32) {
        const int64_t col = col0 + j;
        colexp[j] = (u.col_exp && col < u.N) ? u.col_exp[col] : 0;
    }
    __syncwarp();
    // every lane takes part in the staged loads and stores below; rows past
    // the last one compute garbage that is never stored
    const int rexp = (u.row_exp && row < u.M ? u.row_exp[row] : 0) + p.exp_bias - 37;
    double x[EC];
#pragma unroll
    for (int i = 0; i < EC; ++i) {
        const int e = rexp + colexp[i];
        if (!fixed_to_double(fx[i], e, &x[i]) || !isfinite(fs[i]))
            x[i] = epilogue_rare(fx[i], e, isnan(fs[i]) ? 2 : isinf(fs[i]) ? (fs[i] > 0 ? 1 : -1) : 0);
        if (u.alpha != 1.0) x[i] *= u.alpha;
    }
    double* Cd = reinterpret_cast<double*>(u.C);
    const int64_t r0 = row - lane;
    if (mode != 0) {  // C of the later K chunks / beta C, 8 columns at a time
#pragma unroll
        for (int h = 0; h < EC / 8; ++h) {
            double c[8];
            warp_load_block<double, 8>(Cd, u.ldc, r0, col0 + 8 * h, u.M, u.N, c, stg, lane);
#pragma unroll
            for (int i = 0; i < 8; ++i)
                x[8 * h + i] = mode == 1 ? x[8 * h + i] + c[i] : fma(u.beta, c[i], x[8 * h + i]);
        }
    }
    warp_store_block<double, EC>(Cd, u.ldc, r0, col0, u.M, u.N, u.symmetric != 0, x, stg, lane);
    if (u.symmetric && row < u.M) {
        // the mirror of the lower triangle: lanes are neighbouring rows, so
        // these stores are contiguous along row `col` of C
#pragma unroll
        for (int i = 0; i < EC; ++i) {
            const int64_t col = col0 + i;
            if (col < u.N && col < row) Cd[col * u.ldc + row] = x[i];
        }
    }
}

// f32 epilogue: alpha (acc_0 + sum_{a>0} acc_a) + c with c = beta C (first K
// chunk) or C (later chunks); alpha acc_0 + c is added by an exact two-sum.
template <int BN, int EC>
__device__ __forceinline__ void tc_epilogue_f32(const TcGemmParams& p, const TcUnit& u, uint32_t tbase,
                                                uint64_t* tmem_empty, int64_t row, int64_t col0, int mode,
                                                int lane, float* stg) {
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
    tc_zero_release<BN, EC>(p, tbase, tmem_empty, lane);
    const float af = (float)u.alpha, bf = (float)u.beta;
    float* Cf = reinterpret_cast<float*>(u.C);
    const int64_t r0 = row - lane;
    float c[EC];
    if (mode != 0) warp_load_block<float, EC>(Cf, u.ldc, r0, col0, u.M, u.N, c, stg, lane);
    float y[EC];
#pragma unroll
    for (int i = 0; i < EC; ++i) {
        const float ph = af * s0[i], pl = fmaf(af, s0[i], -ph);
        float ch = 0.f, cl = 0.f;
        if (mode == 1) {
            ch = c[i];
        } else if (mode == 2) {
            ch = bf * c[i];
            cl = fmaf(bf, c[i], -ch);
        }
        const float sh = ph + ch, bb = sh - ph;
        const float se = (ph - (sh - bb)) + (ch - bb);
        y[i] = sh + (se + pl + cl + af * t[i]);
    }
    warp_store_block<float, EC>(Cf, u.ldc, r0, col0, u.M, u.N, u.symmetric != 0, y, stg, lane);
    if (u.symmetric && row < u.M) {
#pragma unroll
        for (int i = 0; i < EC; ++i) {
            const int64_t col = col0 + i;
            if (col < u.N && col < row) Cf[col * u.ldc + row] = y[i];
        }
    }
}

// Dynamic shared memory: the stages, then kTcSmemTail bytes of barriers,
// TMEM slot, abort flag (256 bytes), the epilogue warps' column-exponent
// slots (kTcEpiCols ints each) and their C staging tiles (kTcStageBytes
// each), plus 1024 bytes of alignment slack in front.
constexpr size_t kTcSmemTail = 256 + kTcEpiWarps * kTcEpiCols * 4 + kTcEpiWarps * kTcStageBytes;
constexpr size_t kTcSmemMax = 232448;

template <int KT, int BN, bool F64>
__global__ void __launch_bounds__(kTcThreads, 1) tc_gemm_kernel(const TcGemmParams p) {
    constexpr int EC = kTcEpiCols;  // columns per epilogue warp
    static_assert(BN == kTcBN, "one tile width");
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)p.stages * p.stage_bytes);
    uint64_t* empty = full + kTcMaxStages;
    uint64_t* accum_full = empty + kTcMaxStages;  // per TMEM buffer
    uint64_t* tmem_empty = accum_full + 2;        // per TMEM buffer
    uint64_t* mma_done = tmem_empty + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    int* colexp_all = reinterpret_cast<int*>(reinterpret_cast<uint8_t*>(full) + 256);
    uint8_t* stage_all = reinterpret_cast<uint8_t*>(colexp_all + kTcEpiWarps * kTcEpiCols);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t stages = (uint32_t)p.stages;

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < stages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&accum_full[b], 1);
            tc::mbar_init(&tmem_empty[b], kTcEpiWarps);
        }
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
                    // A: 16 row groups x S slices; B: one 64-row block x S slices
                    const int ga = (u.a_row0 + u.tm * kTcBM) >> 3, bb = (u.b_row0 + u.tn * BN) >> 6;
                    tc::bulk_load(st, p.a_stack + ((size_t)kt * p.a_groups + ga) * p.sa * (8 * KT),
                                  (uint32_t)p.sa * p.a_tile_bytes, &full[s]);
                    tc::bulk_load(st + (size_t)p.sa * p.a_tile_bytes,
                                  p.b_stack + ((size_t)kt * p.b_blocks + bb) * p.sb * (64 * KT),
                                  (uint32_t)p.sb * p.b_tile_bytes, &full[s]);
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
            // the MMA list of one 16-wide K step: stage-relative descriptors
            // (16-byte units), instruction descriptors and TMEM columns.
            // Along K, core matrices are 128 bytes apart; along M the A row
            // groups are S slices apart (A slice a starts a * 16 KT bytes in),
            // along N the B row groups adjacent (B slice b starts b * BN * 2 KT
            // bytes after the S A tiles).
            const uint64_t desc_a = tc::smem_desc_noswizzle(128, (uint32_t)p.sa * 16 * KT);
            const uint64_t desc_b = tc::smem_desc_noswizzle(128, 16 * KT);
            const uint32_t b_base = ((uint32_t)p.sa * p.a_tile_bytes) >> 4, b_step = p.b_tile_bytes >> 4;
            uint32_t pa[kTcMaxMma], pb[kTcMaxMma], pid[kTcMaxMma], pdc[kTcMaxMma];  // low descriptor words
            const int nmma = min(p.nmma, kTcMaxMma);
#pragma unroll
            for (int q = 0; q < kTcMaxMma; ++q) {
                const int qq = q < nmma ? q : 0;
                const uint32_t a = p.mma_a[qq], b0 = p.mma_b0[qq], n = p.mma_n[qq];
                pa[q] = a * KT;
                pb[q] = b_base + b0 * b_step;
                pid[q] = tc::idesc_bf16_f32(kTcBM, BN * n);
                pdc[q] = tmem_base + (a + b0) * BN;
            }
            uint32_t it = 0, unit = 0;
            bool stop = false;
            for (int t = blockIdx.x; t < p.ntiles && !stop; t += gridDim.x) {
                TcUnit u;
                tc_resolve<BN>(p, t, u);
                for (int c0 = 0; c0 < u.k_tiles && !stop; c0 += p.chunk_tiles, ++unit) {
                    // unit u uses TMEM buffer u % nbuf for the (u / nbuf)-th time: the
                    // epilogue has copied out and zeroed that buffer's previous unit
                    const uint32_t buf = unit % (uint32_t)p.nbuf, use = unit / (uint32_t)p.nbuf;
                    if (!tc::mbar_wait(&tmem_empty[buf], use & 1u)) {
                        atomicExch(p.err, kTcErrTmemWait);
                        *abort_flag = 1;
                    }
                    if (*abort_flag) {
                        stop = true;
                        break;
                    }
                    tc::tc_fence_after();
                    const uint32_t dbuf = buf * kTcBufCols;
                    const int c1 = min(c0 + p.chunk_tiles, u.k_tiles);
                    for (int kt = c0; kt < c1; ++kt, ++it) {
                        const uint32_t s = it % stages;
                        const uint32_t ph = (it / stages) & 1u;
                        if (!tc::mbar_wait_spin(&full[s], ph)) {
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
                            // the j-th 16-wide K step starts two core matrices (256 bytes) later
                            const uint32_t k16 = st4 + 16u * j;
#pragma unroll
                            for (int q = 0; q < kTcMaxMma; ++q)
                                if (q < nmma)
                                    tc::mma_f16(pdc[q] + dbuf, desc_a | (uint64_t)(pa[q] + k16),
                                                desc_b | (uint64_t)(pb[q] + k16), pid[q], 1u);
                        }
                        tc::mma_commit(&empty[s]);
                    }
                    if (!stop) tc::mma_commit(&accum_full[buf]);
                }
            }
            // every MMA issued by this thread completes before TMEM is released
            tc::mma_commit(mma_done);
            tc::mbar_wait(mma_done, 0);
        }
        __syncwarp();
    } else {
        // warp w: TMEM lane quadrant w % 4, column part (w - first) / 4
        const int quad = warp & 3, part = (warp - kTcEpiWarp0) >> 2;
        const uint32_t tbase = tmem_base + ((uint32_t)(quad * 32) << 16) + (uint32_t)(part * EC);
        for (int b = 0; b < p.nbuf; ++b)  // the slots start at zero
            tc_zero_release<BN, EC>(p, tbase + (uint32_t)b * kTcBufCols, &tmem_empty[b], lane);
        uint32_t unit = 0;
        bool stop = false;
        for (int t = blockIdx.x; t < p.ntiles && !stop; t += gridDim.x) {
            TcUnit u;
            tc_resolve<BN>(p, t, u);
            const int64_t row = (int64_t)u.tm * kTcBM + quad * 32 + lane;
            const int64_t col0 = (int64_t)u.tn * BN + part * EC;
            for (int c0 = 0; c0 < u.k_tiles; c0 += p.chunk_tiles, ++unit) {
                // converged warp, warp-uniform outcome: the TMEM loads below are
                // warp-collective (lanes past the last row leave the previous
                // unit's stores early)
                __syncwarp();
                const uint32_t buf = unit % (uint32_t)p.nbuf, use = unit / (uint32_t)p.nbuf;
                const bool waited = tc::mbar_wait(&accum_full[buf], use & 1u);
                if (!__all_sync(0xffffffffu, waited && !*abort_flag)) {
                    if (!waited) atomicExch(p.err, kTcErrEpilogueWait);
                    *abort_flag = 1;
                    stop = true;
                    break;
                }
                tc::tc_fence_after();
                const int mode = c0 > 0 ? 1 : (u.beta != 0.0 ? 2 : 0);
                uint8_t* stg = stage_all + (size_t)(warp - kTcEpiWarp0) * kTcStageBytes;
                if constexpr (F64)
                    tc_epilogue_f64<BN, EC>(p, u, tbase + buf * kTcBufCols, &tmem_empty[buf], row, col0, mode, lane,
                                            colexp_all + (warp - kTcEpiWarp0) * EC,
                                            reinterpret_cast<double*>(stg));
                else
                    tc_epilogue_f32<BN, EC>(p, u, tbase + buf * kTcBufCols, &tmem_empty[buf], row, col0, mode, lane,
                                            reinterpret_cast<float*>(stg));
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
// p.a_stack / b_stack / a_groups / b_blocks describe the operand stacks.
int launch_tc_gemm(rstsr_ctx* ctx, int kt, TcGemmParams p, int k_tiles_total, int k_chunk_tiles,
                   int64_t ntiles_grouped = 0);

}  // namespace rstsr
