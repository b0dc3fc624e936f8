// Multi-product tensor-core GEMM for sm_103a (tcgen05 + TMA + TMEM).
//
// One CTA computes a 128 x BN output tile (BN = 128, or 96 when five TMEM
// accumulators are needed). The operands are stacks of bf16 "slices" stored
// K-major ([slices][rows][Kp]): slice s of A occupies rows s*A_rows .. of A's
// 2-D TMA map, likewise for B. Per K tile of width KT, one pipeline stage
// holds every slice of the A and B tiles; the MMA thread then issues a list of
// products (slice of A, slice of B, accumulator), several products summing
// into the same FP32 TMEM accumulator. The epilogue adds the accumulators in
// double precision and applies per-row / per-column power-of-two scales,
// alpha and beta.
//
// This one kernel serves
//   * the Ozaki split for f64 (integer slices, level accumulators),
//   * the three-term bf16 split for f32 (hi/mid/lo products),
//   * a plain bf16 GEMM (one slice each, one product),
// for a single problem or for a list of problems (batched and grouped
// matmul) whose slices share one pair of TMA maps: each CTA then reads its
// (problem, tile) from a device tile list.
//
// Roles (192 threads): warp 0 issues TMA loads, warp 1 owns TMEM and issues
// tcgen05.mma from one thread, warps 2-5 drain TMEM in the epilogue (warp w
// reads TMEM lanes 32*(w%4)..+31). All waits are bounded (tc_ptx.cuh); on a
// timeout the CTA records an error code in p.err and unwinds.
#pragma once

#include "common.cuh"
#include "tc_ptx.cuh"

namespace rstsr {

constexpr int kTcBM = 128;
constexpr int kTcThreads = 192;
constexpr int kTcMaxStages = 8;
constexpr int kTcMaxProducts = 40;
constexpr int kTcMaxAcc = 5;
constexpr uint32_t kTcTmemCols = 512;

// error codes written to p.err
constexpr int kTcErrProducerWait = 1;
constexpr int kTcErrMmaWait = 2;
constexpr int kTcErrEpilogueWait = 3;

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

struct TcGemmParams {
    int32_t M, N;                // single-problem mode: output extent
    int32_t kt_begin, kt_count;  // K tiles processed by this launch (kt_count: single-problem mode)
    int32_t sa, sb;              // slices of A and B
    int32_t a_rows, b_rows;      // rows per slice in the TMA maps
    int32_t nprod, nacc;
    uint8_t prod_a[kTcMaxProducts], prod_b[kTcMaxProducts], prod_acc[kTcMaxProducts];
    int32_t stages;
    uint32_t a_tile_bytes;       // 128 x KT bf16
    uint32_t b_tile_bytes;       // BN x KT bf16
    uint32_t stage_bytes;        // sa A tiles + sb B tiles
    // epilogue
    void* C;
    int64_t ldc;                 // row-major leading dimension of C (elements)
    int32_t out_f64;             // 1: C is f64, 0: C is f32
    double alpha, beta;
    int32_t accumulate;          // 1: C += result (K chunks after the first)
    const int32_t* row_exp;      // per-row power-of-two exponent (or null)
    const int32_t* col_exp;      // per-column exponent (or null)
    int32_t exp_bias;
    int32_t symmetric;           // lower triangle only (row >= col), mirrored
    int32_t tiles_m, tiles_n;
    int32_t group_m;             // raster swizzle: tiles grouped along M
    // grouped mode (tiles != null): blockIdx.x indexes tiles[] = {problem, tm, tn, 0}
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
    // grouped raster: consecutive CTAs share B tiles within a group of rows
    const int per_group = p.group_m * p.tiles_n;
    const int g = bid / per_group;
    const int first_m = g * p.group_m;
    const int gm = min(p.tiles_m - first_m, p.group_m);
    const int in_g = bid - g * per_group;
    tm = first_m + in_g % gm;
    tn = in_g / gm;
}

template <int KT, int BN>
__global__ void __launch_bounds__(kTcThreads, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tma_a, const __grid_constant__ CUtensorMap tma_b,
                   const TcGemmParams p) {
    constexpr uint32_t kRowBytes = KT * 2;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)p.stages * p.stage_bytes);
    uint64_t* empty = full + kTcMaxStages;
    uint64_t* accum_full = empty + kTcMaxStages;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accum_full + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // ---- which tile / problem
    int tm, tn;
    int32_t M = p.M, N = p.N, a_row0 = 0, b_row0 = 0, kt_count = p.kt_count, symmetric = p.symmetric;
    void* Cptr = p.C;
    int64_t ldc = p.ldc;
    double alpha = p.alpha, beta = p.beta;
    const int32_t* row_exp = p.row_exp;
    const int32_t* col_exp = p.col_exp;
    if (p.tiles) {
        const int4 t = p.tiles[blockIdx.x];
        const TcProblem q = p.problems[t.x];
        tm = t.y;
        tn = t.z;
        M = q.M;
        N = q.N;
        a_row0 = q.a_row0;
        b_row0 = q.b_row0;
        kt_count = min(q.k_tiles - p.kt_begin, p.kt_count);
        symmetric = q.symmetric;
        Cptr = q.C;
        ldc = q.ldc;
        alpha = q.alpha;
        beta = q.beta;
        if (row_exp) row_exp += q.row_exp0;
        if (col_exp) col_exp += q.col_exp0;
        if (kt_count <= 0) return;  // this problem has no K tiles in this chunk (uniform per CTA)
    } else {
        tc_tile_coords<BN>(p, blockIdx.x, tm, tn);
    }

    if (threadIdx.x == 0) {
        for (int s = 0; s < p.stages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(accum_full, 1);
        *abort_flag = 0;
        tc::fence_barrier_init();
    }
    if (warp == 1) tc::tmem_alloc(tmem_slot, kTcTmemCols);
    if (warp == 0 && lane == 0) {
        tc::prefetch_tensormap(&tma_a);
        tc::prefetch_tensormap(&tma_b);
    }
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            int issued = 0;
            for (int i = 0; i < kt_count; ++i) {
                const int s = i % p.stages;
                const uint32_t ph = (uint32_t)(i / p.stages) & 1u;
                if (i >= p.stages && !tc::mbar_wait(&empty[s], ph ^ 1u)) {
                    atomicExch(p.err, kTcErrProducerWait);
                    *abort_flag = 1;
                    break;
                }
                if (*abort_flag) break;
                uint8_t* st = smem + (size_t)s * p.stage_bytes;
                tc::mbar_arrive_expect_tx(&full[s], p.stage_bytes);
                const int kx = (p.kt_begin + i) * KT;
                for (int a = 0; a < p.sa; ++a)
                    tc::tma_load_2d(st + (size_t)a * p.a_tile_bytes, &tma_a, &full[s], kx,
                                    a * p.a_rows + a_row0 + tm * kTcBM);
                uint8_t* sb = st + (size_t)p.sa * p.a_tile_bytes;
                for (int b = 0; b < p.sb; ++b)
                    tc::tma_load_2d(sb + (size_t)b * p.b_tile_bytes, &tma_b, &full[s], kx,
                                    b * p.b_rows + b_row0 + tn * BN);
                ++issued;
            }
            // never leave the CTA with copies in flight: wait (bounded) for the
            // last use of every stage that was issued
            for (int s = 0; s < p.stages && s < issued; ++s) {
                const int last = s + ((issued - 1 - s) / p.stages) * p.stages;
                tc::mbar_wait(&full[s], (uint32_t)(last / p.stages) & 1u);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_bf16_f32(kTcBM, BN);
            uint32_t started = 0;  // bit a: accumulator a holds a partial sum
            bool ok = true;
            for (int i = 0; i < kt_count; ++i) {
                const int s = i % p.stages;
                const uint32_t ph = (uint32_t)(i / p.stages) & 1u;
                if (!tc::mbar_wait(&full[s], ph)) {
                    atomicExch(p.err, kTcErrMmaWait);
                    *abort_flag = 1;
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                const uint32_t st = tc::smem_u32(smem + (size_t)s * p.stage_bytes);
                const uint32_t sb = st + (uint32_t)p.sa * p.a_tile_bytes;
                for (int q = 0; q < p.nprod; ++q) {
                    const uint32_t a_addr = st + (uint32_t)p.prod_a[q] * p.a_tile_bytes;
                    const uint32_t b_addr = sb + (uint32_t)p.prod_b[q] * p.b_tile_bytes;
                    const uint32_t acc = p.prod_acc[q];
                    const uint32_t d = tmem_base + acc * BN;
#pragma unroll
                    for (int j = 0; j < KT / 16; ++j) {
                        const uint64_t ad = tc::smem_desc_kmajor(a_addr + j * 32, kRowBytes);
                        const uint64_t bd = tc::smem_desc_kmajor(b_addr + j * 32, kRowBytes);
                        tc::mma_f16(d, ad, bd, idesc, (started >> acc) & 1u);
                        started |= 1u << acc;
                    }
                }
                tc::mma_commit(&empty[s]);
            }
            if (ok) tc::mma_commit(accum_full);
        }
        __syncwarp();
    } else {
        // epilogue: warps 2..5 -> TMEM lane quadrants 2, 3, 0, 1
        const int quad = warp & 3;
        const bool ok = tc::mbar_wait(accum_full, 0);
        if (!ok) {
            atomicExch(p.err, kTcErrEpilogueWait);
        } else {
            tc::tc_fence_after();
            const int r_local = quad * 32 + lane;
            const int64_t row = (int64_t)tm * kTcBM + r_local;
            double rs = alpha;
            if (row_exp && row < M) rs = ldexp(rs, row_exp[row] + p.exp_bias);
#pragma unroll 1
            for (int cc = 0; cc < BN / 32; ++cc) {
                double v[32];
#pragma unroll
                for (int i = 0; i < 32; ++i) v[i] = 0.0;
                for (int a = 0; a < p.nacc; ++a) {
                    uint32_t r[32];
                    tc::tmem_ld_32x32b_x32(
                        tmem_base + ((uint32_t)(quad * 32) << 16) + (uint32_t)(a * BN + cc * 32), r);
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int i = 0; i < 32; ++i) v[i] += (double)__uint_as_float(r[i]);
                }
                if (row >= M) continue;
                const int64_t col0 = (int64_t)tn * BN + cc * 32;
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const int64_t col = col0 + i;
                    if (col >= N) break;
                    if (symmetric && col > row) continue;  // upper triangle: written by the mirror
                    double x = v[i] * rs;
                    if (col_exp) x = ldexp(x, col_exp[col]);
                    if (p.out_f64) {
                        double* Cd = reinterpret_cast<double*>(Cptr);
                        double* dst = Cd + row * ldc + col;
                        double y = x;
                        if (p.accumulate) y += *dst;
                        else if (beta != 0.0) y += beta * *dst;
                        *dst = y;
                        if (symmetric && col != row) Cd[col * ldc + row] = y;
                    } else {
                        float* Cf = reinterpret_cast<float*>(Cptr);
                        float* dst = Cf + row * ldc + col;
                        double y = x;
                        if (p.accumulate) y += (double)*dst;
                        else if (beta != 0.0) y += beta * (double)*dst;
                        *dst = (float)y;
                        if (symmetric && col != row) Cf[col * ldc + row] = (float)y;
                    }
                }
            }
        }
    }
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

// Host side: a 2-D bf16 TMA map over [rows, cols] (cols contiguous, row pitch
// `pitch_elems`), box [box_rows, KT cols] with the swizzle matching KT.
int make_bf16_tma(CUtensorMap* map, const void* base, uint64_t rows, uint64_t cols, uint64_t pitch_elems, int kt,
                  int box_rows);

// Launch tc_gemm_kernel<KT, BN> (BN = 128 when nacc <= 4, else 96) over all
// tiles and K chunks described by p. Grouped mode: p.tiles / p.problems set,
// `ntiles_grouped` tiles, `k_tiles_total` = the largest problem's K tiles.
int launch_tc_gemm(rstsr_ctx* ctx, int kt, const void* a_slices, const void* b_slices, uint64_t kp,
                   TcGemmParams p, int k_tiles_total, int k_chunk_tiles, int64_t ntiles_grouped = 0);

}  // namespace rstsr
