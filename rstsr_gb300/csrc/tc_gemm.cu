// Host launcher of the multi-product tcgen05 GEMM (tc_gemm.cuh).
#include <algorithm>
#include <atomic>
#include <cstring>

#include "tc_gemm.cuh"

namespace rstsr {

template <int KT, bool F64>
static int launch_kt(rstsr_ctx* ctx, const TcGemmParams& p, unsigned grid) {
    const size_t smem = (size_t)p.stages * p.stage_bytes + 1024 /*align*/ + kTcSmemTail;
    grid = std::min<unsigned>(grid, (unsigned)std::max(ctx->num_sms, 1));  // persistent: one CTA per SM
    static std::atomic<uint64_t> attr_set{0};  // bit d: opted in on device d
    const uint64_t bit = 1ull << (ctx->device & 63);
    if (!(attr_set.load() & bit)) {
        RSTSR_CUDA_TRY(cudaFuncSetAttribute(tc_gemm_kernel<KT, kTcBN, F64>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmemMax));
        attr_set.fetch_or(bit);
    }
    tc_gemm_kernel<KT, kTcBN, F64><<<grid, kTcThreads, smem, ctx->stream>>>(p);
    return after_launch(ctx, "tc_gemm_kernel");
}

template <bool F64>
static int launch_out(rstsr_ctx* ctx, int kt, const TcGemmParams& p, unsigned grid) {
    switch (kt) {
        case 64: return launch_kt<64, F64>(ctx, p, grid);
        case 32: return launch_kt<32, F64>(ctx, p, grid);
        default: return launch_kt<16, F64>(ctx, p, grid);
    }
}

int launch_tc_gemm(rstsr_ctx* ctx, int kt, TcGemmParams p, int k_tiles_total, int k_chunk_tiles,
                   int64_t ntiles_grouped) {
    constexpr int BN = kTcBN;
    if (kt != 16 && kt != 32 && kt != 64) return fail(RSTSR_ERR_RUNTIME, "K tile must be 16, 32 or 64");
    if (p.nslots < 1 || p.nslots > kTcMaxSlots || p.nslots * BN > (int)kTcTmemCols)
        return fail(RSTSR_ERR_UNIMPLEMENTED, "too many TMEM level slots");
    if (p.nmma < 1 || p.nmma > kTcMaxMma) return fail(RSTSR_ERR_UNIMPLEMENTED, "too many MMAs per K step");
    for (int q = 0; q < p.nmma; ++q)
        if (p.mma_n[q] < 1 || p.mma_n[q] > kTcMaxStack || p.mma_a[q] >= p.sa || p.mma_b0[q] + p.mma_n[q] > p.sb ||
            p.mma_a[q] + p.mma_b0[q] + p.mma_n[q] > p.nslots)
            return fail(RSTSR_ERR_RUNTIME, "MMA list outside the slices or level slots");
    if ((reinterpret_cast<uintptr_t>(p.a_stack) & 15) || (reinterpret_cast<uintptr_t>(p.b_stack) & 15))
        return fail(RSTSR_ERR_RUNTIME, "operand stacks not 16-byte aligned");
    p.a_tile_bytes = (uint32_t)(kTcBM * kt * 2);
    p.b_tile_bytes = (uint32_t)(BN * kt * 2);
    p.stage_bytes = (uint32_t)p.sa * p.a_tile_bytes + (uint32_t)p.sb * p.b_tile_bytes;
    const size_t budget = kTcSmemMax - 1024 - kTcSmemTail;
    p.stages = (int)std::min<size_t>(kTcMaxStages, budget / p.stage_bytes);
    if (p.stages < 1) return fail(RSTSR_ERR_UNIMPLEMENTED, "too many slices for one pipeline stage");
    int64_t ntiles;
    if (p.tiles) {
        ntiles = ntiles_grouped;
    } else {
        p.tiles_m = (p.M + kTcBM - 1) / kTcBM;
        p.tiles_n = (p.N + BN - 1) / BN;
        const int group = p.group_m;  // 0: defaults (8 row tiles a group, bands of 16)
        p.group_m = group > 0 ? group : 8;
        if (p.symmetric) {
            if (p.M != p.N) return fail(RSTSR_ERR_INVALID_LAYOUT, "symmetric product must be square");
            // bands of at least 16 row tiles (2048 rows), at most kTcMaxBands of them
            p.band_rows = std::max(group > 0 ? group : 16, (p.tiles_m + kTcMaxBands - 1) / kTcMaxBands);
            p.nbands = (p.tiles_m + p.band_rows - 1) / p.band_rows;
            ntiles = 0;
            for (int g = 0; g < p.nbands; ++g) {
                if (ntiles > INT32_MAX) return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, "too many output tiles");
                p.band_first[g] = (int32_t)ntiles;
                const int bs = g * p.band_rows, be = std::min(bs + p.band_rows, p.tiles_m);
                const int jmax = std::min(2 * be, p.tiles_n);
                for (int j = 0; j < jmax; ++j) ntiles += be - std::max(bs, j >> 1);
            }
            p.band_first[p.nbands] = (int32_t)std::min<int64_t>(ntiles, INT32_MAX);
        } else {
            ntiles = (int64_t)p.tiles_m * p.tiles_n;
        }
    }
    if (ntiles == 0) return RSTSR_OK;
    if (ntiles > INT32_MAX) return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, "too many output tiles");
    p.ntiles = (int32_t)ntiles;
    p.nbuf = p.nslots * BN <= (int)kTcBufCols ? 2 : 1;
    p.k_tiles = std::max(k_tiles_total, 1);
    p.chunk_tiles = k_chunk_tiles > 0 ? k_chunk_tiles : p.k_tiles;
    return p.out_f64 ? launch_out<true>(ctx, kt, p, (unsigned)ntiles) : launch_out<false>(ctx, kt, p, (unsigned)ntiles);
}

}  // namespace rstsr
