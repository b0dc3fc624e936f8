// Host launcher of the multi-product tcgen05 GEMM (tc_gemm.cuh) and its TMA
// tensor maps.
#include <algorithm>
#include <cstring>

#include <cudaTypedefs.h>

#include "tc_gemm.cuh"

namespace rstsr {

// cuTensorMapEncodeTiled is resolved through the runtime's driver entry point
// so that the library does not link libcuda directly (it still loads, for the
// host-only entry points, on machines without a driver).
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

int make_bf16_tma(CUtensorMap* map, const void* base, uint64_t rows, uint64_t cols, uint64_t pitch_elems, int kt,
                  int box_rows) {
    memset(map, 0, sizeof(*map));
    if ((reinterpret_cast<uintptr_t>(base) & 15) || (pitch_elems * 2) % 16)
        return fail(RSTSR_ERR_RUNTIME, "TMA operand not 16-byte aligned");
    auto encode = encode_fn();
    if (!encode) return fail(RSTSR_ERR_DEVICE, "cuTensorMapEncodeTiled is not available from the driver");
    cuuint64_t dims[2] = {cols, rows};
    cuuint64_t strides[1] = {pitch_elems * 2};
    cuuint32_t box[2] = {(cuuint32_t)kt, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUtensorMapSwizzle sw = kt == 64   ? CU_TENSOR_MAP_SWIZZLE_128B
                            : kt == 32 ? CU_TENSOR_MAP_SWIZZLE_64B
                                       : CU_TENSOR_MAP_SWIZZLE_32B;
    CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return fail(RSTSR_ERR_DEVICE, "cuTensorMapEncodeTiled failed with CUresult " + std::to_string((int)r));
    return RSTSR_OK;
}

template <int KT, int BN>
static int launch_kt(rstsr_ctx* ctx, const CUtensorMap& ma, const CUtensorMap& mb, const TcGemmParams& p,
                     unsigned grid) {
    const size_t smem = (size_t)p.stages * p.stage_bytes + 1024 /*align*/ + 256 /*barriers*/;
    static bool attr_set = false;
    if (!attr_set) {
        RSTSR_CUDA_TRY(
            cudaFuncSetAttribute(tc_gemm_kernel<KT, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448));
        attr_set = true;
    }
    tc_gemm_kernel<KT, BN><<<grid, kTcThreads, smem, ctx->stream>>>(ma, mb, p);
    return after_launch(ctx, "tc_gemm_kernel");
}

template <int BN>
static int launch_bn(rstsr_ctx* ctx, int kt, const CUtensorMap& ma, const CUtensorMap& mb, const TcGemmParams& p,
                     unsigned grid) {
    switch (kt) {
        case 64: return launch_kt<64, BN>(ctx, ma, mb, p, grid);
        case 32: return launch_kt<32, BN>(ctx, ma, mb, p, grid);
        default: return launch_kt<16, BN>(ctx, ma, mb, p, grid);
    }
}

int launch_tc_gemm(rstsr_ctx* ctx, int kt, const void* a_slices, const void* b_slices, uint64_t kp, TcGemmParams p,
                   int k_tiles_total, int k_chunk_tiles, int64_t ntiles_grouped) {
    const int BN = p.nacc > 4 ? 96 : 128;
    if (p.nacc > kTcMaxAcc || p.nacc * BN > (int)kTcTmemCols)
        return fail(RSTSR_ERR_UNIMPLEMENTED, "too many TMEM accumulators");
    CUtensorMap ma, mb;
    int s = make_bf16_tma(&ma, a_slices, (uint64_t)p.sa * p.a_rows, kp, kp, kt, kTcBM);
    if (s) return s;
    s = make_bf16_tma(&mb, b_slices, (uint64_t)p.sb * p.b_rows, kp, kp, kt, BN);
    if (s) return s;
    p.a_tile_bytes = (uint32_t)(kTcBM * kt * 2);
    p.b_tile_bytes = (uint32_t)(BN * kt * 2);
    p.stage_bytes = (uint32_t)p.sa * p.a_tile_bytes + (uint32_t)p.sb * p.b_tile_bytes;
    const size_t budget = 232448 - 1024 - 256;
    p.stages = (int)std::min<size_t>(kTcMaxStages, budget / p.stage_bytes);
    if (p.stages < 1) return fail(RSTSR_ERR_UNIMPLEMENTED, "too many slices for one pipeline stage");
    int64_t ntiles;
    if (p.tiles) {
        ntiles = ntiles_grouped;
    } else {
        p.tiles_m = (p.M + kTcBM - 1) / kTcBM;
        p.tiles_n = (p.N + BN - 1) / BN;
        if (p.group_m <= 0) p.group_m = 8;
        if (p.symmetric) {
            if (p.M != p.N) return fail(RSTSR_ERR_INVALID_LAYOUT, "symmetric product must be square");
            ntiles = 0;
            for (int j = 0; j < p.tiles_n; ++j) ntiles += p.tiles_m - (j * BN) / kTcBM;
        } else {
            ntiles = (int64_t)p.tiles_m * p.tiles_n;
        }
    }
    if (ntiles == 0) return RSTSR_OK;
    if (ntiles > INT32_MAX) return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, "too many output tiles");
    const int total = std::max(k_tiles_total, 1);
    const int chunk = k_chunk_tiles > 0 ? k_chunk_tiles : total;
    const int accumulate0 = p.accumulate;
    for (int k0 = 0; k0 < total; k0 += chunk) {
        p.kt_begin = k0;
        p.kt_count = std::min(chunk, k_tiles_total - k0);
        p.accumulate = k0 == 0 ? accumulate0 : 1;
        s = BN == 128 ? launch_bn<128>(ctx, kt, ma, mb, p, (unsigned)ntiles)
                      : launch_bn<96>(ctx, kt, ma, mb, p, (unsigned)ntiles);
        if (s) return s;
    }
    return RSTSR_OK;
}

}  // namespace rstsr
