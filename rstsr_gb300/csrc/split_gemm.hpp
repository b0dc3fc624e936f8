// Problem description of the split (Ozaki / three-term bf16) GEMM driver.
#pragma once

#include <climits>
#include <cstdint>
#include <vector>

#include "rstsr_cuda.h"

struct rstsr_ctx;

namespace rstsr {

// One distinct operand matrix, viewed as [R, K] with X[r*s_row + k*s_k];
// `row0` is its first row in the operand stack (slices, exponents).
struct SplitItem {
    const void* ptr;
    int64_t s_row, s_k;
    int32_t R, K;
    int32_t row0;
    // set by split_gemm_run: this item's first block in the statistics and
    // split grids and its blocks along K (32 columns each, K rounded up to 64)
    int32_t blk0, kblk;
};

// C[M,N] (row-major, ldc) = alpha * A[ia] * B[ib]^T + beta * C, where A item
// ia is [M, K] and B item ib is [N, K] (B transposed). With no B items, ib
// indexes the A items (B^T is an A operand).
struct SplitProblem {
    int32_t ia, ib;
    int64_t M, N, K;
    void* C;
    int64_t ldc;
    double alpha, beta;
};

enum class SplitMode { Ozaki, Bf16x3 };

inline bool items_too_large(int rows_a, int rows_b, int maxk) {
    return rows_a > INT32_MAX / 8 || rows_b > INT32_MAX / 8 || maxk > INT32_MAX / 2;
}

// Run every problem with one statistics, one split and one tensor-core
// launch. slices: Ozaki slice count (0 = from the exponent spread) or bf16
// terms (1-3). symmetric: a single problem with B = A^T (no B items), lower
// triangle computed and mirrored.
int split_gemm_run(rstsr_ctx* ctx, SplitMode mode, const std::vector<SplitItem>& a_items,
                   const std::vector<SplitItem>& b_items, const std::vector<SplitProblem>& probs, int slices,
                   bool symmetric);

// Tensor-core kernel configuration chosen by the autotuner (autotune.cu):
// K tile width (16, 32 or 64; 0 = the default rule) and raster group height
// (row tiles per group / symmetric band; 0 = the kernel default). The code
// kt | group << 8 is what rstsr_cuda_autotune_gemm reports.
struct TuneConfig {
    int kt, group;
};
TuneConfig tune_config(SplitMode mode, int slices, int64_t M, int64_t N, int64_t K);

}  // namespace rstsr
