// Placeholder GEMM entry points (replaced by the tensor-core implementation).
#include "common.cuh"

using namespace rstsr;

extern "C" {
int rstsr_cuda_gemm(rstsr_ctx*, rstsr_order, char, char, int64_t, int64_t, int64_t, double, const void*, int64_t,
                    const void*, int64_t, double, void*, int64_t, rstsr_dtype, const rstsr_gemm_opts*) {
    return fail(RSTSR_ERR_UNIMPLEMENTED, "gemm not built");
}
int rstsr_cuda_matmul(rstsr_ctx*, rstsr_dtype, void*, const rstsr_layout*, const void*, const rstsr_layout*,
                      const void*, const rstsr_layout*, double, double, rstsr_order, const rstsr_gemm_opts*) {
    return fail(RSTSR_ERR_UNIMPLEMENTED, "matmul not built");
}
int rstsr_cuda_gemm_grouped(rstsr_ctx*, rstsr_dtype, const rstsr_gemm_problem*, int32_t, const rstsr_gemm_opts*) {
    return fail(RSTSR_ERR_UNIMPLEMENTED, "grouped gemm not built");
}
int32_t rstsr_cuda_last_ozaki_slices(void) { return 0; }
int rstsr_cuda_autotune_gemm(rstsr_ctx*, rstsr_dtype, int64_t, int64_t, int64_t, const rstsr_gemm_opts*, int32_t*) {
    return fail(RSTSR_ERR_UNIMPLEMENTED, "autotune not built");
}
int rstsr_cuda_autotune_save(const char*) { return fail(RSTSR_ERR_UNIMPLEMENTED, "autotune not built"); }
int rstsr_cuda_autotune_load(const char*) { return fail(RSTSR_ERR_UNIMPLEMENTED, "autotune not built"); }
}
