// Reduction kernels instantiated for i32, i64, u64 (usize) and bool inputs.
// Narrower integer types are widened to i64 / u64 before reducing: wrapping
// sums and products modulo 2^n and min / max / count are unchanged by that.
#include "reduce_kernel.cuh"

namespace rstsr {

template <typename T>
static int int_launch(rstsr_ctx* ctx, int kind, const RedParams& p) {
    switch (kind) {
        case kRedSum: return launch_reduce<T, kRedSum>(ctx, p);
        case kRedMin: return launch_reduce<T, kRedMin>(ctx, p);
        case kRedMax: return launch_reduce<T, kRedMax>(ctx, p);
        case kRedProd: return launch_reduce<T, kRedProd>(ctx, p);
        case kRedCount: return launch_reduce<T, kRedCount>(ctx, p);
        case kRedArgMax: return launch_reduce<T, kRedArgMax>(ctx, p);
        case kRedArgMin: return launch_reduce<T, kRedArgMin>(ctx, p);
        default: return fail(RSTSR_ERR_INVALID_VALUE, "reduction not defined on integers");
    }
}

int reduce_launch_i32(rstsr_ctx* ctx, int kind, const RedParams& p) { return int_launch<int32_t>(ctx, kind, p); }
int reduce_launch_i64(rstsr_ctx* ctx, int kind, const RedParams& p) { return int_launch<int64_t>(ctx, kind, p); }
int reduce_launch_u64(rstsr_ctx* ctx, int kind, const RedParams& p) { return int_launch<uint64_t>(ctx, kind, p); }

int reduce_launch_bool(rstsr_ctx* ctx, int kind, const RedParams& p) {
    switch (kind) {
        case kRedAll: return launch_reduce<uint8_t, kRedAll>(ctx, p);
        case kRedAny: return launch_reduce<uint8_t, kRedAny>(ctx, p);
        case kRedCount: return launch_reduce<uint8_t, kRedCount>(ctx, p);
        default: return fail(RSTSR_ERR_INVALID_VALUE, "reduction not defined on bool");
    }
}

}  // namespace rstsr
