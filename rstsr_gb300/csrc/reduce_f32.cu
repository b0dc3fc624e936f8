// Reduction kernels instantiated for f32 inputs.
#include "reduce_kernel.cuh"

namespace rstsr {

int reduce_launch_f32(rstsr_ctx* ctx, int kind, const RedParams& p) {
    switch (kind) {
        case kRedSum: return launch_reduce<float, kRedSum>(ctx, p);
        case kRedMoments: return launch_reduce<float, kRedMoments>(ctx, p);
        case kRedSumSq: return launch_reduce<float, kRedSumSq>(ctx, p);
        case kRedMin: return launch_reduce<float, kRedMin>(ctx, p);
        case kRedMax: return launch_reduce<float, kRedMax>(ctx, p);
        case kRedProd: return launch_reduce<float, kRedProd>(ctx, p);
        case kRedCount: return launch_reduce<float, kRedCount>(ctx, p);
        case kRedArgMax: return launch_reduce<float, kRedArgMax>(ctx, p);
        case kRedArgMin: return launch_reduce<float, kRedArgMin>(ctx, p);
        default: return fail(RSTSR_ERR_INVALID_VALUE, "reduction not defined on f32");
    }
}

}  // namespace rstsr
