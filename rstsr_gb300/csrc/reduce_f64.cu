// Reduction kernels instantiated for f64 inputs.
#include "reduce_kernel.cuh"

namespace rstsr {

int reduce_launch_f64(rstsr_ctx* ctx, int kind, const RedParams& p) {
    switch (kind) {
        case kRedSum: return launch_reduce<double, kRedSum>(ctx, p);
        case kRedMoments: return launch_reduce<double, kRedMoments>(ctx, p);
        case kRedSumSq: return launch_reduce<double, kRedSumSq>(ctx, p);
        case kRedMin: return launch_reduce<double, kRedMin>(ctx, p);
        case kRedMax: return launch_reduce<double, kRedMax>(ctx, p);
        case kRedProd: return launch_reduce<double, kRedProd>(ctx, p);
        case kRedCount: return launch_reduce<double, kRedCount>(ctx, p);
        case kRedArgMax: return launch_reduce<double, kRedArgMax>(ctx, p);
        case kRedArgMin: return launch_reduce<double, kRedArgMin>(ctx, p);
        default: return fail(RSTSR_ERR_INVALID_VALUE, "reduction not defined on f64");
    }
}

}  // namespace rstsr
