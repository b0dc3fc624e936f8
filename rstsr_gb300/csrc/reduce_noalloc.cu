// An allocation-free variant of the axis-sum reduction.
//
// Some hosts cannot let a library allocate device memory: a caller that owns
// every byte of GPU memory through its own arena (so a cudaMalloc behind its
// back would fail or fragment the arena), a latency-critical loop where the
// implicit synchronisation of cudaMalloc/cudaFree is not acceptable, or a
// plugin host that forbids allocations outside its own allocator. The
// regular rstsr_cuda_reduce_axes_into may take scratch memory from the
// context's pool (the per-chunk partial sums of the split reduction) and
// needs a context, whose creation allocates. rstsr_cuda_sum_axes_noalloc runs
// the same kernels on a caller-supplied stream with its scratch in a fixed
// static device array of RSTSR_NOALLOC_SCRATCH_BYTES; every GPU that loads
// the library holds that array until the process exits.
#include <mutex>

#include "reduce_kernel.cuh"

namespace rstsr {

int plan_reduce(rstsr_ctx* ctx, int op, rstsr_dtype t_in, const void* a, const Layout& La, const int64_t* axes,
                int naxes, void* out, const Layout& Lo, RedParams* pp);

// The scratch shared by every call of the allocation-free entry point.
static __device__ __align__(256) unsigned char g_noalloc_scratch[RSTSR_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
static void* g_scratch_addr[kMaxDevices];
static std::mutex g_scratch_mutex;

// Device address of g_noalloc_scratch on the current device, looked up once
// per device (the host-side symbol is only a stand-in, not a device address).
static int scratch_address(int device, void** out) {
    if (device < 0 || device >= kMaxDevices) return fail(RSTSR_ERR_DEVICE, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_scratch_addr[device] = p;
    }
    *out = g_scratch_addr[device];
    return RSTSR_OK;
}

// The planner picks the number of chunks of the reduced range for
// parallelism alone. When their partial sums do not fit the fixed scratch,
// use as many chunks as fit (each chunk a multiple of the vector width, as the
// planner keeps it), down to one unsplit pass that needs no scratch at all: a
// large plan runs with fewer chunks instead of failing.
template <typename T>
static void fit_split_to_scratch(RedParams& p) {
    using Acc = typename Red<T, kRedSum>::Acc;
    if (p.nsplit <= 1) return;
    const size_t per_split = (size_t)p.nout * sizeof(Acc);
    if ((size_t)p.nsplit * per_split <= RSTSR_NOALLOC_SCRATCH_BYTES) return;
    const int64_t fit = (int64_t)(RSTSR_NOALLOC_SCRATCH_BYTES / per_split);
    if (fit < 2) {
        p.nsplit = 1;
        p.chunk = p.nred;
        return;
    }
    constexpr int64_t VEC = 16 / sizeof(T) > 0 ? 16 / sizeof(T) : 1;
    int64_t chunk = (p.nred + fit - 1) / fit;
    chunk = (chunk + VEC - 1) / VEC * VEC;
    p.chunk = chunk;
    p.nsplit = (int32_t)((p.nred + chunk - 1) / chunk);
}

template <typename T>
static int launch_sum_noalloc(cudaStream_t stream, RedParams p, void* scratch) {
    using Acc = typename Red<T, kRedSum>::Acc;
    const int64_t opc = red_outputs_per_cta(p);
    const int64_t gx = (p.nout + opc - 1) / opc;
    if (gx > INT32_MAX || p.nsplit > 65535) return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, "reduction too large");
    fit_split_to_scratch<T>(p);
    if (p.nsplit > 1) {
        // every partial is written by the first kernel before the second
        // reads it, so the scratch needs no clearing
        if ((size_t)p.nsplit * (size_t)p.nout * sizeof(Acc) > RSTSR_NOALLOC_SCRATCH_BYTES)
            return fail(RSTSR_ERR_RUNTIME, "sum_axes_noalloc: split partials exceed the fixed scratch");
        p.partial = scratch;
    } else {
        p.partial = nullptr;
    }
    cudaError_t e = launch_reduce_pass<T, kRedSum>(p, dim3((unsigned)gx, (unsigned)p.nsplit), stream);
    if (e != cudaSuccess) return cuda_fail(e, "reduce pass");
    if (p.nsplit > 1) {
        const int64_t gc = (p.nout + kCombOuts - 1) / kCombOuts;
        reduce_combine_kernel<T, kRedSum><<<(unsigned)gc, kRedThreads, 0, stream>>>(p);
        e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "reduce_combine_kernel");
    }
    return RSTSR_OK;
}

}  // namespace rstsr

using namespace rstsr;

extern "C" int rstsr_cuda_sum_axes_noalloc(void* stream, rstsr_dtype ta, const void* a, const rstsr_layout* la,
                                           const int64_t* axes, int32_t naxes, void* out,
                                           const rstsr_layout* lout) {
    clear_error();
    if (ta != RSTSR_F64 && ta != RSTSR_F32 && ta != RSTSR_I32 && ta != RSTSR_I64)
        return fail(RSTSR_ERR_UNIMPLEMENTED, "sum_axes_noalloc supports f64, f32, i32 and i64");
    int s = check_layout(la, "a");
    if (!s) s = check_layout(lout, "out");
    if (s) return s;
    if (naxes < 0 || (naxes > 0 && !axes)) return fail(RSTSR_ERR_INVALID_VALUE, "bad axes");
    int device = -1;
    RSTSR_CUDA_TRY(cudaGetDevice(&device));
    {
        // the scratch address and the SM count are those of the current
        // device: a stream of another device is refused
        int stream_device = -1;
        RSTSR_CUDA_TRY(cudaStreamGetDevice((cudaStream_t)stream, &stream_device));
        if (stream_device != device)
            return fail(RSTSR_ERR_DEVICE_MISMATCH, "sum_axes_noalloc: the stream belongs to device " +
                                              std::to_string(stream_device) + ", the current device is " +
                                              std::to_string(device));
    }
    void* scratch = nullptr;
    s = scratch_address(device, &scratch);
    if (s) return s;
    // a context on the stack: the planner reads only the stream and the SM
    // count from it, and nothing here allocates
    rstsr_ctx local;
    local.device = device;
    local.stream = (cudaStream_t)stream;
    RSTSR_CUDA_TRY(cudaDeviceGetAttribute(&local.num_sms, cudaDevAttrMultiProcessorCount, device));
    const Layout La = Layout::from_abi(*la), Lo = Layout::from_abi(*lout);
    if (Lo.size() > 0 && !out) return fail(RSTSR_ERR_INVALID_VALUE, "null output pointer");
    if (La.size() > 0 && !a) return fail(RSTSR_ERR_INVALID_VALUE, "null input pointer");
    RedParams p;
    s = plan_reduce(&local, RSTSR_RED_SUM, ta, a, La, axes, naxes, out, Lo, &p);
    if (s || p.nout == 0) return s;
    switch (ta) {
        case RSTSR_F64: return launch_sum_noalloc<double>(local.stream, p, scratch);
        case RSTSR_F32: return launch_sum_noalloc<float>(local.stream, p, scratch);
        case RSTSR_I32: return launch_sum_noalloc<int32_t>(local.stream, p, scratch);
        default: return launch_sum_noalloc<int64_t>(local.stream, p, scratch);
    }
}
