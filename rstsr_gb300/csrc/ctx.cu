// Context, storage, error plumbing, iteration-space planner and CUDA graphs.
#include <algorithm>
#include <cstring>
#include <numeric>

#include "common.cuh"

namespace rstsr {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }
int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
int cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return RSTSR_ERR_DEVICE;
}

int after_launch(rstsr_ctx* ctx, const char* name) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, name);
    ctx->launches.fetch_add(1, std::memory_order_relaxed);
    return RSTSR_OK;
}

int enter(rstsr_ctx* ctx) {
    if (!ctx) return fail(RSTSR_ERR_INVALID_VALUE, "null context");
    // a failed call whose status nobody read (a destructor's, another
    // library's on this thread) must not be reported as this call's launch error
    (void)cudaGetLastError();
    int cur = -1;
    RSTSR_CUDA_TRY(cudaGetDevice(&cur));
    if (cur != ctx->device) RSTSR_CUDA_TRY(cudaSetDevice(ctx->device));
    return RSTSR_OK;
}

int scratch_alloc(rstsr_ctx* ctx, size_t bytes, void** p) {
    *p = nullptr;
    if (bytes == 0) return RSTSR_OK;
    RSTSR_CUDA_TRY(cudaMallocFromPoolAsync(p, bytes, ctx->pool, ctx->stream));
    return RSTSR_OK;
}

void scratch_free(rstsr_ctx* ctx, void* p) {
    if (p) cudaFreeAsync(p, ctx->stream);
}

int check_layout(const rstsr_layout* l, const char* name) {
    if (!l) return fail(RSTSR_ERR_INVALID_LAYOUT, std::string(name) + ": null layout");
    if (l->ndim < 0 || l->ndim > RSTSR_MAX_NDIM)
        return fail(RSTSR_ERR_INVALID_LAYOUT,
                    std::string(name) + ": ndim " + std::to_string(l->ndim) + " outside [0, 8]");
    for (int i = 0; i < l->ndim; ++i)
        if (l->shape[i] < 0) return fail(RSTSR_ERR_INVALID_LAYOUT, std::string(name) + ": negative extent");
    Layout L = Layout::from_abi(*l);
    int64_t lo, hi;
    if (!L.bounds_index(&lo, &hi))
        return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE,
                    std::string(name) + ": layout reaches a negative element index (" + L.repr() + ")");
    return RSTSR_OK;
}

IterSpace make_iter_space(const Layout* const* ls, int nops) {
    IterSpace sp;
    sp.nops = nops;
    const Layout& l0 = *ls[0];
    int n = l0.ndim;
    sp.size = l0.size();
    for (int k = 0; k < nops; ++k) sp.offset[k] = ls[k]->offset;
    if (sp.size == 0) {
        sp.ndim = 0;
        return sp;
    }
    std::vector<int> axes;
    for (int i = 0; i < n; ++i)
        if (l0.shape[i] != 1) axes.push_back(i);
    std::stable_sort(axes.begin(), axes.end(), [&](int a, int b) {
        for (int k = 0; k < nops; ++k) {
            int64_t sa = std::llabs(ls[k]->stride[a]), sb = std::llabs(ls[k]->stride[b]);
            if (sa != sb) return sa < sb;
        }
        return false;
    });
    int nd = 0;
    for (int a : axes) {
        bool merge = nd > 0;
        if (merge) {
            for (int k = 0; k < nops; ++k) {
                if (ls[k]->stride[a] != sp.stride[k][nd - 1] * sp.shape[nd - 1]) {
                    merge = false;
                    break;
                }
            }
        }
        if (merge) {
            sp.shape[nd - 1] *= l0.shape[a];
        } else {
            sp.shape[nd] = l0.shape[a];
            for (int k = 0; k < nops; ++k) sp.stride[k][nd] = ls[k]->stride[a];
            nd++;
        }
    }
    if (nd == 0) {  // every extent is one: a single element
        sp.shape[0] = 1;
        for (int k = 0; k < nops; ++k) sp.stride[k][0] = 0;
        nd = 1;
    }
    sp.ndim = nd;
    return sp;
}

DevDims make_dev_dims(const IterSpace& sp) {
    DevDims d;
    d.ndim = sp.ndim;
    for (int i = 0; i < RSTSR_MAX_NDIM; ++i) {
        d.shape[i] = i < sp.ndim ? (uint32_t)sp.shape[i] : 1u;
        d.div[i] = FastDiv(d.shape[i]);
    }
    return d;
}

bool vec_aligned(const IterSpace& sp, int k, const void* base, size_t esize, int vec) {
    if (vec <= 1) return true;
    if (sp.stride[k][0] != 1) return false;
    if (sp.shape[0] % vec != 0) return false;
    size_t vb = esize * vec;
    uintptr_t addr = reinterpret_cast<uintptr_t>(base) + (uintptr_t)(sp.offset[k] * (int64_t)esize);
    if (addr % vb != 0) return false;
    for (int d = 1; d < sp.ndim; ++d)
        if ((std::llabs(sp.stride[k][d]) * (int64_t)esize) % (int64_t)vb != 0) return false;
    return true;
}

}  // namespace rstsr

using namespace rstsr;

struct rstsr_graph {
    cudaGraphExec_t exec = nullptr;
    int device = 0;
    uint64_t nkernels = 0;  // kernels recorded during capture
};

extern "C" {

const char* rstsr_cuda_last_error(void) { return g_last_error.c_str(); }

const char* rstsr_cuda_version(void) { return "rstsr-cuda 0.1.0 (sm_103a)"; }

int rstsr_cuda_ctx_create(int32_t device, rstsr_ctx** out) {
    clear_error();
    if (!out) return fail(RSTSR_ERR_INVALID_VALUE, "null output pointer");
    *out = nullptr;
    if (int s = load_env_table()) return s;
    int ndev = 0;
    RSTSR_CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev)
        return fail(RSTSR_ERR_INVALID_VALUE, "device " + std::to_string(device) + " not present (" +
                                                 std::to_string(ndev) + " visible)");
    RSTSR_CUDA_TRY(cudaSetDevice(device));
    auto* c = new rstsr_ctx();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "cudaStreamCreateWithFlags");
    }
    c->stream = c->own_stream;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    e = cudaDeviceGetDefaultMemPool(&c->pool, device);
    if (e != cudaSuccess) {
        cudaStreamDestroy(c->own_stream);
        delete c;
        return cuda_fail(e, "cudaDeviceGetDefaultMemPool");
    }
    // Keep freed blocks in the pool: tensors are allocated and dropped at a
    // high rate and returning memory to the driver each time is slow.
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &thr);
    e = cudaMalloc(&c->dev_err, 256);
    if (e == cudaSuccess) e = cudaMemset(c->dev_err, 0, 256);
    if (e != cudaSuccess) {
        cudaStreamDestroy(c->own_stream);
        delete c;
        return cuda_fail(e, "error word allocation");
    }
    *out = c;
    return RSTSR_OK;
}

int rstsr_cuda_ctx_destroy(rstsr_ctx* ctx) {
    clear_error();
    if (!ctx) return RSTSR_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    staging_destroy(ctx);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    if (ctx->dev_err) cudaFree(ctx->dev_err);
    delete ctx;
    return RSTSR_OK;
}

int rstsr_cuda_ctx_sync(rstsr_ctx* ctx) {
    clear_error();
    int s = enter(ctx);
    if (s) return s;
    RSTSR_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    // a kernel that gave up a bounded wait leaves its code in the error word
    int code = 0;
    RSTSR_CUDA_TRY(cudaMemcpy(&code, ctx->dev_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (code != 0) {
        cudaMemset(ctx->dev_err, 0, sizeof(int));
        return fail(RSTSR_ERR_TIMEOUT, "a device-side wait timed out (code " + std::to_string(code) +
                                           "); the results of the affected call are invalid");
    }
    return RSTSR_OK;
}

int rstsr_cuda_ctx_set_stream(rstsr_ctx* ctx, void* stream) {
    clear_error();
    if (!ctx) return fail(RSTSR_ERR_INVALID_VALUE, "null context");
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return RSTSR_OK;
}

void* rstsr_cuda_ctx_get_stream(rstsr_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int32_t rstsr_cuda_ctx_device(const rstsr_ctx* ctx) { return ctx ? ctx->device : -1; }

uint64_t rstsr_cuda_ctx_launch_count(const rstsr_ctx* ctx) {
    return ctx ? ctx->launches.load(std::memory_order_relaxed) : 0;
}

int rstsr_cuda_malloc(rstsr_ctx* ctx, size_t nbytes, void** out) {
    clear_error();
    if (!out) return fail(RSTSR_ERR_INVALID_VALUE, "null output pointer");
    *out = nullptr;
    int s = enter(ctx);
    if (s) return s;
    if (nbytes == 0) return RSTSR_OK;
    RSTSR_CUDA_TRY(cudaMallocFromPoolAsync(out, nbytes, ctx->pool, ctx->stream));
    return RSTSR_OK;
}

int rstsr_cuda_free(rstsr_ctx* ctx, void* ptr) {
    clear_error();
    int s = enter(ctx);
    if (s) return s;
    if (!ptr) return RSTSR_OK;
    RSTSR_CUDA_TRY(cudaFreeAsync(ptr, ctx->stream));
    return RSTSR_OK;
}

int rstsr_cuda_memcpy_h2d(rstsr_ctx* ctx, void* dst, const void* src, size_t nbytes) {
    clear_error();
    int s = enter(ctx);
    if (s) return s;
    if (nbytes == 0) return RSTSR_OK;
    if (!dst || !src) return fail(RSTSR_ERR_INVALID_VALUE, "null pointer in memcpy_h2d");
    RSTSR_CUDA_TRY(cudaMemcpyAsync(dst, src, nbytes, cudaMemcpyHostToDevice, ctx->stream));
    return RSTSR_OK;
}

int rstsr_cuda_memcpy_d2h(rstsr_ctx* ctx, void* dst, const void* src, size_t nbytes) {
    clear_error();
    int s = enter(ctx);
    if (s) return s;
    if (nbytes == 0) return RSTSR_OK;
    if (!dst || !src) return fail(RSTSR_ERR_INVALID_VALUE, "null pointer in memcpy_d2h");
    RSTSR_CUDA_TRY(cudaMemcpyAsync(dst, src, nbytes, cudaMemcpyDeviceToHost, ctx->stream));
    RSTSR_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return RSTSR_OK;
}

int rstsr_cuda_memcpy_d2d(rstsr_ctx* ctx, void* dst, const void* src, size_t nbytes) {
    clear_error();
    int s = enter(ctx);
    if (s) return s;
    if (nbytes == 0) return RSTSR_OK;
    if (!dst || !src) return fail(RSTSR_ERR_INVALID_VALUE, "null pointer in memcpy_d2d");
    // cudaMemcpyDefault: with unified addressing either side may also be
    // pinned host memory, which makes this the asynchronous device->host copy
    RSTSR_CUDA_TRY(cudaMemcpyAsync(dst, src, nbytes, cudaMemcpyDefault, ctx->stream));
    return RSTSR_OK;
}

int rstsr_cuda_graph_begin(rstsr_ctx* ctx) {
    clear_error();
    int s = enter(ctx);
    if (s) return s;
    if (ctx->capturing) return fail(RSTSR_ERR_RUNTIME, "graph capture already active on this context");
    if (ctx->stream == nullptr) return fail(RSTSR_ERR_RUNTIME, "cannot capture the legacy default stream");
    RSTSR_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    ctx->capturing = true;
    ctx->launches_at_capture = ctx->launches.load();
    return RSTSR_OK;
}

int rstsr_cuda_graph_end(rstsr_ctx* ctx, rstsr_graph** out) {
    clear_error();
    if (!out) return fail(RSTSR_ERR_INVALID_VALUE, "null output pointer");
    *out = nullptr;
    int s = enter(ctx);
    if (s) return s;
    if (!ctx->capturing) return fail(RSTSR_ERR_RUNTIME, "no graph capture active on this context");
    ctx->capturing = false;
    cudaGraph_t g = nullptr;
    RSTSR_CUDA_TRY(cudaStreamEndCapture(ctx->stream, &g));
    auto* rg = new rstsr_graph();
    rg->device = ctx->device;
    // kernels recorded during capture did not run; they run on each replay
    uint64_t now = ctx->launches.load();
    rg->nkernels = now - ctx->launches_at_capture;
    ctx->launches.store(ctx->launches_at_capture);
    cudaError_t e = cudaGraphInstantiate(&rg->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        delete rg;
        return cuda_fail(e, "cudaGraphInstantiate");
    }
    *out = rg;
    return RSTSR_OK;
}

int rstsr_cuda_graph_launch(rstsr_ctx* ctx, rstsr_graph* g) {
    clear_error();
    int s = enter(ctx);
    if (s) return s;
    if (!g) return fail(RSTSR_ERR_INVALID_VALUE, "null graph");
    if (g->device != ctx->device) return fail(RSTSR_ERR_DEVICE_MISMATCH, "graph built on another device");
    RSTSR_CUDA_TRY(cudaGraphLaunch(g->exec, ctx->stream));
    ctx->launches.fetch_add(g->nkernels, std::memory_order_relaxed);
    return RSTSR_OK;
}

int rstsr_cuda_graph_destroy(rstsr_graph* g) {
    clear_error();
    if (!g) return RSTSR_OK;
    cudaSetDevice(g->device);
    cudaGraphExecDestroy(g->exec);
    delete g;
    return RSTSR_OK;
}

}  // extern "C"
