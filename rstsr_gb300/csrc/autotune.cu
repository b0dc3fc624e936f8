// GEMM autotuner: times the tensor-core kernel configurations of the split
// GEMM (K tile width, raster group height) on one problem shape and keeps the
// fastest per shape class in a process-wide table that the split GEMM driver
// consults (tune_config). The table is saved and loaded as text, one entry a
// line:
//   <mode: ozaki | bf16x3> <slices> <log2 m> <log2 n> <log2 k> <kt> <group>
// with the log2 values rounded up. A process started with
// RSTSR_CUDA_AUTOTUNE_TABLE=<file> has that file loaded by its first context
// creation, which fails with the load's error if the file is missing or
// malformed. The reference has no counterpart: rstsr's CPU GEMMs take their
// blocking from faer / the BLAS library.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "split_gemm.hpp"
#include "tc_gemm.cuh"

namespace rstsr {

int ozaki_dgemm(rstsr_ctx* ctx, int64_t M, int64_t N, int64_t K, double alpha, Operand A, Operand Bt, double beta,
                double* C, int64_t ldc, int slices, bool symmetric);
int split_sgemm(rstsr_ctx* ctx, int64_t M, int64_t N, int64_t K, double alpha, Operand A, Operand Bt, double beta,
                float* C, int64_t ldc, int terms, bool symmetric);

namespace {

using TuneKey = std::tuple<int, int, int, int, int>;  // mode, slices, log2 m, log2 n, log2 k

std::mutex g_mu;
std::map<TuneKey, TuneConfig> g_table;
thread_local TuneConfig g_force = {0, 0};  // set while the autotuner times a candidate

int ceil_log2(int64_t x) {
    int l = 0;
    while (l < 62 && (int64_t(1) << l) < x) ++l;
    return l;
}

TuneKey key_of(SplitMode mode, int slices, int64_t M, int64_t N, int64_t K) {
    return TuneKey{mode == SplitMode::Ozaki ? 0 : 1, slices, ceil_log2(M), ceil_log2(N), ceil_log2(K)};
}

bool valid(const TuneConfig& c) {
    return (c.kt == 16 || c.kt == 32 || c.kt == 64) && c.group >= 1 && c.group <= 64;
}

// uniform values in (-1, 1) from a hash of the index (operands to time with)
template <typename T>
__global__ void fill_uniform_kernel(T* __restrict__ x, int64_t n, uint32_t seed) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t h = (uint32_t)i * 2654435761u ^ seed;
        h ^= h >> 16;
        h *= 0x7feb352du;
        h ^= h >> 15;
        h *= 0x846ca68bu;
        h ^= h >> 16;
        x[i] = (T)((double)h * (2.0 / 4294967296.0) - 1.0);
    }
}

}  // namespace

int load_env_table() {
    static std::once_flag once;
    static int status = RSTSR_OK;
    static std::string msg;
    std::call_once(once, [] {
        const char* path = std::getenv("RSTSR_CUDA_AUTOTUNE_TABLE");
        if (!path || !*path) return;
        status = rstsr_cuda_autotune_load(path);
        if (status != RSTSR_OK) msg = rstsr_cuda_last_error();
    });
    return status == RSTSR_OK ? RSTSR_OK : fail(status, "RSTSR_CUDA_AUTOTUNE_TABLE: " + msg);
}

TuneConfig tune_config(SplitMode mode, int slices, int64_t M, int64_t N, int64_t K) {
    if (g_force.kt) return g_force;
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_table.find(key_of(mode, slices, M, N, K));
    return it == g_table.end() ? TuneConfig{0, 0} : it->second;
}

}  // namespace rstsr

using namespace rstsr;

extern "C" {

int rstsr_cuda_autotune_gemm(rstsr_ctx* ctx, rstsr_dtype t, int64_t m, int64_t n, int64_t k,
                             const rstsr_gemm_opts* opts, int32_t* best_config) {
    if (int e = enter(ctx)) return e;
    if (!best_config) return fail(RSTSR_ERR_INVALID_VALUE, "best_config is null");
    *best_config = 0;
    const int prec = opts ? opts->precision : RSTSR_PREC_AUTO;
    SplitMode mode;
    int slices;
    size_t esz;
    if (t == RSTSR_F64 && (prec == RSTSR_PREC_AUTO || prec == RSTSR_PREC_OZAKI)) {
        mode = SplitMode::Ozaki;
        slices = opts && opts->ozaki_slices > 0 ? std::min(opts->ozaki_slices, 8) : 7;
        esz = 8;
    } else if (t == RSTSR_F32 && (prec == RSTSR_PREC_AUTO || prec == RSTSR_PREC_BF16X3)) {
        mode = SplitMode::Bf16x3;
        slices = opts && opts->reserved[0] > 0 ? std::min<int>(opts->reserved[0], 3) : 3;
        esz = 4;
    } else {
        return fail(RSTSR_ERR_INVALID_VALUE, "autotuning covers the f64 Ozaki and f32 bf16 split GEMMs");
    }
    if (m < 1 || n < 1 || k < 1 || m > 65536 || n > 65536 || k > 65536)
        return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, "autotune shape must be within [1, 65536] per extent");
    cudaStreamCaptureStatus cs;
    if (cudaStreamIsCapturing(ctx->stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
        return fail(RSTSR_ERR_RUNTIME, "cannot autotune while the stream is captured into a graph");

    void *A = nullptr, *B = nullptr, *Cm = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int s = RSTSR_OK;
    auto cleanup = [&]() {
        if (A) scratch_free(ctx, A);
        if (B) scratch_free(ctx, B);
        if (Cm) scratch_free(ctx, Cm);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        g_force = TuneConfig{0, 0};
    };
    if ((s = scratch_alloc(ctx, (size_t)m * k * esz, &A)) || (s = scratch_alloc(ctx, (size_t)n * k * esz, &B)) ||
        (s = scratch_alloc(ctx, (size_t)m * n * esz, &Cm)))
        return cleanup(), s;
    const unsigned grid = (unsigned)std::max(ctx->num_sms, 1) * 4;
    if (esz == 8) {
        fill_uniform_kernel<double><<<grid, 256, 0, ctx->stream>>>((double*)A, m * k, 0x1234u);
        fill_uniform_kernel<double><<<grid, 256, 0, ctx->stream>>>((double*)B, n * k, 0x9876u);
    } else {
        fill_uniform_kernel<float><<<grid, 256, 0, ctx->stream>>>((float*)A, m * k, 0x1234u);
        fill_uniform_kernel<float><<<grid, 256, 0, ctx->stream>>>((float*)B, n * k, 0x9876u);
    }
    if ((s = after_launch(ctx, "fill_uniform_kernel"))) return cleanup(), s;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return cleanup(), fail(RSTSR_ERR_DEVICE, "cudaEventCreate failed");

    // row-major A [m, k], B^T [n, k], C [m, n]
    const Operand opA{A, k, 1}, opB{B, k, 1};
    auto run = [&]() {
        return esz == 8 ? ozaki_dgemm(ctx, m, n, k, 1.0, opA, opB, 0.0, (double*)Cm, n, slices, false)
                        : split_sgemm(ctx, m, n, k, 1.0, opA, opB, 0.0, (float*)Cm, n, slices, false);
    };
    const size_t budget = kTcSmemMax - 1024 - kTcSmemTail;
    TuneConfig best{0, 0};
    float best_ms = 0.f;
    for (int kt : {16, 32, 64}) {
        if (budget / ((size_t)slices * (kTcBM + kTcBN) * kt * 2) < 2) continue;  // at least two stages
        for (int group : {4, 8, 16, 32}) {
            g_force = TuneConfig{kt, group};
            if ((s = run())) return cleanup(), s;  // warm-up
            cudaEventRecord(e0, ctx->stream);
            for (int r = 0; r < 3; ++r)
                if ((s = run())) return cleanup(), s;
            cudaEventRecord(e1, ctx->stream);
            if (cudaEventSynchronize(e1) != cudaSuccess)
                return cleanup(), cuda_fail(cudaGetLastError(), "autotune timing");
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (!best.kt || ms < best_ms) best = g_force, best_ms = ms;
        }
    }
    cleanup();
    if (!best.kt) return fail(RSTSR_ERR_UNIMPLEMENTED, "no kernel configuration fits this slice count");
    {
        std::lock_guard<std::mutex> lk(g_mu);
        g_table[key_of(mode, slices, m, n, k)] = best;
    }
    *best_config = best.kt | (best.group << 8);
    return RSTSR_OK;
}

int rstsr_cuda_autotune_save(const char* path) {
    clear_error();
    if (!path) return fail(RSTSR_ERR_INVALID_VALUE, "path is null");
    FILE* f = fopen(path, "w");
    if (!f) return fail(RSTSR_ERR_RUNTIME, std::string("cannot open ") + path + " for writing");
    std::lock_guard<std::mutex> lk(g_mu);
    fprintf(f, "# rstsr_gb300 GEMM autotune table: mode slices log2m log2n log2k kt group\n");
    for (const auto& [key, c] : g_table)
        fprintf(f, "%s %d %d %d %d %d %d\n", std::get<0>(key) == 0 ? "ozaki" : "bf16x3", std::get<1>(key),
                std::get<2>(key), std::get<3>(key), std::get<4>(key), c.kt, c.group);
    const bool ok = fflush(f) == 0;
    fclose(f);
    return ok ? RSTSR_OK : fail(RSTSR_ERR_RUNTIME, std::string("cannot write ") + path);
}

int rstsr_cuda_autotune_load(const char* path) {
    clear_error();
    if (!path) return fail(RSTSR_ERR_INVALID_VALUE, "path is null");
    FILE* f = fopen(path, "r");
    if (!f) return fail(RSTSR_ERR_RUNTIME, std::string("cannot open ") + path);
    std::map<TuneKey, TuneConfig> table;
    char line[256];
    int lineno = 0;
    while (fgets(line, sizeof(line), f)) {
        ++lineno;
        const char* q = line;
        while (*q == ' ' || *q == '\t') ++q;
        if (*q == '#' || *q == '\n' || *q == '\r' || *q == 0) continue;
        char mode[16];
        int sl, lm, ln, lk, kt, group;
        if (sscanf(q, "%15s %d %d %d %d %d %d", mode, &sl, &lm, &ln, &lk, &kt, &group) != 7 ||
            (strcmp(mode, "ozaki") != 0 && strcmp(mode, "bf16x3") != 0) || sl < 1 || sl > 8 || lm < 0 || lm > 62 ||
            ln < 0 || ln > 62 || lk < 0 || lk > 62 || !valid(TuneConfig{kt, group})) {
            fclose(f);
            return fail(RSTSR_ERR_INVALID_VALUE, std::string(path) + ":" + std::to_string(lineno) +
                                                     ": malformed autotune entry");
        }
        table[TuneKey{strcmp(mode, "ozaki") == 0 ? 0 : 1, sl, lm, ln, lk}] = TuneConfig{kt, group};
    }
    fclose(f);
    std::lock_guard<std::mutex> lk(g_mu);
    g_table = std::move(table);
    return RSTSR_OK;
}

}  // extern "C"
