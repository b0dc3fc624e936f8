// Host <-> device moves of DeviceChangeAPI (rstsr-core/src/storage/conversion.rs:3-21:
// to_cpu_vec / from_cpu_vec / outof_cpu_vec) for any host memory.
//
// Page-locked host memory (cudaHostAlloc / cudaHostRegister, torch's
// pin_memory) is copied by one stream-ordered cudaMemcpyAsync. Ordinary
// pageable memory -- a Rust Vec<T>, a numpy array -- goes through the
// context's staging ring: kRing page-locked buffers of kChunk bytes each.
// Host to device: chunk i is copied by the host into buffer i % kRing (after
// the device has drained that buffer's previous chunk, an event wait) and
// sent with one cudaMemcpyAsync, so the host copy of chunk i+1 overlaps the
// transfer of chunk i. Device to host: up to kRing chunks are in flight into
// the ring while the host copies finished ones out. The host-side copies are
// split over a few worker threads: one thread's memcpy is several times
// slower than the chip-to-chip link.
#include <condition_variable>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"

namespace rstsr {

namespace {

constexpr size_t kChunk = size_t(8) << 20;
constexpr int kRing = 4;
// below this size one thread copies (waking the workers costs more)
constexpr size_t kParallelMin = size_t(1) << 20;

// A fixed team of worker threads that copy disjoint parts of one buffer.
class CopyTeam {
  public:
    explicit CopyTeam(int nworkers) {
        for (int i = 0; i < nworkers; ++i) threads_.emplace_back([this, i] { work(i); });
    }
    ~CopyTeam() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& t : threads_) t.join();
    }
    // dst[0, n) = src[0, n), split over the workers and the calling thread
    void copy(void* dst, const void* src, size_t n) {
        const int parts = (int)threads_.size() + 1;
        if (n < kParallelMin || parts == 1) {
            memcpy(dst, src, n);
            return;
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            dst_ = static_cast<char*>(dst);
            src_ = static_cast<const char*>(src);
            n_ = n;
            parts_ = parts;
            pending_ = (int)threads_.size();
            ++gen_;
        }
        cv_.notify_all();
        do_part(parts - 1);
        std::unique_lock<std::mutex> lk(mu_);
        done_cv_.wait(lk, [this] { return pending_ == 0; });
    }

  private:
    void do_part(int p) {
        // parts of 64-byte multiples
        const size_t per = ((n_ + parts_ - 1) / parts_ + 63) / 64 * 64;
        const size_t b = std::min(n_, per * (size_t)p), e = std::min(n_, b + per);
        if (e > b) memcpy(dst_ + b, src_ + b, e - b);
    }
    void work(int id) {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
            }
            do_part(id);
            std::lock_guard<std::mutex> lk(mu_);
            if (--pending_ == 0) done_cv_.notify_one();
        }
    }
    std::vector<std::thread> threads_;
    std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    bool stop_ = false;
    uint64_t gen_ = 0;
    char* dst_ = nullptr;
    const char* src_ = nullptr;
    size_t n_ = 0;
    int parts_ = 1, pending_ = 0;
};

}  // namespace

struct StagingRing {
    std::mutex mu;  // one staged transfer at a time per context
    void* buf[kRing] = {};
    cudaEvent_t ev[kRing] = {};
    CopyTeam* team = nullptr;
};

static int staging_get(rstsr_ctx* ctx, StagingRing** out) {
    std::lock_guard<std::mutex> lk(ctx->staging_mu);
    if (!ctx->staging) {
        auto* r = new StagingRing();
        for (int i = 0; i < kRing; ++i) {
            cudaError_t e = cudaHostAlloc(&r->buf[i], kChunk, cudaHostAllocPortable);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->ev[i], cudaEventDisableTiming);
            if (e != cudaSuccess) {
                for (int j = 0; j <= i; ++j) {
                    if (r->buf[j]) cudaFreeHost(r->buf[j]);
                    if (r->ev[j]) cudaEventDestroy(r->ev[j]);
                }
                delete r;
                return cuda_fail(e, "staging ring allocation");
            }
        }
        // one thread's memcpy moves about 9 GB/s on the Grace host: the ring
        // (72 GB/s with eight threads) was bound by them, not by the link
        const unsigned hw = std::thread::hardware_concurrency();
        r->team = new CopyTeam((int)std::min(15u, hw > 1 ? hw - 1 : 0u));
        ctx->staging = r;
    }
    *out = ctx->staging;
    return RSTSR_OK;
}

void staging_destroy(rstsr_ctx* ctx) {
    StagingRing* r = ctx->staging;
    if (!r) return;
    for (int i = 0; i < kRing; ++i) {
        if (r->ev[i]) {
            cudaEventSynchronize(r->ev[i]);
            cudaEventDestroy(r->ev[i]);
        }
        if (r->buf[i]) cudaFreeHost(r->buf[i]);
    }
    delete r->team;
    delete r;
    ctx->staging = nullptr;
}

// Host memory that the copy engines can reach directly (page-locked or
// registered), or device / managed memory.
static int is_pageable(const void* p, bool* pageable) {
    cudaPointerAttributes at;
    cudaError_t e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess) return cuda_fail(e, "cudaPointerGetAttributes");
    *pageable = at.type == cudaMemoryTypeUnregistered;
    return RSTSR_OK;
}

static int refuse_capture(rstsr_ctx* ctx, const char* what) {
    cudaStreamCaptureStatus cs;
    if (cudaStreamIsCapturing(ctx->stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
        return fail(RSTSR_ERR_RUNTIME, std::string(what) +
                                           ": a staged copy of pageable host memory waits on the host and cannot "
                                           "be captured into a graph");
    return RSTSR_OK;
}

}  // namespace rstsr

using namespace rstsr;

extern "C" {

int rstsr_cuda_memcpy_h2d_async(rstsr_ctx* ctx, void* dst, const void* src, size_t nbytes) {
    clear_error();
    int s = enter(ctx);
    if (s) return s;
    if (nbytes == 0) return RSTSR_OK;
    if (!dst || !src) return fail(RSTSR_ERR_INVALID_VALUE, "null pointer in memcpy_h2d_async");
    bool pageable = false;
    if ((s = is_pageable(src, &pageable))) return s;
    if (!pageable) {
        RSTSR_CUDA_TRY(cudaMemcpyAsync(dst, src, nbytes, cudaMemcpyDefault, ctx->stream));
        return RSTSR_OK;
    }
    if ((s = refuse_capture(ctx, "memcpy_h2d_async"))) return s;
    StagingRing* r = nullptr;
    if ((s = staging_get(ctx, &r))) return s;
    std::lock_guard<std::mutex> lk(r->mu);
    const char* h = static_cast<const char*>(src);
    char* d = static_cast<char*>(dst);
    for (size_t off = 0, i = 0; off < nbytes; off += kChunk, ++i) {
        const int j = (int)(i % kRing);
        const size_t len = std::min(kChunk, nbytes - off);
        // the device has drained this buffer's previous chunk
        RSTSR_CUDA_TRY(cudaEventSynchronize(r->ev[j]));
        r->team->copy(r->buf[j], h + off, len);
        RSTSR_CUDA_TRY(cudaMemcpyAsync(d + off, r->buf[j], len, cudaMemcpyHostToDevice, ctx->stream));
        RSTSR_CUDA_TRY(cudaEventRecord(r->ev[j], ctx->stream));
    }
    return RSTSR_OK;
}

int rstsr_cuda_memcpy_d2h_async(rstsr_ctx* ctx, void* dst, const void* src, size_t nbytes) {
    clear_error();
    int s = enter(ctx);
    if (s) return s;
    if (nbytes == 0) return RSTSR_OK;
    if (!dst || !src) return fail(RSTSR_ERR_INVALID_VALUE, "null pointer in memcpy_d2h_async");
    bool pageable = false;
    if ((s = is_pageable(dst, &pageable))) return s;
    if (!pageable) {
        RSTSR_CUDA_TRY(cudaMemcpyAsync(dst, src, nbytes, cudaMemcpyDefault, ctx->stream));
        return RSTSR_OK;
    }
    if ((s = refuse_capture(ctx, "memcpy_d2h_async"))) return s;
    StagingRing* r = nullptr;
    if ((s = staging_get(ctx, &r))) return s;
    std::lock_guard<std::mutex> lk(r->mu);
    char* h = static_cast<char*>(dst);
    const char* d = static_cast<const char*>(src);
    const size_t nchunks = (nbytes + kChunk - 1) / kChunk;
    auto issue = [&](size_t i) -> int {
        const int j = (int)(i % kRing);
        const size_t off = i * kChunk, len = std::min(kChunk, nbytes - off);
        RSTSR_CUDA_TRY(cudaMemcpyAsync(r->buf[j], d + off, len, cudaMemcpyDeviceToHost, ctx->stream));
        RSTSR_CUDA_TRY(cudaEventRecord(r->ev[j], ctx->stream));
        return RSTSR_OK;
    };
    // a ring buffer may still be read by an earlier host-to-device chunk
    for (int j = 0; j < kRing; ++j) RSTSR_CUDA_TRY(cudaEventSynchronize(r->ev[j]));
    for (size_t i = 0; i < nchunks && i < (size_t)kRing; ++i)
        if ((s = issue(i))) return s;
    for (size_t i = 0; i < nchunks; ++i) {
        const int j = (int)(i % kRing);
        const size_t off = i * kChunk, len = std::min(kChunk, nbytes - off);
        RSTSR_CUDA_TRY(cudaEventSynchronize(r->ev[j]));
        r->team->copy(h + off, r->buf[j], len);
        if (i + kRing < nchunks && (s = issue(i + kRing))) return s;
    }
    return RSTSR_OK;
}

}  // extern "C"
