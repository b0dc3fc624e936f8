// index_select: c[..., k, ...] = a[..., indices[k], ...] along one axis,
// replacing rstsr-native-impl/src/cpu_serial/adv_indexing.rs:3-69
// (index_select_cpu_serial) and cpu_rayon/adv_indexing.rs behind
// DeviceIndexSelectAPI (rstsr-core/src/operators/adv_indexing.rs:8-23).
//
// The reference walks two cases (indexed axis contiguous in c: an inner loop
// over the indices; otherwise one strided assign per selected slice). Here
// both are one gather kernel over a collapsed iteration space of c: the
// indexed axis stays its own dim (never merged) and maps its coordinate k to
// indices[k] * a_stride; every other axis is collapsed as in the element-wise
// kernels. When the innermost dim is contiguous in both c and a (selecting
// rows, slabs or blocks), elements move as 16/8/4/2-byte words; when the
// indexed axis is innermost, stores stay coalesced and loads gather.
//
// The index list arrives in HOST memory (the reference's `&[usize]`). Up to
// kIdxInline indices (as int32, extents below 2^31) ride in the kernel
// parameters (no copy, valid inside a graph capture: the list is baked into
// the captured launch); longer lists are copied to stream-ordered scratch first.
#include <atomic>

#include "ew_kernel.cuh"
#include "tc_ptx.cuh"

namespace rstsr {

namespace {

constexpr int kIdxInline = 512;
constexpr int kIsThreads = 256;
constexpr int kIsUnroll = 4;
constexpr int64_t kStageMaxBytes = 96 * 1024;  // source row staged in shared memory (two CTAs per SM)
constexpr int kBulkThreads = 512;
constexpr int64_t kBulkMinRow = 4096;           // rows staged by bulk copies: 4 KiB ..
constexpr int64_t kBulkSmem = 220 * 1024;       // .. with 2-4 row buffers (+ the index list) in this much
constexpr int64_t kBulkIdxMax = 8192;           // indices kept in shared memory as int32 (else read from global)
constexpr uint32_t kBulkChunk = 32 * 1024;      // bytes per cp.async.bulk
constexpr int kIsErrStageWait = 5;              // error word: a staged-row wait gave up

struct IsParams {
    DevDims dims;            // inner first
    int axis_dim;            // dims index of the indexed axis, -1 if folded away
    int big;                 // 64-bit index decomposition
    int64_t total;
    uint32_t nrows;          // product of dims 1.. (row kernel)
    int64_t sc[RSTSR_MAX_NDIM], sa[RSTSR_MAX_NDIM];
    int64_t off_c, off_a;
    int64_t row_len;         // staged kernel: source elements per row (the axis extent)
    int stage_vec;           // staged kernel: rows load as 16-byte words
    int nbuf;                // bulk kernel: row buffers (0: not the bulk kernel)
    uint32_t buf_stride;     // bulk kernel: bytes between row buffers
    int idx_smem;            // bulk kernel: the index list is staged in shared memory
    int* err;                // device error word
    int nidx;                // indices held inline (0: use idx)
    const int64_t* idx;      // device copy of the indices (long lists)
    int32_t inl[kIdxInline];  // inline indices (int32: the parameter block stays below 4 KB)
};

static_assert(sizeof(IsParams) < 4096, "the kernel parameter block stays within 4 KB");

template <typename W>
__global__ void __launch_bounds__(kIsThreads)
    index_select_kernel(W* __restrict__ c, const W* __restrict__ a, const __grid_constant__ IsParams p) {
    __shared__ int64_t sidx[kIdxInline];
    for (int i = threadIdx.x; i < p.nidx; i += blockDim.x) sidx[i] = p.inl[i];
    __syncthreads();
    const int64_t* ix = p.nidx ? sidx : p.idx;
    const int64_t step = (int64_t)gridDim.x * kIsThreads;
    for (int64_t base = (int64_t)blockIdx.x * kIsThreads * kIsUnroll + threadIdx.x; base < p.total;
         base += step * kIsUnroll) {
        W v[kIsUnroll];
        int64_t oc[kIsUnroll];
#pragma unroll
        for (int u = 0; u < kIsUnroll; ++u) {
            const int64_t e = base + (int64_t)u * kIsThreads;
            oc[u] = -1;
            if (e >= p.total) continue;
            int64_t offc = p.off_c, offa = p.off_a;
            if (p.big) {
                uint64_t rem = (uint64_t)e;
                for (int d = 0; d < p.dims.ndim; ++d) {
                    const uint64_t q = d + 1 < p.dims.ndim ? rem / p.dims.shape[d] : 0;
                    const int64_t k = (int64_t)(rem - q * p.dims.shape[d]);
                    rem = q;
                    offc += k * p.sc[d];
                    offa += (d == p.axis_dim ? ix[k] : k) * p.sa[d];
                }
            } else {
                uint32_t rem = (uint32_t)e;
                for (int d = 0; d < p.dims.ndim; ++d) {
                    const uint32_t q = d + 1 < p.dims.ndim ? p.dims.div[d].div(rem) : 0;
                    const int64_t k = (int64_t)(rem - q * p.dims.shape[d]);
                    rem = q;
                    offc += k * p.sc[d];
                    offa += (d == p.axis_dim ? ix[k] : k) * p.sa[d];
                }
            }
            oc[u] = offc;
            v[u] = a[offa];
        }
#pragma unroll
        for (int u = 0; u < kIsUnroll; ++u)
            if (oc[u] >= 0) c[oc[u]] = v[u];
    }
}

// Innermost dim long (>= one CTA width): a CTA walks whole rows of it, the
// outer multi-index decomposed once per row; four loads in flight per thread.
template <typename W>
__global__ void __launch_bounds__(kIsThreads, 6)
    index_select_rows_kernel(W* __restrict__ c, const W* __restrict__ a, const __grid_constant__ IsParams p) {
    __shared__ int64_t sidx[kIdxInline];
    for (int i = threadIdx.x; i < p.nidx; i += blockDim.x) sidx[i] = p.inl[i];
    __syncthreads();
    const int64_t* ix = p.nidx ? sidx : p.idx;
    const int64_t n0 = p.dims.shape[0], sc0 = p.sc[0], sa0 = p.sa[0];
    const bool ax0 = p.axis_dim == 0;
    for (uint32_t row = blockIdx.x; row < p.nrows; row += gridDim.x) {
        int64_t offc = p.off_c, offa = p.off_a;
        uint32_t rem = row;
        for (int d = 1; d < p.dims.ndim; ++d) {
            const uint32_t q = d + 1 < p.dims.ndim ? p.dims.div[d].div(rem) : 0;
            const int64_t k = (int64_t)(rem - q * p.dims.shape[d]);
            rem = q;
            offc += k * p.sc[d];
            offa += (d == p.axis_dim ? ix[k] : k) * p.sa[d];
        }
        for (int64_t k0 = threadIdx.x; k0 < n0; k0 += kIsThreads * kIsUnroll) {
            W v[kIsUnroll];
#pragma unroll
            for (int u = 0; u < kIsUnroll; ++u) {
                const int64_t k = k0 + (int64_t)u * kIsThreads;
                if (k < n0) v[u] = a[offa + (ax0 ? ix[k] : k) * sa0];
            }
#pragma unroll
            for (int u = 0; u < kIsUnroll; ++u) {
                const int64_t k = k0 + (int64_t)u * kIsThreads;
                if (k < n0) c[offc + k * sc0] = v[u];
            }
        }
    }
}

// Indexed axis innermost, contiguous in the source, and the selection dense
// (at least one index per four source elements): gathering straight from
// global memory would fetch a 32-byte sector per element in random order, so
// the CTA first copies the whole source row into shared memory with coalesced
// (16-byte where aligned) loads, then gathers from there with coalesced
// stores. Two CTAs per SM overlap one's row load with the other's gather.
template <typename W>
__global__ void __launch_bounds__(kIsThreads)
    index_select_staged_kernel(W* __restrict__ c, const W* __restrict__ a, const __grid_constant__ IsParams p) {
    extern __shared__ uint4 stage_raw[];
    __shared__ int64_t sidx[kIdxInline];
    for (int i = threadIdx.x; i < p.nidx; i += blockDim.x) sidx[i] = p.inl[i];
    const int64_t* ix = p.nidx ? sidx : p.idx;
    W* row = reinterpret_cast<W*>(stage_raw);
    const int64_t n0 = p.dims.shape[0], sc0 = p.sc[0], L = p.row_len;
    const int64_t nvec = L * (int64_t)sizeof(W) / 16;
    for (uint32_t r = blockIdx.x; r < p.nrows; r += gridDim.x) {
        int64_t offc = p.off_c, offa = p.off_a;
        uint32_t rem = r;
        for (int d = 1; d < p.dims.ndim; ++d) {
            const uint32_t q = d + 1 < p.dims.ndim ? p.dims.div[d].div(rem) : 0;
            const int64_t k = (int64_t)(rem - q * p.dims.shape[d]);
            rem = q;
            offc += k * p.sc[d];
            offa += (d == p.axis_dim ? ix[k] : k) * p.sa[d];
        }
        __syncthreads();  // the previous row's gathers are done with the stage
        if (p.stage_vec) {
            const uint4* src = reinterpret_cast<const uint4*>(a + offa);
            for (int64_t q0 = threadIdx.x; q0 < nvec; q0 += kIsThreads * kIsUnroll) {
                uint4 v[kIsUnroll];
#pragma unroll
                for (int u = 0; u < kIsUnroll; ++u)
                    if (q0 + u * kIsThreads < nvec) v[u] = src[q0 + u * kIsThreads];
#pragma unroll
                for (int u = 0; u < kIsUnroll; ++u)
                    if (q0 + u * kIsThreads < nvec) stage_raw[q0 + u * kIsThreads] = v[u];
            }
        } else {
            for (int64_t q0 = threadIdx.x; q0 < L; q0 += kIsThreads * kIsUnroll) {
                W v[kIsUnroll];
#pragma unroll
                for (int u = 0; u < kIsUnroll; ++u)
                    if (q0 + u * kIsThreads < L) v[u] = a[offa + q0 + u * kIsThreads];
#pragma unroll
                for (int u = 0; u < kIsUnroll; ++u)
                    if (q0 + u * kIsThreads < L) row[q0 + u * kIsThreads] = v[u];
            }
        }
        __syncthreads();
        for (int64_t k = threadIdx.x; k < n0; k += kIsThreads) c[offc + k * sc0] = row[ix[k]];
    }
}

// The staged gather with the rows moved by the copy engine: one CTA per SM
// keeps nbuf source rows in flight as cp.async.bulk copies (completion counted
// on one mbarrier per buffer) and gathers from the oldest while the others
// fill. Every wait is bounded; a CTA that gives up records kIsErrStageWait,
// waits (bounded) for its copies still in flight, and returns.
template <typename W>
__global__ void __launch_bounds__(kBulkThreads)
    index_select_bulk_kernel(W* __restrict__ c, const W* __restrict__ a, const __grid_constant__ IsParams p) {
    extern __shared__ __align__(128) uint8_t stage[];
    __shared__ __align__(8) uint64_t full[4];
    const int nbuf = p.nbuf;
    const int64_t n0 = p.dims.shape[0], sc0 = p.sc[0];
    const uint32_t row_bytes = (uint32_t)(p.row_len * (int64_t)sizeof(W));
    // the index list as int32 behind the row buffers (indices < row_len <= 96 Ki)
    int32_t* sidx = reinterpret_cast<int32_t*>(stage + (size_t)nbuf * p.buf_stride);
    if (p.idx_smem)
        for (int64_t k = threadIdx.x; k < n0; k += kBulkThreads) sidx[k] = (int32_t)(p.nidx ? p.inl[k] : p.idx[k]);
    if (threadIdx.x == 0) {
        for (int b = 0; b < nbuf; ++b) tc::mbar_init(&full[b], 1);
        tc::fence_barrier_init();
    }
    __syncthreads();
    const uint32_t nmine = (p.nrows - blockIdx.x + gridDim.x - 1) / gridDim.x;
    auto offsets = [&](uint32_t j, int64_t& offc, int64_t& offa) {
        uint32_t rem = blockIdx.x + j * gridDim.x;
        offc = p.off_c;
        offa = p.off_a;
        for (int d = 1; d < p.dims.ndim; ++d) {
            const uint32_t q = d + 1 < p.dims.ndim ? p.dims.div[d].div(rem) : 0;
            const int64_t k = (int64_t)(rem - q * p.dims.shape[d]);
            rem = q;
            offc += k * p.sc[d];
            offa += k * p.sa[d];  // the indexed axis is dim 0 here
        }
    };
    auto issue = [&](uint32_t j) {
        int64_t oc, oa;
        offsets(j, oc, oa);
        uint64_t* bar = &full[j % nbuf];
        const uint8_t* src = reinterpret_cast<const uint8_t*>(a + oa);
        uint8_t* dst = stage + (size_t)(j % nbuf) * p.buf_stride;
        tc::mbar_arrive_expect_tx(bar, row_bytes);
        for (uint32_t o = 0; o < row_bytes; o += kBulkChunk)
            tc::bulk_load(dst + o, src + o, row_bytes - o < kBulkChunk ? row_bytes - o : kBulkChunk, bar);
    };
    if (threadIdx.x == 0)
        for (uint32_t j = 0; j < (uint32_t)nbuf && j < nmine; ++j) issue(j);
    for (uint32_t j = 0; j < nmine; ++j) {
        const bool ok = tc::mbar_wait(&full[j % nbuf], (j / nbuf) & 1u);
        if (!__syncthreads_and(ok)) {
            if (threadIdx.x == 0) {
                atomicExch(p.err, kIsErrStageWait);
                for (uint32_t q = j; q < j + (uint32_t)nbuf && q < nmine; ++q)
                    (void)tc::mbar_wait(&full[q % nbuf], (q / nbuf) & 1u);
            }
            return;
        }
        int64_t offc, offa;
        offsets(j, offc, offa);
        const W* row = reinterpret_cast<const W*>(stage + (size_t)(j % nbuf) * p.buf_stride);
        for (int64_t k0 = threadIdx.x; k0 < n0; k0 += kBulkThreads * kIsUnroll) {
            W v[kIsUnroll];
#pragma unroll
            for (int u = 0; u < kIsUnroll; ++u) {
                const int64_t k = k0 + (int64_t)u * kBulkThreads;
                if (k < n0) v[u] = row[p.idx_smem ? (int64_t)sidx[k] : (p.nidx ? (int64_t)p.inl[k] : p.idx[k])];
            }
#pragma unroll
            for (int u = 0; u < kIsUnroll; ++u) {
                const int64_t k = k0 + (int64_t)u * kBulkThreads;
                if (k < n0) c[offc + k * sc0] = v[u];
            }
        }
        __syncthreads();  // every thread is done with this buffer
        if (threadIdx.x == 0 && j + nbuf < nmine) issue(j + nbuf);
    }
}

struct IsDim {
    int64_t shape, sc, sa;
    bool axis;
};

template <typename W>
int launch_is(rstsr_ctx* ctx, const IsParams& p, void* c, const void* a) {
    if (p.nbuf > 0) {
        const size_t smem = (size_t)p.nbuf * p.buf_stride + (p.idx_smem ? (size_t)p.dims.shape[0] * 4 : 0);
        static std::atomic<uint64_t> attr_set{0};  // bit d: opted in on device d
        const uint64_t bit = 1ull << (ctx->device & 63);
        if (!(attr_set.load() & bit)) {
            RSTSR_CUDA_TRY(cudaFuncSetAttribute(index_select_bulk_kernel<W>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBulkSmem));
            attr_set.fetch_or(bit);
        }
        const uint32_t cap = (uint32_t)ctx->num_sms;
        index_select_bulk_kernel<W><<<p.nrows < cap ? p.nrows : cap, kBulkThreads, smem, ctx->stream>>>(
            static_cast<W*>(c), static_cast<const W*>(a), p);
        return after_launch(ctx, "index_select_bulk_kernel");
    }
    if (p.row_len > 0) {
        const size_t smem = (size_t)((p.row_len * (int64_t)sizeof(W) + 15) / 16 * 16);
        static std::atomic<uint64_t> attr_set{0};  // bit d: opted in on device d
        const uint64_t bit = 1ull << (ctx->device & 63);
        if (!(attr_set.load() & bit)) {
            RSTSR_CUDA_TRY(cudaFuncSetAttribute(index_select_staged_kernel<W>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStageMaxBytes));
            attr_set.fetch_or(bit);
        }
        const uint32_t cap = (uint32_t)ctx->num_sms * 2;
        index_select_staged_kernel<W><<<p.nrows < cap ? p.nrows : cap, kIsThreads, smem, ctx->stream>>>(
            static_cast<W*>(c), static_cast<const W*>(a), p);
        return after_launch(ctx, "index_select_staged_kernel");
    }
    if (p.nrows > 0) {
        const uint32_t cap = (uint32_t)ctx->num_sms * 6;  // the resident CTAs (40 registers)
        index_select_rows_kernel<W><<<p.nrows < cap ? p.nrows : cap, kIsThreads, 0, ctx->stream>>>(
            static_cast<W*>(c), static_cast<const W*>(a), p);
        return after_launch(ctx, "index_select_rows_kernel");
    }
    const int64_t per_cta = (int64_t)kIsThreads * kIsUnroll;
    int64_t grid = (p.total + per_cta - 1) / per_cta;
    const int64_t cap = (int64_t)ctx->num_sms * 8;
    if (grid > cap) grid = cap;
    index_select_kernel<W><<<(int)grid, kIsThreads, 0, ctx->stream>>>(static_cast<W*>(c),
                                                                         static_cast<const W*>(a), p);
    return after_launch(ctx, "index_select_kernel");
}

}  // namespace

}  // namespace rstsr

using namespace rstsr;

extern "C" {

int rstsr_cuda_index_select(rstsr_ctx* ctx, rstsr_dtype t, void* c, const rstsr_layout* lc, const void* a,
                            const rstsr_layout* la, int32_t axis, const uint64_t* indices, int64_t nindices) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(lc, "c"));
    RSTSR_TRY(check_layout(la, "a"));
    if (!dtype_valid(t)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    Layout Lc = Layout::from_abi(*lc), La = Layout::from_abi(*la);
    if (Lc.ndim != La.ndim) return fail(RSTSR_ERR_INVALID_LAYOUT, "index_select: input and output ndim differ");
    if (axis < 0 || axis >= La.ndim)
        return fail(RSTSR_ERR_AXIS, "index_select: axis " + std::to_string(axis) + " out of range for ndim " +
                                        std::to_string(La.ndim));
    if (nindices < 0 || Lc.shape[axis] != nindices)
        return fail(RSTSR_ERR_INVALID_LAYOUT, "index_select: output extent on the axis is not the index count");
    for (int d = 0; d < La.ndim; ++d)
        if (d != axis && Lc.shape[d] != La.shape[d])
            return fail(RSTSR_ERR_INVALID_LAYOUT,
                        "index_select: extents off the axis differ (" + Lc.repr() + ", " + La.repr() + ")");
    if (nindices > 0 && !indices) return fail(RSTSR_ERR_INVALID_VALUE, "index_select: null index list");
    for (int64_t k = 0; k < nindices; ++k)
        if (indices[k] >= (uint64_t)La.shape[axis])
            return fail(RSTSR_ERR_INDEX, "index_select: index " + std::to_string(indices[k]) +
                                             " out of range for extent " + std::to_string(La.shape[axis]));
    RSTSR_TRY(check_write_layout(Lc, "index_select"));
    if (Lc.size() == 0) return RSTSR_OK;
    if (!c || !a) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");

    // collapse c's iteration space; the indexed axis is never merged
    int64_t off_c = Lc.offset, off_a = La.offset;
    std::vector<IsDim> dims;
    for (int d = 0; d < La.ndim; ++d) {
        if (d == axis) {
            if (nindices == 1)
                off_a += (int64_t)indices[0] * La.stride[d];
            else
                dims.push_back({nindices, Lc.stride[d], La.stride[d], true});
        } else if (La.shape[d] != 1) {
            dims.push_back({La.shape[d], Lc.stride[d], La.stride[d], false});
        }
    }
    std::stable_sort(dims.begin(), dims.end(), [](const IsDim& x, const IsDim& y) {
        if (std::llabs(x.sc) != std::llabs(y.sc)) return std::llabs(x.sc) < std::llabs(y.sc);
        return std::llabs(x.sa) < std::llabs(y.sa);
    });
    std::vector<IsDim> merged;
    for (const IsDim& d : dims) {
        if (!merged.empty()) {
            IsDim& m = merged.back();
            if (!m.axis && !d.axis && m.shape * m.sc == d.sc && m.shape * m.sa == d.sa) {
                m.shape *= d.shape;
                continue;
            }
        }
        merged.push_back(d);
    }
    // element word: widen along a contiguous inner dim when everything aligns
    const size_t es = dtype_size(t);
    int64_t vec = 1;
    if (!merged.empty() && !merged[0].axis && merged[0].sc == 1 && merged[0].sa == 1) {
        for (int64_t v = 16 / (int64_t)es; v >= 2; v /= 2) {
            bool ok = merged[0].shape % v == 0 && off_c % v == 0 && off_a % v == 0 &&
                      reinterpret_cast<uintptr_t>(c) % (v * es) == 0 && reinterpret_cast<uintptr_t>(a) % (v * es) == 0;
            for (size_t d = 1; d < merged.size() && ok; ++d) ok = merged[d].sc % v == 0 && merged[d].sa % v == 0;
            if (ok) {
                vec = v;
                break;
            }
        }
    }
    if (vec > 1) {
        merged[0].shape /= vec;
        merged[0].sc = merged[0].sa = 1;
        for (size_t d = 1; d < merged.size(); ++d) {
            merged[d].sc /= vec;
            merged[d].sa /= vec;
        }
        off_c /= vec;
        off_a /= vec;
    }
    if ((int)merged.size() > RSTSR_MAX_NDIM) return fail(RSTSR_ERR_INVALID_LAYOUT, "index_select: too many dims");

    IsParams p;
    std::memset(&p, 0, sizeof(p));
    p.dims.ndim = (int)merged.size();
    p.axis_dim = -1;
    p.total = 1;
    for (size_t d = 0; d < merged.size(); ++d) {
        p.total *= merged[d].shape;
        p.sc[d] = merged[d].sc;
        p.sa[d] = merged[d].sa;
        if (merged[d].axis) p.axis_dim = (int)d;
    }
    p.big = p.total > INT32_MAX;
    for (size_t d = 0; d < merged.size(); ++d) {
        if (merged[d].shape > UINT32_MAX)
            return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, "index_select: one collapsed extent above 2^32");
        p.dims.shape[d] = (uint32_t)merged[d].shape;
        p.dims.div[d] = FastDiv((uint32_t)merged[d].shape);
    }
    // rows of the innermost dim when it fills a CTA and the rows count fits
    if (!merged.empty() && merged[0].shape >= kIsThreads && p.total / merged[0].shape <= INT32_MAX)
        p.nrows = (uint32_t)(p.total / merged[0].shape);
    // dense selection along a contiguous innermost source axis: stage the row
    const int64_t axis_len = La.shape[axis];
    if (p.nrows > 0 && p.axis_dim == 0 && merged[0].sa == 1 && axis_len * (int64_t)es <= kStageMaxBytes &&
        nindices * 4 >= axis_len) {
        p.row_len = axis_len;
        bool vec_ok = (axis_len * (int64_t)es) % 16 == 0 && reinterpret_cast<uintptr_t>(a) % 16 == 0 &&
                      (off_a * (int64_t)es) % 16 == 0;
        for (size_t d = 1; d < merged.size() && vec_ok; ++d)
            if (!merged[d].axis) vec_ok = (merged[d].sa * (int64_t)es) % 16 == 0;
        p.stage_vec = vec_ok ? 1 : 0;
        const int64_t row_bytes = axis_len * (int64_t)es;
        if (vec_ok && row_bytes >= kBulkMinRow) {
            p.buf_stride = (uint32_t)((row_bytes + 127) / 128 * 128);
            p.idx_smem = nindices <= kBulkIdxMax ? 1 : 0;
            int64_t nb = (kBulkSmem - (p.idx_smem ? nindices * 4 : 0)) / p.buf_stride;
            if (nb < 2 && p.idx_smem) {  // a long row and a long list: keep the list in global memory
                p.idx_smem = 0;
                nb = kBulkSmem / p.buf_stride;
            }
            p.nbuf = (int)(nb > 4 ? 4 : nb);  // >= 2: rows are at most kStageMaxBytes
        }
    }
    p.err = ctx->dev_err;
    p.off_c = off_c;
    p.off_a = off_a;

    int64_t* dev_idx = nullptr;
    if (p.axis_dim >= 0) {
        if (nindices <= kIdxInline && La.shape[axis] <= INT32_MAX) {
            p.nidx = (int)nindices;
            for (int64_t k = 0; k < nindices; ++k) p.inl[k] = (int32_t)indices[k];
        } else {
            if (ctx->capturing)
                return fail(RSTSR_ERR_UNIMPLEMENTED,
                            "index_select: more than 512 indices cannot be captured into a graph "
                            "(the host list would be read again at every replay)");
            std::vector<int64_t> host(indices, indices + nindices);
            RSTSR_TRY(scratch_alloc(ctx, nindices * sizeof(int64_t), reinterpret_cast<void**>(&dev_idx)));
            cudaError_t e = cudaMemcpyAsync(dev_idx, host.data(), nindices * sizeof(int64_t),
                                            cudaMemcpyHostToDevice, ctx->stream);
            if (e != cudaSuccess) {
                scratch_free(ctx, dev_idx);
                return cuda_fail(e, "index_select index upload");
            }
            p.idx = dev_idx;
        }
    }
    int rc;
    switch (es * vec) {
        case 1: rc = launch_is<uint8_t>(ctx, p, c, a); break;
        case 2: rc = launch_is<uint16_t>(ctx, p, c, a); break;
        case 4: rc = launch_is<uint32_t>(ctx, p, c, a); break;
        case 8: rc = launch_is<uint64_t>(ctx, p, c, a); break;
        case 16: rc = launch_is<uint4>(ctx, p, c, a); break;
        default: rc = fail(RSTSR_ERR_INVALID_VALUE, "unsupported element size");
    }
    if (dev_idx) {
        // the pageable source was staged by the runtime before cudaMemcpyAsync
        // returned, so the host vector may go; the scratch is freed in stream order
        scratch_free(ctx, dev_idx);
    }
    return rc;
}

}  // extern "C"
