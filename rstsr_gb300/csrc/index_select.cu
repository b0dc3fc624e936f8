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
// kIdxInline indices ride in the kernel parameters (no copy, valid inside a
// graph capture: the list is baked into the captured launch); longer lists
// are copied to stream-ordered scratch first.
#include "ew_kernel.cuh"

namespace rstsr {

namespace {

constexpr int kIdxInline = 512;
constexpr int kIsThreads = 256;
constexpr int kIsUnroll = 4;

struct IsParams {
    DevDims dims;            // inner first
    int axis_dim;            // dims index of the indexed axis, -1 if folded away
    int big;                 // 64-bit index decomposition
    int64_t total;
    int64_t sc[RSTSR_MAX_NDIM], sa[RSTSR_MAX_NDIM];
    int64_t off_c, off_a;
    int nidx;                // indices held inline (0: use idx)
    const int64_t* idx;      // device copy of the indices (long lists)
    int64_t inl[kIdxInline];
};

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

struct IsDim {
    int64_t shape, sc, sa;
    bool axis;
};

template <typename W>
int launch_is(rstsr_ctx* ctx, const IsParams& p, void* c, const void* a) {
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
        if (!p.big) p.dims.div[d] = FastDiv((uint32_t)merged[d].shape);
    }
    p.off_c = off_c;
    p.off_a = off_a;

    int64_t* dev_idx = nullptr;
    if (p.axis_dim >= 0) {
        if (nindices <= kIdxInline) {
            p.nidx = (int)nindices;
            for (int64_t k = 0; k < nindices; ++k) p.inl[k] = (int64_t)indices[k];
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
