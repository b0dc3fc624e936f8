// assign / assign_arbitrary / fill: the copies behind to_contig, to_layout,
// reshape and the storage conversions, replacing
// rstsr-native-impl/src/cpu_rayon/assignment.rs (assign_arbitary_*_cpu_rayon
// :14-93, assign_*_cpu_rayon :95-171, fill_promote_cpu_rayon :181-225).
//
// Four kernels: the shared strided element-wise kernel moving raw element bits
// (vector copy when both sides are contiguous along the innermost collapsed
// dim); a shared-memory tile transpose when the source is contiguous along a
// different dim than the destination (axis-permuted layouts); an index-walk
// kernel for copies between different shapes (reshape-like assign_arbitrary);
// and one runtime-typed kernel for copies that convert between dtypes with
// Rust `as` semantics (DTypeCastAPI, rstsr-dtype-traits/src/promotion.rs:160-230).
#include "ew_kernel.cuh"

namespace rstsr {

template <typename T>
struct CopyF {
    __device__ __forceinline__ T operator()(const T* v) const { return v[0]; }
};

template <typename T>
struct ConstF {
    T value;
    __device__ __forceinline__ T operator()(const T*) const { return value; }
};

// ------------------------------------------------------------ transpose

constexpr int kTile = 32;
constexpr int kTileRows = 8;

struct TrParams {
    int64_t n0, nj;
    int64_t in_s0, in_sj, out_sj;
    int64_t in_off, out_off;
    int nb;
    uint32_t bshape[RSTSR_MAX_NDIM];
    FastDiv bdiv[RSTSR_MAX_NDIM];
    int64_t in_bs[RSTSR_MAX_NDIM], out_bs[RSTSR_MAX_NDIM];
    FastDiv div_t0, div_tj;
    uint32_t tiles0, tilesj;
    uint32_t ntiles;
    // transpose2_kernel: dim j folded with the batch dim that continues it in
    // the source (source stride nj_in): column ij of the tile writes at
    // (ij mod nj_in) * out_sj + (ij / nj_in) * out_sjo; jlog = log2(nj_in), 0 = no fold
    int jlog;
    int64_t out_sjo;
};

// Source contiguous along dim j, destination along dim 0: reads coalesce along
// j, writes along 0, and the exchange goes through a padded shared tile.
template <typename T>
__global__ void __launch_bounds__(kTile * kTileRows)
    transpose_kernel(T* __restrict__ out, const T* __restrict__ in, const TrParams p) {
    __shared__ T tile[kTile][kTile + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (uint32_t t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
        uint32_t rest = p.div_t0.div(t);
        const uint32_t t0 = t - rest * p.tiles0;
        uint32_t b = p.div_tj.div(rest);
        const uint32_t tj = rest - b * p.tilesj;
        int64_t ib = p.in_off, ob = p.out_off;
        for (int i = 0; i < p.nb; ++i) {
            uint32_t q = p.bdiv[i].div(b);
            int64_t idx = b - q * p.bshape[i];
            b = q;
            ib += idx * p.in_bs[i];
            ob += idx * p.out_bs[i];
        }
        const int64_t i0b = (int64_t)t0 * kTile, ijb = (int64_t)tj * kTile;
        T vals[kTile / kTileRows];
#pragma unroll
        for (int r = 0; r < kTile / kTileRows; ++r) {
            const int64_t i0 = i0b + ty + r * kTileRows, ij = ijb + tx;
            if (i0 < p.n0 && ij < p.nj) vals[r] = in[ib + i0 * p.in_s0 + ij * p.in_sj];
        }
#pragma unroll
        for (int r = 0; r < kTile / kTileRows; ++r) tile[ty + r * kTileRows][tx] = vals[r];
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kTile / kTileRows; ++r) {
            const int64_t ij = ijb + ty + r * kTileRows, i0 = i0b + tx;
            if (i0 < p.n0 && ij < p.nj) out[ob + i0 + ij * p.out_sj] = tile[tx][ty + r * kTileRows];
        }
        __syncthreads();
    }
}

// 4-byte elements: 64 x 64 tiles moved as 8-byte pairs (neighbours along j
// when read, along dim 0 when written), sixteen elements a thread. Needs both
// extents even and every offset and stride (but the unit ones) even, so that
// each pair is 8-byte aligned and lies inside the tensor. The 32 x 32 tile of
// transpose_kernel left each thread four 4-byte loads in flight (0.57 of HBM
// for the F-ordered f32 to_contig of [32,64,128,128]).
constexpr int kTile2 = 64;

__global__ void __launch_bounds__(32 * kTileRows)
    transpose2_kernel(uint32_t* __restrict__ out, const uint32_t* __restrict__ in, const TrParams p) {
    __shared__ uint32_t tile[kTile2][kTile2 + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (uint32_t t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
        uint32_t rest = p.div_t0.div(t);
        const uint32_t t0 = t - rest * p.tiles0;
        uint32_t b = p.div_tj.div(rest);
        const uint32_t tj = rest - b * p.tilesj;
        int64_t ib = p.in_off, ob = p.out_off;
        for (int i = 0; i < p.nb; ++i) {
            uint32_t q = p.bdiv[i].div(b);
            int64_t idx = b - q * p.bshape[i];
            b = q;
            ib += idx * p.in_bs[i];
            ob += idx * p.out_bs[i];
        }
        const int64_t i0b = (int64_t)t0 * kTile2, ijb = (int64_t)tj * kTile2;
        uint2 v[kTile2 / kTileRows];
#pragma unroll
        for (int r = 0; r < kTile2 / kTileRows; ++r) {
            const int64_t i0 = i0b + ty + r * kTileRows, ij = ijb + 2 * tx;
            if (i0 < p.n0 && ij < p.nj) v[r] = *reinterpret_cast<const uint2*>(in + ib + i0 * p.in_s0 + ij);
        }
#pragma unroll
        for (int r = 0; r < kTile2 / kTileRows; ++r) {
            tile[ty + r * kTileRows][2 * tx] = v[r].x;
            tile[ty + r * kTileRows][2 * tx + 1] = v[r].y;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kTile2 / kTileRows; ++r) {
            const int64_t ij = ijb + ty + r * kTileRows, i0 = i0b + 2 * tx;
            if (i0 < p.n0 && ij < p.nj) {
                uint2 w;
                w.x = tile[2 * tx][ty + r * kTileRows];
                w.y = tile[2 * tx + 1][ty + r * kTileRows];
                const int64_t oj = p.jlog ? (ij & ((1 << p.jlog) - 1)) * p.out_sj + (ij >> p.jlog) * p.out_sjo
                                          : ij * p.out_sj;
                *reinterpret_cast<uint2*>(out + ob + i0 + oj) = w;
            }
        }
        __syncthreads();
    }
}

// Use the tile transpose when the destination is contiguous along dim 0, the
// source strides along dim 0 by more than a few elements, and the source is
// (nearly) contiguous along another dim j with both extents large enough to
// fill a tile. Returns j, or -1.
static int transpose_dim(const IterSpace& sp) {
    if (sp.ndim < 2 || sp.stride[0][0] != 1) return -1;
    const int64_t s0 = std::llabs(sp.stride[1][0]);
    if (s0 <= 4) return -1;
    int best = -1;
    int64_t bs = s0;
    for (int d = 1; d < sp.ndim; ++d) {
        int64_t s = std::llabs(sp.stride[1][d]);
        if (s != 0 && s < bs) {
            bs = s;
            best = d;
        }
    }
    if (best < 0 || bs > 2) return -1;
    if (sp.shape[0] < 16 || sp.shape[best] < 16) return -1;
    return best;
}

template <typename T>
static int launch_transpose(rstsr_ctx* ctx, const IterSpace& sp, int j, void* out, const void* in) {
    TrParams p;
    memset(&p, 0, sizeof(p));
    p.n0 = sp.shape[0];
    p.nj = sp.shape[j];
    p.in_s0 = sp.stride[1][0];
    p.in_sj = sp.stride[1][j];
    p.out_sj = sp.stride[0][j];
    p.in_off = sp.offset[1];
    p.out_off = sp.offset[0];
    int nb = 0;
    int64_t nbatch = 1;
    for (int d = 1; d < sp.ndim; ++d) {
        if (d == j) continue;
        p.bshape[nb] = (uint32_t)sp.shape[d];
        p.bdiv[nb] = FastDiv((uint32_t)sp.shape[d]);
        p.in_bs[nb] = sp.stride[1][d];
        p.out_bs[nb] = sp.stride[0][d];
        nbatch *= sp.shape[d];
        nb++;
    }
    p.nb = nb;
    // 4-byte elements in 8-byte pairs (transpose2_kernel) where every pair is aligned
    bool pairs = sizeof(T) == 4 && p.in_sj == 1 && (p.n0 % 2) == 0 && (p.nj % 2) == 0 && (p.in_s0 % 2) == 0 &&
                 (p.out_sj % 2) == 0 && (p.in_off % 2) == 0 && (p.out_off % 2) == 0 &&
                 (reinterpret_cast<uintptr_t>(in) % 8) == 0 && (reinterpret_cast<uintptr_t>(out) % 8) == 0;
    for (int i = 0; pairs && i < nb; ++i) pairs = (p.in_bs[i] % 2) == 0 && (p.out_bs[i] % 2) == 0;
    // a contiguous source run shorter than the 64-wide tile (a power of two):
    // fold the batch dim that continues it in the source into the tile's
    // columns, so that the tile stays full (an F-ordered [32, ...] source
    // otherwise left half of every tile empty)
    if (pairs && p.nj < kTile2 && (p.nj & (p.nj - 1)) == 0) {
        for (int i = 0; i < nb; ++i) {
            if (p.in_bs[i] != p.nj || p.bshape[i] < 2) continue;
            int lg = 0;
            while ((int64_t(1) << lg) < p.nj) ++lg;
            p.jlog = lg;
            p.out_sjo = p.out_bs[i];
            p.nj *= p.bshape[i];
            nbatch /= p.bshape[i];
            for (int k = i; k + 1 < nb; ++k) {
                p.bshape[k] = p.bshape[k + 1];
                p.bdiv[k] = p.bdiv[k + 1];
                p.in_bs[k] = p.in_bs[k + 1];
                p.out_bs[k] = p.out_bs[k + 1];
            }
            --nb;
            p.nb = nb;
            break;
        }
    }
    const int tile = pairs ? kTile2 : kTile;
    p.tiles0 = (uint32_t)((p.n0 + tile - 1) / tile);
    p.tilesj = (uint32_t)((p.nj + tile - 1) / tile);
    p.div_t0 = FastDiv(p.tiles0);
    p.div_tj = FastDiv(p.tilesj);
    const int64_t ntiles = (int64_t)p.tiles0 * p.tilesj * nbatch;
    if (ntiles >= (int64_t(1) << 31)) return -1;  // caller falls back to the generic kernel
    p.ntiles = (uint32_t)ntiles;
    const int64_t maxgrid = (int64_t)ctx->num_sms * 16;
    const unsigned grid = (unsigned)std::min<int64_t>(ntiles, maxgrid);
    if (pairs) {
        transpose2_kernel<<<grid, dim3(32, kTileRows), 0, ctx->stream>>>((uint32_t*)out, (const uint32_t*)in, p);
        return after_launch(ctx, "transpose2_kernel");
    }
    transpose_kernel<T><<<grid, dim3(kTile, kTileRows), 0, ctx->stream>>>((T*)out, (const T*)in, p);
    return after_launch(ctx, "transpose_kernel");
}

// ------------------------------------------------------- arbitrary assign

struct ArbParams {
    DevDims dc, da;
    int64_t sc[RSTSR_MAX_NDIM], sa[RSTSR_MAX_NDIM];
    int64_t oc, oa;
    int64_t n;
};

// c and a walked in the same logical order over their own (different) shapes:
// element e of the walk is decomposed once per operand.
template <typename T>
__global__ void __launch_bounds__(kThreads) arb_kernel(T* __restrict__ c, const T* __restrict__ a,
                                                       const ArbParams p) {
    for (int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x; e < p.n; e += (int64_t)gridDim.x * kThreads) {
        int64_t offc = p.oc, offa = p.oa;
        uint32_t rem = (uint32_t)e;
        for (int i = 0; i < p.dc.ndim - 1; ++i) {
            uint32_t q = p.dc.div[i].div(rem);
            offc += (int64_t)(rem - q * p.dc.shape[i]) * p.sc[i];
            rem = q;
        }
        offc += (int64_t)rem * p.sc[p.dc.ndim - 1];
        rem = (uint32_t)e;
        for (int i = 0; i < p.da.ndim - 1; ++i) {
            uint32_t q = p.da.div[i].div(rem);
            offa += (int64_t)(rem - q * p.da.shape[i]) * p.sa[i];
            rem = q;
        }
        offa += (int64_t)rem * p.sa[p.da.ndim - 1];
        c[offc] = a[offa];
    }
}

// Collapse a layout for a walk in logical C order (reversed axes) or F order:
// inner-first dims, extent-1 axes dropped, contiguous neighbours merged.
static IterSpace walk_space(const Layout& l, rstsr_order order) {
    Layout w = order == RSTSR_ROW_MAJOR ? l.reverse_axes() : l;
    IterSpace sp;
    sp.nops = 1;
    sp.size = w.size();
    sp.offset[0] = w.offset;
    int nd = 0;
    for (int i = 0; i < w.ndim; ++i) {
        if (w.shape[i] == 1) continue;
        if (nd > 0 && w.stride[i] == sp.stride[0][nd - 1] * sp.shape[nd - 1]) {
            sp.shape[nd - 1] *= w.shape[i];
        } else {
            sp.shape[nd] = w.shape[i];
            sp.stride[0][nd] = w.stride[i];
            nd++;
        }
    }
    if (nd == 0) {
        sp.shape[0] = 1;
        sp.stride[0][0] = 0;
        nd = 1;
    }
    sp.ndim = nd;
    return sp;
}

// ------------------------------------------------------------ casting copy

// Runtime-typed conversion c = a as TC. The source value is widened to a
// double (float types, exact), int64 or uint64 (integer types) and then
// narrowed to the destination with one rounding, saturating float->int
// conversions and NaN -> 0, bool as 0/1, x != 0 -> true.
struct CastParams {
    DevDims dims;
    int64_t n;
    int64_t sc[RSTSR_MAX_NDIM], sa[RSTSR_MAX_NDIM];
    int64_t oc, oa;
    int32_t tc, ta, big;
};

__device__ __forceinline__ void cast_one(void* c, int64_t ic, int tc, const void* a, int64_t ia, int ta) {
    double fv = 0;
    int64_t iv = 0;
    uint64_t uv = 0;
    int kind;  // 0 float, 1 signed, 2 unsigned
    switch (ta) {
        case RSTSR_F64: fv = ((const double*)a)[ia]; kind = 0; break;
        case RSTSR_F32: fv = ((const float*)a)[ia]; kind = 0; break;
        case RSTSR_F16: fv = __half2float(((const __half*)a)[ia]); kind = 0; break;
        case RSTSR_BF16: fv = __bfloat162float(((const __nv_bfloat16*)a)[ia]); kind = 0; break;
        case RSTSR_I8: iv = ((const int8_t*)a)[ia]; kind = 1; break;
        case RSTSR_I16: iv = ((const int16_t*)a)[ia]; kind = 1; break;
        case RSTSR_I32: iv = ((const int32_t*)a)[ia]; kind = 1; break;
        case RSTSR_I64: iv = ((const int64_t*)a)[ia]; kind = 1; break;
        case RSTSR_U8: uv = ((const uint8_t*)a)[ia]; kind = 2; break;
        case RSTSR_U16: uv = ((const uint16_t*)a)[ia]; kind = 2; break;
        case RSTSR_U32: uv = ((const uint32_t*)a)[ia]; kind = 2; break;
        case RSTSR_U64: uv = ((const uint64_t*)a)[ia]; kind = 2; break;
        default: uv = ((const uint8_t*)a)[ia] != 0; kind = 2; break;  // bool
    }
    // integer view of the value for integer destinations (wrapping)
    const uint64_t bits = kind == 1 ? (uint64_t)iv : uv;
    switch (tc) {
        case RSTSR_F64:
            ((double*)c)[ic] = kind == 0 ? fv : kind == 1 ? __ll2double_rn(iv) : __ull2double_rn(uv);
            break;
        case RSTSR_F32:
            ((float*)c)[ic] = kind == 0 ? __double2float_rn(fv) : kind == 1 ? __ll2float_rn(iv) : __ull2float_rn(uv);
            break;
        case RSTSR_F16:
            ((__half*)c)[ic] = kind == 0 ? __double2half(fv)
                                         : __float2half_rn(kind == 1 ? __ll2float_rn(iv) : __ull2float_rn(uv));
            break;
        case RSTSR_BF16:
            ((__nv_bfloat16*)c)[ic] = kind == 0 ? __double2bfloat16(fv)
                                                : __float2bfloat16_rn(kind == 1 ? __ll2float_rn(iv) : __ull2float_rn(uv));
            break;
        case RSTSR_I8:
            ((int8_t*)c)[ic] = kind == 0 ? float_to_int_sat<int8_t>(fv, -128.0, 127.0, INT8_MIN, INT8_MAX) : (int8_t)bits;
            break;
        case RSTSR_I16:
            ((int16_t*)c)[ic] =
                kind == 0 ? float_to_int_sat<int16_t>(fv, -32768.0, 32767.0, INT16_MIN, INT16_MAX) : (int16_t)bits;
            break;
        case RSTSR_I32:
            ((int32_t*)c)[ic] = kind == 0 ? float_to_int_sat<int32_t>(fv, -2147483648.0, 2147483647.0, INT32_MIN, INT32_MAX)
                                          : (int32_t)bits;
            break;
        case RSTSR_I64:
            ((int64_t*)c)[ic] = kind == 0 ? float_to_int_sat<int64_t>(fv, -9223372036854775808.0, 9223372036854775807.0,
                                                                      INT64_MIN, INT64_MAX)
                                          : (int64_t)bits;
            break;
        case RSTSR_U8:
            ((uint8_t*)c)[ic] = kind == 0 ? float_to_int_sat<uint8_t>(fv, 0.0, 255.0, 0, UINT8_MAX) : (uint8_t)bits;
            break;
        case RSTSR_U16:
            ((uint16_t*)c)[ic] = kind == 0 ? float_to_int_sat<uint16_t>(fv, 0.0, 65535.0, 0, UINT16_MAX) : (uint16_t)bits;
            break;
        case RSTSR_U32:
            ((uint32_t*)c)[ic] =
                kind == 0 ? float_to_int_sat<uint32_t>(fv, 0.0, 4294967295.0, 0, UINT32_MAX) : (uint32_t)bits;
            break;
        case RSTSR_U64:
            ((uint64_t*)c)[ic] =
                kind == 0 ? float_to_int_sat<uint64_t>(fv, 0.0, 18446744073709551615.0, 0, UINT64_MAX) : bits;
            break;
        default:  // bool
            ((uint8_t*)c)[ic] = kind == 0 ? (fv != 0.0) : (bits != 0);
            break;
    }
}

__global__ void __launch_bounds__(kThreads) cast_kernel(void* __restrict__ c, const void* __restrict__ a,
                                                        const CastParams p) {
    for (int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x; e < p.n; e += (int64_t)gridDim.x * kThreads) {
        int64_t offc = p.oc, offa = p.oa;
        if (p.big) {
            uint64_t rem = (uint64_t)e;
            for (int i = 0; i < p.dims.ndim - 1; ++i) {
                uint64_t q = rem / p.dims.shape[i];
                int64_t idx = (int64_t)(rem - q * p.dims.shape[i]);
                offc += idx * p.sc[i];
                offa += idx * p.sa[i];
                rem = q;
            }
            offc += (int64_t)rem * p.sc[p.dims.ndim - 1];
            offa += (int64_t)rem * p.sa[p.dims.ndim - 1];
        } else {
            uint32_t rem = (uint32_t)e;
            for (int i = 0; i < p.dims.ndim - 1; ++i) {
                uint32_t q = p.dims.div[i].div(rem);
                int64_t idx = (int64_t)(rem - q * p.dims.shape[i]);
                offc += idx * p.sc[i];
                offa += idx * p.sa[i];
                rem = q;
            }
            offc += (int64_t)rem * p.sc[p.dims.ndim - 1];
            offa += (int64_t)rem * p.sa[p.dims.ndim - 1];
        }
        cast_one(c, offc, p.tc, a, offa, p.ta);
    }
}

// ------------------------------------------------------------- dispatch

template <typename T>
static int copy_typed(rstsr_ctx* ctx, const IterSpace& sp, void* c, const void* a) {
    int j = transpose_dim(sp);
    if (j > 0 && sp.size < (int64_t(1) << 31)) {
        int s = launch_transpose<T>(ctx, sp, j, c, a);
        if (s >= 0) return s;
    }
    EwInput ins[1] = {{a, nullptr}};
    return launch_ew<T, T, 1>(ctx, sp, c, ins, CopyF<T>{}, "assign");
}

static int copy_dispatch(rstsr_ctx* ctx, rstsr_dtype tc, rstsr_dtype ta, const IterSpace& sp, void* c,
                         const void* a) {
    if (tc == ta) {
        switch (dtype_size(tc)) {
            case 8: return copy_typed<uint64_t>(ctx, sp, c, a);
            case 4: return copy_typed<uint32_t>(ctx, sp, c, a);
            case 2: return copy_typed<uint16_t>(ctx, sp, c, a);
            default: return copy_typed<uint8_t>(ctx, sp, c, a);
        }
    }
    if (sp.size == 0) return RSTSR_OK;
    if (!inner_extents_fit_u32(sp))
        return fail(RSTSR_ERR_UNIMPLEMENTED, "casting copy: an inner extent of 2^32 or more elements");
    CastParams p;
    memset(&p, 0, sizeof(p));
    p.dims = make_dev_dims(sp);
    p.n = sp.size;
    for (int i = 0; i < RSTSR_MAX_NDIM; ++i) {
        p.sc[i] = i < sp.ndim ? sp.stride[0][i] : 0;
        p.sa[i] = i < sp.ndim ? sp.stride[1][i] : 0;
    }
    p.oc = sp.offset[0];
    p.oa = sp.offset[1];
    p.tc = tc;
    p.ta = ta;
    p.big = sp.size >= (int64_t(1) << 31);
    const unsigned grid =
        (unsigned)std::min<int64_t>((p.n + kThreads - 1) / kThreads, (int64_t)ctx->num_sms * 32);
    cast_kernel<<<grid, kThreads, 0, ctx->stream>>>(c, a, p);
    return after_launch(ctx, "cast_kernel");
}

template <typename T>
static int fill_typed(rstsr_ctx* ctx, const IterSpace& sp, void* c, const void* value) {
    T v;
    memcpy(&v, value, sizeof(T));
    EwInput ins[1] = {{nullptr, nullptr}};
    return launch_ew<T, T, 0>(ctx, sp, c, ins, ConstF<T>{v}, "fill");
}

}  // namespace rstsr

using namespace rstsr;

extern "C" {

int rstsr_cuda_assign(rstsr_ctx* ctx, void* c, const rstsr_layout* lc, rstsr_dtype tc, const void* a,
                      const rstsr_layout* la, rstsr_dtype ta) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(lc, "c"));
    RSTSR_TRY(check_layout(la, "a"));
    if (!dtype_valid(tc) || !dtype_valid(ta)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    Layout Lc = Layout::from_abi(*lc), La = Layout::from_abi(*la);
    RSTSR_TRY(check_same_shape3(Lc, La, nullptr, "assign"));
    RSTSR_TRY(check_write_layout(Lc, "assign"));
    if (Lc.size() == 0) return RSTSR_OK;
    if (!c || !a) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    const Layout* ls[2] = {&Lc, &La};
    IterSpace sp = make_iter_space(ls, 2);
    return copy_dispatch(ctx, tc, ta, sp, c, a);
}

int rstsr_cuda_assign_arbitrary(rstsr_ctx* ctx, void* c, const rstsr_layout* lc, rstsr_dtype tc, const void* a,
                                const rstsr_layout* la, rstsr_dtype ta, rstsr_order order) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(lc, "c"));
    RSTSR_TRY(check_layout(la, "a"));
    if (!dtype_valid(tc) || !dtype_valid(ta)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    if (order != RSTSR_ROW_MAJOR && order != RSTSR_COL_MAJOR) return fail(RSTSR_ERR_INVALID_VALUE, "bad order");
    Layout Lc = Layout::from_abi(*lc), La = Layout::from_abi(*la);
    if (Lc.size() != La.size())
        return fail(RSTSR_ERR_INVALID_LAYOUT,
                    "assign_arbitrary: sizes differ (" + Lc.repr() + " vs " + La.repr() + ")");
    RSTSR_TRY(check_write_layout(Lc, "assign_arbitrary"));
    if (Lc.size() == 0) return RSTSR_OK;
    if (!c || !a) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    if (same_shape(Lc, La)) {
        // equal shapes: the i-th elements of both walks share one multi-index,
        // so any iteration order gives the same result
        const Layout* ls[2] = {&Lc, &La};
        IterSpace sp = make_iter_space(ls, 2);
        return copy_dispatch(ctx, tc, ta, sp, c, a);
    }
    if (tc != ta) {
        // casting reshape: cast into a contiguous temporary of the source
        // shape, then walk-copy without casting
        void* tmp = nullptr;
        const int64_t n = La.size();
        RSTSR_TRY(scratch_alloc(ctx, (size_t)n * dtype_size(tc), &tmp));
        Layout Lt = order == RSTSR_COL_MAJOR ? Layout::f_contig(La.shape, La.ndim) : Layout::c_contig(La.shape, La.ndim);
        rstsr_layout lt = Lt.to_abi();
        int s = rstsr_cuda_assign(ctx, tmp, &lt, tc, a, la, ta);
        if (s == RSTSR_OK) s = rstsr_cuda_assign_arbitrary(ctx, c, lc, tc, tmp, &lt, tc, order);
        scratch_free(ctx, tmp);
        return s;
    }
    IterSpace sc = walk_space(Lc, order), sa = walk_space(La, order);
    if (sc.ndim == 1 && sa.ndim == 1) {
        // both walks are single strided runs: a 1-D same-shape copy
        IterSpace sp;
        sp.nops = 2;
        sp.ndim = 1;
        sp.size = sc.size;
        sp.shape[0] = sc.shape[0];
        sp.stride[0][0] = sc.stride[0][0];
        sp.stride[1][0] = sa.stride[0][0];
        sp.offset[0] = sc.offset[0];
        sp.offset[1] = sa.offset[0];
        return copy_dispatch(ctx, tc, ta, sp, c, a);
    }
    if (Lc.size() >= (int64_t(1) << 31))
        return fail(RSTSR_ERR_UNIMPLEMENTED, "assign_arbitrary between different shapes above 2^31 elements");
    ArbParams p;
    memset(&p, 0, sizeof(p));
    p.dc = make_dev_dims(sc);
    p.da = make_dev_dims(sa);
    for (int i = 0; i < RSTSR_MAX_NDIM; ++i) {
        p.sc[i] = i < sc.ndim ? sc.stride[0][i] : 0;
        p.sa[i] = i < sa.ndim ? sa.stride[0][i] : 0;
    }
    p.oc = sc.offset[0];
    p.oa = sa.offset[0];
    p.n = Lc.size();
    const unsigned grid =
        (unsigned)std::min<int64_t>((p.n + kThreads - 1) / kThreads, (int64_t)ctx->num_sms * 32);
    switch (dtype_size(tc)) {
        case 8: arb_kernel<uint64_t><<<grid, kThreads, 0, ctx->stream>>>((uint64_t*)c, (const uint64_t*)a, p); break;
        case 4: arb_kernel<uint32_t><<<grid, kThreads, 0, ctx->stream>>>((uint32_t*)c, (const uint32_t*)a, p); break;
        case 2: arb_kernel<uint16_t><<<grid, kThreads, 0, ctx->stream>>>((uint16_t*)c, (const uint16_t*)a, p); break;
        default: arb_kernel<uint8_t><<<grid, kThreads, 0, ctx->stream>>>((uint8_t*)c, (const uint8_t*)a, p); break;
    }
    return after_launch(ctx, "assign_arbitrary");
}

int rstsr_cuda_fill(rstsr_ctx* ctx, void* c, const rstsr_layout* lc, rstsr_dtype tc, const void* value) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(lc, "c"));
    if (!dtype_valid(tc)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    if (!value) return fail(RSTSR_ERR_INVALID_VALUE, "null fill value");
    Layout Lc = Layout::from_abi(*lc);
    if (Lc.size() == 0) return RSTSR_OK;
    if (!c) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    // G order (rstsr-native-impl/src/cpu_serial/assignment.rs:137): axes the
    // destination broadcasts over are written once
    int perm[RSTSR_MAX_NDIM];
    Layout g = greedy_layout(Lc, false, perm);
    const Layout* ls[1] = {&g};
    IterSpace sp = make_iter_space(ls, 1);
    switch (dtype_size(tc)) {
        case 8: return fill_typed<uint64_t>(ctx, sp, c, value);
        case 4: return fill_typed<uint32_t>(ctx, sp, c, value);
        case 2: return fill_typed<uint16_t>(ctx, sp, c, value);
        default: return fill_typed<uint8_t>(ctx, sp, c, value);
    }
}

}  // extern "C"
