// pack_tri / unpack_tri: packed triangular storage of the trailing matrix
// axes, replacing rstsr-native-impl/src/cpu_serial/op_tri.rs
// (pack_tri_cpu_serial :73-144, the inner_unpack_tri{l,u}_* loops :148-410)
// and their rayon forms in cpu_rayon/op_tri.rs, behind OpPackTriAPI /
// OpUnpackTriAPI (rstsr-core/src/operators/ops/op_tri.rs:3-30).
//
// Packed order (row-major view, the reference's loops): lower packs row i's
// columns 0..=i, so element (i, j), j <= i, sits at i(i+1)/2 + j; upper packs
// row i's columns i..n, so (i, j), j >= i, sits at i(2n-i-1)/2 + j. ColMajor
// devices reverse every axis and flip uplo first (feature_rayon/auto_impl/
// op_tri.rs:20-26, :49-55); the host code below does the same.
//
// One kernel shape for both directions: a CTA owns one 32x32 tile of one
// matrix's triangle (the grid strides over tile pairs x batch), stages it in a
// padded shared tile and moves it so that global loads and stores both run
// along the smaller-stride axis of the side they touch. For unpack with a
// symmetry, the same staged tile is also written transposed into the mirror
// tile, so every packed element is read once. Elements move as raw bits; the
// anti-symmetric forms negate by flipping the sign bit (IEEE negation, as
// Rust's `-x` on floats), writing +0 on the diagonal.
#include "ew_kernel.cuh"

namespace rstsr {

namespace {

constexpr int kTriTile = 32;
constexpr int kTriRows = 8;  // threads along y; each covers kTriTile / kTriRows rows

struct TriParams {
    int64_t n;               // matrix order
    int64_t s_i, s_j;        // matrix strides along rows and columns (elements)
    int64_t s_p;             // packed-axis stride
    int64_t off_m, off_p;    // offsets of the first matrix / packed vector
    int lower;               // 1: (i, j) with j <= i; 0: j >= i
    int negate;              // mirror = -value (anti-symmetric), diagonal = 0
    int mirror;              // write the other triangle (symm != N)
    int cols_fast;           // 1: |s_j| <= |s_i|, matrix accesses run along j
    uint32_t tiles;          // tiles along one matrix axis
    uint32_t pairs;          // tile pairs of one triangle: tiles (tiles + 1) / 2
    FastDiv div_pairs;
    uint32_t total;          // pairs * batches
    uint32_t rows_total;     // n * batches (row kernel)
    FastDiv div_n;
    int nb;                  // collapsed batch dims (inner first)
    uint32_t bshape[RSTSR_MAX_NDIM];
    FastDiv bdiv[RSTSR_MAX_NDIM];
    int64_t m_bs[RSTSR_MAX_NDIM], p_bs[RSTSR_MAX_NDIM];
};

// Sign-bit mask of an element stored as an unsigned word of its width.
template <typename W>
__device__ __forceinline__ W sign_bit() {
    return W(W(1) << (sizeof(W) * 8 - 1));
}

// Tile pair t -> (P, Q), P >= Q, in the order (0,0), (1,0), (1,1), (2,0), ...
// The FP32 root is within one of P for t < 2^31 (GB300's FP64 pipe is far too
// slow to spend per tile); the integer steps make it exact.
__device__ __forceinline__ void tri_pair(uint32_t t, uint32_t* P, uint32_t* Q) {
    uint32_t p = (uint32_t)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
    while ((uint64_t)p * (p + 1) / 2 > t) --p;
    while ((uint64_t)(p + 1) * (p + 2) / 2 <= t) ++p;
    *P = p;
    *Q = (uint32_t)(t - (uint64_t)p * (p + 1) / 2);
}

// First packed index of row i (the element at column j is row_base + j).
__device__ __forceinline__ int64_t tri_row_base(int64_t i, int64_t n, int lower) {
    return lower ? i * (i + 1) / 2 : i * (2 * n - i - 1) / 2;
}

struct TriTile {
    int32_t R, C;      // tile row / column (in tiles)
    bool diag;
    int64_t mb, pb;    // matrix / packed base offsets of this batch element
};

__device__ __forceinline__ TriTile tri_tile(const TriParams& p, uint32_t t) {
    const uint32_t batch = p.div_pairs.div(t);
    uint32_t P, Q;
    tri_pair(t - batch * p.pairs, &P, &Q);
    TriTile tt;
    tt.R = (int32_t)(p.lower ? P : Q);
    tt.C = (int32_t)(p.lower ? Q : P);
    tt.diag = P == Q;
    tt.mb = p.off_m;
    tt.pb = p.off_p;
    uint32_t b = batch;
    for (int d = 0; d < p.nb; ++d) {
        const uint32_t q = p.bdiv[d].div(b);
        const int64_t idx = b - q * p.bshape[d];
        b = q;
        tt.mb += idx * p.m_bs[d];
        tt.pb += idx * p.p_bs[d];
    }
    return tt;
}

__device__ __forceinline__ bool in_tri(int64_t i, int64_t j, int64_t n, int lower) {
    return i < n && j < n && (lower ? j <= i : j >= i);
}

constexpr int kTriPer = kTriTile / kTriRows;  // rows of a tile per thread

// A tile lies wholly inside the triangle and the matrix: no per-element test.
__device__ __forceinline__ bool tri_full(const TriParams& p, const TriTile& tt) {
    return !tt.diag && (int64_t)(tt.R + 1) * kTriTile <= p.n && (int64_t)(tt.C + 1) * kTriTile <= p.n;
}

// Matrix (.., n, n) -> packed (.., n(n+1)/2), matrix contiguous along j and
// n >= 64: one warp per matrix row copies the row's part of the triangle,
// both sides contiguous, four loads in flight per lane, no exchange.
template <typename W>
__global__ void __launch_bounds__(256)
    pack_tri_rows_kernel(W* __restrict__ packed, const W* __restrict__ mat, const TriParams p) {
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < p.rows_total; w += nw) {
        uint32_t b = p.div_n.div(w);
        const int64_t i = (int64_t)(w - b * (uint32_t)p.n);
        int64_t mb = p.off_m, pb = p.off_p;
        for (int d = 0; d < p.nb; ++d) {
            const uint32_t q = p.bdiv[d].div(b);
            const int64_t idx = b - q * p.bshape[d];
            b = q;
            mb += idx * p.m_bs[d];
            pb += idx * p.p_bs[d];
        }
        const int64_t j0 = p.lower ? 0 : i, j1 = p.lower ? i + 1 : p.n;
        const W* src = mat + mb + i * p.s_i;
        W* dst = packed + pb + tri_row_base(i, p.n, p.lower) * p.s_p;
        for (int64_t j = j0 + lane; j < j1; j += 4 * 32) {
            W v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (j + 32 * u < j1) v[u] = src[(j + 32 * u) * p.s_j];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (j + 32 * u < j1) dst[(j + 32 * u) * p.s_p] = v[u];
        }
    }
}

// Matrix -> packed through a shared tile (the matrix is contiguous along i,
// or n < 64): the shape of the element-wise transpose kernel (32 x 32 tiles,
// four elements per thread, small register footprint so that eight CTAs share
// an SM and their loads overlap).
template <typename W>
__global__ void __launch_bounds__(kTriTile* kTriRows, 8)
    pack_tri_kernel(W* __restrict__ packed, const W* __restrict__ mat, const TriParams p) {
    __shared__ W tile[kTriTile][kTriTile + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (uint32_t t = blockIdx.x; t < p.total; t += gridDim.x) {
        const TriTile tt = tri_tile(p, t);
        const int64_t i0 = (int64_t)tt.R * kTriTile, j0 = (int64_t)tt.C * kTriTile;
        const bool full = tri_full(p, tt);
#pragma unroll
        for (int k = 0; k < kTriPer; ++k) {
            const int a = ty + k * kTriRows;
            const int r = p.cols_fast ? a : tx, c = p.cols_fast ? tx : a;
            const int64_t i = i0 + r, j = j0 + c;
            if (full || in_tri(i, j, p.n, p.lower)) tile[r][c] = mat[tt.mb + i * p.s_i + j * p.s_j];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kTriPer; ++k) {
            const int r = ty + k * kTriRows, c = tx;
            const int64_t i = i0 + r, j = j0 + c;
            if (full || in_tri(i, j, p.n, p.lower))
                packed[tt.pb + (tri_row_base(i, p.n, p.lower) + j) * p.s_p] = tile[r][c];
        }
        __syncthreads();
    }
}

// Packed (.., n(n+1)/2) -> matrix (.., n, n), mirrored by the symmetry, in the
// same transpose-kernel shape: the packed tile is read once into shared
// memory, then written to its own position and, transposed, to the mirror.
template <typename W>
__global__ void __launch_bounds__(kTriTile* kTriRows, 8)
    unpack_tri_kernel(W* __restrict__ mat, const W* __restrict__ packed, const TriParams p) {
    __shared__ W tile[kTriTile][kTriTile + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const W flip = p.negate ? sign_bit<W>() : W(0);
    for (uint32_t t = blockIdx.x; t < p.total; t += gridDim.x) {
        const TriTile tt = tri_tile(p, t);
        const int64_t i0 = (int64_t)tt.R * kTriTile, j0 = (int64_t)tt.C * kTriTile;
        const bool full = tri_full(p, tt);
#pragma unroll
        for (int k = 0; k < kTriPer; ++k) {
            const int r = ty + k * kTriRows;
            const int64_t i = i0 + r, j = j0 + tx;
            if (full || in_tri(i, j, p.n, p.lower))
                tile[r][tx] = packed[tt.pb + (tri_row_base(i, p.n, p.lower) + j) * p.s_p];
        }
        __syncthreads();
        W* const mbase = mat + tt.mb;
        if (full) {
            // element (i, j) = tile[i - i0][j - j0]; tx runs along the written fast axis
            {
                W* dst = p.cols_fast ? mbase + (i0 + ty) * p.s_i + (j0 + tx) * p.s_j
                                     : mbase + (i0 + tx) * p.s_i + (j0 + ty) * p.s_j;
                const int64_t step = (int64_t)kTriRows * (p.cols_fast ? p.s_i : p.s_j);
#pragma unroll
                for (int k = 0; k < kTriPer; ++k) {
                    const int a = ty + k * kTriRows;
                    *dst = p.cols_fast ? tile[a][tx] : tile[tx][a];
                    dst += step;
                }
            }
            if (p.mirror) {
                // element (j, i), at j * s_i + i * s_j, = op(tile[i - i0][j - j0])
                W* dst = p.cols_fast ? mbase + (j0 + ty) * p.s_i + (i0 + tx) * p.s_j
                                     : mbase + (j0 + tx) * p.s_i + (i0 + ty) * p.s_j;
                const int64_t step = (int64_t)kTriRows * (p.cols_fast ? p.s_i : p.s_j);
#pragma unroll
                for (int k = 0; k < kTriPer; ++k) {
                    const int a = ty + k * kTriRows;
                    *dst = (p.cols_fast ? tile[tx][a] : tile[a][tx]) ^ flip;
                    dst += step;
                }
            }
        } else {
            // edge or diagonal tile: per-element tests
#pragma unroll
            for (int k = 0; k < kTriPer; ++k) {
                const int a = ty + k * kTriRows;
                const int r = p.cols_fast ? a : tx, c = p.cols_fast ? tx : a;
                const int64_t i = i0 + r, j = j0 + c;
                if (i >= p.n || j >= p.n) continue;
                W w;
                if (i == j) {
                    w = p.negate ? W(0) : tile[r][c];
                } else if (in_tri(i, j, p.n, p.lower)) {
                    w = tile[r][c];
                } else if (p.mirror) {  // diagonal tile only: (j, i) is staged at [c][r]
                    w = tile[c][r] ^ flip;
                } else {
                    continue;
                }
                mbase[i * p.s_i + j * p.s_j] = w;
            }
            if (p.mirror && !tt.diag) {
#pragma unroll
                for (int k = 0; k < kTriPer; ++k) {
                    const int a = ty + k * kTriRows;
                    const int r = p.cols_fast ? tx : a, c = p.cols_fast ? a : tx;
                    const int64_t i = i0 + r, j = j0 + c;
                    if (i < p.n && j < p.n) mbase[j * p.s_i + i * p.s_j] = tile[r][c] ^ flip;
                }
            }
        }
        __syncthreads();
    }
}

// Matrix / packed pair after the order normalisation, ready to launch.
struct TriPlan {
    TriParams p;
    bool empty;
};

// lm: (..., n, n) matrix layout, lp: (..., n(n+1)/2) packed layout (row-major
// view). Fills the batch collapse and the tile counts.
int tri_plan(const Layout& lm, const Layout& lp, bool lower, const char* what, TriPlan* out) {
    if (lm.ndim < 2 || lp.ndim != lm.ndim - 1)
        return fail(RSTSR_ERR_INVALID_LAYOUT,
                    std::string(what) + ": the matrix needs two more axes than the batch and the packed side one (" +
                        lm.repr() + ", " + lp.repr() + ")");
    const int nb = lp.ndim - 1;
    const int64_t n = lm.shape[lm.ndim - 1];
    if (lm.shape[lm.ndim - 2] != n)
        return fail(RSTSR_ERR_INVALID_LAYOUT, std::string(what) + ": the two matrix axes differ (" + lm.repr() + ")");
    if (n > (int64_t(1) << 31))
        return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE, std::string(what) + ": matrix order above 2^31");
    if (lp.shape[nb] != n * (n + 1) / 2)
        return fail(RSTSR_ERR_INVALID_LAYOUT,
                    std::string(what) + ": packed axis " + std::to_string(lp.shape[nb]) + " is not n(n+1)/2 for n = " +
                        std::to_string(n));
    for (int d = 0; d < nb; ++d)
        if (lm.shape[d] != lp.shape[d])
            return fail(RSTSR_ERR_INVALID_LAYOUT,
                        std::string(what) + ": batch axes differ (" + lm.repr() + ", " + lp.repr() + ")");
    Layout bm, bp;
    bm.ndim = bp.ndim = nb;
    bm.offset = lm.offset;
    bp.offset = lp.offset;
    for (int d = 0; d < nb; ++d) {
        bm.shape[d] = bp.shape[d] = lm.shape[d];
        bm.stride[d] = lm.stride[d];
        bp.stride[d] = lp.stride[d];
    }
    const Layout* ls[2] = {&bm, &bp};
    IterSpace sp = make_iter_space(ls, 2);
    TriParams& p = out->p;
    p = TriParams{};
    out->empty = sp.size == 0 || n == 0;
    if (out->empty) return RSTSR_OK;
    const uint64_t tiles = (uint64_t)((n + kTriTile - 1) / kTriTile);
    const uint64_t pairs = tiles * (tiles + 1) / 2;
    if (pairs * (uint64_t)sp.size > INT32_MAX)
        return fail(RSTSR_ERR_VALUE_OUT_OF_RANGE,
                    std::string(what) + ": more than 2^31 tiles of 32 x 32 over the batch (split the batch)");
    p.n = n;
    p.s_i = lm.stride[lm.ndim - 2];
    p.s_j = lm.stride[lm.ndim - 1];
    p.s_p = lp.stride[nb];
    p.off_m = sp.offset[0];
    p.off_p = sp.offset[1];
    p.lower = lower ? 1 : 0;
    p.cols_fast = std::llabs(p.s_j) <= std::llabs(p.s_i) ? 1 : 0;
    p.tiles = (uint32_t)tiles;
    p.pairs = (uint32_t)pairs;
    p.div_pairs = FastDiv(p.pairs);
    p.total = (uint32_t)(pairs * (uint64_t)sp.size);
    const uint64_t rows_total = (uint64_t)n * (uint64_t)sp.size;
    p.rows_total = rows_total > INT32_MAX ? 0 : (uint32_t)rows_total;  // 0: row kernel unusable
    p.div_n = FastDiv((uint32_t)n);
    p.nb = sp.ndim;
    for (int d = 0; d < sp.ndim; ++d) {
        p.bshape[d] = (uint32_t)sp.shape[d];
        p.bdiv[d] = FastDiv((uint32_t)sp.shape[d]);
        p.m_bs[d] = sp.stride[0][d];
        p.p_bs[d] = sp.stride[1][d];
    }
    return RSTSR_OK;
}

int tri_grid(rstsr_ctx* ctx, uint32_t total) {
    const uint32_t cap = (uint32_t)ctx->num_sms * 16;
    return (int)(total < cap ? total : cap);
}

template <typename W>
int launch_pack(rstsr_ctx* ctx, const TriParams& p, void* packed, const void* mat) {
    if (p.cols_fast && p.n >= 64 && p.rows_total > 0) {
        const uint32_t warps = p.rows_total, cap = (uint32_t)ctx->num_sms * 64;
        const uint32_t grid = ((warps < cap ? warps : cap) + 7) / 8;
        pack_tri_rows_kernel<W><<<grid, 256, 0, ctx->stream>>>(static_cast<W*>(packed),
                                                               static_cast<const W*>(mat), p);
        return after_launch(ctx, "pack_tri_rows_kernel");
    }
    pack_tri_kernel<W><<<tri_grid(ctx, p.total), dim3(kTriTile, kTriRows), 0, ctx->stream>>>(
        static_cast<W*>(packed), static_cast<const W*>(mat), p);
    return after_launch(ctx, "pack_tri_kernel");
}

template <typename W>
int launch_unpack(rstsr_ctx* ctx, const TriParams& p, void* mat, const void* packed) {
    unpack_tri_kernel<W><<<tri_grid(ctx, p.total), dim3(kTriTile, kTriRows), 0, ctx->stream>>>(
        static_cast<W*>(mat), static_cast<const W*>(packed), p);
    return after_launch(ctx, "unpack_tri_kernel");
}

int parse_uplo(char uplo, bool* lower) {
    if (uplo == 'L' || uplo == 'l') {
        *lower = true;
        return RSTSR_OK;
    }
    if (uplo == 'U' || uplo == 'u') {
        *lower = false;
        return RSTSR_OK;
    }
    return fail(RSTSR_ERR_INVALID_VALUE, std::string("uplo must be 'L' or 'U', got '") + uplo + "'");
}

// Row-major view of both layouts (ColMajor reverses the axes, flips uplo).
void tri_normalise(Layout* lm, Layout* lp, bool* lower, rstsr_order order) {
    if (order == RSTSR_COL_MAJOR) {
        *lm = lm->reverse_axes();
        *lp = lp->reverse_axes();
        *lower = !*lower;
    }
}

}  // namespace

}  // namespace rstsr

using namespace rstsr;

extern "C" {

int rstsr_cuda_pack_tri(rstsr_ctx* ctx, rstsr_dtype t, void* a, const rstsr_layout* la, const void* b,
                        const rstsr_layout* lb, char uplo, rstsr_order order) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(la, "a"));
    RSTSR_TRY(check_layout(lb, "b"));
    if (!dtype_valid(t)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    if (order != RSTSR_ROW_MAJOR && order != RSTSR_COL_MAJOR) return fail(RSTSR_ERR_INVALID_VALUE, "unknown order");
    bool lower;
    RSTSR_TRY(parse_uplo(uplo, &lower));
    Layout Lp = Layout::from_abi(*la), Lm = Layout::from_abi(*lb);
    RSTSR_TRY(check_write_layout(Lp, "pack_tri"));
    tri_normalise(&Lm, &Lp, &lower, order);
    TriPlan plan;
    RSTSR_TRY(tri_plan(Lm, Lp, lower, "pack_tri", &plan));
    if (plan.empty) return RSTSR_OK;
    if (!a || !b) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    switch (dtype_size(t)) {
        case 1: return launch_pack<uint8_t>(ctx, plan.p, a, b);
        case 2: return launch_pack<uint16_t>(ctx, plan.p, a, b);
        case 4: return launch_pack<uint32_t>(ctx, plan.p, a, b);
        case 8: return launch_pack<uint64_t>(ctx, plan.p, a, b);
        default: return fail(RSTSR_ERR_INVALID_VALUE, "unsupported element size");
    }
}

int rstsr_cuda_unpack_tri(rstsr_ctx* ctx, rstsr_dtype t, void* a, const rstsr_layout* la, const void* b,
                          const rstsr_layout* lb, char uplo, rstsr_symm symm, rstsr_order order) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(la, "a"));
    RSTSR_TRY(check_layout(lb, "b"));
    if (!dtype_valid(t)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    if (!is_float_dtype(t))
        return fail(RSTSR_ERR_INVALID_VALUE,
                    std::string("unpack_tri: element type must be a float type, got ") + dtype_name(t));
    if (order != RSTSR_ROW_MAJOR && order != RSTSR_COL_MAJOR) return fail(RSTSR_ERR_INVALID_VALUE, "unknown order");
    if (symm < RSTSR_SYMM_SY || symm > RSTSR_SYMM_N) return fail(RSTSR_ERR_INVALID_VALUE, "unknown symmetry flag");
    bool lower;
    RSTSR_TRY(parse_uplo(uplo, &lower));
    Layout Lm = Layout::from_abi(*la), Lp = Layout::from_abi(*lb);
    RSTSR_TRY(check_write_layout(Lm, "unpack_tri"));
    tri_normalise(&Lm, &Lp, &lower, order);
    TriPlan plan;
    RSTSR_TRY(tri_plan(Lm, Lp, lower, "unpack_tri", &plan));
    if (plan.empty) return RSTSR_OK;
    if (!a || !b) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    // real element types: He == Sy and Ah == Ay (conjugation is the identity)
    plan.p.negate = (symm == RSTSR_SYMM_AY || symm == RSTSR_SYMM_AH) ? 1 : 0;
    plan.p.mirror = symm != RSTSR_SYMM_N ? 1 : 0;
    switch (dtype_size(t)) {
        case 2: return launch_unpack<uint16_t>(ctx, plan.p, a, b);
        case 4: return launch_unpack<uint32_t>(ctx, plan.p, a, b);
        case 8: return launch_unpack<uint64_t>(ctx, plan.p, a, b);
        default: return fail(RSTSR_ERR_INVALID_VALUE, "unsupported element size");
    }
}

}  // extern "C"
