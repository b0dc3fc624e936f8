// BLAS-3 drivers beyond GEMM: SYRK, SYMM and TRSM, the device forms of
// rstsr-blas-traits/src/blas3/{gemm.rs, syhemm.rs, trsm.rs} (driver_syhemm,
// driver_trsm; SYRK as DeviceSYRKAPI, rstsr-core/src/operators/matmul.rs:64-78).
//
// All three work on strided matrix views (order + leading dimension become a
// layout), so every case reduces to a few cases by transposed views:
//  * SYRK: W = alpha op(A) op(A)^T by the symmetric split GEMM, then the uplo
//    triangle of C = W + beta C through the packed-triangle kernels (pack, axpby
//    on the packed vectors, unpack with symmetry N), which never touch the
//    other triangle of C;
//  * SYMM: the full symmetric A is rebuilt from its uplo triangle (pack +
//    unpack with symmetry Sy) into scratch, then one matmul with alpha / beta;
//  * TRSM: side R becomes side L on the transposed views and op(A) = A^T a
//    transposed view of A, so only L X = B (forward) and U X = B (backward)
//    remain; they are solved by recursive halving down to blocks of
//    kTrsmBlock rows: a small kernel solves each diagonal block in the
//    operands' own precision (one thread per right-hand side column, the block
//    of A in shared memory), and between the halves one split-GEMM matmul
//    B' -= A' X (alpha = -1, beta = 1) updates the half still to solve.
#include "ew_kernel.cuh"

namespace rstsr {

namespace {

constexpr int kTrsmBlock = 64;

// X := T^{-1} X for a kTrsmBlock-or-smaller triangular block T (lower: forward
// substitution, upper: backward), X the block's rows of B, in the
// right-looking order: once x_q is final every later row subtracts
// T[i][q] x_q. Four threads share a column, thread k holding rows
// i = 4 j + k (j < 16) in registers (a cyclic split: each does a quarter of
// the updates at every step); the owner of row q scales it by the diagonal's
// reciprocal and a shuffle hands x_q to the other three. T sits transposed in
// shared memory (a quad's four rows of one column are neighbours: no bank
// conflicts), padded to an identity triangle when nb < 64. Measured on GB300:
// a warp issues FP64 at one SM sub-partition's share, so one thread per
// column (32 warps for 1024 columns) left the FP64 units 85 % idle and a
// 64-row leaf took 105 us; an earlier kernel also re-read every solved entry
// from global memory inside a left-looking loop (leaves 72 % of a 4096 TRSM).
constexpr int kTrsmLanes = 4;                          // threads per column
constexpr int kTrsmRowsPerLane = kTrsmBlock / kTrsmLanes;
constexpr int kTrsmLeafThreads = 128;

template <typename T>
__global__ void __launch_bounds__(kTrsmLeafThreads) trsm_diag_kernel(const T* __restrict__ a, int64_t a_si,
                                                                     int64_t a_sj, T* __restrict__ b, int64_t b_si,
                                                                     int64_t b_sj, int nb, int64_t ncols, int lower,
                                                                     int unit) {
    __shared__ T tt[kTrsmBlock][kTrsmBlock];  // tt[q][i] = T[i][q]
    __shared__ T rdiag[kTrsmBlock];
    for (int idx = threadIdx.x; idx < kTrsmBlock * kTrsmBlock; idx += blockDim.x) {
        const int i = idx / kTrsmBlock, q = idx % kTrsmBlock;
        tt[q][i] = (i < nb && q < nb) ? a[i * a_si + q * a_sj] : (i == q ? (T)1 : (T)0);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kTrsmBlock; i += blockDim.x) rdiag[i] = unit ? (T)1 : (T)1 / tt[i][i];
    __syncthreads();
    const int k = threadIdx.x & (kTrsmLanes - 1);
    const int64_t col = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / kTrsmLanes;
    const bool live = col < ncols;  // every lane stays for the shuffles
    T* xc = b + (live ? col : 0) * b_sj;
    const int lead = (threadIdx.x & 31) & ~(kTrsmLanes - 1);
    T x[kTrsmRowsPerLane];
#pragma unroll
    for (int j = 0; j < kTrsmRowsPerLane; ++j) {
        const int i = kTrsmLanes * j + k;
        x[j] = (live && i < nb) ? xc[i * b_si] : (T)0;
    }
    if (lower) {
#pragma unroll
        for (int q = 0; q < kTrsmBlock; ++q) {
            const int jq = q / kTrsmLanes;
            const T xq = __shfl_sync(0xffffffffu, x[jq] * rdiag[q], lead | (q % kTrsmLanes));
            if (k == q % kTrsmLanes) x[jq] = xq;
#pragma unroll
            for (int j = 0; j < kTrsmRowsPerLane; ++j) {
                const int i0 = kTrsmLanes * j;  // this slot's rows are i0 .. i0 + 3
                if (i0 + kTrsmLanes - 1 <= q) continue;
                if (i0 > q || i0 + k > q) x[j] -= tt[q][i0 + k] * xq;
            }
        }
    } else {
#pragma unroll
        for (int q = kTrsmBlock - 1; q >= 0; --q) {
            const int jq = q / kTrsmLanes;
            const T xq = __shfl_sync(0xffffffffu, x[jq] * rdiag[q], lead | (q % kTrsmLanes));
            if (k == q % kTrsmLanes) x[jq] = xq;
#pragma unroll
            for (int j = 0; j < kTrsmRowsPerLane; ++j) {
                const int i0 = kTrsmLanes * j;
                if (i0 >= q) continue;
                if (i0 + kTrsmLanes - 1 < q || i0 + k < q) x[j] -= tt[q][i0 + k] * xq;
            }
        }
    }
    if (live) {
#pragma unroll
        for (int j = 0; j < kTrsmRowsPerLane; ++j) {
            const int i = kTrsmLanes * j + k;
            if (i < nb) xc[i * b_si] = x[j];
        }
    }
}

// A matrix view rows x cols of a BLAS operand in `order` with leading dimension ld.
Layout mat_view(rstsr_order order, int64_t rows, int64_t cols, int64_t ld) {
    Layout l;
    l.ndim = 2;
    l.shape[0] = rows;
    l.shape[1] = cols;
    l.stride[0] = order == RSTSR_ROW_MAJOR ? ld : 1;
    l.stride[1] = order == RSTSR_ROW_MAJOR ? 1 : ld;
    return l;
}

Layout transposed(const Layout& l) {
    Layout t = l;
    std::swap(t.shape[0], t.shape[1]);
    std::swap(t.stride[0], t.stride[1]);
    return t;
}

Layout sub_view(const Layout& l, int64_t r0, int64_t r1, int64_t c0, int64_t c1) {
    Layout v = l;
    v.offset = l.offset + r0 * l.stride[0] + c0 * l.stride[1];
    v.shape[0] = r1 - r0;
    v.shape[1] = c1 - c0;
    return v;
}

bool blas_float(rstsr_dtype t) { return t == RSTSR_F64 || t == RSTSR_F32; }

int check_ld(rstsr_order order, int64_t rows, int64_t cols, int64_t ld, const char* what) {
    const int64_t need = order == RSTSR_ROW_MAJOR ? cols : rows;
    if (ld < std::max<int64_t>(need, 1))
        return fail(RSTSR_ERR_INVALID_VALUE, std::string(what) + ": leading dimension too small");
    return RSTSR_OK;
}

int upper_lower(char c, bool* lower) {
    if (c == 'L' || c == 'l') *lower = true;
    else if (c == 'U' || c == 'u') *lower = false;
    else return fail(RSTSR_ERR_INVALID_VALUE, "uplo must be 'L' or 'U'");
    return RSTSR_OK;
}

int trans_flag(char c, bool* tr) {
    if (c == 'N' || c == 'n') *tr = false;
    else if (c == 'T' || c == 't' || c == 'C' || c == 'c') *tr = true;
    else return fail(RSTSR_ERR_INVALID_VALUE, "trans must be 'N', 'T' or 'C'");
    return RSTSR_OK;
}

const void* scalar_of(rstsr_dtype t, double v, double* d, float* f) {
    *d = v;
    *f = (float)v;
    return t == RSTSR_F64 ? (const void*)d : (const void*)f;
}

}  // namespace

}  // namespace rstsr

using namespace rstsr;

extern "C" {

int rstsr_cuda_syrk(rstsr_ctx* ctx, rstsr_order order, char uplo, char trans, int64_t n, int64_t k, double alpha,
                    const void* a, int64_t lda, double beta, void* c, int64_t ldc, rstsr_dtype t,
                    const rstsr_gemm_opts* opts) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    if (!blas_float(t)) return fail(RSTSR_ERR_INVALID_VALUE, "syrk: F64 or F32");
    bool lower, tr;
    RSTSR_TRY(upper_lower(uplo, &lower));
    RSTSR_TRY(trans_flag(trans, &tr));
    if (n < 0 || k < 0) return fail(RSTSR_ERR_INVALID_VALUE, "syrk: negative dimension");
    RSTSR_TRY(check_ld(order, tr ? k : n, tr ? n : k, lda, "syrk A"));
    RSTSR_TRY(check_ld(order, n, n, ldc, "syrk C"));
    if (n == 0) return RSTSR_OK;
    if (!a || !c) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    const size_t es = dtype_size(t);
    const Layout lc = mat_view(order, n, n, ldc);
    Layout la = mat_view(order, tr ? k : n, tr ? n : k, lda);
    if (tr) la = transposed(la);  // op(A), n x k
    const int64_t ntp = n * (n + 1) / 2;
    void *w = nullptr, *pw = nullptr, *pc = nullptr;
    auto cleanup = [&](int rc) {
        if (w) scratch_free(ctx, w);
        if (pw) scratch_free(ctx, pw);
        if (pc) scratch_free(ctx, pc);
        return rc;
    };
    int rc = scratch_alloc(ctx, (size_t)n * n * es, &w);
    if (rc == RSTSR_OK) rc = scratch_alloc(ctx, (size_t)ntp * es, &pw);
    if (rc == RSTSR_OK && beta != 0.0) rc = scratch_alloc(ctx, (size_t)ntp * es, &pc);
    if (rc != RSTSR_OK) return cleanup(rc);
    // W = alpha op(A) op(A)^T (the symmetric split GEMM: b is the transpose view of a)
    const int64_t sw[2] = {n, n};
    const Layout lw = Layout::c_contig(sw, 2);
    const Layout lat = transposed(la);
    rstsr_layout l0 = lw.to_abi(), l1 = la.to_abi(), l2 = lat.to_abi();
    if (k == 0) {
        double d;
        float f;
        rc = rstsr_cuda_fill(ctx, w, &l0, t, scalar_of(t, 0.0, &d, &f));
    } else {
        rc = rstsr_cuda_matmul(ctx, t, w, &l0, a, &l1, a, &l2, alpha, 0.0, RSTSR_ROW_MAJOR, opts);
    }
    if (rc != RSTSR_OK) return cleanup(rc);
    // the uplo triangle of C = W + beta C on packed vectors
    const int64_t sp[1] = {ntp};
    const Layout lp = Layout::c_contig(sp, 1);
    rstsr_layout lpa = lp.to_abi(), lwa = lw.to_abi(), lca = lc.to_abi();
    const char u = lower ? 'L' : 'U';
    rc = rstsr_cuda_pack_tri(ctx, t, pw, &lpa, w, &lwa, u, RSTSR_ROW_MAJOR);
    void* src = pw;
    if (rc == RSTSR_OK && beta != 0.0) {
        double d;
        float f;
        rc = rstsr_cuda_pack_tri(ctx, t, pc, &lpa, c, &lca, u, RSTSR_ROW_MAJOR);
        if (rc == RSTSR_OK && beta != 1.0)
            rc = rstsr_cuda_binary_scalar(ctx, RSTSR_OP_MUL, t, pc, &lpa, pc, &lpa, scalar_of(t, beta, &d, &f), 0);
        if (rc == RSTSR_OK) rc = rstsr_cuda_binary(ctx, RSTSR_OP_ADD, t, pc, &lpa, pc, &lpa, pw, &lpa);
        src = pc;
    }
    if (rc == RSTSR_OK) rc = rstsr_cuda_unpack_tri(ctx, t, c, &lca, src, &lpa, u, RSTSR_SYMM_N, RSTSR_ROW_MAJOR);
    return cleanup(rc);
}

int rstsr_cuda_symm(rstsr_ctx* ctx, rstsr_order order, char side, char uplo, int64_t m, int64_t n, double alpha,
                    const void* a, int64_t lda, const void* b, int64_t ldb, double beta, void* c, int64_t ldc,
                    rstsr_dtype t, const rstsr_gemm_opts* opts) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    if (!blas_float(t)) return fail(RSTSR_ERR_INVALID_VALUE, "symm: F64 or F32");
    bool lower;
    RSTSR_TRY(upper_lower(uplo, &lower));
    const bool left = side == 'L' || side == 'l';
    if (!left && side != 'R' && side != 'r') return fail(RSTSR_ERR_INVALID_VALUE, "side must be 'L' or 'R'");
    if (m < 0 || n < 0) return fail(RSTSR_ERR_INVALID_VALUE, "symm: negative dimension");
    const int64_t na = left ? m : n;
    RSTSR_TRY(check_ld(order, na, na, lda, "symm A"));
    RSTSR_TRY(check_ld(order, m, n, ldb, "symm B"));
    RSTSR_TRY(check_ld(order, m, n, ldc, "symm C"));
    if (m == 0 || n == 0) return RSTSR_OK;
    if (!a || !b || !c) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    const size_t es = dtype_size(t);
    const int64_t ntp = na * (na + 1) / 2;
    void *full = nullptr, *pk = nullptr;
    auto cleanup = [&](int rc) {
        if (full) scratch_free(ctx, full);
        if (pk) scratch_free(ctx, pk);
        return rc;
    };
    int rc = scratch_alloc(ctx, (size_t)na * na * es, &full);
    if (rc == RSTSR_OK) rc = scratch_alloc(ctx, (size_t)ntp * es, &pk);
    if (rc != RSTSR_OK) return cleanup(rc);
    const Layout la = mat_view(order, na, na, lda);
    const int64_t sf[2] = {na, na}, sp[1] = {ntp};
    const Layout lf = Layout::c_contig(sf, 2), lp = Layout::c_contig(sp, 1);
    rstsr_layout l_a = la.to_abi(), l_f = lf.to_abi(), l_p = lp.to_abi();
    const char u = lower ? 'L' : 'U';
    rc = rstsr_cuda_pack_tri(ctx, t, pk, &l_p, a, &l_a, u, RSTSR_ROW_MAJOR);
    if (rc == RSTSR_OK) rc = rstsr_cuda_unpack_tri(ctx, t, full, &l_f, pk, &l_p, u, RSTSR_SYMM_SY, RSTSR_ROW_MAJOR);
    if (rc != RSTSR_OK) return cleanup(rc);
    const Layout lb = mat_view(order, m, n, ldb), lc = mat_view(order, m, n, ldc);
    rstsr_layout l_b = lb.to_abi(), l_c = lc.to_abi();
    if (left)
        rc = rstsr_cuda_matmul(ctx, t, c, &l_c, full, &l_f, b, &l_b, alpha, beta, RSTSR_ROW_MAJOR, opts);
    else
        rc = rstsr_cuda_matmul(ctx, t, c, &l_c, b, &l_b, full, &l_f, alpha, beta, RSTSR_ROW_MAJOR, opts);
    return cleanup(rc);
}

int rstsr_cuda_trsm(rstsr_ctx* ctx, rstsr_order order, char side, char uplo, char transa, char diag, int64_t m,
                    int64_t n, double alpha, const void* a, int64_t lda, void* b, int64_t ldb, rstsr_dtype t,
                    const rstsr_gemm_opts* opts) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    if (!blas_float(t)) return fail(RSTSR_ERR_INVALID_VALUE, "trsm: F64 or F32");
    bool lower, tr;
    RSTSR_TRY(upper_lower(uplo, &lower));
    RSTSR_TRY(trans_flag(transa, &tr));
    const bool left = side == 'L' || side == 'l';
    if (!left && side != 'R' && side != 'r') return fail(RSTSR_ERR_INVALID_VALUE, "side must be 'L' or 'R'");
    const bool unit = diag == 'U' || diag == 'u';
    if (!unit && diag != 'N' && diag != 'n') return fail(RSTSR_ERR_INVALID_VALUE, "diag must be 'U' or 'N'");
    if (m < 0 || n < 0) return fail(RSTSR_ERR_INVALID_VALUE, "trsm: negative dimension");
    const int64_t na = left ? m : n;
    RSTSR_TRY(check_ld(order, na, na, lda, "trsm A"));
    RSTSR_TRY(check_ld(order, m, n, ldb, "trsm B"));
    if (m == 0 || n == 0) return RSTSR_OK;
    if (!a || !b) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    // op(A) as a view, then side R -> side L: X op(A) = B  <=>  op(A)^T X^T = B^T
    Layout A = mat_view(order, na, na, lda);
    Layout B = mat_view(order, m, n, ldb);
    if (tr) {
        A = transposed(A);
        lower = !lower;
    }
    if (!left) {
        A = transposed(A);
        lower = !lower;
        B = transposed(B);
    }
    const int64_t rows = B.shape[0], cols = B.shape[1];
    const size_t es = dtype_size(t);
    double d;
    float f;
    int rc = RSTSR_OK;
    rstsr_layout lb_full = B.to_abi();
    if (alpha != 1.0)
        rc = rstsr_cuda_binary_scalar(ctx, RSTSR_OP_MUL, t, b, &lb_full, b, &lb_full, scalar_of(t, alpha, &d, &f), 0);
    if (rc != RSTSR_OK) return rc;
    // Recursive halving (split points on kTrsmBlock boundaries): solve one half,
    // update the other with one GEMM of K = that half, solve the other half. The
    // same flops as a block-by-block sweep, but in GEMMs weighted towards large K
    // (one of K = rows / 2, two of rows / 4, ...), which the split GEMM runs far
    // more efficiently than many K = kTrsmBlock updates.
    auto solve_block = [&](int64_t r0, int64_t r1) -> int {
        const Layout Ad = sub_view(A, r0, r1, r0, r1), Bd = sub_view(B, r0, r1, 0, cols);
        const int64_t threads = cols * kTrsmLanes;
        const unsigned grid = (unsigned)((threads + kTrsmLeafThreads - 1) / kTrsmLeafThreads);
        if (t == RSTSR_F64)
            trsm_diag_kernel<double><<<grid, kTrsmLeafThreads, 0, ctx->stream>>>(
                (const double*)a + Ad.offset, Ad.stride[0], Ad.stride[1], (double*)b + Bd.offset, Bd.stride[0],
                Bd.stride[1], (int)(r1 - r0), cols, lower ? 1 : 0, unit ? 1 : 0);
        else
            trsm_diag_kernel<float><<<grid, kTrsmLeafThreads, 0, ctx->stream>>>(
                (const float*)a + Ad.offset, Ad.stride[0], Ad.stride[1], (float*)b + Bd.offset, Bd.stride[0],
                Bd.stride[1], (int)(r1 - r0), cols, lower ? 1 : 0, unit ? 1 : 0);
        return after_launch(ctx, "trsm_diag_kernel");
    };
    // B[u0:u1] -= A[u0:u1, s0:s1] X[s0:s1]
    auto update = [&](int64_t u0, int64_t u1, int64_t s0, int64_t s1) -> int {
        const Layout Bu = sub_view(B, u0, u1, 0, cols), Au = sub_view(A, u0, u1, s0, s1);
        const Layout Bs = sub_view(B, s0, s1, 0, cols);
        rstsr_layout l0 = Bu.to_abi(), l1 = Au.to_abi(), l2 = Bs.to_abi();
        return rstsr_cuda_matmul(ctx, t, b, &l0, a, &l1, b, &l2, -1.0, 1.0, RSTSR_ROW_MAJOR, opts);
    };
    // an explicit stack of row ranges (depth log2(rows / kTrsmBlock)); a range
    // is pushed with phase 0 (split it) and revisited with phase 1 (update
    // between its halves, then its second half)
    struct Frame {
        int64_t r0, r1, mid;
        int phase;
    };
    std::vector<Frame> stack;
    stack.push_back({0, rows, 0, 0});
    while (!stack.empty()) {
        Frame& f = stack.back();
        if (f.r1 - f.r0 <= kTrsmBlock) {
            const int64_t r0 = f.r0, r1 = f.r1;
            stack.pop_back();
            RSTSR_TRY(solve_block(r0, r1));
            continue;
        }
        if (f.phase == 0) {
            const int64_t half = (f.r1 - f.r0 + 1) / 2;
            f.mid = f.r0 + (half + kTrsmBlock - 1) / kTrsmBlock * kTrsmBlock;
            f.phase = 1;
            // lower: the top half first; upper: the bottom half first
            const Frame first = lower ? Frame{f.r0, f.mid, 0, 0} : Frame{f.mid, f.r1, 0, 0};
            stack.push_back(first);
            continue;
        }
        // phase 1: the first half is solved; update the second half and solve it
        const int64_t r0 = f.r0, r1 = f.r1, mid = f.mid;
        stack.pop_back();
        if (lower)
            rc = update(mid, r1, r0, mid);
        else
            rc = update(r0, mid, mid, r1);
        if (rc != RSTSR_OK) return rc;
        stack.push_back(lower ? Frame{mid, r1, 0, 0} : Frame{r0, mid, 0, 0});
    }
    (void)es;
    return RSTSR_OK;
}

}  // extern "C"
