// Reduction planner and C ABI: Op{Sum,Mean,Var,Std,Min,Max,Prod,L2Norm,All,
// Any,CountNonZero}API::{*_all, *_axes} and Op{ArgMax,ArgMin}API
// (rstsr-core/src/operators/reduction.rs:3-33; CPU semantics in
// rstsr-core/src/feature_rayon/auto_impl/reduction.rs:7-716).
//
// The planner splits the input layout into reduced and kept axes
// (dim_split_axes, rstsr-common/src/layout/indexer.rs:453), picks the output
// layout layout_for_array_copy(kept, K) exactly as the reference does
// (rstsr-native-impl/src/cpu_serial/reduction.rs:210-215), collapses both
// spaces and chooses the row or column regime and the chunk split of
// reduce_kernel.cuh.
#include <algorithm>
#include <cstring>

#include "reduce_kernel.cuh"

namespace rstsr {

static bool is_f(rstsr_dtype t) { return t == RSTSR_F64 || t == RSTSR_F32 || t == RSTSR_F16 || t == RSTSR_BF16; }
static bool is_signed_int(rstsr_dtype t) {
    return t == RSTSR_I8 || t == RSTSR_I16 || t == RSTSR_I32 || t == RSTSR_I64;
}
static bool is_unsigned_int(rstsr_dtype t) {
    return t == RSTSR_U8 || t == RSTSR_U16 || t == RSTSR_U32 || t == RSTSR_U64;
}

// How a reduction of dtype ta is evaluated: the dtype the kernel reads (after
// an exact widening copy if it differs), the accumulator kind, the dtype the
// kernel writes and the dtype the caller receives (a narrowing copy follows
// when the two differ).
struct RedPlan {
    rstsr_dtype t_in;
    int kind;
    rstsr_dtype t_kout;
    rstsr_dtype t_out;
};

static int plan_dtypes(int op, rstsr_dtype ta, RedPlan* rp) {
    if (!dtype_valid(ta)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    const bool f = is_f(ta), si = is_signed_int(ta), ui = is_unsigned_int(ta), b = ta == RSTSR_BOOL;
    // widened reading dtype
    rstsr_dtype tw = ta;
    if (ta == RSTSR_F16 || ta == RSTSR_BF16) tw = RSTSR_F32;
    if (ta == RSTSR_I8 || ta == RSTSR_I16) tw = RSTSR_I64;
    if (ta == RSTSR_U8 || ta == RSTSR_U16 || ta == RSTSR_U32) tw = RSTSR_U64;
    auto bad = [&]() {
        return fail(RSTSR_ERR_INVALID_VALUE,
                    std::string("reduction ") + std::to_string(op) + " is not defined on " + dtype_name(ta));
    };
    switch (op) {
        case RSTSR_RED_SUM:
            if (b) {  // OpSumBoolAPI: count of true values as usize
                *rp = {RSTSR_BOOL, kRedCount, RSTSR_U64, RSTSR_U64};
                return RSTSR_OK;
            }
            *rp = {tw, kRedSum, tw, ta};
            return RSTSR_OK;
        case RSTSR_RED_MEAN:
            if (!f) return bad();
            *rp = {tw, kRedSum, tw, ta};
            return RSTSR_OK;
        case RSTSR_RED_VAR:
        case RSTSR_RED_STD:
            if (!f) return bad();
            *rp = {tw, kRedMoments, tw, ta};
            return RSTSR_OK;
        case RSTSR_RED_L2NORM:
            if (!f) return bad();
            *rp = {tw, kRedSumSq, tw, ta};
            return RSTSR_OK;
        case RSTSR_RED_MIN:
        case RSTSR_RED_MAX:
        case RSTSR_RED_PROD:
            if (b) return bad();
            *rp = {tw, op == RSTSR_RED_MIN ? kRedMin : op == RSTSR_RED_MAX ? kRedMax : kRedProd, tw, ta};
            return RSTSR_OK;
        case RSTSR_RED_ALL:
        case RSTSR_RED_ANY:
            if (!b) return bad();
            *rp = {RSTSR_BOOL, op == RSTSR_RED_ALL ? kRedAll : kRedAny, RSTSR_BOOL, RSTSR_BOOL};
            return RSTSR_OK;
        case RSTSR_RED_COUNT_NONZERO:
            *rp = {b ? RSTSR_BOOL : tw, kRedCount, RSTSR_U64, RSTSR_U64};
            return RSTSR_OK;
        default:
            return fail(RSTSR_ERR_INVALID_VALUE, "unknown reduction");
    }
    (void)si;
    (void)ui;
}

static int plan_arg_dtypes(rstsr_dtype ta, int is_max, RedPlan* rp) {
    if (!dtype_valid(ta)) return fail(RSTSR_ERR_INVALID_VALUE, "unknown dtype");
    if (ta == RSTSR_BOOL) return fail(RSTSR_ERR_INVALID_VALUE, "arg reductions are not defined on bool");
    rstsr_dtype tw = ta;
    if (ta == RSTSR_F16 || ta == RSTSR_BF16) tw = RSTSR_F32;  // exact, order and ties preserved
    if (ta == RSTSR_I8 || ta == RSTSR_I16) tw = RSTSR_I64;
    if (ta == RSTSR_U8 || ta == RSTSR_U16 || ta == RSTSR_U32) tw = RSTSR_U64;
    *rp = {tw, is_max ? kRedArgMax : kRedArgMin, RSTSR_U64, RSTSR_U64};
    return RSTSR_OK;
}

static int launch_kind(rstsr_ctx* ctx, rstsr_dtype t, int kind, const RedParams& p) {
    switch (t) {
        case RSTSR_F64: return reduce_launch_f64(ctx, kind, p);
        case RSTSR_F32: return reduce_launch_f32(ctx, kind, p);
        case RSTSR_I32: return reduce_launch_i32(ctx, kind, p);
        case RSTSR_I64: return reduce_launch_i64(ctx, kind, p);
        case RSTSR_U64: return reduce_launch_u64(ctx, kind, p);
        case RSTSR_BOOL: return reduce_launch_bool(ctx, kind, p);
        default: return fail(RSTSR_ERR_INVALID_VALUE, "no reduction kernel for this dtype");
    }
}

// Collapse the reduced axes: extent-1 axes dropped, sorted by |stride|,
// neighbours merged when contiguous in memory AND in logical C order of the
// reduced shape (needed to report arg indices).
static void build_red_space(const Layout& ls, RedSpace* r) {
    int64_t lstr[RSTSR_MAX_NDIM];
    {
        int64_t acc = 1;
        for (int i = ls.ndim - 1; i >= 0; --i) {
            lstr[i] = acc;
            acc *= std::max<int64_t>(ls.shape[i], 1);
        }
    }
    std::vector<int> axes;
    for (int i = 0; i < ls.ndim; ++i)
        if (ls.shape[i] != 1) axes.push_back(i);
    std::stable_sort(axes.begin(), axes.end(),
                     [&](int a, int b) { return std::llabs(ls.stride[a]) < std::llabs(ls.stride[b]); });
    int nd = 0;
    int64_t shape[RSTSR_MAX_NDIM], st[RSTSR_MAX_NDIM], lst[RSTSR_MAX_NDIM];
    for (int a : axes) {
        if (nd > 0 && ls.stride[a] == st[nd - 1] * shape[nd - 1] && lstr[a] == lst[nd - 1] * shape[nd - 1]) {
            shape[nd - 1] *= ls.shape[a];
        } else {
            shape[nd] = ls.shape[a];
            st[nd] = ls.stride[a];
            lst[nd] = lstr[a];
            nd++;
        }
    }
    if (nd == 0) {
        shape[0] = 1;
        st[0] = 0;
        lst[0] = 0;
        nd = 1;
    }
    memset(r, 0, sizeof(*r));
    r->nd = nd;
    for (int i = 0; i < RSTSR_MAX_NDIM; ++i) {
        r->shape[i] = i < nd ? (uint32_t)shape[i] : 1u;
        r->div[i] = FastDiv(r->shape[i]);
        r->stride[i] = i < nd ? st[i] : 0;
        r->lstride[i] = i < nd ? lst[i] : 0;
    }
}

// Plan a reduction of `a` (dtype t_in, layout La) over `axes` into `out`
// (layout Lo with the kept shape): fills every field of *pp except the
// scratch pointer. Allocates nothing. pp->nout == 0 means nothing to do.
int plan_reduce(rstsr_ctx* ctx, int op, rstsr_dtype t_in, const void* a, const Layout& La, const int64_t* axes,
                int naxes, void* out, const Layout& Lo, RedParams* pp) {
    Layout ls, lm;
    Error e;
    if (!split_axes(La, axes, naxes, &ls, &lm, nullptr, &e)) return fail(e.code, e.msg);
    if (lm.ndim != Lo.ndim || !std::equal(lm.shape, lm.shape + lm.ndim, Lo.shape))
        return fail(RSTSR_ERR_INVALID_LAYOUT, "reduction output shape does not match the kept axes (" +
                                                  Lo.repr() + " vs " + lm.repr() + ")");
    RedParams& p = *pp;
    memset(&p, 0, sizeof(p));
    p.nred = ls.size();
    p.nout = lm.size();
    if (p.nout == 0) return RSTSR_OK;
    if (p.nred >= (int64_t(1) << 32) || p.nout >= (int64_t(1) << 32))
        return fail(RSTSR_ERR_UNIMPLEMENTED, "reductions over 2^32 or more elements per output");
    build_red_space(ls, &p.r);
    // the flattened reduced index is the logical (C-order) index: every walk
    // in index order visits the logical indices in increasing order
    {
        int64_t acc = 1;
        bool mono = true;
        for (int i = 0; i < p.r.nd; ++i) {
            mono = mono && (p.r.shape[i] == 1 || p.r.lstride[i] == acc);
            acc *= p.r.shape[i];
        }
        p.mono = mono ? 1 : 0;
    }
    // kept space: operand 0 = input (drives the order), operand 1 = output
    {
        Layout lmi = lm, loo = Lo;
        lmi.offset = 0;
        loo.offset = 0;
        const Layout* ops[2] = {&lmi, &loo};
        IterSpace sk = make_iter_space(ops, 2);
        p.k.nd = sk.ndim;
        for (int i = 0; i < RSTSR_MAX_NDIM; ++i) {
            p.k.shape[i] = i < sk.ndim ? (uint32_t)sk.shape[i] : 1u;
            p.k.div[i] = FastDiv(p.k.shape[i]);
            p.k.in_stride[i] = i < sk.ndim ? sk.stride[0][i] : 0;
            p.k.out_stride[i] = i < sk.ndim ? sk.stride[1][i] : 0;
        }
        if (lm.ndim == 0) p.k.nd = 0;
    }
    p.in_off = La.offset;
    p.out_off = Lo.offset;
    p.in = a;
    p.out = out;
    p.op = op;
    const size_t es = dtype_size(t_in);
    const int VEC = (int)std::max<size_t>(1, 16 / es);
    const int64_t rin = std::llabs(p.r.stride[0]);
    const int64_t kin = p.k.nd > 0 ? std::llabs(p.k.in_stride[0]) : INT64_MAX;
    const int64_t target = 2 * (int64_t)ctx->num_sms;
    if (p.nred == 0) {
        // empty reduced set: one pass writes init -> f_out per output
        p.glog = 0;
        p.nsplit = 1;
        p.chunk = 1;
    } else if (rin <= kin) {
        // row regime. Group size from the vector loads per output (nvec):
        // short runs give each lane about 16 of them, long runs about 32
        // (a CTA that issues only one round of loads spends most of its life
        // waiting for it); 8-byte elements twice as many (their rounds are
        // four loads, and their folds are integer-pipe work that the longer
        // walks overlap with the loads). G <= 256. Measured on GB300 over the
        // [32,64,128,128] workload against 8 / 32 vectors a lane for every
        // type: f64 argmax over the last axis 0.57 -> 0.67 of HBM (C and
        // permuted), f64 sums over axes (1, 3) 0.59 -> 0.64, the step-2
        // sliced argmax 0.35 -> 0.37 (4-byte) and 0.40 -> 0.44 (f64).
        const bool s2_shape = VEC >= 4 && p.r.stride[0] == 2 && (p.r.shape[0] % (VEC / 2)) == 0;
        const int64_t W = p.r.stride[0] == 1 && (p.r.shape[0] % VEC) == 0 ? VEC : s2_shape ? VEC / 2 : 1;
        const int64_t nvec = (p.nred + W - 1) / W;
        const int64_t per_lane = (nvec <= 1024 ? 16 : 32) * (es >= 8 ? 2 : 1);
        int G = 1, glog = 0;
        while (G < 256 && (int64_t)G * 2 * per_lane <= nvec) {
            G <<= 1;
            ++glog;
        }
        if (nvec <= 1024 && G > 32) {
            G = 32;
            glog = 5;
        }
        p.glog = glog;
        p.row = 1;
        const int64_t gx = (p.nout + (kRedThreads / G) - 1) / (kRedThreads / G);
        int64_t nsplit = 1;
        if (gx < target && p.nred > (int64_t)G * VEC * 8)
            nsplit = std::min<int64_t>((target + gx - 1) / gx, (p.nred + (int64_t)G * VEC * 8 - 1) / ((int64_t)G * VEC * 8));
        nsplit = std::max<int64_t>(1, std::min<int64_t>(nsplit, 65535));
        int64_t chunk = (p.nred + nsplit - 1) / nsplit;
        chunk = (chunk + VEC - 1) / VEC * VEC;
        nsplit = (p.nred + chunk - 1) / chunk;
        p.nsplit = (int32_t)nsplit;
        p.chunk = chunk;
        // vector loads along reduced dim 0
        bool vec = VEC > 1 && p.r.stride[0] == 1 && (p.r.shape[0] % VEC) == 0 && (p.chunk % VEC) == 0;
        const int64_t vb = 16;
        if (vec) vec = ((reinterpret_cast<uintptr_t>(a) + (uintptr_t)(La.offset * (int64_t)es)) % vb) == 0;
        for (int i = 1; vec && i < p.r.nd; ++i) vec = (std::llabs(p.r.stride[i]) * (int64_t)es) % vb == 0;
        for (int i = 0; vec && i < p.k.nd; ++i) vec = (std::llabs(p.k.in_stride[i]) * (int64_t)es) % vb == 0;
        p.vec = vec ? 1 : 0;
        // step-2 rows of 4-byte or smaller elements: 16-byte loads of which
        // every other element is used (the other half of each sector is read
        // anyway), aligned like the contiguous case; no negative strides, so
        // that the view's largest offset bounds every load
        bool s2 = !vec && s2_shape && (p.chunk % VEC) == 0 &&
                  ((reinterpret_cast<uintptr_t>(a) + (uintptr_t)(La.offset * (int64_t)es)) % vb) == 0;
        for (int i = 1; s2 && i < p.r.nd; ++i) s2 = p.r.stride[i] > 0 && (p.r.stride[i] * (int64_t)es) % vb == 0;
        for (int i = 0; s2 && i < p.k.nd; ++i) s2 = p.k.in_stride[i] > 0 && (p.k.in_stride[i] * (int64_t)es) % vb == 0;
        if (s2) {
            int64_t mx = La.offset;
            for (int i = 0; i < La.ndim; ++i)
                if (La.shape[i] > 0) mx += (La.shape[i] - 1) * std::max<int64_t>(La.stride[i], 0);
            p.max_off = mx;
        }
        p.s2 = s2 ? 1 : 0;
        // the group's step over the reduced elements as (rows, columns) of dim 0
        const uint32_t step = (uint32_t)G * (uint32_t)(vec ? VEC : s2 ? VEC / 2 : 1);
        p.adv_row = step / p.r.shape[0];
        p.adv_c = step % p.r.shape[0];
    } else {
        // column regime: a warp reads 32 neighbouring outputs' elements per
        // step. When kept dim 0 is contiguous in the input (and everything is
        // aligned), each thread takes OV neighbouring outputs with one
        // OV-wide vector load per reduced element; measured on GB300 the
        // scalar form reached 22 % of DRAM bandwidth (f32 sum_axes over an
        // F-ordered tensor, 4096 outputs), latency-bound with ~20 KB in
        // flight per SM. A CTA keeps 256 x 8 vector loads in flight (32 KB)
        // or 256 x 4 scalar ones.
        p.glog = 0;
        const int OV = es >= 16 ? 1 : (16 / (int)es >= 4 ? 4 : 16 / (int)es);
        bool cv = OV > 1 && p.k.nd > 0 && p.k.in_stride[0] == 1 && (p.k.shape[0] % OV) == 0;
        const int64_t vbytes = (int64_t)OV * (int64_t)es;
        if (cv) cv = ((reinterpret_cast<uintptr_t>(a) + (uintptr_t)(La.offset * (int64_t)es)) % vbytes) == 0;
        for (int i = 1; cv && i < p.k.nd; ++i) cv = (std::llabs(p.k.in_stride[i]) * (int64_t)es) % vbytes == 0;
        for (int i = 0; cv && i < p.r.nd; ++i) cv = (std::llabs(p.r.stride[i]) * (int64_t)es) % vbytes == 0;
        p.ocol = cv ? OV : 1;
        const int64_t opc = (int64_t)kRedThreads * p.ocol;
        const int64_t gx = (p.nout + opc - 1) / opc;
        const int64_t col_target = 4 * (int64_t)ctx->num_sms;
        // With vector loads, split the reduced range only when the outputs
        // alone give fewer CTAs than SMs: with one CTA per SM or more the
        // loads in flight cover the HBM latency, and a split's partials (24
        // bytes per output and chunk for an arg reduction) and combine pass
        // cost more than they bring (f32 argmax over the last axis of an
        // F-ordered [32,64,128,128]: 48.9 us in three chunks, 30.7 us
        // unsplit). Scalar walks aim for four CTAs per SM, each walking a
        // long chunk.
        const int64_t split_below = p.ocol > 1 ? (int64_t)ctx->num_sms : col_target;
        int64_t nsplit = 1;
        if (gx < split_below && p.nred > 16)
            nsplit = std::min<int64_t>((col_target + gx - 1) / gx, (p.nred + 15) / 16);
        nsplit = std::max<int64_t>(1, std::min<int64_t>(nsplit, 65535));
        int64_t chunk = (p.nred + nsplit - 1) / nsplit;
        nsplit = (p.nred + chunk - 1) / chunk;
        p.nsplit = (int32_t)nsplit;
        p.chunk = chunk;
        p.vec = 0;
    }
    return RSTSR_OK;
}

// Plan and launch a reduction of `a` (dtype t_in, layout La) over `axes`
// into `out` (dtype t_kout, layout Lo with the kept shape).
static int run_reduce(rstsr_ctx* ctx, int op, rstsr_dtype t_in, int kind, const void* a, const Layout& La,
                      const int64_t* axes, int naxes, void* out, const Layout& Lo) {
    RedParams p;
    int s = plan_reduce(ctx, op, t_in, a, La, axes, naxes, out, Lo, &p);
    if (s || p.nout == 0) return s;
    return launch_kind(ctx, t_in, kind, p);
}

// Full reduction entry: widening copy in, kernel, narrowing copy out.
static int reduce_into(rstsr_ctx* ctx, int op, const RedPlan& rp, rstsr_dtype ta, const void* a, const Layout& La,
                       const int64_t* axes, int naxes, void* out, const Layout& Lo) {
    const void* src = a;
    Layout Ls = La;
    void* wide = nullptr;
    if (rp.t_in != ta) {
        const int64_t n = La.size();
        int s = scratch_alloc(ctx, (size_t)std::max<int64_t>(n, 1) * dtype_size(rp.t_in), &wide);
        if (s) return s;
        Ls = Layout::c_contig(La.shape, La.ndim);
        rstsr_layout lw = Ls.to_abi(), la = La.to_abi();
        s = rstsr_cuda_assign(ctx, wide, &lw, rp.t_in, a, &la, ta);
        if (s) {
            scratch_free(ctx, wide);
            return s;
        }
        src = wide;
    }
    int s;
    if (rp.t_kout == rp.t_out) {
        s = run_reduce(ctx, op, rp.t_in, rp.kind, src, Ls, axes, naxes, out, Lo);
    } else {
        void* tmp = nullptr;
        Layout Lt = Layout::c_contig(Lo.shape, Lo.ndim);
        s = scratch_alloc(ctx, (size_t)std::max<int64_t>(Lo.size(), 1) * dtype_size(rp.t_kout), &tmp);
        if (!s) s = run_reduce(ctx, op, rp.t_in, rp.kind, src, Ls, axes, naxes, tmp, Lt);
        if (!s && Lo.size() > 0) {
            rstsr_layout lo = Lo.to_abi(), lt = Lt.to_abi();
            s = rstsr_cuda_assign(ctx, out, &lo, rp.t_out, tmp, &lt, rp.t_kout);
        }
        if (tmp) scratch_free(ctx, tmp);
    }
    if (wide) scratch_free(ctx, wide);
    return s;
}

static int check_nonempty(int op, const Layout& La) {
    if (La.size() == 0 && (op == RSTSR_RED_MIN || op == RSTSR_RED_MAX))
        return fail(RSTSR_ERR_INVALID_VALUE,
                    std::string("zero-size array is not supported for ") + (op == RSTSR_RED_MIN ? "min" : "max"));
    return RSTSR_OK;
}

}  // namespace rstsr

using namespace rstsr;

#define RSTSR_TRY(expr)                \
    do {                               \
        int _s = (expr);               \
        if (_s != RSTSR_OK) return _s; \
    } while (0)

extern "C" {

int rstsr_cuda_reduce_out_dtype(rstsr_reduce_op op, rstsr_dtype ta, rstsr_dtype* tout) {
    clear_error();
    if (!tout) return fail(RSTSR_ERR_INVALID_VALUE, "null output");
    RedPlan rp;
    RSTSR_TRY(plan_dtypes(op, ta, &rp));
    *tout = rp.t_out;
    return RSTSR_OK;
}

int rstsr_cuda_reduce_axes_into(rstsr_ctx* ctx, rstsr_reduce_op op, rstsr_dtype ta, const void* a,
                                const rstsr_layout* la, const int64_t* axes, int32_t naxes, void* out,
                                const rstsr_layout* lout) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(la, "a"));
    RSTSR_TRY(check_layout(lout, "out"));
    if (naxes < 0 || (naxes > 0 && !axes)) return fail(RSTSR_ERR_INVALID_VALUE, "bad axes");
    RedPlan rp;
    RSTSR_TRY(plan_dtypes(op, ta, &rp));
    Layout La = Layout::from_abi(*la), Lo = Layout::from_abi(*lout);
    RSTSR_TRY(check_nonempty(op, La));
    if (Lo.size() > 0 && !out) return fail(RSTSR_ERR_INVALID_VALUE, "null output pointer");
    if (La.size() > 0 && !a) return fail(RSTSR_ERR_INVALID_VALUE, "null input pointer");
    return reduce_into(ctx, op, rp, ta, a, La, axes, naxes, out, Lo);
}

int rstsr_cuda_reduce_axes(rstsr_ctx* ctx, rstsr_reduce_op op, rstsr_dtype ta, const void* a, const rstsr_layout* la,
                           const int64_t* axes, int32_t naxes, void** out, rstsr_layout* lout) {
    clear_error();
    if (!out || !lout) return fail(RSTSR_ERR_INVALID_VALUE, "null output");
    *out = nullptr;
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(la, "a"));
    RedPlan rp;
    RSTSR_TRY(plan_dtypes(op, ta, &rp));
    RSTSR_TRY(rstsr_cuda_reduce_axes_layout(la, axes, naxes, lout));
    Layout Lo = Layout::from_abi(*lout);
    void* buf = nullptr;
    RSTSR_TRY(rstsr_cuda_malloc(ctx, (size_t)std::max<int64_t>(Lo.size(), 1) * dtype_size(rp.t_out), &buf));
    int s = rstsr_cuda_reduce_axes_into(ctx, op, ta, a, la, axes, naxes, buf, lout);
    if (s) {
        rstsr_cuda_free(ctx, buf);
        return s;
    }
    *out = buf;
    return RSTSR_OK;
}

int rstsr_cuda_reduce_all(rstsr_ctx* ctx, rstsr_reduce_op op, rstsr_dtype ta, const void* a, const rstsr_layout* la,
                          void* out_host) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(la, "a"));
    if (!out_host) return fail(RSTSR_ERR_INVALID_VALUE, "null output");
    RedPlan rp;
    RSTSR_TRY(plan_dtypes(op, ta, &rp));
    Layout La = Layout::from_abi(*la);
    RSTSR_TRY(check_nonempty(op, La));
    if (La.size() > 0 && !a) return fail(RSTSR_ERR_INVALID_VALUE, "null input pointer");
    int64_t axes[RSTSR_MAX_NDIM];
    for (int i = 0; i < La.ndim; ++i) axes[i] = i;
    Layout Lo;  // 0-dim
    void* dev = nullptr;
    RSTSR_TRY(scratch_alloc(ctx, 16, &dev));
    int s = reduce_into(ctx, op, rp, ta, a, La, axes, La.ndim, dev, Lo);
    if (s == RSTSR_OK) {
        cudaError_t e = cudaMemcpyAsync(out_host, dev, dtype_size(rp.t_out), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) s = cuda_fail(e, "reduce_all result copy");
    }
    scratch_free(ctx, dev);
    return s;
}

int rstsr_cuda_argreduce_axes_into(rstsr_ctx* ctx, int32_t is_max, rstsr_dtype ta, const void* a,
                                   const rstsr_layout* la, const int64_t* axes, int32_t naxes, void* out,
                                   const rstsr_layout* lout) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(la, "a"));
    RSTSR_TRY(check_layout(lout, "out"));
    if (naxes < 0 || (naxes > 0 && !axes)) return fail(RSTSR_ERR_INVALID_VALUE, "bad axes");
    RedPlan rp;
    RSTSR_TRY(plan_arg_dtypes(ta, is_max, &rp));
    Layout La = Layout::from_abi(*la), Lo = Layout::from_abi(*lout);
    if (La.size() == 0) return fail(RSTSR_ERR_INVALID_LAYOUT, "empty sequence is not allowed for reduce_arg.");
    if (!a || !out) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
    return reduce_into(ctx, is_max ? RSTSR_RED_MAX : RSTSR_RED_MIN, rp, ta, a, La, axes, naxes, out, Lo);
}

int rstsr_cuda_argreduce_axes(rstsr_ctx* ctx, int32_t is_max, rstsr_dtype ta, const void* a, const rstsr_layout* la,
                              const int64_t* axes, int32_t naxes, void** out, rstsr_layout* lout) {
    clear_error();
    if (!out || !lout) return fail(RSTSR_ERR_INVALID_VALUE, "null output");
    *out = nullptr;
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(la, "a"));
    RSTSR_TRY(rstsr_cuda_reduce_axes_layout(la, axes, naxes, lout));
    Layout Lo = Layout::from_abi(*lout);
    void* buf = nullptr;
    RSTSR_TRY(rstsr_cuda_malloc(ctx, (size_t)std::max<int64_t>(Lo.size(), 1) * 8, &buf));
    int s = rstsr_cuda_argreduce_axes_into(ctx, is_max, ta, a, la, axes, naxes, buf, lout);
    if (s) {
        rstsr_cuda_free(ctx, buf);
        return s;
    }
    *out = buf;
    return RSTSR_OK;
}

int rstsr_cuda_argreduce_all(rstsr_ctx* ctx, int32_t is_max, rstsr_dtype ta, const void* a, const rstsr_layout* la,
                             uint64_t* out_host) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(la, "a"));
    if (!out_host) return fail(RSTSR_ERR_INVALID_VALUE, "null output");
    Layout La = Layout::from_abi(*la);
    int64_t axes[RSTSR_MAX_NDIM];
    for (int i = 0; i < La.ndim; ++i) axes[i] = i;
    Layout Lo;
    rstsr_layout lo = Lo.to_abi();
    void* dev = nullptr;
    RSTSR_TRY(scratch_alloc(ctx, 16, &dev));
    int s = rstsr_cuda_argreduce_axes_into(ctx, is_max, ta, a, la, axes, La.ndim, dev, &lo);
    if (s == RSTSR_OK) {
        cudaError_t e = cudaMemcpyAsync(out_host, dev, 8, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) s = cuda_fail(e, "argreduce_all result copy");
    }
    scratch_free(ctx, dev);
    return s;
}

}  // extern "C"
