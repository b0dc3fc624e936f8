// einsum / tensordot / vecdot on the device.
//
// The reference contracts through TBLIS (crates-plugin/rstsr-tblis/src/
// einsum_impl.rs:146-199, tensordot_impl.rs:33-58 with the subscript builder
// rstsr-common/src/tensordot_to_einsum.rs:18-112; TBLIS 0.2 and
// opt-einsum-path 0.2 are third-party and not vendored), and vecdot through
// rstsr-native-impl/src/cpu_serial/vecdot.rs (DeviceVecdotAPI,
// rstsr-core/src/operators/linalg.rs:3-20).
//
// Here a host planner turns an einsum into calls of this library's own
// kernels, with the tensor cores doing every contraction:
//   1. repeated labels in one operand become a diagonal view (the strides of
//      the repeated axes add up; no copy);
//   2. labels that occur in one operand only and not in the output are summed
//      out with the reduction kernels;
//   3. while two or more operands remain, the pair whose result is smallest
//      (ties: the larger contraction) is contracted: labels split into batch
//      (both operands, kept), contracted (both, not kept) and free (one
//      operand, kept); the operands are viewed as [batch, M, K] x [batch, K, N]
//      when their axes merge (else copied contiguous first) and multiplied by
//      one batched matmul launch (Ozaki split for f64, bf16 split for f32);
//      with nothing contracted the product is the broadcast multiply kernel;
//   4. the last operand is permuted into the output by the copy kernels,
//      unless the last contraction could write the output directly.
// Labels are Unicode code points (the reference's own example uses Greek
// letters); whitespace is ignored; "->" is optional (implicit output: the
// labels seen once, in code-point order, as numpy does).
#include <algorithm>
#include <map>
#include <set>

#include "ew_kernel.cuh"

namespace rstsr {

namespace {

struct EinOp {
    const void* ptr = nullptr;
    Layout l;
    std::vector<int> lab;
    void* owned = nullptr;  // intermediate storage of this operand (freed when consumed)
};

// UTF-8 to code points; returns false on a malformed sequence.
bool utf8_decode(const char* s, std::vector<int>& out) {
    const unsigned char* p = reinterpret_cast<const unsigned char*>(s);
    while (*p) {
        int c = *p, n = 0;
        if (c < 0x80) {
            n = 0;
        } else if ((c & 0xE0) == 0xC0) {
            c &= 0x1F;
            n = 1;
        } else if ((c & 0xF0) == 0xE0) {
            c &= 0x0F;
            n = 2;
        } else if ((c & 0xF8) == 0xF0) {
            c &= 0x07;
            n = 3;
        } else {
            return false;
        }
        ++p;
        for (int k = 0; k < n; ++k, ++p) {
            if ((*p & 0xC0) != 0x80) return false;
            c = (c << 6) | (*p & 0x3F);
        }
        out.push_back(c);
    }
    return true;
}

bool is_space(int c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }

// "ij,jk->ik": input label lists and the output list.
int parse_subscripts(const char* subscripts, int nops, std::vector<std::vector<int>>& ins, std::vector<int>& out) {
    if (!subscripts) return fail(RSTSR_ERR_INVALID_VALUE, "einsum: null subscripts");
    std::vector<int> cps;
    if (!utf8_decode(subscripts, cps)) return fail(RSTSR_ERR_INVALID_VALUE, "einsum: subscripts are not UTF-8");
    ins.assign(1, {});
    bool arrow = false;
    for (size_t i = 0; i < cps.size(); ++i) {
        const int c = cps[i];
        if (is_space(c)) continue;
        if (c == '.') return fail(RSTSR_ERR_UNIMPLEMENTED, "einsum: ellipsis broadcasting is not supported");
        if (c == '-') {
            if (i + 1 >= cps.size() || cps[i + 1] != '>' || arrow)
                return fail(RSTSR_ERR_INVALID_VALUE, "einsum: malformed '->' in subscripts");
            arrow = true;
            ++i;
            continue;
        }
        if (c == ',') {
            if (arrow) return fail(RSTSR_ERR_INVALID_VALUE, "einsum: ',' after '->'");
            ins.emplace_back();
            continue;
        }
        if (c == '>') return fail(RSTSR_ERR_INVALID_VALUE, "einsum: stray '>' in subscripts");
        if (arrow)
            out.push_back(c);
        else
            ins.back().push_back(c);
    }
    if ((int)ins.size() != nops)
        return fail(RSTSR_ERR_INVALID_VALUE, "einsum: " + std::to_string(ins.size()) + " subscript groups for " +
                                                 std::to_string(nops) + " operands");
    if (!arrow) {
        std::map<int, int> count;
        for (auto& v : ins)
            for (int c : v) count[c]++;
        for (auto& kv : count)
            if (kv.second == 1) out.push_back(kv.first);  // std::map: code-point order
    }
    std::set<int> seen;
    for (int c : out)
        if (!seen.insert(c).second) return fail(RSTSR_ERR_INVALID_VALUE, "einsum: an output label repeats");
    std::set<int> all;
    for (auto& v : ins) all.insert(v.begin(), v.end());
    for (int c : out)
        if (!all.count(c)) return fail(RSTSR_ERR_INVALID_VALUE, "einsum: an output label is in no operand");
    return RSTSR_OK;
}

// Extent of every label, checked consistent across operands.
int label_extents(const std::vector<std::vector<int>>& ins, const std::vector<Layout>& ls, std::map<int, int64_t>& ext) {
    for (size_t k = 0; k < ins.size(); ++k) {
        if ((int)ins[k].size() != ls[k].ndim)
            return fail(RSTSR_ERR_INVALID_LAYOUT, "einsum: operand " + std::to_string(k) + " has " +
                                                      std::to_string(ls[k].ndim) + " axes but " +
                                                      std::to_string(ins[k].size()) + " labels");
        for (size_t a = 0; a < ins[k].size(); ++a) {
            auto it = ext.find(ins[k][a]);
            if (it == ext.end())
                ext[ins[k][a]] = ls[k].shape[a];
            else if (it->second != ls[k].shape[a])
                return fail(RSTSR_ERR_INVALID_LAYOUT, "einsum: a label has extents " + std::to_string(it->second) +
                                                          " and " + std::to_string(ls[k].shape[a]));
        }
    }
    return RSTSR_OK;
}

// Merge a repeated label into one axis (the diagonal view).
void take_diagonals(EinOp& op) {
    std::vector<int> lab;
    Layout l;
    l.offset = op.l.offset;
    for (int a = 0; a < op.l.ndim; ++a) {
        auto it = std::find(lab.begin(), lab.end(), op.lab[a]);
        if (it == lab.end()) {
            lab.push_back(op.lab[a]);
            l.shape[l.ndim] = op.l.shape[a];
            l.stride[l.ndim] = op.l.stride[a];
            l.ndim++;
        } else {
            l.stride[it - lab.begin()] += op.l.stride[a];
        }
    }
    op.l = l;
    op.lab = lab;
}

void release(rstsr_ctx* ctx, EinOp& op) {
    if (op.owned) scratch_free(ctx, op.owned);
    op.owned = nullptr;
}

int64_t prod_ext(const std::vector<int>& labs, const std::map<int, int64_t>& ext) {
    int64_t p = 1;
    for (int c : labs) p *= ext.at(c);
    return p;
}

// Sum out the axes whose labels are not in `keep`.
int sum_unkept(rstsr_ctx* ctx, rstsr_dtype t, EinOp& op, const std::set<int>& keep) {
    std::vector<int64_t> axes;
    std::vector<int> lab;
    for (int a = 0; a < op.l.ndim; ++a) {
        if (keep.count(op.lab[a]))
            lab.push_back(op.lab[a]);
        else
            axes.push_back(a);
    }
    if (axes.empty()) return RSTSR_OK;
    // the kept axes, C-contiguous, in their current order
    std::vector<int64_t> kshape;
    for (int a = 0; a < op.l.ndim; ++a)
        if (keep.count(op.lab[a])) kshape.push_back(op.l.shape[a]);
    Layout lo = Layout::c_contig(kshape.data(), (int)kshape.size());
    const int64_t n = std::max<int64_t>(lo.size(), 1);
    void* buf = nullptr;
    RSTSR_TRY(scratch_alloc(ctx, (size_t)n * dtype_size(t), &buf));
    rstsr_layout la = op.l.to_abi(), lab_o = lo.to_abi();
    int rc = rstsr_cuda_reduce_axes_into(ctx, RSTSR_RED_SUM, t, op.ptr, &la, axes.data(), (int32_t)axes.size(), buf,
                                         &lab_o);
    if (rc != RSTSR_OK) {
        scratch_free(ctx, buf);
        return rc;
    }
    release(ctx, op);
    op.ptr = buf;
    op.owned = buf;
    op.l = lo;
    op.lab = lab;
    return RSTSR_OK;
}

// View the axes `axes` (in this order) of l as one axis; false if they do not
// merge. Extent-1 axes never block a merge; no axes gives extent 1.
bool merge_axes(const Layout& l, const std::vector<int>& axes, int64_t* ext, int64_t* stride) {
    int64_t e = 1, s = 1;
    bool have = false;
    for (int k = (int)axes.size() - 1; k >= 0; --k) {  // innermost last in the list
        const int a = axes[k];
        if (l.shape[a] == 1) continue;
        if (!have) {
            s = l.stride[a];
            e = l.shape[a];
            have = true;
        } else {
            if (l.stride[a] != s * e) return false;
            e *= l.shape[a];
        }
    }
    *ext = e;
    *stride = s;
    return true;
}

// Copy op into C-contiguous scratch with its axes permuted to `order`.
int make_contig(rstsr_ctx* ctx, rstsr_dtype t, EinOp& op, const std::vector<int>& order) {
    Layout src;
    src.ndim = (int)order.size();
    src.offset = op.l.offset;
    std::vector<int64_t> shp;
    std::vector<int> lab;
    for (size_t k = 0; k < order.size(); ++k) {
        src.shape[k] = op.l.shape[order[k]];
        src.stride[k] = op.l.stride[order[k]];
        shp.push_back(src.shape[k]);
        lab.push_back(op.lab[order[k]]);
    }
    Layout dst = Layout::c_contig(shp.data(), (int)shp.size());
    const int64_t n = std::max<int64_t>(dst.size(), 1);
    void* buf = nullptr;
    RSTSR_TRY(scratch_alloc(ctx, (size_t)n * dtype_size(t), &buf));
    rstsr_layout ld = dst.to_abi(), ls = src.to_abi();
    int rc = rstsr_cuda_assign(ctx, buf, &ld, t, op.ptr, &ls, t);
    if (rc != RSTSR_OK) {
        scratch_free(ctx, buf);
        return rc;
    }
    release(ctx, op);
    op.ptr = buf;
    op.owned = buf;
    op.l = dst;
    op.lab = lab;
    return RSTSR_OK;
}

int axis_of(const EinOp& op, int c) { return (int)(std::find(op.lab.begin(), op.lab.end(), c) - op.lab.begin()); }

bool has(const std::vector<int>& v, int c) { return std::find(v.begin(), v.end(), c) != v.end(); }

// Merge the axes of `op` carrying `labs` (outer to inner).
bool merge_labels(const EinOp& op, const std::vector<int>& labs, int64_t* e, int64_t* st) {
    std::vector<int> axes;
    for (int c : labs) axes.push_back(axis_of(op, c));
    return merge_axes(op.l, axes, e, st);
}

// Labels ordered by decreasing |stride| in op (outer first; extent-1 last).
std::vector<int> by_stride(const EinOp& op, std::vector<int> labs) {
    std::stable_sort(labs.begin(), labs.end(), [&](int x, int y) {
        const int ax = axis_of(op, x), ay = axis_of(op, y);
        const bool ux = op.l.shape[ax] == 1, uy = op.l.shape[ay] == 1;
        if (ux != uy) return uy;
        return std::llabs(op.l.stride[ax]) > std::llabs(op.l.stride[ay]);
    });
    return labs;
}

// The longest inner run of `labs` (ordered by stride) that merges in op; the
// labels before it are returned in `moved` (they become batch axes).
std::vector<int> merged_suffix(const EinOp& op, const std::vector<int>& labs, std::vector<int>* moved) {
    moved->clear();
    for (size_t cut = 0; cut < labs.size(); ++cut) {
        std::vector<int> tail(labs.begin() + cut, labs.end());
        int64_t e, st;
        if (merge_labels(op, tail, &e, &st)) {
            moved->assign(labs.begin(), labs.begin() + cut);
            return tail;
        }
    }
    return {};
}

// Contract A and B over their shared labels not in `keep` with one batched
// matmul. Matmul views: A as [batch..., M, K], B as [batch..., K, N], the
// batch axes being the labels both keep plus free labels whose axes do not
// merge into M (or N) -- those get stride 0 in the other operand, so that the
// matmul broadcasts instead of a copy. K's labels are ordered so that they
// merge in both operands; an operand is copied contiguous only when no order
// works. The result's labels are batch, M's, N's. When `out` is given and its
// layout fits that label order, the product is written there directly.
int contract_pair(rstsr_ctx* ctx, rstsr_dtype t, EinOp& A, EinOp& B, const std::set<int>& keep,
                  const std::map<int, int64_t>& ext, const std::vector<int>& pref, const rstsr_gemm_opts* opts,
                  EinOp* res, void* out, const Layout* lout, const std::vector<int>* out_lab, bool* wrote_out) {
    *wrote_out = false;
    std::vector<int> batch, con, fa, fb;
    for (int c : A.lab) {
        if (has(B.lab, c) && keep.count(c))
            batch.push_back(c);
        else if (has(B.lab, c))
            con.push_back(c);
        else
            fa.push_back(c);
    }
    for (int c : B.lab)
        if (!has(A.lab, c)) fb.push_back(c);
    auto by_pref = [&](std::vector<int>& v) {
        std::stable_sort(v.begin(), v.end(), [&](int x, int y) {
            return std::find(pref.begin(), pref.end(), x) < std::find(pref.begin(), pref.end(), y);
        });
    };
    by_pref(batch);
    by_pref(fa);
    by_pref(fb);
    const int64_t k = prod_ext(con, ext);

    // the labels of the matmul axes
    std::vector<int> mlab, klab, nlab, movedA, movedB;
    if (!con.empty()) {
        auto k_ok = [&](const std::vector<int>& ord) {
            int64_t e, st;
            return merge_labels(A, ord, &e, &st) && merge_labels(B, ord, &e, &st);
        };
        // copy X contiguous as [batch, free, K] (A) or [batch, K, free] (B)
        auto copy_operand = [&](bool is_a) {
            EinOp& X = is_a ? A : B;
            std::vector<int> order;
            for (int c : batch) order.push_back(axis_of(X, c));
            if (is_a) {
                for (int c : fa) order.push_back(axis_of(X, c));
                for (int c : klab) order.push_back(axis_of(X, c));
            } else {
                for (int c : klab) order.push_back(axis_of(X, c));
                for (int c : fb) order.push_back(axis_of(X, c));
            }
            return make_contig(ctx, t, X, order);
        };
        klab = by_stride(A, con);
        if (!k_ok(klab)) {
            klab = by_stride(B, con);
            if (!k_ok(klab)) {
                // copy the smaller operand with K in the other's order; the other too if needed
                const bool copy_a = A.l.size() <= B.l.size();
                klab = by_stride(copy_a ? B : A, con);
                RSTSR_TRY(copy_operand(copy_a));
                if (!k_ok(klab)) RSTSR_TRY(copy_operand(!copy_a));
            }
        }
        mlab = fa.empty() ? fa : merged_suffix(A, by_stride(A, fa), &movedA);
        nlab = fb.empty() ? fb : merged_suffix(B, by_stride(B, fb), &movedB);
    } else {
        mlab = fa;
        nlab = fb;
    }
    std::vector<int> bl = batch;
    bl.insert(bl.end(), movedA.begin(), movedA.end());
    bl.insert(bl.end(), movedB.begin(), movedB.end());
    std::vector<int> rlab = bl;
    rlab.insert(rlab.end(), mlab.begin(), mlab.end());
    rlab.insert(rlab.end(), nlab.begin(), nlab.end());
    if ((int)rlab.size() > RSTSR_MAX_NDIM || (int)bl.size() + 2 > RSTSR_MAX_NDIM)
        return fail(RSTSR_ERR_UNIMPLEMENTED, "einsum: an intermediate would have more than 8 axes");
    const int64_t nres = prod_ext(rlab, ext);

    // the product's destination: the output itself when its axes fit, else scratch
    void* owned = nullptr;
    void* cptr = nullptr;
    Layout lres;  // result over rlab
    if (out && out_lab && *out_lab == rlab) {
        cptr = out;
        lres = *lout;
        *wrote_out = true;
    } else {
        std::vector<int64_t> shp;
        for (int c : rlab) shp.push_back(ext.at(c));
        lres = Layout::c_contig(shp.data(), (int)shp.size());
        RSTSR_TRY(scratch_alloc(ctx, (size_t)std::max<int64_t>(nres, 1) * dtype_size(t), &owned));
        cptr = owned;
    }
    auto fail_free = [&](int rc) {
        if (owned) scratch_free(ctx, owned);
        *wrote_out = false;
        return rc;
    };
    // a view of X over `labs` (stride 0 for labels X lacks)
    auto view_over = [&](const EinOp& X, const std::vector<int>& labs) {
        Layout v;
        v.ndim = (int)labs.size();
        v.offset = X.l.offset;
        for (size_t q = 0; q < labs.size(); ++q) {
            v.shape[q] = ext.at(labs[q]);
            v.stride[q] = has(X.lab, labs[q]) ? X.l.stride[axis_of(X, labs[q])] : 0;
        }
        return v;
    };
    int rc = RSTSR_OK;
    if (nres == 0) {
        // nothing to write
    } else if (k == 0) {
        rstsr_layout l = lres.to_abi();
        const double zero = 0.0;
        const float zf = 0.0f;
        const int64_t zi = 0;
        const void* z = t == RSTSR_F64 ? (const void*)&zero : t == RSTSR_F32 ? (const void*)&zf : (const void*)&zi;
        rc = rstsr_cuda_fill(ctx, cptr, &l, t, z);
    } else if (con.empty()) {
        // nothing contracted: the broadcast multiply over the result's axes
        Layout xa = view_over(A, rlab), xb = view_over(B, rlab);
        rstsr_layout l0 = lres.to_abi(), l1 = xa.to_abi(), l2 = xb.to_abi();
        rc = rstsr_cuda_binary(ctx, RSTSR_OP_MUL, t, cptr, &l0, A.ptr, &l1, B.ptr, &l2);
    } else {
        // [batch..., M, K] x [batch..., K, N] -> [batch..., M, N]
        const int nbd = (int)bl.size();
        Layout va = view_over(A, bl), vb = view_over(B, bl), vc;
        vc.ndim = nbd + 2;
        vc.offset = lres.offset;
        for (int q = 0; q < nbd; ++q) {
            vc.shape[q] = lres.shape[q];
            vc.stride[q] = lres.stride[q];
        }
        va.ndim = vb.ndim = nbd + 2;
        int64_t e, st;
        bool ok = true;
        // M and N of C: merge its axes nbd.. (the M labels) and the rest (the N labels)
        {
            std::vector<int> axm, axn;
            for (size_t q = 0; q < mlab.size(); ++q) axm.push_back(nbd + (int)q);
            for (size_t q = 0; q < nlab.size(); ++q) axn.push_back(nbd + (int)mlab.size() + (int)q);
            ok = merge_axes(lres, axm, &vc.shape[nbd], &vc.stride[nbd]) &&
                 merge_axes(lres, axn, &vc.shape[nbd + 1], &vc.stride[nbd + 1]);
        }
        if (!ok) {
            // the output's axes do not merge: compute into scratch instead
            if (*wrote_out) {
                *wrote_out = false;
                std::vector<int64_t> shp;
                for (int c : rlab) shp.push_back(ext.at(c));
                lres = Layout::c_contig(shp.data(), (int)shp.size());
                RSTSR_TRY(scratch_alloc(ctx, (size_t)std::max<int64_t>(nres, 1) * dtype_size(t), &owned));
                cptr = owned;
                for (int q = 0; q < nbd; ++q) vc.stride[q] = lres.stride[q];
                vc.offset = 0;
                std::vector<int> axm, axn;
                for (size_t q = 0; q < mlab.size(); ++q) axm.push_back(nbd + (int)q);
                for (size_t q = 0; q < nlab.size(); ++q) axn.push_back(nbd + (int)mlab.size() + (int)q);
                merge_axes(lres, axm, &vc.shape[nbd], &vc.stride[nbd]);
                merge_axes(lres, axn, &vc.shape[nbd + 1], &vc.stride[nbd + 1]);
            } else {
                return fail_free(fail(RSTSR_ERR_RUNTIME, "einsum: scratch result did not merge"));
            }
        }
        // an empty M keeps C row-major for the grouped kernel (the stride of an extent-1 axis is free)
        if (mlab.empty()) vc.stride[nbd] = vc.shape[nbd + 1] * std::max<int64_t>(vc.stride[nbd + 1], 1);
        ok = merge_labels(A, mlab, &va.shape[nbd], &va.stride[nbd]) &&
             merge_labels(A, klab, &va.shape[nbd + 1], &va.stride[nbd + 1]) &&
             merge_labels(B, klab, &vb.shape[nbd], &vb.stride[nbd]) &&
             merge_labels(B, nlab, &vb.shape[nbd + 1], &vb.stride[nbd + 1]);
        if (!ok) return fail_free(fail(RSTSR_ERR_RUNTIME, "einsum: operand axes did not merge"));
        (void)e;
        (void)st;
        rstsr_layout l0 = vc.to_abi(), l1 = va.to_abi(), l2 = vb.to_abi();
        rc = rstsr_cuda_matmul(ctx, t, cptr, &l0, A.ptr, &l1, B.ptr, &l2, 1.0, 0.0, RSTSR_ROW_MAJOR, opts);
    }
    if (rc != RSTSR_OK) return fail_free(rc);
    release(ctx, A);
    release(ctx, B);
    if (!*wrote_out) {
        res->l = lres;
        res->ptr = cptr;
        res->owned = owned;
        res->lab = rlab;
    }
    return RSTSR_OK;
}

bool einsum_dtype_ok(rstsr_dtype t) {
    return t == RSTSR_F64 || t == RSTSR_F32 || t == RSTSR_I32 || t == RSTSR_I64;
}

int einsum_impl(rstsr_ctx* ctx, rstsr_dtype t, const std::vector<std::vector<int>>& ins, const std::vector<int>& olab,
                int nops, const void* const* ptrs, const std::vector<Layout>& ls, void* out, const Layout& lout,
                const rstsr_gemm_opts* opts) {
    std::map<int, int64_t> ext;
    RSTSR_TRY(label_extents(ins, ls, ext));
    if (lout.ndim != (int)olab.size())
        return fail(RSTSR_ERR_INVALID_LAYOUT, "einsum: the output has " + std::to_string(lout.ndim) + " axes for " +
                                                  std::to_string(olab.size()) + " output labels");
    for (size_t a = 0; a < olab.size(); ++a)
        if (lout.shape[a] != ext[olab[a]])
            return fail(RSTSR_ERR_INVALID_LAYOUT, "einsum: output extent differs from the label's");
    RSTSR_TRY(check_write_layout(lout, "einsum"));
    if (lout.size() == 0) return RSTSR_OK;
    for (int k = 0; k < nops; ++k)
        if (!ptrs[k] && ls[k].size() > 0) return fail(RSTSR_ERR_INVALID_VALUE, "einsum: null operand pointer");
    if (!out) return fail(RSTSR_ERR_INVALID_VALUE, "einsum: null output pointer");

    std::vector<EinOp> ops(nops);
    for (int k = 0; k < nops; ++k) {
        ops[k].ptr = ptrs[k];
        ops[k].l = ls[k];
        ops[k].lab = ins[k];
        take_diagonals(ops[k]);
    }
    const std::set<int> oset(olab.begin(), olab.end());
    auto keep_for = [&](size_t self, size_t other) {
        std::set<int> keep = oset;
        for (size_t q = 0; q < ops.size(); ++q)
            if (q != self && q != other) keep.insert(ops[q].lab.begin(), ops[q].lab.end());
        return keep;
    };
    auto cleanup = [&](int rc) {
        for (auto& o : ops) release(ctx, o);
        return rc;
    };
    // 2. labels of one operand only
    for (size_t k = 0; k < ops.size(); ++k) {
        std::set<int> keep = keep_for(k, k);
        int rc = sum_unkept(ctx, t, ops[k], keep);
        if (rc != RSTSR_OK) return cleanup(rc);
    }
    // 3. pairwise contractions, smallest result first
    while (ops.size() > 1) {
        size_t bi = 0, bj = 1;
        int64_t best_size = -1, best_k = 0;
        for (size_t i = 0; i < ops.size(); ++i)
            for (size_t j = i + 1; j < ops.size(); ++j) {
                const std::set<int> keep = keep_for(i, j);
                std::set<int> rl;
                int64_t kk = 1;
                for (int c : ops[i].lab) {
                    const bool inb = std::find(ops[j].lab.begin(), ops[j].lab.end(), c) != ops[j].lab.end();
                    if (!inb || keep.count(c))
                        rl.insert(c);
                    else
                        kk *= ext[c];
                }
                for (int c : ops[j].lab) rl.insert(c);
                for (auto it = rl.begin(); it != rl.end();)
                    it = (!keep.count(*it) && std::find(ops[i].lab.begin(), ops[i].lab.end(), *it) != ops[i].lab.end() &&
                          std::find(ops[j].lab.begin(), ops[j].lab.end(), *it) != ops[j].lab.end())
                             ? rl.erase(it)
                             : std::next(it);
                int64_t sz = 1;
                for (int c : rl) sz *= ext[c];
                if (best_size < 0 || sz < best_size || (sz == best_size && kk > best_k)) {
                    best_size = sz;
                    best_k = kk;
                    bi = i;
                    bj = j;
                }
            }
        const std::set<int> keep = keep_for(bi, bj);
        const bool last = ops.size() == 2;
        // the last contraction: let the output order decide which operand is A
        if (last) {
            auto first_free = [&](const EinOp& x, const EinOp& y) {
                for (int c : olab) {
                    const bool inx = std::find(x.lab.begin(), x.lab.end(), c) != x.lab.end();
                    const bool iny = std::find(y.lab.begin(), y.lab.end(), c) != y.lab.end();
                    if (inx && !iny) return 0;
                    if (iny && !inx) return 1;
                }
                return 0;
            };
            if (first_free(ops[bi], ops[bj]) == 1) std::swap(bi, bj);
        }
        EinOp res;
        bool wrote = false;
        int rc = contract_pair(ctx, t, ops[bi], ops[bj], keep, ext, olab, opts, &res, last ? out : nullptr,
                               last ? &lout : nullptr, last ? &olab : nullptr, &wrote);
        if (rc != RSTSR_OK) return cleanup(rc);
        const size_t hi = std::max(bi, bj), lo = std::min(bi, bj);
        ops.erase(ops.begin() + hi);
        ops.erase(ops.begin() + lo);
        if (wrote) return cleanup(RSTSR_OK);
        ops.push_back(res);
    }
    // 4. permute the last operand into the output
    EinOp& f = ops[0];
    int rc = sum_unkept(ctx, t, f, oset);
    if (rc != RSTSR_OK) return cleanup(rc);
    Layout src;
    src.ndim = (int)olab.size();
    src.offset = f.l.offset;
    for (size_t a = 0; a < olab.size(); ++a) {
        const int ax = (int)(std::find(f.lab.begin(), f.lab.end(), olab[a]) - f.lab.begin());
        src.shape[a] = f.l.shape[ax];
        src.stride[a] = f.l.stride[ax];
    }
    rstsr_layout lo = lout.to_abi(), lsrc = src.to_abi();
    rc = rstsr_cuda_assign(ctx, out, &lo, t, f.ptr, &lsrc, t);
    return cleanup(rc);
}

int read_layouts(int nops, const rstsr_layout* lops, std::vector<Layout>& ls) {
    if (nops < 1) return fail(RSTSR_ERR_INVALID_VALUE, "einsum: at least one operand is required");
    if (!lops) return fail(RSTSR_ERR_INVALID_VALUE, "einsum: null layouts");
    for (int k = 0; k < nops; ++k) {
        RSTSR_TRY(check_layout(&lops[k], "operand"));
        ls.push_back(Layout::from_abi(lops[k]));
    }
    return RSTSR_OK;
}

// Labels of tensordot (rstsr-common/src/tensordot_to_einsum.rs:18-112):
// contracted pairs first, then A's remaining axes, then B's; the output keeps
// A's free axes then B's.
int tensordot_labels(int nda, int ndb, const int64_t* axes_a, const int64_t* axes_b, int naxes,
                     std::vector<std::vector<int>>& ins, std::vector<int>& out) {
    if (naxes < 0 || naxes > nda || naxes > ndb)
        return fail(RSTSR_ERR_INVALID_LAYOUT, "tensordot: more contracted axes than dimensions");
    std::vector<int> la(nda, -1), lb(ndb, -1);
    int next = 'a';
    for (int q = 0; q < naxes; ++q) {
        int64_t x = axes_a[q] < 0 ? axes_a[q] + nda : axes_a[q];
        int64_t y = axes_b[q] < 0 ? axes_b[q] + ndb : axes_b[q];
        if (x < 0 || x >= nda || y < 0 || y >= ndb) return fail(RSTSR_ERR_AXIS, "tensordot: axis out of range");
        if (la[x] >= 0 || lb[y] >= 0) return fail(RSTSR_ERR_INVALID_VALUE, "tensordot: an axis repeats");
        la[x] = lb[y] = next++;
    }
    for (int i = 0; i < nda; ++i)
        if (la[i] < 0) {
            la[i] = next++;
            out.push_back(la[i]);
        }
    for (int j = 0; j < ndb; ++j)
        if (lb[j] < 0) {
            lb[j] = next++;
            out.push_back(lb[j]);
        }
    ins = {la, lb};
    return RSTSR_OK;
}

// Fused dot products: one warp per output element c[r] = sum_k a[r, k] b[r, k]
// over a contracted axis contiguous in both operands (stride 1), four loads
// of each operand in flight per lane, a shuffle reduction at the end. The
// outputs' multi-indices (broadcast operands: stride 0) are decomposed from
// the warp's row number.
struct DotParams {
    DevDims dims;  // the output's collapsed dims (inner first)
    int64_t sc[RSTSR_MAX_NDIM], sa[RSTSR_MAX_NDIM], sb[RSTSR_MAX_NDIM];
    int64_t oc, oa, ob;
    int64_t K;
    uint32_t rows;
};

template <typename T> struct DotAcc { using type = T; };
template <> struct DotAcc<int32_t> { using type = uint32_t; };  // wrapping sums
template <> struct DotAcc<int64_t> { using type = uint64_t; };

template <typename T>
__global__ void __launch_bounds__(256) vecdot_rows_kernel(T* __restrict__ c, const T* __restrict__ a,
                                                          const T* __restrict__ b, const DotParams p) {
    using A = typename DotAcc<T>::type;
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < p.rows; w += nw) {
        int64_t oc = p.oc, oa = p.oa, ob = p.ob;
        uint32_t rem = w;
        for (int d = 0; d < p.dims.ndim; ++d) {
            const uint32_t q = d + 1 < p.dims.ndim ? p.dims.div[d].div(rem) : 0;
            const int64_t i = (int64_t)(rem - q * p.dims.shape[d]);
            rem = q;
            oc += i * p.sc[d];
            oa += i * p.sa[d];
            ob += i * p.sb[d];
        }
        const T* x = a + oa;
        const T* y = b + ob;
        A acc[4] = {A(0), A(0), A(0), A(0)};
        for (int64_t k = lane; k < p.K; k += 128) {
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int64_t kk = k + 32 * u;
                if (kk < p.K) acc[u] += (A)x[kk] * (A)y[kk];
            }
        }
        A s = (acc[0] + acc[1]) + (acc[2] + acc[3]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) c[oc] = (T)s;
    }
}

template <typename T>
int launch_vecdot_rows(rstsr_ctx* ctx, const DotParams& p, void* c, const void* a, const void* b) {
    const uint32_t cap = (uint32_t)ctx->num_sms * 64;  // warps
    const uint32_t warps = p.rows < cap ? p.rows : cap;
    vecdot_rows_kernel<T><<<(warps + 7) / 8, 256, 0, ctx->stream>>>(static_cast<T*>(c), static_cast<const T*>(a),
                                                                      static_cast<const T*>(b), p);
    return after_launch(ctx, "vecdot_rows_kernel");
}

}  // namespace

}  // namespace rstsr

using namespace rstsr;

extern "C" {

int rstsr_cuda_einsum_output_shape(const char* subscripts, int32_t nops, const rstsr_layout* lops,
                                   int32_t* ndim_out, int64_t* shape_out) {
    clear_error();
    std::vector<Layout> ls;
    RSTSR_TRY(read_layouts(nops, lops, ls));
    std::vector<std::vector<int>> ins;
    std::vector<int> olab;
    RSTSR_TRY(parse_subscripts(subscripts, nops, ins, olab));
    std::map<int, int64_t> ext;
    RSTSR_TRY(label_extents(ins, ls, ext));
    if ((int)olab.size() > RSTSR_MAX_NDIM) return fail(RSTSR_ERR_INVALID_VALUE, "einsum: output has too many axes");
    if (!ndim_out || !shape_out) return fail(RSTSR_ERR_INVALID_VALUE, "einsum: null output arguments");
    *ndim_out = (int32_t)olab.size();
    for (size_t a = 0; a < olab.size(); ++a) shape_out[a] = ext[olab[a]];
    return RSTSR_OK;
}

int rstsr_cuda_einsum(rstsr_ctx* ctx, rstsr_dtype t, const char* subscripts, int32_t nops, const void* const* ops,
                      const rstsr_layout* lops, void* out, const rstsr_layout* lout, const rstsr_gemm_opts* opts) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    if (!einsum_dtype_ok(t))
        return fail(RSTSR_ERR_INVALID_VALUE, std::string("einsum: unsupported element type ") + dtype_name(t));
    std::vector<Layout> ls;
    RSTSR_TRY(read_layouts(nops, lops, ls));
    RSTSR_TRY(check_layout(lout, "out"));
    if (!ops) return fail(RSTSR_ERR_INVALID_VALUE, "einsum: null operand list");
    std::vector<std::vector<int>> ins;
    std::vector<int> olab;
    RSTSR_TRY(parse_subscripts(subscripts, nops, ins, olab));
    return einsum_impl(ctx, t, ins, olab, nops, ops, ls, out, Layout::from_abi(*lout), opts);
}

int rstsr_cuda_tensordot(rstsr_ctx* ctx, rstsr_dtype t, void* c, const rstsr_layout* lc, const void* a,
                         const rstsr_layout* la, const void* b, const rstsr_layout* lb, const int64_t* axes_a,
                         const int64_t* axes_b, int32_t naxes, const rstsr_gemm_opts* opts) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    if (!einsum_dtype_ok(t))
        return fail(RSTSR_ERR_INVALID_VALUE, std::string("tensordot: unsupported element type ") + dtype_name(t));
    RSTSR_TRY(check_layout(lc, "c"));
    RSTSR_TRY(check_layout(la, "a"));
    RSTSR_TRY(check_layout(lb, "b"));
    if (naxes > 0 && (!axes_a || !axes_b)) return fail(RSTSR_ERR_INVALID_VALUE, "tensordot: null axes");
    std::vector<Layout> ls = {Layout::from_abi(*la), Layout::from_abi(*lb)};
    std::vector<std::vector<int>> ins;
    std::vector<int> olab;
    RSTSR_TRY(tensordot_labels(ls[0].ndim, ls[1].ndim, axes_a, axes_b, naxes, ins, olab));
    const void* ptrs[2] = {a, b};
    return einsum_impl(ctx, t, ins, olab, 2, ptrs, ls, c, Layout::from_abi(*lc), opts);
}

int rstsr_cuda_vecdot(rstsr_ctx* ctx, rstsr_dtype t, void* c, const rstsr_layout* lc, const void* a,
                      const rstsr_layout* la, const void* b, const rstsr_layout* lb, const int64_t* axes_a,
                      const int64_t* axes_b, int32_t naxes, rstsr_order order) {
    clear_error();
    RSTSR_TRY(enter(ctx));
    RSTSR_TRY(check_layout(lc, "c"));
    RSTSR_TRY(check_layout(la, "a"));
    RSTSR_TRY(check_layout(lb, "b"));
    if (!dtype_valid(t) || t == RSTSR_BOOL) return fail(RSTSR_ERR_INVALID_VALUE, "vecdot: unsupported dtype");
    if (naxes < 1 || !axes_a || !axes_b) return fail(RSTSR_ERR_INVALID_VALUE, "vecdot: no contracted axes");
    Layout A = Layout::from_abi(*la), B = Layout::from_abi(*lb), Cl = Layout::from_abi(*lc);
    Layout as, am, bs, bm;
    Error err;
    std::vector<int> norm_a, norm_b;
    if (!split_axes(A, axes_a, naxes, &as, &am, &norm_a, &err) || !split_axes(B, axes_b, naxes, &bs, &bm, &norm_b, &err))
        return fail(err.code, "vecdot: " + err.msg);
    if (!same_shape(as, bs))
        return fail(RSTSR_ERR_INVALID_LAYOUT,
                    "vecdot: the dimensions of a and b along the contracted axes should be the same");
    // remaining parts broadcast to c (broadcast_layout_to_first, cpu_serial/vecdot.rs:37-40)
    Layout cb, amb, bmb;
    if (!broadcast_layouts(Cl, am, order, &cb, &amb, &err) || !same_shape(cb, Cl) ||
        !broadcast_layouts(Cl, bm, order, &cb, &bmb, &err) || !same_shape(cb, Cl))
        return fail(RSTSR_ERR_INVALID_LAYOUT, "vecdot: a and b do not broadcast to c after the axis sum");
    RSTSR_TRY(check_write_layout(Cl, "vecdot"));
    if (Cl.size() == 0) return RSTSR_OK;
    // fused path: the contracted axes merge into one axis of stride 1 in both
    // operands, it is long enough for a warp, and the rows fit 32-bit indexing
    {
        std::vector<int> ax(as.ndim);
        for (int d = 0; d < as.ndim; ++d) ax[d] = d;
        int64_t ka, sa1, kb, sb1;
        const bool fused_type = t == RSTSR_F64 || t == RSTSR_F32 || t == RSTSR_I32 || t == RSTSR_I64;
        if (fused_type && merge_axes(as, ax, &ka, &sa1) && merge_axes(bs, ax, &kb, &sb1) && ka == kb &&
            (sa1 == 1 || ka == 1) && (sb1 == 1 || kb == 1) && ka >= 32 && Cl.size() <= INT32_MAX) {
            const Layout* ls[3] = {&Cl, &amb, &bmb};
            IterSpace sp = make_iter_space(ls, 3);
            DotParams p;
            std::memset(&p, 0, sizeof(p));
            p.dims = make_dev_dims(sp);
            for (int d = 0; d < sp.ndim; ++d) {
                p.sc[d] = sp.stride[0][d];
                p.sa[d] = sp.stride[1][d];
                p.sb[d] = sp.stride[2][d];
            }
            p.oc = sp.offset[0];
            p.oa = sp.offset[1] + (as.offset - A.offset);
            p.ob = sp.offset[2] + (bs.offset - B.offset);
            p.K = ka;
            p.rows = (uint32_t)Cl.size();
            if (!a || !b || !c) return fail(RSTSR_ERR_INVALID_VALUE, "null data pointer");
            switch (t) {
                case RSTSR_F64: return launch_vecdot_rows<double>(ctx, p, c, a, b);
                case RSTSR_F32: return launch_vecdot_rows<float>(ctx, p, c, a, b);
                case RSTSR_I32: return launch_vecdot_rows<int32_t>(ctx, p, c, a, b);
                default: return launch_vecdot_rows<int64_t>(ctx, p, c, a, b);
            }
        }
    }
    // product over [c's axes..., contracted axes...] then the sum over the contracted axes
    Layout P, PA, PB;
    P.ndim = PA.ndim = PB.ndim = Cl.ndim + as.ndim;
    if (P.ndim > RSTSR_MAX_NDIM) return fail(RSTSR_ERR_INVALID_LAYOUT, "vecdot: too many axes");
    std::vector<int64_t> pshape;
    for (int d = 0; d < Cl.ndim; ++d) pshape.push_back(Cl.shape[d]);
    for (int d = 0; d < as.ndim; ++d) pshape.push_back(as.shape[d]);
    P = Layout::c_contig(pshape.data(), (int)pshape.size());
    PA.offset = amb.offset;
    PB.offset = bmb.offset;
    for (int d = 0; d < Cl.ndim; ++d) {
        PA.shape[d] = PB.shape[d] = Cl.shape[d];
        PA.stride[d] = amb.stride[d];
        PB.stride[d] = bmb.stride[d];
    }
    for (int d = 0; d < as.ndim; ++d) {
        PA.shape[Cl.ndim + d] = PB.shape[Cl.ndim + d] = as.shape[d];
        PA.stride[Cl.ndim + d] = as.stride[d];
        PB.stride[Cl.ndim + d] = bs.stride[d];
    }
    PA.offset += as.offset - A.offset;  // split_axes keeps the offset on both parts
    PB.offset += bs.offset - B.offset;
    const int64_t n = std::max<int64_t>(P.size(), 1);
    void* buf = nullptr;
    RSTSR_TRY(scratch_alloc(ctx, (size_t)n * dtype_size(t), &buf));
    rstsr_layout l0 = P.to_abi(), l1 = PA.to_abi(), l2 = PB.to_abi();
    int rc = rstsr_cuda_binary(ctx, RSTSR_OP_MUL, t, buf, &l0, a, &l1, b, &l2);
    if (rc == RSTSR_OK) {
        std::vector<int64_t> axes;
        for (int d = 0; d < as.ndim; ++d) axes.push_back(Cl.ndim + d);
        rc = rstsr_cuda_reduce_axes_into(ctx, RSTSR_RED_SUM, t, buf, &l0, axes.data(), (int32_t)axes.size(), c, lc);
    }
    scratch_free(ctx, buf);
    return rc;
}

}  // extern "C"
