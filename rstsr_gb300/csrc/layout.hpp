// Host-side layout algebra of the CUDA device backend.
//
// A restatement, in C++, of the parts of rstsr-common's layout module that a
// device implementation needs to plan a launch and to produce output layouts
// that are identical to the CPU devices':
//   rstsr-common/src/layout/layoutbase.rs   (Layout, contiguity tests, bounds)
//   rstsr-common/src/layout/rearrangement.rs (greedy_layout, layout_for_array_copy,
//                                             translate_to_col_major*, axes composition,
//                                             get_layout_for_binary_op)
//   rstsr-common/src/layout/broadcast.rs    (broadcast_layout)
//   rstsr-common/src/layout/indexer.rs:453  (dim_split_axes)
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "rstsr_cuda.h"

namespace rstsr {

struct Error {
    int code;
    std::string msg;
};

// Error reporting across the C ABI: a thread-local message and a status code.
void set_error(const std::string& msg);
void clear_error();
int fail(int code, const std::string& msg);

// Layout<IxD> with shape/stride/offset in elements.
struct Layout {
    int ndim = 0;
    int64_t offset = 0;
    int64_t shape[RSTSR_MAX_NDIM] = {0};
    int64_t stride[RSTSR_MAX_NDIM] = {0};

    static Layout from_abi(const rstsr_layout& l);
    rstsr_layout to_abi() const;
    static Layout c_contig(const int64_t* shp, int n, int64_t offset = 0);
    static Layout f_contig(const int64_t* shp, int n, int64_t offset = 0);

    int64_t size() const;
    bool c_contig() const { return ndim == ndim_of_c_contig(); }
    bool f_contig() const { return ndim == ndim_of_f_contig(); }
    int ndim_of_f_contig() const;  // layoutbase.rs:152
    int ndim_of_c_contig() const;  // layoutbase.rs:172
    bool f_prefer() const;         // layoutbase.rs:89
    bool c_prefer() const;         // layoutbase.rs:119
    int64_t size_non_broadcast() const;  // broadcast.rs:255
    // [min, max) element bounds (layoutbase.rs:237); false if min < 0.
    bool bounds_index(int64_t* lo, int64_t* hi) const;
    // No two multi-indices map to the same element (layoutbase.rs:285).
    bool check_strides(bool skip_zero) const;
    Layout transpose(const int* axes) const;  // layoutbase.rs:443
    Layout reverse_axes() const;              // layoutbase.rs:476
    // Reverse the direction of axis n (dim_narrow(n, ::-1), indexer.rs:126).
    Layout flip_axis(int n) const;
    bool same_as(const Layout& o) const;      // PartialEq, layoutbase.rs:553
    std::string repr() const;
};

// greedy_layout (rearrangement.rs:36-113). perm receives the transpose index.
Layout greedy_layout(const Layout& l, bool keep_shape, int* perm);
// layout_for_array_copy with TensorIterOrder K (rearrangement.rs:125-152).
Layout layout_for_array_copy_k(const Layout& l);
Layout layout_for_array_copy(const Layout& l, char order /* 'C','F','K' */);
// get_axes_composition (rearrangement.rs:335-372).
void axes_composition(const Layout& l, std::vector<int>& c1, std::vector<int>& c0,
                      std::vector<int>& cc, std::vector<int>& cd);
// get_layout_for_binary_op (rearrangement.rs:394-459).
bool layout_for_binary_op(const Layout& la, const Layout& lb, rstsr_order order, Layout* out,
                          Error* err);
// normalize_axes_index + dim_split_axes (indexer.rs:453-475).
bool split_axes(const Layout& l, const int64_t* axes, int naxes, Layout* ls, Layout* lm,
                std::vector<int>* axes_norm, Error* err);
// broadcast_layout, row-major (broadcast.rs:166-245).
bool broadcast_layouts(const Layout& a, const Layout& b, rstsr_order order, Layout* oa,
                       Layout* ob, Error* err);

// Matmul layout rules (rstsr-common/src/layout/matmul.rs:70-460): output
// layout for operands la, lb in the given order.
bool matmul_output_layout(const Layout& la, const Layout& lb, rstsr_order order, Layout* lc, Error* err);

size_t dtype_size(rstsr_dtype t);
bool dtype_valid(int t);
const char* dtype_name(rstsr_dtype t);

}  // namespace rstsr
