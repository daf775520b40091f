// Hierarchical matrices: cluster / block trees, ACA and the H-matrix mat-vec.
#pragma once
#include <memory>

#include "common.cuh"

namespace bem {

struct HMatrixDev;

struct Forest;

void solve_surface_hmatrix(Context& c, const Problem& p, const double2* d_rhs_inc, double2* d_phi, double2* d_vn,
                           bem_solve_report* rep);

// One leaf of a built FP64 H-matrix: rows rows[row_off .. + m), columns
// cols[col_off .. + n) (global indices, in the cluster's order); dense leaves
// store m x n entries at store_off, admissible ones U (m x kmax) then V
// (n x kmax), column-major, of which the first `rank` columns are used.
struct HLeafView {
    int64_t row_off, m, col_off, n, store_off;
    int32_t adm, kmax, rank;
    double norm;
};
struct HBuilt {
    std::shared_ptr<void> keep;  // owns the device data below
    int64_t n = 0;
    double norm = 0;             // h_matrix.rs:189-196 (dense leaves, then low-rank)
    std::vector<HLeafView> leaves;
    std::vector<int64_t> rows, cols;
    const int64_t *d_rows = nullptr, *d_cols = nullptr;
    const double2* d_store = nullptr;
};
// h_matrix.rs:127-148 HMatrix::new_from at the problem's current frequency
// (side 1: lhs factors, 0: rhs factors), leaf size, eta and ACA tolerance
// from the problem.
// tree_cache (may be null): holds the problem's cluster / block trees between
// calls for several frequencies of one body (built on the first call).
HBuilt hmatrix_build_view(Context& c, const Problem& p, int side, std::shared_ptr<void>* tree_cache = nullptr);
// The problem's cluster tree at its H-matrix leaf size (cluster.rs:35-105,
// built on the device), through the same cache as hmatrix_build_view.
std::shared_ptr<const Forest> hmatrix_forest(Context& c, const Problem& p, std::shared_ptr<void>* tree_cache);
// out = H 1 (n entries, device) for the H-matrix of `side`.
void hmatrix_row_sums(Context& c, const Problem& p, int side, double2* out);

}  // namespace bem
