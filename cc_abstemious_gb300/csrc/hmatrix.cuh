// Hierarchical matrices: cluster / block trees, ACA and the H-matrix mat-vec.
#pragma once
#include "common.cuh"

namespace bem {

struct HMatrixDev;

// Leaves of the cluster tree of cluster.rs:35-105 (bounding-box bisection).
struct LeafCluster {
    std::vector<int64_t> idx;
    double lo[3], hi[3], diam;
};
std::vector<LeafCluster> cluster_leaves(const std::vector<double>& pts, int64_t stride, int64_t leaf);
double box_distance(const LeafCluster& a, const LeafCluster& b);

void solve_surface_hmatrix(Context& c, const Problem& p, const double2* d_rhs_inc, double2* d_phi, double2* d_vn,
                           bem_solve_report* rep);

}  // namespace bem
