// Cluster trees (cluster.rs:35-105) and block trees (block.rs:38-93) built on
// the device, for one body or for every body of a batch at once.
#pragma once

#include <memory>
#include <vector>

#include "common.cuh"

namespace bem {

// One cluster: its points are perm[begin .. end) of its body.
struct TreeNode {
    int64_t begin, end;
    double lo[3], hi[3];
    double diam;         // diagonal of the bounding box (cluster.rs:84-91)
    int32_t son0, son1;  // -1 for a leaf
    int32_t body, depth;
};

// One leaf of a block tree: clusters r (rows) and c (columns) of one body.
struct BlockLeaf {
    int32_t r, c, adm, body;
};

// The cluster trees of several point sets.  Node b (b < nbodies) is the root
// of body b.  perm lists body b's point indices (local to the body) at
// positions pt0[b] .. pt0[b + 1] - 1 in cluster order: every cluster of the
// body is the range pt0[b] + begin .. pt0[b] + end - 1, and the leaves follow
// one another depth-first.
struct Forest {
    int nbodies = 0;
    int64_t leaf = 0;
    std::vector<int64_t> pt0;
    std::vector<int64_t> perm;
    std::vector<TreeNode> nodes;
    std::vector<int32_t> leaves;     // leaf clusters, depth-first per body, bodies in order
    std::vector<int32_t> leaf0;      // first entry of each body in `leaves`
    DevBuf d_perm;                   // perm on the device (body-local indices)
    int64_t n(int b) const { return pt0[(size_t)b + 1] - pt0[(size_t)b]; }
    const TreeNode& root(int b) const { return nodes[(size_t)b]; }
};

// Builds the trees of `nb` point sets: set b has npts[b] points at
// pts[b][stride * i + 0..2] (host memory).  Leaf clusters hold at most `leaf`
// points.  Throws BEM_ERR_BAD_INPUT where points cannot be separated
// (coincident points) or a tree would exceed 200 levels.
std::shared_ptr<Forest> build_forest(Context& c, int nb, const double* const* pts, const int64_t* npts,
                                     int64_t stride, int64_t leaf);
// The same for the collocation points of several problems (read from their
// device geometry).
std::shared_ptr<Forest> build_forest(Context& c, const std::vector<const Problem*>& bodies, int64_t leaf);
// The block-tree leaves of every body (pairs of its clusters, root with root),
// depth-first per body as block.rs:76-93 flattens them, bodies in order;
// admissible when min(diam) <= eta * dist (block.rs:38-55).
std::vector<BlockLeaf> forest_block_leaves(Context& c, const Forest& F, double eta);

// Host copies of the two box functions the trees use (cluster.rs:84-101),
// with the same operation order as the device.
double node_distance(const TreeNode& a, const TreeNode& b);

}  // namespace bem
