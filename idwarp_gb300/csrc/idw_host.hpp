// Host-side set-up of the surface tree: duplicate merging and the kd-tree
// build.  Runs once per surface definition; the per-warp work is on the GPU.
#pragma once
#include <cstdint>
#include <vector>

namespace idw {

// Merge points within tol (squared distance <= tol^2).  Semantics of
// src/utils/pointReduce.F90:27-77: scanning points in order, the first
// not-yet-linked point opens a new unique point (its own coordinates) and every
// point within tol of it is (re)linked to that id.  link is 1-based.
int point_reduce(const double *pts, int n, double tol, double *uniquePts, int32_t *link);

// Flat kd-tree in preorder.  Node k covers tree-order points [l, u]; its
// subtree occupies preorder ids [k, escape).  Interior nodes have their left
// child at k+1 and their right child at escape(k+1).
struct FlatTree {
    int n = 0;                  // points
    int bucket = 8;
    int maxDepth = 1;
    std::vector<int32_t> perm;  // tree order -> input (lexsorted unique) index
    std::vector<int32_t> l, u, escape, leaf, depth;
    std::vector<double> X;      // 3 per node: unweighted centroid
    std::vector<double> oradius;
    int nodes() const { return int(l.size()); }
};

// Median kd-split on the axis of largest (sampled) spread, exactly as
// build_tree (src/modules/kd_tree.F90:123-300): the spread uses the first
// min(u, l+200) points of the range, the split index is (l+u)/2 and the
// partition is the reference's selection scheme, so the same input gives the
// same tree.  Centroids/radii as setCenters (kd_tree.F90:558-593).
void build_kdtree(const double *pts, int n, int bucket, FlatTree &t);

}  // namespace idw
