// Host tree builders and the flattening into the device layout.
//
// Both builders produce the same tree as the reference (node boxes, split
// planes, leaf triangle lists in the same order), so that the GPU's
// (distance, DFS leaf position) tie rule picks the triangle the reference's
// depth-first traversal picks:
//   median: KDTree::buildRecursive, src/kd_tree.cpp:48-84 (object split at the
//           centroid median, tight node boxes, children may overlap)
//   sah:    KDTreeSAH::buildRecursive, src/kd_tree_sah.cpp:92-138 (event sweep,
//           voxel node boxes, straddling triangles referenced on both sides)
#pragma once

#include <cstdint>
#include <vector>

#include "geom.h"

namespace pray_gpu {

enum TreeKind : int { kTreeMedian = 0, kTreeSah = 1 };

struct TreeOptions {
    int kind = kTreeMedian;
    int leaf_size = 32;   // leaf when a node has at most this many triangles
    int max_depth = 20;   // leaf at this depth
    float sah_ct = 5.f;   // SAH traversal cost
    float sah_ci = 1.5f;  // SAH intersection cost
    int threads = 0;      // 0: hardware concurrency
};

// One node in depth-first pre-order (left subtree before right).
struct FlatNode {
    Aabb box{};
    int32_t left = -1, right = -1;  // pre-order indices of the children, -1 for a leaf
    int32_t axis = 255;
    float split = 0.f;
    uint32_t first = 0, count = 0;  // leaf triangle references [first, first+count)
};

struct BuiltTree {
    std::vector<FlatNode> nodes;  // pre-order; nodes[0] is the root
    std::vector<uint32_t> refs;   // triangle indices, leaves concatenated in DFS order
    // KDTree statistics as the reference logs them (include/kd_tree.h:122-132)
    uint64_t maxdepth = 0, leaf_nodes = 0, empty_leaves = 0;
};

std::vector<TriPre> precompute_triangles(const float *verts, uint64_t n, int threads);

BuiltTree build_tree(const std::vector<TriPre> &tris, const TreeOptions &opt);

}  // namespace pray_gpu
