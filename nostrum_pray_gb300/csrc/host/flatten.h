// Flattening of a built tree into the device layout (device_layout.h).
//
// The reference's tree is copied node for node: its boxes are tested on the
// GPU with the reference's slab arithmetic, so the GPU visits exactly the
// leaves the reference's depth-first traversal would reach. Large leaves of
// that tree (more than `leaf_refine` references) are then refined into a small
// bounding-volume hierarchy over their own triangles, whose boxes are the
// triangles' bounds padded by a relative 2^-16: a ray skips a sub-box only if
// it cannot come within that pad of any triangle inside, so every triangle the
// one-sided Moeller-Trumbore test could report as hit is still tested. Each
// triangle record keeps its depth-first position in the reference's leaf order
// as the tie-break key, so the refined leaves return the same triangle as a
// linear scan in the reference's order.
//
// A second copy of the nodes (nodes_tight) has the same topology, but an
// interior node of the reference's tree carries the padded bounds of the
// triangles below it instead of the reference's box (for the SAH tree, a
// voxel with much empty space) wherever those bounds have the smaller surface
// area. Leaves keep the reference's box. It is used
// for rays whose inverse direction is finite: for them the reference's slab
// test is monotone in the box (a box inside another gives an interval inside
// the other's), and the reference's boxes are nested, so the reference
// reaches a leaf exactly when the leaf's own box passes; an interior box then
// only needs to keep every triangle the ray can hit, which either the
// reference's box or the padded triangle bounds do. Rays with an infinite
// inverse component (NaN cases of the reference's test) use the exact copy.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../device_layout.h"
#include "geom.h"
#include "kdtree.h"

namespace pray_gpu {

struct DeviceImage {
    std::vector<GNode> nodes;        // reference boxes (exact slab decisions)
    std::vector<GNode> nodes_tight;  // same topology; interior reference nodes bound their triangles (padded)
    std::vector<GTri> tris;
    uint64_t refined_leaves = 0;  // reference leaves split into a sub-hierarchy
    uint64_t sub_nodes = 0;       // nodes added by the refinement
};

// leaf_refine <= 0 keeps every reference leaf as one linear leaf.
void flatten_for_device(const BuiltTree &t, const std::vector<TriPre> &pre, int leaf_refine, DeviceImage &out);

// Structural check before upload: child pairs and leaf ranges in bounds, each
// node reached once, depth within the kernels' traversal stack (the deepest
// node's depth goes to *max_depth when given).
bool validate_device_image(const DeviceImage &img, std::string &why, int *max_depth = nullptr);

}  // namespace pray_gpu
