// Flattening of a built tree into the device layout (device_layout.h).
//
// The reference's tree is copied node for node: its boxes are tested on the
// GPU with the reference's slab arithmetic, so the GPU visits exactly the
// leaves the reference's depth-first traversal would reach. Each triangle
// record keeps its depth-first position in the reference's leaf order as the
// tie-break key, so a leaf returns the same triangle as the reference's linear
// scan in whatever order its records are stored.
//
// Two copies of the nodes share one topology. The exact copy (nodes) keeps
// every box of the reference and scans every leaf linearly. The culling copy
// (nodes_tight) is for rays whose inverse direction is finite and whose
// origin lies within cull_radius2 of cull_center:
// - Large leaves (more than `leaf_refine` references) are refined into a small
//   bounding-volume hierarchy over their own triangles, whose boxes are the
//   triangles' bounds padded by a relative 2^-16 and by 2^-16 of the scene's
//   diagonal: a ray skips a sub-box only if it cannot come within that pad of
//   any triangle inside, and for such origins the pad exceeds the float error
//   of the slab test and the distance by which a hit that the one-sided
//   Moeller-Trumbore test reports can lie off its triangle (up to grazing
//   angles; flatten.cpp gives the bounds), so those triangles are still
//   tested.
// - An interior node of the reference's tree carries the padded bounds of the
//   triangles below it instead of the reference's box (for the SAH tree, a
//   voxel with much empty space) wherever those bounds have the smaller surface
//   area. For finite inverse directions the reference's slab test is monotone
//   in the box (a box inside another gives an interval inside the other's),
//   and the reference's boxes are nested, so the reference reaches a leaf
//   exactly when the leaf's own box passes; an interior box then only needs to
//   keep every triangle the ray can hit, which either the reference's box or
//   the padded triangle bounds do. Leaves keep the reference's box.
// Rays with an infinite inverse component (NaN cases of the reference's test)
// or a distant origin use the exact copy.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../device_layout.h"
#include "geom.h"
#include "kdtree.h"

namespace pray_gpu {

struct DeviceImage {
    std::vector<GNode> nodes;        // reference boxes (exact slab decisions), linear leaves
    std::vector<GNode> nodes_tight;  // culling copy: refined leaves, interior nodes bounding their triangles
    float cull_center[3] = {0.f, 0.f, 0.f};
    float cull_radius2 = -1.f;  // origins within sqrt of this of cull_center may use nodes_tight
    std::vector<GTri> tris;
    uint64_t refined_leaves = 0;  // reference leaves split into a sub-hierarchy
    uint64_t sub_nodes = 0;       // nodes added by the refinement
};

// leaf_refine <= 0 keeps every reference leaf as one linear leaf.
void flatten_for_device(const BuiltTree &t, const std::vector<TriPre> &pre, int leaf_refine, DeviceImage &out);

// Structural check of both copies before upload: child pairs and leaf ranges
// in bounds, each node reached once, every triangle reference reached once,
// depth within the kernels' traversal stack (the deepest node's depth goes to
// *max_depth when given).
bool validate_device_image(const DeviceImage &img, std::string &why, int *max_depth = nullptr);

}  // namespace pray_gpu
