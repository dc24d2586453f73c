// Device-resident scene layout (shared by the host flattener and the kernels).
//
// Nodes: 32-byte records, the two children of an interior node stored side by
// side (one 64-byte, 64-byte-aligned pair), so one visit fetches both child
// boxes and tests them before descending (root at index 0, slot 1 unused).
//   interior: a = index of the first child of its pair, b = 0
//   leaf:     a = first triangle reference, b = kLeafFlag | reference count
// Every node keeps its own box (tight triangle bounds for the median tree,
// the voxel for the SAH tree) so the kernels apply the reference's slab test
// to exactly the boxes the reference tests.
//
// Triangle references: 48 bytes each, one per leaf entry, in depth-first leaf
// order (a triangle referenced by two SAH leaves is stored twice). The
// position of a reference in this array is the reference's depth-first visit
// order, which breaks distance ties.
//   v0 = (a.xyz, triangle id as bits), e1 = (b - a, 0), e2 = (c - a, 0)
// Shading records: per triangle id, normal (w: 1 for emitters) and colour.
#pragma once

#include <cstdint>

#include <vector_types.h>

namespace pray_gpu {

constexpr uint32_t kLeafFlag = 0x80000000u;
constexpr int kMaxTreeDepth = 30;        // deepest reference tree the API accepts
constexpr int kMaxTraversalDepth = 62;   // deepest device hierarchy (reference tree + leaf refinement)

struct alignas(16) GNode {
    float lo[3];
    uint32_t a;
    float hi[3];
    uint32_t b;
};
static_assert(sizeof(GNode) == 32, "GNode must be 32 bytes");

struct alignas(16) GTri {
    float v0[4];
    float e1[4];
    float e2[4];
};
static_assert(sizeof(GTri) == 48, "GTri must be 48 bytes");

struct alignas(16) GShade {
    float n[4];
    float c[4];
};

// Split records of the culling copy (8 bytes per node, same slots as the
// GNode copy), for the warp-packet walk over SAH voxel trees. Where a node's
// children are exactly its voxel cut by one axis-aligned plane, a visit needs
// only that plane: each lane clips its own entry/exit interval at the plane's
// distance instead of testing two boxes.
//   split node:   x = split position (float bits), y = axis << 30 | index of the children's pair
//   linear leaf:  x = first triangle reference,    y = 3 << 30 | reference count
//   box node:     x = index of the children's pair (their boxes in the GNode copy), y = 3 << 30 | 1 << 29
constexpr uint32_t kKindBox = 3u << 30;
constexpr uint32_t kKindBoxInterior = 1u << 29;
constexpr uint32_t kKdCountMask = kKindBoxInterior - 1u;

// Launch-time view of a device scene.
struct DevScene {
    const GNode *nodes;  // n_nodes nodes with the reference's boxes and linear leaves, then the culling
                         // copy (same topology, refined leaves, interior boxes bounding their triangles;
                         // for finite-direction rays whose origin is within cull_r2 of cull_c)
    const GTri *tris;
    const GShade *shade;
    uint32_t n_nodes, n_refs, n_tris;
    float tol;  // absolute distance tolerance for culling boxes behind the origin
    uint32_t depth;  // deepest node level of the hierarchy (root 0): a traversal pushes at most this many nodes
    float cull_c[3], cull_r2;  // centre and squared radius of the region of origins served by the culling copy
    // emitting triangles (for next-event estimation): geometry as GTri (v0.w
    // = triangle id) and the inclusive prefix sums of their areas
    const GTri *emit_tris;
    const float *emit_cdf;
    uint32_t n_emit;
    float emit_area;
    // split records of the culling copy (n_nodes of them), or NULL where the
    // tree has no split nodes (median trees); kd_pad = 2^-16 of the scene's
    // diagonal, the absolute part of a split plane's padding
    const uint2 *knodes;
    float kd_pad;
};

}  // namespace pray_gpu
