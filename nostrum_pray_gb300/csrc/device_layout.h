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

namespace pray_gpu {

constexpr uint32_t kLeafFlag = 0x80000000u;
constexpr int kMaxTreeDepth = 30;        // deepest reference tree the API accepts
constexpr int kMaxTraversalDepth = 62;   // deepest device hierarchy (reference tree + leaf refinement)

struct alignas(32) GNode {  // 32-byte aligned: one 256-bit load per node (traverse.cuh ldg_node)
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
};

}  // namespace pray_gpu
