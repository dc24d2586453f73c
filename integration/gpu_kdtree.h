// Reference-side binding: the spatial database of the reference
// (class SpatialDatabase, include/spatial.h:10-39 of nicmue/nostrum_pray)
// answered by this library's GPU kd tree.
//
// This file is meant to be compiled inside the reference's source tree, with
// the reference's include/ directory and this repository's include/ on the
// include path, and linked with nostrum_pray_gb300/_build/libnostrum_pray.so.
// It uses only the reference's public types (Triangle, Ray, Vec3) and the
// C ABI of include/nostrum_pray.h.
//
// build() takes the triangles exactly as the reference's KDTree::build does
// (include/kd_tree.h: the tree owns them afterwards; `scene.triangles` is
// moved in by preprocessScene, src/scene_preprocessor.cpp:60) and builds the
// same median or SAH tree on the GPU that the reference would build on the
// host (the choice by triangle count of src/scene_preprocessor.cpp:52-57).
// intersect() returns the same triangle and distance as KDTree::intersect
// (src/kd_tree.cpp:142-279), ties included. It may be called from many
// OpenMP threads at once, as the reference's renderers do: the library
// serialises calls on one scene. A GPU call per ray is slow; renderers that
// can collect rays should use intersectBatch, or hand the whole frame to
// pray_render_rt_host / pray_render_pt_host (see renderOnGpu in
// gpu_kdtree.cpp).
#pragma once

#include <cstdint>
#include <vector>

#include "nostrum_pray.h"
#include "pray.h"
#include "spatial.h"

namespace pray {

class GpuKDTree : public SpatialDatabase {
  public:
    // det_epsilon: the one-sided Moeller-Trumbore threshold; the reference
    // compiles it in as EPSILON (include/geometry.h:12).
    explicit GpuKDTree(int32_t device = 0, float det_epsilon = EPSILON);
    // Frees the GPU scene. The reference's SpatialDatabase declares no
    // virtual destructor (include/spatial.h:10-39), so a GpuKDTree deleted
    // through scene.triangleDB (a std::unique_ptr<SpatialDatabase>) only runs
    // this when the reference adds `virtual ~SpatialDatabase() = default;`.
    ~GpuKDTree();
    GpuKDTree(const GpuKDTree &) = delete;
    GpuKDTree &operator=(const GpuKDTree &) = delete;

    void build(const std::vector<Triangle> &triangles) override;
    void build(std::vector<Triangle> &&triangles) override;

    bool intersect(const Ray &ray, Triangle &triangle, float &dist) const override;

    // Closest hits of many rays in one GPU call: ids[i] is the index of the
    // hit triangle in triangles() or -1, dists[i] its distance (FLT_MAX on a
    // miss).
    void intersectBatch(const std::vector<Ray> &rays, std::vector<int32_t> &ids, std::vector<float> &dists) const;

#if defined(ENABLE_AVX)
    __m256 intersect(const __m256 &rayPosX, const __m256 &rayPosY, const __m256 &rayPosZ, const __m256 &rayDirX,
                     const __m256 &rayDirY, const __m256 &rayDirZ, const __m256 &rayMask,
                     std::array<Triangle, 8> &trs, __m256 &distance) const override;
#elif defined(ENABLE_SSE)
    __m128 intersect(const __m128 &rayPosX, const __m128 &rayPosY, const __m128 &rayPosZ, const __m128 &rayDirX,
                     const __m128 &rayDirY, const __m128 &rayDirZ, const __m128 &rayMask, std::vector<Triangle> &trs,
                     __m128 &distance) const override;
#endif

    bool isEmpty() const override { return triangles_.empty(); }
    size_t size() const override { return triangles_.size(); }

    const std::vector<Triangle> &triangles() const { return triangles_; }
    pray_scene *handle() const { return scene_; }

  private:
    // Closest hits of n rays packed as 9 floats each (position, direction,
    // inverse direction); throws std::runtime_error with pray_last_error().
    void trace(const float *rays9, uint64_t n, int32_t *ids, float *dists) const;
    // Lanes of a SIMD packet as rays (the inverse direction computed as the
    // reference's Ray constructor does, include/geometry.h:84-87).
    void tracePacket(const float *px, const float *py, const float *pz, const float *dx, const float *dy,
                     const float *dz, int lanes, int mask, int32_t *ids, float *dists) const;

    int32_t device_;
    float eps_;
    pray_scene *scene_ = nullptr;
    std::vector<Triangle> triangles_;
};

// The whole frame of `scene` on the GPU, for render() (src/pray.cpp:617-637):
// ray tracing through pray_render_rt_host, path tracing through
// pray_render_pt_host (Kajiya mode for max_depth > 1, the branching mode
// otherwise, as preprocessScene chooses, src/scene_preprocessor.cpp:34-40).
// scene.triangleDB must be a GpuKDTree. image: 3 x width x height bytes.
void renderOnGpu(Image &image, const Scene &scene, uint64_t seed = 0);

}  // namespace pray
