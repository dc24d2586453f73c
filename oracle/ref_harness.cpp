// Oracle support (test infrastructure only): a thin extern "C" harness around the
// reference's own scene preprocessing, KD-tree builders, scalar intersector and
// ray-tracing renderer, compiled from the reference's sources by build_ref.sh.
// It is used in the development container to pin the CPU restatement in
// pray_oracle.cpp and to write the golden fixtures under tests/golden/.
// Nothing in the product links or loads it.
//
// Reference entry points reached from here:
//   initialiseTriangles          src/scene_preprocessor.cpp:74-96
//   calculatePrimRays            src/scene_preprocessor.cpp:98-136
//   KDTree::build / buildRecursive        src/kd_tree.cpp:18-84
//   KDTreeSAH::build / buildRecursive     src/kd_tree_sah.cpp:25-138
//   KDTree::intersectRecursive   src/kd_tree.cpp:237-279 (private; reached with
//                                an access override below)
//   render / rayTrace            src/pray.cpp:380-637
//   buildGPUTreeFromKDTree       src/gpu_util.cpp:7-57 (device layout of the
//                                reference's GPU path tracer)
//   evaluatePathRecursive        src/pray.cpp:342-364 (Kajiya path tracer)
//   evaluatePathRecursiveDiffuse src/pray.cpp:315-340 (branching path tracer)
//   readSceneDescription         src/io.cpp:27-137
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <experimental/filesystem>
#include <fstream>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <random>
#include <string>
#include <vector>

#define private public
#define protected public
#include "pray.h"
#include "kd_tree.h"
#include "kd_tree_sah.h"
#include "scene_preprocessor.h"
#include "io.h"
#include "gpu_util.h"
#undef private
#undef protected

using namespace pray;

// Defined in src/pray.cpp with external linkage but not declared in its headers.
namespace pray {
Vec3 evaluatePathRecursive(const Ray &ray, const Scene &scene, size_t depth);
Vec3 evaluatePathRecursiveDiffuse(const Ray &ray, const Scene &scene, size_t depth);
}  // namespace pray

namespace {

struct Handle {
    Scene scene;
    bool prepared = false;
};

void dfs_dump(const KDTreeElement *n, std::vector<const KDTreeElement *> &order) {
    order.push_back(n);
    if (n->left) dfs_dump(n->left.get(), order);
    if (n->right) dfs_dump(n->right.get(), order);
}

const KDTree &tree_of(Handle *h) { return dynamic_cast<const KDTree &>(*h->scene.triangleDB); }

void silence_begin(std::streambuf *&saved) {
    saved = std::cout.rdbuf();
    static std::ofstream null_sink("/dev/null");
    std::cout.rdbuf(null_sink.rdbuf());
}
void silence_end(std::streambuf *saved) { std::cout.rdbuf(saved); }

}  // namespace

extern "C" {

// Constants this variant was compiled with: leaf threshold, max depth,
// SAH traversal cost, SAH intersection cost, det epsilon.
void ref_constants(double *out) {
    struct Probe : KDTreeSAH {
        float ct() const { return traversalCost; }
        float ci() const { return triangleIntersectionCost; }
    } p;
    out[0] = (double)KDTree::THRESHOLD;
    out[1] = (double)KDTree::MAX_DEPTH;
    out[2] = p.ct();
    out[3] = p.ci();
    out[4] = pray::EPSILON;
}

void *ref_scene_from_tris(const float *verts, const float *colors, const uint8_t *emit, size_t n) {
    auto *h = new Handle();
    h->scene.triangles.reserve(n);
    for (size_t i = 0; i < n; i++) {
        const float *v = verts + 9 * i;
        h->scene.triangles.push_back(Triangle(Vec3(v[0], v[1], v[2]), Vec3(v[3], v[4], v[5]),
                                              Vec3(v[6], v[7], v[8]),
                                              Vec3(colors[3 * i], colors[3 * i + 1], colors[3 * i + 2]),
                                              emit ? emit[i] != 0 : false));
    }
    return h;
}

void *ref_scene_from_json(const char *path) {
    auto *h = new Handle();
    std::streambuf *saved;
    silence_begin(saved);
    readSceneDescription(std::experimental::filesystem::path(path), h->scene);
    silence_end(saved);
    return h;
}

// width, height, fov, mode, maxDepth, numSamples, cam_pos[3], cam_look[3], bg[3],
// n_lights, n_triangles
void ref_scene_info(void *vh, double *out) {
    auto *h = static_cast<Handle *>(vh);
    const Scene &s = h->scene;
    out[0] = (double)s.width;
    out[1] = (double)s.height;
    out[2] = (double)s.field_of_view;
    out[3] = (double)s.mode;
    out[4] = (double)s.maxDepth;
    out[5] = (double)s.numSamples;
    out[6] = s.camera_position.x;
    out[7] = s.camera_position.y;
    out[8] = s.camera_position.z;
    out[9] = s.camera_look.x;
    out[10] = s.camera_look.y;
    out[11] = s.camera_look.z;
    out[12] = s.backgroundColor.x;
    out[13] = s.backgroundColor.y;
    out[14] = s.backgroundColor.z;
    out[15] = (double)s.lights.size();
    out[16] = (double)(h->prepared ? h->scene.triangleDB->size() : s.triangles.size());
}

void ref_scene_get(void *vh, float *verts, float *colors, uint8_t *emit, float *lights) {
    auto *h = static_cast<Handle *>(vh);
    const std::vector<Triangle> &tris = h->prepared ? tree_of(h).triangles : h->scene.triangles;
    for (size_t i = 0; i < tris.size(); i++) {
        const Triangle &t = tris[i];
        float *v = verts + 9 * i;
        v[0] = t.a.x; v[1] = t.a.y; v[2] = t.a.z;
        v[3] = t.b.x; v[4] = t.b.y; v[5] = t.b.z;
        v[6] = t.c.x; v[7] = t.c.y; v[8] = t.c.z;
        colors[3 * i] = t.color.x; colors[3 * i + 1] = t.color.y; colors[3 * i + 2] = t.color.z;
        emit[i] = t.isEmitting ? 1 : 0;
    }
    for (size_t i = 0; i < h->scene.lights.size(); i++) {
        const LightSource &l = h->scene.lights[i];
        float *o = lights + 6 * i;
        o[0] = l.position.x; o[1] = l.position.y; o[2] = l.position.z;
        o[3] = l.color.x; o[4] = l.color.y; o[5] = l.color.z;
    }
}

// Per-triangle precompute of initialiseTriangles, read back:
// bbox min[3], bbox max[3], midpoint[3], ab[3], ac[3], normal[3] (18 floats/tri).
void ref_triangle_precompute(void *vh, float *out) {
    auto *h = static_cast<Handle *>(vh);
    const std::vector<Triangle> &tris = tree_of(h).triangles;
    for (size_t i = 0; i < tris.size(); i++) {
        const Triangle &t = tris[i];
        float *o = out + 18 * i;
        const Vec3 *vs[6] = {&t.boundingBox.min, &t.boundingBox.max, &t.midPoint, &t.ab, &t.ac, &t.normal};
        for (int k = 0; k < 6; k++) {
            o[3 * k] = vs[k]->x; o[3 * k + 1] = vs[k]->y; o[3 * k + 2] = vs[k]->z;
        }
    }
}

// initialiseTriangles + tree build (sah != 0: KDTreeSAH, else the median KDTree).
void ref_scene_prepare(void *vh, int sah) {
    auto *h = static_cast<Handle *>(vh);
    std::streambuf *saved;
    silence_begin(saved);
    initialiseTriangles(h->scene);
    if (sah)
        h->scene.triangleDB = std::make_unique<KDTreeSAH>();
    else
        h->scene.triangleDB = std::make_unique<KDTree>();
    h->scene.triangleDB->build(std::move(h->scene.triangles));
    silence_end(saved);
    h->prepared = true;
}

void ref_scene_free(void *vh) { delete static_cast<Handle *>(vh); }

// nnodes, maxdepth, leafNodes, emptyLeafNodes, total leaf references
void ref_tree_stats(void *vh, uint64_t *out) {
    auto *h = static_cast<Handle *>(vh);
    const KDTree &t = tree_of(h);
    std::vector<const KDTreeElement *> order;
    dfs_dump(t.root.get(), order);
    uint64_t refs = 0;
    for (auto *n : order) refs += n->triangleIndices.size();
    out[0] = order.size();
    out[1] = t.maxdepth;
    out[2] = t.leafNodes;
    out[3] = t.emptyLeafNodes;
    out[4] = refs;
}

// DFS pre-order (left before right) dump: per node box[6], split distance,
// info[4] = {is_leaf, split axis, n_tris, first ref}; refs = leaf triangle
// indices concatenated in DFS order.
void ref_tree_dump(void *vh, float *boxes, float *split, int32_t *info, int64_t *refs) {
    auto *h = static_cast<Handle *>(vh);
    const KDTree &t = tree_of(h);
    std::vector<const KDTreeElement *> order;
    dfs_dump(t.root.get(), order);
    int64_t r = 0;
    for (size_t i = 0; i < order.size(); i++) {
        const KDTreeElement *n = order[i];
        float *b = boxes + 6 * i;
        b[0] = n->boundingBox.min.x; b[1] = n->boundingBox.min.y; b[2] = n->boundingBox.min.z;
        b[3] = n->boundingBox.max.x; b[4] = n->boundingBox.max.y; b[5] = n->boundingBox.max.z;
        split[i] = n->splitPlane.distance;
        int32_t *o = info + 4 * i;
        o[0] = n->isLeaf() ? 1 : 0;
        o[1] = n->splitPlane.axis;
        o[2] = (int32_t)n->triangleIndices.size();
        o[3] = (int32_t)r;
        for (size_t k = 0; k < n->triangleIndices.size(); k++) refs[r++] = (int64_t)n->triangleIndices[k];
    }
}

// Primary rays of calculatePrimRays: per pixel position[3], direction[3], inverse[3].
void ref_primary_rays(uint64_t width, uint64_t height, uint64_t fov, const float *cam_pos,
                      const float *cam_look, float *out) {
    Scene s;
    s.width = width;
    s.height = height;
    s.field_of_view = fov;
    s.camera_position = Vec3(cam_pos[0], cam_pos[1], cam_pos[2]);
    s.camera_look = Vec3(cam_look[0], cam_look[1], cam_look[2]);
    calculatePrimRays(s);
    for (size_t i = 0; i < s.primRays.size(); i++) {
        const Ray &r = s.primRays[i];
        float *o = out + 9 * i;
        o[0] = r.position.x; o[1] = r.position.y; o[2] = r.position.z;
        o[3] = r.direction.x; o[4] = r.direction.y; o[5] = r.direction.z;
        o[6] = r.inverseDirection.x; o[7] = r.inverseDirection.y; o[8] = r.inverseDirection.z;
    }
}

// Closest hit per ray through the reference's scalar recursive traversal.
// rays: position[3], direction[3], inverse direction[3] (taken as given).
// ids: triangle index or -1; ts: distance (FLT_MAX on a miss).
void ref_trace(void *vh, const float *rays, size_t n, int64_t *ids, float *ts) {
    auto *h = static_cast<Handle *>(vh);
    const KDTree &t = tree_of(h);
#pragma omp parallel for schedule(dynamic, 1024)
    for (size_t i = 0; i < n; i++) {
        const float *r = rays + 9 * i;
        Ray ray;
        ray.position = Vec3(r[0], r[1], r[2]);
        ray.direction = Vec3(r[3], r[4], r[5]);
        ray.inverseDirection = Vec3(r[6], r[7], r[8]);
        size_t idx = 0;
        float dist = std::numeric_limits<float>::max();
        bool hit = !t.triangles.empty() && t.intersectRecursive(t.root, ray, idx, dist);
        ids[i] = hit ? (int64_t)idx : -1;
        ts[i] = dist;
    }
}

// The reference ray-tracing renderer (scalar build) on the prepared scene.
// lights: n_lights x (position[3], color[3]). Writes width*height*3 bytes.
void ref_render_rt(void *vh, uint64_t width, uint64_t height, uint64_t fov, const float *cam_pos,
                   const float *cam_look, const float *lights, int n_lights, const float *bg,
                   uint8_t *out) {
    auto *h = static_cast<Handle *>(vh);
    Scene &s = h->scene;
    s.mode = Mode::RAYTRACING;
    s.width = width;
    s.height = height;
    s.field_of_view = fov;
    s.camera_position = Vec3(cam_pos[0], cam_pos[1], cam_pos[2]);
    s.camera_look = Vec3(cam_look[0], cam_look[1], cam_look[2]);
    s.backgroundColor = Vec3(bg[0], bg[1], bg[2]);
    s.lights.clear();
    for (int i = 0; i < n_lights; i++) {
        const float *l = lights + 6 * i;
        s.lights.push_back(LightSource(Vec3(l[0], l[1], l[2]), Vec3(l[3], l[4], l[5])));
    }
    calculatePrimRays(s);
    Image image(3 * width * height);
    render(image, s);
    std::memcpy(out, image.data(), image.size());
}

// Per-pixel moments of the reference's own path-tracing estimators on the
// prepared scene: for every pixel, `runs` independent calls of
// evaluatePathRecursive (diffuse == 0; src/pray.cpp:342-364, one Kajiya path
// with max_depth bounces) or evaluatePathRecursiveDiffuse (diffuse != 0;
// src/pray.cpp:315-340, a branching tree with `branching` rays per hit) on the
// pixel's primary ray, unclamped. sum and sumsq (width*height*3 doubles each)
// receive the sums of the values and of their squares. The reference seeds a
// fresh mt19937_64 from the system clock inside every call
// (src/pray.cpp:331,357), so these are samples of its estimator, not a
// reproducible stream.
void ref_path_moments(void *vh, uint64_t width, uint64_t height, uint64_t fov, const float *cam_pos,
                      const float *cam_look, const float *bg, uint64_t max_depth, uint64_t branching,
                      int diffuse, uint64_t runs, double *sum, double *sumsq) {
    auto *h = static_cast<Handle *>(vh);
    Scene &s = h->scene;
    s.mode = Mode::PATHTRACING;
    s.ptMode = diffuse ? PtMode::DIFFUSE : PtMode::NORMAL;
    s.maxDepth = max_depth;
    s.numSamples = branching;
    s.width = width;
    s.height = height;
    s.field_of_view = fov;
    s.camera_position = Vec3(cam_pos[0], cam_pos[1], cam_pos[2]);
    s.camera_look = Vec3(cam_look[0], cam_look[1], cam_look[2]);
    s.backgroundColor = Vec3(bg[0], bg[1], bg[2]);
    calculatePrimRays(s);
    const int64_t n = (int64_t)(width * height);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < n; i++) {
        double a[3] = {0, 0, 0}, q[3] = {0, 0, 0};
        for (uint64_t k = 0; k < runs; k++) {
            const Vec3 v = diffuse ? evaluatePathRecursiveDiffuse(s.primRays[i], s, 0)
                                   : evaluatePathRecursive(s.primRays[i], s, 0);
            const double c[3] = {v.x, v.y, v.z};
            for (int j = 0; j < 3; j++) {
                a[j] += c[j];
                q[j] += c[j] * c[j];
            }
        }
        for (int j = 0; j < 3; j++) {
            sum[3 * i + j] = a[j];
            sumsq[3 * i + j] = q[j];
        }
    }
}

// The breadth-first device tree of the reference's GPU path tracer
// (buildGPUTreeFromKDTree) over the prepared median tree, field by field:
// per node left, right (int32), is_leaf (uint8), first, count (uint64),
// box[6] (float), axis (uint8), split (float), ropes[6] (int32); indices: the
// concatenated leaf triangle indices. Call ref_gpu_tree_size first for the
// sizes. The reference moves the tree's triangles into its result, so the
// handle is not usable afterwards.
void ref_gpu_tree_size(void *vh, uint64_t *n_nodes, uint64_t *n_indices) {
    auto *h = static_cast<Handle *>(vh);
    const KDTree &t = tree_of(h);
    *n_nodes = t.nnodes;
    uint64_t refs = 0;
    std::vector<const KDTreeElement *> order;
    dfs_dump(t.root.get(), order);
    for (auto *n : order) refs += n->triangleIndices.size();
    *n_indices = refs;
}

void ref_gpu_tree(void *vh, int32_t *left, int32_t *right, uint8_t *is_leaf, uint64_t *first, uint64_t *count,
                  float *box, uint8_t *axis, float *split, int32_t *ropes, uint64_t *indices) {
    auto *h = static_cast<Handle *>(vh);
    KDTreeGPU g = buildGPUTreeFromKDTree(h->scene.triangleDB);
    for (size_t i = 0; i < g.nodes.size(); i++) {
        const KDTreeGPUNode &n = g.nodes[i];
        left[i] = n.leftChildIndex;
        right[i] = n.rightChildIndex;
        is_leaf[i] = n.isLeaf ? 1 : 0;
        first[i] = n.firstTriangleIdxIdx;
        count[i] = n.numTriangles;
        const float b[6] = {n.bb.min.x, n.bb.min.y, n.bb.min.z, n.bb.max.x, n.bb.max.y, n.bb.max.z};
        for (int k = 0; k < 6; k++) box[6 * i + k] = b[k];
        axis[i] = n.splitPlane.axis;
        split[i] = n.splitPlane.distance;
        for (int k = 0; k < 6; k++) ropes[6 * i + k] = n.ropes[k];
    }
    for (size_t i = 0; i < g.triangleIndices.size(); i++) indices[i] = g.triangleIndices[i];
}

}  // extern "C"
