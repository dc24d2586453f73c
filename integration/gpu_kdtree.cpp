// Reference-side binding (see gpu_kdtree.h): SpatialDatabase on the GPU kd
// tree of libnostrum_pray, and a GPU render() for the reference's Scene.
#include "gpu_kdtree.h"

#include <algorithm>
#include <array>
#include <cfloat>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace pray {

namespace {

void check(pray_status st, const char *what) {
    if (st != PRAY_OK) throw std::runtime_error(std::string(what) + ": " + pray_last_error());
}

void put_ray(float *o, const Vec3 &p, const Vec3 &d, const Vec3 &inv) {
    o[0] = p.x, o[1] = p.y, o[2] = p.z;
    o[3] = d.x, o[4] = d.y, o[5] = d.z;
    o[6] = inv.x, o[7] = inv.y, o[8] = inv.z;
}

}  // namespace

GpuKDTree::GpuKDTree(int32_t device, float det_epsilon) : device_(device), eps_(det_epsilon) {}

GpuKDTree::~GpuKDTree() { pray_scene_destroy(scene_); }

void GpuKDTree::build(const std::vector<Triangle> &triangles) {
    std::vector<Triangle> copy = triangles;
    build(std::move(copy));
}

void GpuKDTree::build(std::vector<Triangle> &&triangles) {
    const size_t n = triangles.size();
    std::vector<float> verts(9 * n), colors(3 * n);
    std::vector<uint8_t> emit(n);
    for (size_t i = 0; i < n; i++) {
        const Triangle &t = triangles[i];
        const Vec3 *p[3] = {&t.a, &t.b, &t.c};
        for (int k = 0; k < 3; k++) {
            verts[9 * i + 3 * k] = p[k]->x;
            verts[9 * i + 3 * k + 1] = p[k]->y;
            verts[9 * i + 3 * k + 2] = p[k]->z;
        }
        colors[3 * i] = t.color.x, colors[3 * i + 1] = t.color.y, colors[3 * i + 2] = t.color.z;
        emit[i] = t.isEmitting ? 1 : 0;
    }
    pray_tree_options o;
    pray_tree_options_default(&o);
    // the tree preprocessScene would build (src/scene_preprocessor.cpp:52-57)
    o.tree = (n >= MIN_NUM_TRIANGLES_SAH && n < MAX_NUM_TRIANGLES_SAH) ? PRAY_TREE_SAH : PRAY_TREE_MEDIAN;
    pray_scene *created = nullptr;
    check(pray_scene_create(verts.data(), colors.data(), emit.data(), n, &o, device_, &created), "pray_scene_create");
    pray_scene_destroy(scene_);
    scene_ = created;
    triangles_ = std::move(triangles);
    uint64_t st[8];
    check(pray_scene_stats(scene_, st), "pray_scene_stats");
    nnodes = st[0];
    maxdepth = st[1];
    leafNodes = st[2];
    emptyLeafNodes = st[3];
    triangleCount = triangles_.size();
}

void GpuKDTree::trace(const float *rays9, uint64_t n, int32_t *ids, float *dists) const {
    if (n == 0) return;
    if (!scene_) {
        std::fill(ids, ids + n, -1);
        std::fill(dists, dists + n, FLT_MAX);
        return;
    }
    check(pray_trace_closest_host(scene_, rays9, n, eps_, ids, dists), "pray_trace_closest_host");
}

bool GpuKDTree::intersect(const Ray &ray, Triangle &triangle, float &dist) const {
    float r[9];
    put_ray(r, ray.position, ray.direction, ray.inverseDirection);
    int32_t id = -1;
    float t = FLT_MAX;
    trace(r, 1, &id, &t);
    if (id < 0) return false;
    triangle = triangles_[(size_t)id];
    dist = t;
    return true;
}

void GpuKDTree::intersectBatch(const std::vector<Ray> &rays, std::vector<int32_t> &ids,
                               std::vector<float> &dists) const {
    std::vector<float> packed(9 * rays.size());
    for (size_t i = 0; i < rays.size(); i++)
        put_ray(&packed[9 * i], rays[i].position, rays[i].direction, rays[i].inverseDirection);
    ids.assign(rays.size(), -1);
    dists.assign(rays.size(), FLT_MAX);
    trace(packed.data(), rays.size(), ids.data(), dists.data());
}

void GpuKDTree::tracePacket(const float *px, const float *py, const float *pz, const float *dx, const float *dy,
                            const float *dz, int lanes, int mask, int32_t *ids, float *dists) const {
    std::array<float, 9 * 8> packed{};
    std::array<int, 8> lane_of{};
    int m = 0;
    for (int j = 0; j < lanes; j++) {
        ids[j] = -1;
        dists[j] = FLT_MAX;
        if (!((mask >> j) & 1)) continue;
        Vec3 d(dx[j], dy[j], dz[j]);
        put_ray(&packed[9 * m], Vec3(px[j], py[j], pz[j]), d, d.inverse());
        lane_of[m++] = j;
    }
    std::array<int32_t, 8> hid{};
    std::array<float, 8> ht{};
    trace(packed.data(), (uint64_t)m, hid.data(), ht.data());
    for (int k = 0; k < m; k++) ids[lane_of[k]] = hid[k], dists[lane_of[k]] = ht[k];
}

#if defined(ENABLE_AVX)
// The 8-lane packet query of KDTree::intersect (src/kd_tree.cpp:282-299):
// lanes outside rayMask are not traced; returns the mask of lanes that hit,
// with their triangles and distances (FLT_MAX elsewhere).
__m256 GpuKDTree::intersect(const __m256 &rayPosX, const __m256 &rayPosY, const __m256 &rayPosZ,
                            const __m256 &rayDirX, const __m256 &rayDirY, const __m256 &rayDirZ,
                            const __m256 &rayMask, std::array<Triangle, 8> &trs, __m256 &distance) const {
    alignas(32) float px[8], py[8], pz[8], dx[8], dy[8], dz[8], d[8], hit[8];
    _mm256_store_ps(px, rayPosX), _mm256_store_ps(py, rayPosY), _mm256_store_ps(pz, rayPosZ);
    _mm256_store_ps(dx, rayDirX), _mm256_store_ps(dy, rayDirY), _mm256_store_ps(dz, rayDirZ);
    int32_t ids[8];
    tracePacket(px, py, pz, dx, dy, dz, 8, _mm256_movemask_ps(rayMask), ids, d);
    for (int j = 0; j < 8; j++) {
        uint32_t bits = ids[j] >= 0 ? 0xffffffffu : 0u;
        std::memcpy(&hit[j], &bits, 4);
        if (ids[j] >= 0) trs[j] = triangles_[(size_t)ids[j]];
    }
    distance = _mm256_load_ps(d);
    return _mm256_load_ps(hit);
}
#elif defined(ENABLE_SSE)
// The 4-lane packet query of the SSE build (include/spatial.h:33-36).
__m128 GpuKDTree::intersect(const __m128 &rayPosX, const __m128 &rayPosY, const __m128 &rayPosZ,
                            const __m128 &rayDirX, const __m128 &rayDirY, const __m128 &rayDirZ,
                            const __m128 &rayMask, std::vector<Triangle> &trs, __m128 &distance) const {
    alignas(16) float px[4], py[4], pz[4], dx[4], dy[4], dz[4], d[4], hit[4];
    _mm_store_ps(px, rayPosX), _mm_store_ps(py, rayPosY), _mm_store_ps(pz, rayPosZ);
    _mm_store_ps(dx, rayDirX), _mm_store_ps(dy, rayDirY), _mm_store_ps(dz, rayDirZ);
    int32_t ids[4];
    tracePacket(px, py, pz, dx, dy, dz, 4, _mm_movemask_ps(rayMask), ids, d);
    if (trs.size() < 4) trs.resize(4);
    for (int j = 0; j < 4; j++) {
        uint32_t bits = ids[j] >= 0 ? 0xffffffffu : 0u;
        std::memcpy(&hit[j], &bits, 4);
        if (ids[j] >= 0) trs[j] = triangles_[(size_t)ids[j]];
    }
    distance = _mm_load_ps(d);
    return _mm_load_ps(hit);
}
#endif

void renderOnGpu(Image &image, const Scene &scene, uint64_t seed) {
    const auto *db = dynamic_cast<const GpuKDTree *>(scene.triangleDB.get());
    if (!db) throw std::runtime_error("renderOnGpu: scene.triangleDB is not a GpuKDTree");
    image.resize(3 * scene.width * scene.height);
    const Vec3 &cp = scene.camera_position, &cl = scene.camera_look, &bg = scene.backgroundColor;
    if (scene.mode == Mode::RAYTRACING) {
        std::vector<float> lights(6 * scene.lights.size());
        for (size_t i = 0; i < scene.lights.size(); i++) {
            const LightSource &l = scene.lights[i];
            float *o = &lights[6 * i];
            o[0] = l.position.x, o[1] = l.position.y, o[2] = l.position.z;
            o[3] = l.color.x, o[4] = l.color.y, o[5] = l.color.z;
        }
        pray_rt_params p{};
        p.width = scene.width, p.height = scene.height, p.fov = scene.field_of_view;
        p.camera_position[0] = cp.x, p.camera_position[1] = cp.y, p.camera_position[2] = cp.z;
        p.camera_look[0] = cl.x, p.camera_look[1] = cl.y, p.camera_look[2] = cl.z;
        p.background[0] = bg.x, p.background[1] = bg.y, p.background[2] = bg.z;
        p.lights = lights.data();
        p.n_lights = (int32_t)scene.lights.size();
        p.det_epsilon = EPSILON;
        check(pray_render_rt_host(db->handle(), &p, image.data(), nullptr), "pray_render_rt_host");
        return;
    }
    pray_pt_params p{};
    p.width = scene.width, p.height = scene.height, p.fov = scene.field_of_view;
    p.camera_position[0] = cp.x, p.camera_position[1] = cp.y, p.camera_position[2] = cp.z;
    p.camera_look[0] = cl.x, p.camera_look[1] = cl.y, p.camera_look[2] = cl.z;
    p.background[0] = bg.x, p.background[1] = bg.y, p.background[2] = bg.z;
    p.max_depth = (uint32_t)scene.maxDepth;
    p.num_samples = (uint32_t)scene.numSamples;
    p.seed = seed;
    p.det_epsilon = EPSILON;
    p.mode = scene.maxDepth > MAX_DEPTH_DIFFUSE ? PRAY_PT_KAJIYA : PRAY_PT_DIFFUSE;
    p.scheduler = PRAY_SCHED_PIXEL;
    check(pray_render_pt_host(db->handle(), &p, image.data(), nullptr, nullptr), "pray_render_pt_host");
}

}  // namespace pray
