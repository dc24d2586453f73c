// C-ABI entry points (include/nostrum_pray.h): scene build and upload, error
// reporting, and the tracing launches.
#include "../../include/nostrum_pray.h"

#include <cfloat>
#include <cmath>
#include <algorithm>
#include <atomic>
#include <cstring>
#include <exception>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "batch_launch.h"
#include "capi_internal.h"
#include "denoise_net.h"
#include "device_layout.h"
#include "host/camera.h"
#include "host/flatten.h"
#include "host/kdtree.h"
#include "trace_launch.h"

using namespace pray_gpu;

namespace {

thread_local std::string g_error;

}  // namespace

namespace pray_gpu {

pray_status set_error(pray_status st, const std::string &msg) {
    g_error = msg;
    return st;
}

pray_status cuda_error(cudaError_t e, const char *what) {
    return set_error(e == cudaErrorMemoryAllocation ? PRAY_ERR_OUT_OF_MEMORY : PRAY_ERR_CUDA,
                     std::string(what) + ": " + cudaGetErrorString(e));
}

bool valid_options(const pray_tree_options *opt, std::string &why) {
    if (opt->tree != PRAY_TREE_MEDIAN && opt->tree != PRAY_TREE_SAH) {
        why = "tree must be PRAY_TREE_MEDIAN or PRAY_TREE_SAH";
        return false;
    }
    if (opt->leaf_size < 1) {
        why = "leaf_size must be >= 1";
        return false;
    }
    if (opt->max_depth < 0 || opt->max_depth > kMaxTreeDepth) {
        why = "max_depth must be in [0, 30]";
        return false;
    }
    if (opt->leaf_refine < 0) {
        why = "leaf_refine must be >= 0";
        return false;
    }
    if (!(opt->sah_traversal_cost >= 0.f) || !(opt->sah_intersection_cost > 0.f)) {
        why = "SAH costs must be finite, traversal >= 0 and intersection > 0";
        return false;
    }
    return true;
}

TreeOptions to_options(const pray_tree_options *opt) {
    TreeOptions o;
    o.kind = opt->tree;
    o.leaf_size = opt->leaf_size;
    o.max_depth = opt->max_depth;
    o.sah_ct = opt->sah_traversal_cost;
    o.sah_ci = opt->sah_intersection_cost;
    o.threads = opt->build_threads;
    return o;
}

}  // namespace pray_gpu

struct pray_host_tree {
    std::vector<TriPre> tris;
    BuiltTree tree;
};

struct pray_scene {
    int device = 0;
    uint64_t n_tris = 0;
    BuiltTree tree;  // host copy (statistics, dumps)
    GNode *d_nodes = nullptr;
    GTri *d_tris = nullptr;
    GShade *d_shade = nullptr;
    GTri *d_emit = nullptr;
    float *d_emit_cdf = nullptr;
    uint32_t n_emit = 0;
    float emit_area = 0.f;
    uint32_t n_gnodes = 0;
    uint64_t refined_leaves = 0;
    int device_depth = 0;  // deepest node of the device hierarchy
    float tol = 0.f;
    float cull_c[3] = {0.f, 0.f, 0.f}, cull_r2 = -1.f;
    std::atomic<int> rt_packets{PRAY_TRAVERSAL_AUTO};  // pray_traversal of the ray-traced frames
    uint64_t device_bytes = 0;
    // wavefront path tracer: scratch (path pool, queues), private stream,
    // events and the captured frame graph
    void *d_wf = nullptr;
    uint64_t wf_bytes = 0;
    uint64_t wf_capacity = 0, wf_pixels = 0;
    cudaStream_t wf_stream = nullptr;
    cudaEvent_t wf_ev_in = nullptr, wf_ev_out = nullptr;
    // second stream and fork / join events of a recorded wavefront frame
    // (each bounce's occlusion pass beside the next bounce's extend pass)
    cudaStream_t wf_side = nullptr;
    cudaEvent_t wf_fork = nullptr, wf_join = nullptr;
    cudaGraphExec_t wf_exec = nullptr;
    PtLaunch wf_key;
    uint64_t wf_key_cap = 0;
    int sm_count = 0;
    // frame buffers of the host-memory entry points, grown on demand
    uint8_t *d_rgb = nullptr;
    uint64_t rgb_cap = 0;
    unsigned long long *d_counters = nullptr;
    unsigned long long *d_pt_next = nullptr;  // work counter of the per-pixel path tracer
    // staging of pray_trace_closest_host (rays, ids, distances), grown on
    // demand; the mutex serialises host threads that share the scene
    std::mutex trace_mu;
    void *d_trace = nullptr;
    uint64_t trace_cap = 0;

    DevScene view() const {
        DevScene v;
        v.nodes = d_nodes;
        v.tris = d_tris;
        v.shade = d_shade;
        v.n_nodes = n_gnodes;
        v.n_refs = (uint32_t)tree.refs.size();
        v.n_tris = (uint32_t)n_tris;
        v.tol = tol;
        v.depth = (uint32_t)device_depth;
        for (int k = 0; k < 3; k++) v.cull_c[k] = cull_c[k];
        v.cull_r2 = cull_r2;
        v.emit_tris = d_emit;
        v.emit_cdf = d_emit_cdf;
        v.n_emit = n_emit;
        v.emit_area = emit_area;
        return v;
    }
    void release() {
        cudaFree(d_nodes);
        cudaFree(d_tris);
        cudaFree(d_shade);
        cudaFree(d_rgb);
        cudaFree(d_counters);
        cudaFree(d_emit);
        cudaFree(d_emit_cdf);
        cudaFree(d_wf);
        cudaFree(d_pt_next);
        cudaFree(d_trace);
        d_pt_next = nullptr;
        d_trace = nullptr;
        trace_cap = 0;
        if (wf_exec) cudaGraphExecDestroy(wf_exec);
        if (wf_stream) cudaStreamDestroy(wf_stream);
        if (wf_ev_in) cudaEventDestroy(wf_ev_in);
        if (wf_ev_out) cudaEventDestroy(wf_ev_out);
        if (wf_side) cudaStreamDestroy(wf_side);
        if (wf_fork) cudaEventDestroy(wf_fork);
        if (wf_join) cudaEventDestroy(wf_join);
        d_wf = nullptr, wf_exec = nullptr, wf_stream = nullptr, wf_ev_in = nullptr, wf_ev_out = nullptr;
        wf_side = nullptr, wf_fork = nullptr, wf_join = nullptr;
        wf_bytes = 0;
        d_nodes = nullptr, d_tris = nullptr, d_shade = nullptr, d_rgb = nullptr, d_counters = nullptr;
        d_emit = nullptr, d_emit_cdf = nullptr;
    }
};

namespace {

#define PRAY_TRY(...)                                                           \
    try {                                                                       \
        __VA_ARGS__                                                             \
    } catch (const std::bad_alloc &) {                                          \
        return set_error(PRAY_ERR_OUT_OF_MEMORY, "host allocation failed");     \
    } catch (const std::exception &e) {                                         \
        return set_error(PRAY_ERR_INVALID_ARGUMENT, e.what());                  \
    }

void dump_tree(const BuiltTree &t, float *boxes, float *split, int32_t *info, int64_t *refs) {
    for (size_t i = 0; i < t.nodes.size(); i++) {
        const FlatNode &n = t.nodes[i];
        for (int k = 0; k < 3; k++) boxes[6 * i + k] = n.box.lo[k], boxes[6 * i + 3 + k] = n.box.hi[k];
        split[i] = n.split;
        const bool leaf = n.left < 0;
        info[4 * i] = leaf ? 1 : 0;
        info[4 * i + 1] = n.axis;
        info[4 * i + 2] = leaf ? (int32_t)n.count : 0;
        info[4 * i + 3] = (int32_t)n.first;
    }
    for (size_t i = 0; i < t.refs.size(); i++) refs[i] = t.refs[i];
}

void tree_stats(const BuiltTree &t, uint64_t *out) {
    out[0] = t.nodes.size();
    out[1] = t.maxdepth;
    out[2] = t.leaf_nodes;
    out[3] = t.empty_leaves;
    out[4] = t.refs.size();
}

pray_status check_params(const pray_rt_params *p) {
    if (!p) return set_error(PRAY_ERR_INVALID_ARGUMENT, "params is NULL");
    if (p->width == 0 || p->height == 0 || p->width > 65536 || p->height > 65536)
        return set_error(PRAY_ERR_INVALID_ARGUMENT, "width and height must be in [1, 65536]");
    if (p->n_lights < 0 || p->n_lights > kMaxLights)
        return set_error(PRAY_ERR_INVALID_ARGUMENT, "n_lights must be in [0, 64]");
    if (p->n_lights > 0 && !p->lights) return set_error(PRAY_ERR_INVALID_ARGUMENT, "lights is NULL");
    return PRAY_OK;
}

// A ray-traced frame with the scene's traversal. The first frame of a scene
// renders with each traversal (per lane, packets, packets for the primary
// rays only) twice, times the second of each pair and keeps the fastest for
// the scene (the frames are identical; coherent surfaces favour packets,
// occlusion rays from the scattered hits of a triangle soup the per-lane
// walk); it synchronises `stream`.
cudaError_t render_rt(pray_scene *s, RtLaunch L, cudaStream_t stream) {
    if (s->rt_packets.load() < 0) {
        constexpr int kModes = 3;
        const int modes[kModes] = {PRAY_TRAVERSAL_LANES, PRAY_TRAVERSAL_PACKETS, PRAY_TRAVERSAL_PRIMARY_PACKETS};
        RtLaunch C = L;
        C.counters = nullptr;
        C.count_fetches = 0;
        cudaEvent_t ev[2 * kModes] = {};
        cudaError_t e = cudaSuccess;
        for (cudaEvent_t &x : ev)
            if (e == cudaSuccess) e = cudaEventCreate(&x);
        for (int rep = 0; rep < 2 && e == cudaSuccess; rep++)
            for (int m = 0; m < kModes && e == cudaSuccess; m++) {
                C.packets = modes[m];
                if (rep == 1) e = cudaEventRecord(ev[2 * m], stream);
                if (e == cudaSuccess) e = launch_render_rt(s->view(), C, stream);
                if (rep == 1 && e == cudaSuccess) e = cudaEventRecord(ev[2 * m + 1], stream);
            }
        if (e == cudaSuccess) e = cudaEventSynchronize(ev[2 * kModes - 1]);
        int best = 0;
        float best_ms = 0.f;
        for (int m = 0; m < kModes && e == cudaSuccess; m++) {
            float ms = 0.f;
            e = cudaEventElapsedTime(&ms, ev[2 * m], ev[2 * m + 1]);
            if (m == 0 || ms < best_ms) best = m, best_ms = ms;
        }
        for (cudaEvent_t x : ev)
            if (x) cudaEventDestroy(x);
        if (e != cudaSuccess) return e;
        s->rt_packets.store(modes[best]);
    }
    L.packets = s->rt_packets.load();
    return launch_render_rt(s->view(), L, stream);
}

pray_status check_pt_params(const pray_pt_params *p) {
    if (!p) return set_error(PRAY_ERR_INVALID_ARGUMENT, "params is NULL");
    if (p->width == 0 || p->height == 0 || p->width > 65536 || p->height > 65536)
        return set_error(PRAY_ERR_INVALID_ARGUMENT, "width and height must be in [1, 65536]");
    if (p->num_samples == 0) return set_error(PRAY_ERR_INVALID_ARGUMENT, "num_samples must be >= 1");
    if (p->max_depth >= (uint32_t)kMaxPtDepth)
        return set_error(PRAY_ERR_UNSUPPORTED, "max_depth must be below 64");
    if (p->mode != PRAY_PT_KAJIYA && p->mode != PRAY_PT_NEE && p->mode != PRAY_PT_DIFFUSE)
        return set_error(PRAY_ERR_INVALID_ARGUMENT, "mode must be PRAY_PT_KAJIYA, PRAY_PT_NEE or PRAY_PT_DIFFUSE");
    if (p->mode == PRAY_PT_DIFFUSE && p->max_depth > (uint32_t)kMaxDiffuseDepth)
        return set_error(PRAY_ERR_UNSUPPORTED, "PRAY_PT_DIFFUSE: max_depth must be at most 8");
    if (p->scheduler != PRAY_SCHED_PIXEL && p->scheduler != PRAY_SCHED_WAVEFRONT && p->scheduler != PRAY_SCHED_AUTO)
        return set_error(PRAY_ERR_INVALID_ARGUMENT,
                         "scheduler must be PRAY_SCHED_PIXEL, PRAY_SCHED_WAVEFRONT or PRAY_SCHED_AUTO");
    if (p->scheduler == PRAY_SCHED_WAVEFRONT && p->mode != PRAY_PT_NEE)
        return set_error(PRAY_ERR_UNSUPPORTED, "the wavefront scheduler runs PRAY_PT_NEE only");
    if ((uint64_t)p->sample_offset + p->num_samples > 0xFFFFFFFFull)
        return set_error(PRAY_ERR_INVALID_ARGUMENT, "sample_offset + num_samples must fit in 32 bits");
    return PRAY_OK;
}

PtLaunch make_pt_launch(const pray_pt_params *p) {
    PtLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.cam = make_camera(p->width, p->height, p->fov, p->camera_position, p->camera_look);
    for (int k = 0; k < 3; k++) L.bg[k] = p->background[k];
    L.max_depth = p->max_depth;
    L.num_samples = p->num_samples;
    L.rr_depth = p->rr_depth;
    L.mode = p->mode;
    L.seed = p->seed;
    L.eps = p->det_epsilon;
    L.sample_offset = p->sample_offset;
    return L;
}

RtLaunch make_launch(const pray_rt_params *p) {
    RtLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.cam = make_camera(p->width, p->height, p->fov, p->camera_position, p->camera_look);
    L.n_lights = p->n_lights;
    for (int i = 0; i < p->n_lights; i++)
        for (int k = 0; k < 6; k++) L.lights[i][k] = p->lights[6 * i + k];
    for (int k = 0; k < 3; k++) L.bg[k] = p->background[k];
    L.eps = p->det_epsilon;
    return L;
}

}  // namespace

// Grows the frame buffer of the host-memory entry points to `bytes` (plus
// alignment slack) and makes sure the ray counters exist.
pray_status ensure_frame(pray_scene *s, uint64_t bytes) {
    cudaError_t e;
    bytes += 16;
    if (bytes > s->rgb_cap) {
        cudaFree(s->d_rgb);
        s->d_rgb = nullptr;
        s->rgb_cap = 0;
        if ((e = cudaMalloc(&s->d_rgb, bytes)) != cudaSuccess) return cuda_error(e, "cudaMalloc (frame)");
        s->rgb_cap = bytes;
    }
    if (!s->d_counters && (e = cudaMalloc(&s->d_counters, 8 * sizeof(unsigned long long))) != cudaSuccess)
        return cuda_error(e, "cudaMalloc (counters)");
    return PRAY_OK;
}

// Most paths a wavefront round keeps in flight (at least one per pixel).
constexpr uint64_t kWavefrontMaxPaths = 1ull << 23;

// Paths per frame from which PRAY_SCHED_AUTO picks the wavefront scheduler:
// below it the per-pixel kernel is faster (one launch instead of three per
// bounce; at 512 x 512 it wins at 1 sample per pixel and loses at 2).
constexpr uint64_t kAutoWavefrontPaths = 1ull << 19;

// Runs a path-tracing launch with the chosen scheduler on `stream`.
pray_status run_pt(pray_scene *s, const PtLaunch &L, int scheduler, uint32_t wavefront_paths, cudaStream_t stream) {
    cudaError_t e;
    if (scheduler == PRAY_SCHED_AUTO)
        scheduler = (L.mode == PRAY_PT_NEE &&
                     (uint64_t)L.cam.width * L.cam.height * L.num_samples >= kAutoWavefrontPaths)
                        ? PRAY_SCHED_WAVEFRONT
                        : PRAY_SCHED_PIXEL;
    // both schedulers run on the scene's private stream (their scratch and
    // work counters are the scene's), ordered after the caller's work
    if (!s->wf_stream) {
        if ((e = cudaStreamCreateWithFlags(&s->wf_stream, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&s->wf_ev_in, cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&s->wf_ev_out, cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaStreamCreateWithFlags(&s->wf_side, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&s->wf_fork, cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&s->wf_join, cudaEventDisableTiming)) != cudaSuccess)
            return cuda_error(e, "path-tracer stream set-up");
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, dev);
    }
    if (scheduler == PRAY_SCHED_PIXEL) {
        if (!s->d_pt_next && (e = cudaMalloc(&s->d_pt_next, sizeof(unsigned long long))) != cudaSuccess)
            return cuda_error(e, "cudaMalloc (pixel counter)");
        PtLaunch P = L;
        P.next_pixel = s->d_pt_next;
        if ((e = cudaEventRecord(s->wf_ev_in, stream)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(s->wf_stream, s->wf_ev_in, 0)) != cudaSuccess ||
            (e = cudaMemsetAsync(s->d_pt_next, 0, sizeof(unsigned long long), s->wf_stream)) != cudaSuccess ||
            (e = launch_render_pt(s->view(), P, s->sm_count, s->wf_stream)) != cudaSuccess ||
            (e = cudaEventRecord(s->wf_ev_out, s->wf_stream)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(stream, s->wf_ev_out, 0)) != cudaSuccess)
            return cuda_error(e, "render_pt launch");
        return PRAY_OK;
    }
    const uint64_t P = (uint64_t)L.cam.width * L.cam.height;
    const uint64_t max_paths = wavefront_paths ? wavefront_paths : kWavefrontMaxPaths;
    const uint64_t cap = std::max<uint64_t>(P, std::min<uint64_t>(P * L.num_samples, max_paths));
    if (cap >= (1ull << 32)) return set_error(PRAY_ERR_UNSUPPORTED, "frame too large for the wavefront scheduler");
    if (s->wf_capacity < cap || s->wf_pixels < P) {
        const uint64_t ncap = std::max(cap, s->wf_capacity), npx = std::max(P, s->wf_pixels);
        const uint64_t bytes = wavefront_scratch_bytes(ncap, npx);
        if ((e = cudaStreamSynchronize(s->wf_stream)) != cudaSuccess) return cuda_error(e, "wavefront sync");
        cudaFree(s->d_wf);
        s->d_wf = nullptr;
        s->wf_capacity = s->wf_pixels = 0;
        if ((e = cudaMalloc(&s->d_wf, bytes)) != cudaSuccess) return cuda_error(e, "cudaMalloc (wavefront)");
        s->wf_capacity = ncap;
        s->wf_pixels = npx;
        s->wf_bytes = bytes;
        if (s->wf_exec) cudaGraphExecDestroy(s->wf_exec);
        s->wf_exec = nullptr;
    }
    if (!s->wf_exec || std::memcmp(&s->wf_key, &L, sizeof(L)) != 0 || s->wf_key_cap != cap) {
        if (s->wf_exec) cudaGraphExecDestroy(s->wf_exec);
        s->wf_exec = nullptr;
        WavefrontScratch w = wavefront_carve(s->d_wf, s->wf_capacity, s->wf_pixels);
        w.capacity = cap;
        cudaGraph_t g = nullptr;
        if ((e = cudaStreamBeginCapture(s->wf_stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
            return cuda_error(e, "graph capture");
        cudaError_t le = record_wavefront_frame(s->view(), L, w, s->sm_count, s->wf_stream, s->wf_side, s->wf_fork,
                                                s->wf_join);
        e = cudaStreamEndCapture(s->wf_stream, &g);
        if (le != cudaSuccess || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_error(le != cudaSuccess ? le : e, "wavefront capture");
        }
        e = cudaGraphInstantiate(&s->wf_exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            s->wf_exec = nullptr;
            return cuda_error(e, "graph instantiate");
        }
        std::memcpy(&s->wf_key, &L, sizeof(L));
        s->wf_key_cap = cap;
    }
    // order the private stream after the caller's work, and the caller's
    // later work after the frame
    if ((e = cudaEventRecord(s->wf_ev_in, stream)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(s->wf_stream, s->wf_ev_in, 0)) != cudaSuccess ||
        (e = cudaGraphLaunch(s->wf_exec, s->wf_stream)) != cudaSuccess ||
        (e = cudaEventRecord(s->wf_ev_out, s->wf_stream)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(stream, s->wf_ev_out, 0)) != cudaSuccess)
        return cuda_error(e, "wavefront launch");
    return PRAY_OK;
}

extern "C" {

const char *pray_last_error(void) { return g_error.c_str(); }

int32_t pray_api_version(void) { return PRAY_API_VERSION; }

void pray_tree_options_default(pray_tree_options *opt) {
    if (!opt) return;
    opt->tree = PRAY_TREE_MEDIAN;
    opt->leaf_size = 32;
    opt->max_depth = 20;
    opt->sah_traversal_cost = 5.f;
    opt->sah_intersection_cost = 1.5f;
    opt->build_threads = 0;
    opt->leaf_refine = 8;
}

pray_status pray_host_tree_build(const float *verts, uint64_t n, const pray_tree_options *opt,
                                 pray_host_tree **out) {
    if (!out || !opt || (n > 0 && !verts)) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n >= (1ull << 31)) return set_error(PRAY_ERR_INVALID_ARGUMENT, "too many triangles (max 2^31-1)");
    std::string why;
    if (!valid_options(opt, why)) return set_error(PRAY_ERR_INVALID_ARGUMENT, why);
    PRAY_TRY({
        auto t = std::make_unique<pray_host_tree>();
        t->tris = precompute_triangles(verts, n, opt->build_threads);
        t->tree = build_tree(t->tris, to_options(opt));
        *out = t.release();
        return PRAY_OK;
    })
}

void pray_host_tree_destroy(pray_host_tree *t) { delete t; }

pray_status pray_host_tree_stats(const pray_host_tree *t, uint64_t *out) {
    if (!t || !out) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    tree_stats(t->tree, out);
    return PRAY_OK;
}

pray_status pray_host_tree_dump(const pray_host_tree *t, float *boxes, float *split, int32_t *info,
                                int64_t *refs) {
    if (!t || !boxes || !split || !info || !refs) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    dump_tree(t->tree, boxes, split, info, refs);
    return PRAY_OK;
}

pray_status pray_host_tree_precompute(const pray_host_tree *t, float *out) {
    if (!t || !out) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    for (size_t i = 0; i < t->tris.size(); i++) {
        const TriPre &p = t->tris[i];
        const F3 *vs[6] = {&p.box.lo, &p.box.hi, &p.mid, &p.ab, &p.ac, &p.normal};
        for (int k = 0; k < 6; k++)
            for (int c = 0; c < 3; c++) out[18 * i + 3 * k + c] = (*vs[k])[c];
    }
    return PRAY_OK;
}

pray_status pray_host_tree_device_layout(const pray_host_tree *t, int32_t leaf_refine, uint64_t *out) {
    if (!t || !out) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    if (leaf_refine < 0) return set_error(PRAY_ERR_INVALID_ARGUMENT, "leaf_refine must be >= 0");
    PRAY_TRY({
        DeviceImage img;
        flatten_for_device(t->tree, t->tris, leaf_refine, img);
        std::string bad;
        if (!validate_device_image(img, bad)) return set_error(PRAY_ERR_UNSUPPORTED, "device layout: " + bad);
        out[0] = img.nodes.size();
        out[1] = img.tris.size();
        out[2] = img.refined_leaves;
        out[3] = img.sub_nodes;
        return PRAY_OK;
    })
}

pray_status pray_camera(uint64_t width, uint64_t height, uint64_t fov, const float *pos, const float *look,
                        float *out) {
    if (!pos || !look || !out) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    if (width == 0 || height == 0) return set_error(PRAY_ERR_INVALID_ARGUMENT, "empty image");
    CameraConsts c = make_camera(width, height, fov, pos, look);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) out[3 * i + j] = c.m[i][j];
    out[9] = c.inv_w;
    out[10] = c.inv_h;
    out[11] = c.aspect;
    out[12] = c.angle;
    return PRAY_OK;
}

pray_status pray_scene_create(const float *verts, const float *colors, const uint8_t *emit, uint64_t n,
                              const pray_tree_options *opt, int32_t device, pray_scene **out) {
    if (!out || !opt || (n > 0 && (!verts || !colors))) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n >= (1ull << 31)) return set_error(PRAY_ERR_INVALID_ARGUMENT, "too many triangles (max 2^31-1)");
    std::string why;
    if (!valid_options(opt, why)) return set_error(PRAY_ERR_INVALID_ARGUMENT, why);
    *out = nullptr;
    std::unique_ptr<pray_scene> s;
    std::vector<TriPre> pre;
    std::vector<GNode> gnodes;
    std::vector<GTri> gtris;
    std::vector<GShade> gshade;
    std::vector<GTri> gemit;
    std::vector<float> gcdf;
    PRAY_TRY({
        s = std::make_unique<pray_scene>();
        s->device = device;
        s->n_tris = n;
        pre = precompute_triangles(verts, n, opt->build_threads);
        s->tree = build_tree(pre, to_options(opt));
        if (s->tree.refs.size() >= (1ull << 31))
            return set_error(PRAY_ERR_UNSUPPORTED, "more than 2^31-1 leaf references");
        DeviceImage img;
        flatten_for_device(s->tree, pre, opt->leaf_refine, img);
        std::string bad;
        if (!validate_device_image(img, bad, &s->device_depth))
            return set_error(PRAY_ERR_UNSUPPORTED, "device layout: " + bad);
        gnodes.swap(img.nodes);
        gnodes.insert(gnodes.end(), img.nodes_tight.begin(), img.nodes_tight.end());  // both copies, one buffer
        for (int k = 0; k < 3; k++) s->cull_c[k] = img.cull_center[k];
        s->cull_r2 = img.cull_radius2;
        gtris.swap(img.tris);
        s->refined_leaves = img.refined_leaves;
        gshade.resize(n);
        for (uint64_t i = 0; i < n; i++) {
            GShade &g = gshade[i];
            for (int k = 0; k < 3; k++) g.n[k] = pre[i].normal[k], g.c[k] = colors[3 * i + k];
            g.n[3] = (emit && emit[i]) ? 1.f : 0.f;
            g.c[3] = 0.f;
        }
        // emitters for next-event estimation: geometry and area prefix sums
        // (area = |ab x ac| / 2 in double, summed in double)
        double acc = 0.0;
        for (uint64_t i = 0; i < n; i++) {
            if (!(emit && emit[i])) continue;
            const TriPre &p = pre[i];
            const F3 c = cross3(p.ab, p.ac);
            const double area = 0.5 * std::sqrt((double)c[0] * c[0] + (double)c[1] * c[1] + (double)c[2] * c[2]);
            if (!(area > 0.0)) continue;
            acc += area;
            GTri g;
            uint32_t idbits = (uint32_t)i;
            float idf;
            std::memcpy(&idf, &idbits, 4);
            g.v0[0] = p.a[0], g.v0[1] = p.a[1], g.v0[2] = p.a[2], g.v0[3] = idf;
            g.e1[0] = p.ab[0], g.e1[1] = p.ab[1], g.e1[2] = p.ab[2], g.e1[3] = 0.f;
            g.e2[0] = p.ac[0], g.e2[1] = p.ac[1], g.e2[2] = p.ac[2], g.e2[3] = 0.f;
            gemit.push_back(g);
            gcdf.push_back((float)acc);
        }
        s->emit_area = gcdf.empty() ? 0.f : gcdf.back();
        // box-behind-origin margin: 1e-5 of the scene's diagonal
        const Aabb &rb = s->tree.nodes[0].box;
        float diag = 0.f;
        if (n > 0) {
            for (int k = 0; k < 3; k++) {
                const float e = rb.hi[k] - rb.lo[k];
                diag += e * e;
            }
            diag = std::sqrt(diag);
        }
        s->tol = std::isfinite(diag) ? diag * 1e-5f : FLT_MAX;
    })
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    const size_t nb = gnodes.size() * sizeof(GNode), tb = std::max<size_t>(gtris.size(), 1) * sizeof(GTri),
                 sb = std::max<size_t>(gshade.size(), 1) * sizeof(GShade);
    if ((e = cudaMalloc(&s->d_nodes, nb)) != cudaSuccess || (e = cudaMalloc(&s->d_tris, tb)) != cudaSuccess ||
        (e = cudaMalloc(&s->d_shade, sb)) != cudaSuccess) {
        s->release();
        return cuda_error(e, "cudaMalloc (scene)");
    }
    if ((e = cudaMemcpy(s->d_nodes, gnodes.data(), nb, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (!gtris.empty() &&
         (e = cudaMemcpy(s->d_tris, gtris.data(), gtris.size() * sizeof(GTri), cudaMemcpyHostToDevice)) !=
             cudaSuccess) ||
        (!gshade.empty() && (e = cudaMemcpy(s->d_shade, gshade.data(), gshade.size() * sizeof(GShade),
                                            cudaMemcpyHostToDevice)) != cudaSuccess)) {
        s->release();
        return cuda_error(e, "cudaMemcpy (scene upload)");
    }
    if (!gemit.empty()) {
        if ((e = cudaMalloc(&s->d_emit, gemit.size() * sizeof(GTri))) != cudaSuccess ||
            (e = cudaMalloc(&s->d_emit_cdf, gcdf.size() * sizeof(float))) != cudaSuccess ||
            (e = cudaMemcpy(s->d_emit, gemit.data(), gemit.size() * sizeof(GTri), cudaMemcpyHostToDevice)) !=
                cudaSuccess ||
            (e = cudaMemcpy(s->d_emit_cdf, gcdf.data(), gcdf.size() * sizeof(float), cudaMemcpyHostToDevice)) !=
                cudaSuccess) {
            s->release();
            return cuda_error(e, "emitter upload");
        }
        s->n_emit = (uint32_t)gemit.size();
    }
    s->n_gnodes = (uint32_t)(gnodes.size() / 2);
    s->device_bytes = nb + tb + sb + gemit.size() * (sizeof(GTri) + sizeof(float));
    *out = s.release();
    return PRAY_OK;
}

pray_status pray_scene_destroy(pray_scene *s) {
    if (!s) return PRAY_OK;
    cudaSetDevice(s->device);
    s->release();
    delete s;
    return PRAY_OK;
}

pray_status pray_scene_set_traversal(pray_scene *s, int32_t traversal) {
    if (!s) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    if (traversal < PRAY_TRAVERSAL_AUTO || traversal > PRAY_TRAVERSAL_PRIMARY_PACKETS)
        return set_error(PRAY_ERR_INVALID_ARGUMENT,
                         "traversal must be PRAY_TRAVERSAL_AUTO, _LANES, _PACKETS or _PRIMARY_PACKETS");
    s->rt_packets.store(traversal);
    return PRAY_OK;
}

pray_status pray_scene_traversal(const pray_scene *s, int32_t *traversal) {
    if (!s || !traversal) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    *traversal = s->rt_packets.load();
    return PRAY_OK;
}

pray_status pray_scene_stats(const pray_scene *s, uint64_t *out) {
    if (!s || !out) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    tree_stats(s->tree, out);
    out[5] = s->n_tris;
    out[6] = s->device_bytes;
    out[7] = s->n_gnodes;
    return PRAY_OK;
}

pray_status pray_trace_closest(pray_scene *s, const float *rays, uint64_t n, float eps, int32_t *ids, float *ts,
                               void *stream) {
    if (!s || (n > 0 && (!rays || !ids || !ts))) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n >= (1ull << 40)) return set_error(PRAY_ERR_INVALID_ARGUMENT, "too many rays");
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    e = launch_trace_closest(s->view(), rays, n, eps, ids, ts, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_error(e, "trace_closest launch");
    return PRAY_OK;
}

pray_status pray_trace_occluded(pray_scene *s, const float *rays, const float *dist2, uint64_t n, float eps,
                                uint8_t *occluded, void *stream) {
    if (!s || (n > 0 && (!rays || !dist2 || !occluded))) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n >= (1ull << 40)) return set_error(PRAY_ERR_INVALID_ARGUMENT, "too many rays");
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    e = launch_trace_occluded(s->view(), rays, dist2, n, eps, occluded, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_error(e, "trace_occluded launch");
    return PRAY_OK;
}

pray_status pray_trace_closest_host(pray_scene *s, const float *rays_host, uint64_t n, float eps, int32_t *ids_host,
                                    float *t_host) {
    if (!s || (n > 0 && (!rays_host || !ids_host || !t_host))) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n >= (1ull << 32)) return set_error(PRAY_ERR_INVALID_ARGUMENT, "too many rays for one call");
    if (n == 0) return PRAY_OK;
    std::lock_guard<std::mutex> lock(s->trace_mu);
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    // one buffer: n x 9 floats of rays, then n ids, then n distances (all 4-byte words)
    if (n > s->trace_cap) {
        cudaFree(s->d_trace);
        s->d_trace = nullptr;
        s->trace_cap = 0;
        const uint64_t cap = std::max<uint64_t>(n, 1024);
        if ((e = cudaMalloc(&s->d_trace, cap * 11 * sizeof(float))) != cudaSuccess)
            return cuda_error(e, "cudaMalloc (trace staging)");
        s->trace_cap = cap;
    }
    float *d_rays = static_cast<float *>(s->d_trace);
    int32_t *d_ids = reinterpret_cast<int32_t *>(d_rays + 9 * s->trace_cap);
    float *d_t = reinterpret_cast<float *>(d_ids + s->trace_cap);
    if ((e = cudaMemcpy(d_rays, rays_host, n * 9 * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_error(e, "cudaMemcpy (rays)");
    if ((e = launch_trace_closest(s->view(), d_rays, n, eps, d_ids, d_t, 0)) != cudaSuccess)
        return cuda_error(e, "trace_closest launch");
    if ((e = cudaMemcpy(ids_host, d_ids, n * sizeof(int32_t), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_error(e, "cudaMemcpy (ids)");
    if ((e = cudaMemcpy(t_host, d_t, n * sizeof(float), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_error(e, "cudaMemcpy (distances)");
    return PRAY_OK;
}

pray_status pray_render_rt(pray_scene *s, const pray_rt_params *p, uint8_t *rgb, int32_t *ids, float *ts,
                           unsigned long long *counters, void *stream) {
    if (!s || !rgb) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    if ((ids == nullptr) != (ts == nullptr))
        return set_error(PRAY_ERR_INVALID_ARGUMENT, "ids and t must both be given or both be NULL");
    pray_status st = check_params(p);
    if (st != PRAY_OK) return st;
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    RtLaunch L = make_launch(p);
    L.rgb = rgb;
    L.ids = ids;
    L.ts = ts;
    L.counters = counters;
    e = render_rt(s, L, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_error(e, "render_rt launch");
    return PRAY_OK;
}

pray_status pray_render_rt_host(pray_scene *s, const pray_rt_params *p, uint8_t *rgb_host, uint64_t *rays_cast) {
    if (!s || !rgb_host) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    pray_status st = check_params(p);
    if (st != PRAY_OK) return st;
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    const uint64_t bytes = 3ull * p->width * p->height;
    if ((st = ensure_frame(s, bytes)) != PRAY_OK) return st;
    if ((e = cudaMemsetAsync(s->d_counters, 0, 2 * sizeof(unsigned long long), 0)) != cudaSuccess)
        return cuda_error(e, "cudaMemsetAsync");
    RtLaunch L = make_launch(p);
    L.rgb = s->d_rgb;
    L.counters = s->d_counters;
    if ((e = render_rt(s, L, 0)) != cudaSuccess) return cuda_error(e, "render_rt launch");
    if ((e = cudaMemcpy(rgb_host, s->d_rgb, bytes, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_error(e, "cudaMemcpy (frame)");
    if (rays_cast) {
        unsigned long long c[2];
        if ((e = cudaMemcpy(c, s->d_counters, sizeof(c), cudaMemcpyDeviceToHost)) != cudaSuccess)
            return cuda_error(e, "cudaMemcpy (counters)");
        rays_cast[0] = c[0];
        rays_cast[1] = c[1];
    }
    return PRAY_OK;
}

pray_status pray_render_rt_counts(pray_scene *s, const pray_rt_params *p, uint64_t *out) {
    if (!s || !out) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    pray_status st = check_params(p);
    if (st != PRAY_OK) return st;
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    if ((st = ensure_frame(s, 3ull * p->width * p->height)) != PRAY_OK) return st;
    if ((e = cudaMemsetAsync(s->d_counters, 0, 8 * sizeof(unsigned long long), 0)) != cudaSuccess)
        return cuda_error(e, "cudaMemsetAsync");
    RtLaunch L = make_launch(p);
    L.rgb = s->d_rgb;
    L.counters = s->d_counters;
    L.count_fetches = 1;
    if ((e = render_rt(s, L, 0)) != cudaSuccess) return cuda_error(e, "render_rt launch");
    unsigned long long c[5];
    if ((e = cudaMemcpy(c, s->d_counters, sizeof(c), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_error(e, "cudaMemcpy (counters)");
    for (int k = 0; k < 5; k++) out[k] = c[k];
    return PRAY_OK;
}

pray_status pray_render_pt(pray_scene *s, const pray_pt_params *p, uint8_t *rgb, float *radiance,
                           unsigned long long *counters, void *stream) {
    if (!s || (!rgb && !radiance)) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    pray_status st = check_pt_params(p);
    if (st != PRAY_OK) return st;
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    PtLaunch L = make_pt_launch(p);
    L.rgb = rgb;
    L.radiance = radiance;
    L.counters = counters;
    return run_pt(s, L, p->scheduler, p->wavefront_paths, (cudaStream_t)stream);
}

pray_status pray_accumulate_pt(pray_scene *s, const pray_pt_params *p, double *sum, unsigned long long *counters,
                               void *stream) {
    if (!s || !sum) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    pray_status st = check_pt_params(p);
    if (st != PRAY_OK) return st;
    if (p->mode == PRAY_PT_DIFFUSE)
        return set_error(PRAY_ERR_UNSUPPORTED, "PRAY_PT_DIFFUSE makes one estimate per pixel; nothing to accumulate");
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    PtLaunch L = make_pt_launch(p);
    L.sum64 = sum;
    L.counters = counters;
    return run_pt(s, L, p->scheduler, p->wavefront_paths, (cudaStream_t)stream);
}

pray_status pray_render_pt_noalloc(pray_scene *s, const pray_pt_params *p, uint8_t *rgb, float *radiance,
                                   unsigned long long *counters, void *stream) {
    if (!s || (!rgb && !radiance)) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    pray_status st = check_pt_params(p);
    if (st != PRAY_OK) return st;
    if (p->mode != PRAY_PT_NEE)
        return set_error(PRAY_ERR_UNSUPPORTED, "the allocation-free path tracer runs PRAY_PT_NEE only");
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    PtLaunch L = make_pt_launch(p);
    L.rgb = rgb;
    L.radiance = radiance;
    L.counters = counters;
    std::string why;
    e = launch_wavefront_noalloc(s->view(), L, p->wavefront_paths, (cudaStream_t)stream, why);
    if (e != cudaSuccess) {
        if (!why.empty()) return set_error(e == cudaErrorInvalidValue ? PRAY_ERR_INVALID_ARGUMENT : PRAY_ERR_CUDA, why);
        return cuda_error(e, "allocation-free render_pt");
    }
    return PRAY_OK;
}

}  // extern "C"

struct pray_batch {
    int device = 0;
    std::vector<pray_scene *> scenes;
    std::vector<BatchItem> items;  // host copy; first_tile follows the tile shape
    BatchItem *d_items = nullptr;
    unsigned long long *d_next = nullptr;
    uint64_t total_tiles = 0;
    int max_depth = 0;
    int sm_count = 0;
    bool kajiya = true;  // every item runs PRAY_PT_KAJIYA
    pray_batch_config cfg{8, 4, 128, 0, 64};
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long *exec_counters = nullptr;
    void release() {
        if (exec) cudaGraphExecDestroy(exec);
        if (stream) cudaStreamDestroy(stream);
        if (ev_in) cudaEventDestroy(ev_in);
        if (ev_out) cudaEventDestroy(ev_out);
        cudaFree(d_items);
        cudaFree(d_next);
        exec = nullptr, stream = nullptr, ev_in = ev_out = nullptr, d_items = nullptr, d_next = nullptr;
    }
};

namespace {

bool valid_batch_config(const pray_batch *b, const pray_batch_config &c, std::string &why) {
    if (c.tile_w < 1 || c.tile_h < 1 || c.tile_w * c.tile_h != 32) {
        why = "tile_w * tile_h must be 32";
        return false;
    }
    if (c.block_threads < 32 || c.block_threads > 1024 || c.block_threads % 32) {
        why = "block_threads must be a multiple of 32 in [32, 1024]";
        return false;
    }
    if (c.stack_entries != 32 && c.stack_entries != 64) {
        why = "stack_entries must be 32 or 64";
        return false;
    }
    if (c.stack_entries == 32 && b->max_depth >= 32) {
        why = "a scene's device hierarchy is too deep for a 32-entry stack";
        return false;
    }
    if (c.blocks_per_sm < 0) {
        why = "blocks_per_sm must be >= 0";
        return false;
    }
    return true;
}

// Tile numbering for the batch's tile shape, uploaded with the items.
pray_status upload_batch(pray_batch *b) {
    uint64_t t = 0;
    for (BatchItem &it : b->items) {
        it.first_tile = t;
        const uint64_t tx = (it.L.cam.width + b->cfg.tile_w - 1) / b->cfg.tile_w;
        const uint64_t ty = (it.L.cam.height + b->cfg.tile_h - 1) / b->cfg.tile_h;
        t += tx * ty;
    }
    b->total_tiles = t;
    cudaError_t e = cudaMemcpy(b->d_items, b->items.data(), b->items.size() * sizeof(BatchItem),
                               cudaMemcpyHostToDevice);
    return e == cudaSuccess ? PRAY_OK : cuda_error(e, "batch upload");
}

int batch_blocks(pray_batch *b, const pray_batch_config &c) {
    int per_sm = 0;
    if (batch_max_blocks_per_sm(c.block_threads, c.stack_entries, b->kajiya, &per_sm) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    if (c.blocks_per_sm > 0) per_sm = std::min(per_sm, c.blocks_per_sm);
    return per_sm * std::max(1, b->sm_count);
}

BatchLaunch batch_view(const pray_batch *b, unsigned long long *counters) {
    BatchLaunch B;
    B.items = b->d_items;
    B.n_items = (int)b->items.size();
    B.total_tiles = b->total_tiles;
    B.next_tile = b->d_next;
    B.tile_w = (uint32_t)b->cfg.tile_w;
    B.tile_h = (uint32_t)b->cfg.tile_h;
    B.counters = counters;
    B.kajiya = b->kajiya;
    return B;
}

}  // namespace

extern "C" {

pray_status pray_batch_create(pray_scene *const *scenes, const pray_pt_params *params, uint8_t *const *rgb,
                              float *const *radiance, int32_t n, pray_batch **out) {
    if (!scenes || !params || !out || n <= 0) return set_error(PRAY_ERR_INVALID_ARGUMENT, "empty or NULL batch");
    *out = nullptr;
    auto b = std::make_unique<pray_batch>();
    b->device = scenes[0] ? scenes[0]->device : 0;
    for (int i = 0; i < n; i++) {
        pray_scene *s = scenes[i];
        if (!s) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL scene in batch");
        if (s->device != b->device) return set_error(PRAY_ERR_INVALID_ARGUMENT, "batch scenes on different devices");
        pray_pt_params p = params[i];
        p.scheduler = PRAY_SCHED_PIXEL;
        pray_status st = check_pt_params(&p);
        if (st != PRAY_OK) return st;
        if (p.mode == PRAY_PT_DIFFUSE)
            return set_error(PRAY_ERR_UNSUPPORTED, "batches run PRAY_PT_KAJIYA or PRAY_PT_NEE");
        uint8_t *o8 = rgb ? rgb[i] : nullptr;
        float *of = radiance ? radiance[i] : nullptr;
        if (!o8 && !of) return set_error(PRAY_ERR_INVALID_ARGUMENT, "batch item without an output");
        BatchItem it;
        std::memset(&it, 0, sizeof(it));
        it.s = s->view();
        it.L = make_pt_launch(&p);
        it.L.rgb = o8;
        it.L.radiance = of;
        b->items.push_back(it);
        b->scenes.push_back(s);
        b->kajiya = b->kajiya && p.mode == PRAY_PT_KAJIYA;
        b->max_depth = std::max(b->max_depth, s->device_depth);
    }
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device);
    if (b->max_depth >= 32) b->cfg.stack_entries = 64;
    if ((e = cudaMalloc(&b->d_items, b->items.size() * sizeof(BatchItem))) != cudaSuccess ||
        (e = cudaMalloc(&b->d_next, sizeof(unsigned long long))) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->ev_out, cudaEventDisableTiming)) != cudaSuccess) {
        b->release();
        return cuda_error(e, "batch set-up");
    }
    pray_status st = upload_batch(b.get());
    if (st != PRAY_OK) {
        b->release();
        return st;
    }
    *out = b.release();
    return PRAY_OK;
}

pray_status pray_batch_destroy(pray_batch *b) {
    if (!b) return PRAY_OK;
    cudaSetDevice(b->device);
    b->release();
    delete b;
    return PRAY_OK;
}

pray_status pray_batch_set_config(pray_batch *b, const pray_batch_config *cfg) {
    if (!b || !cfg) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    std::string why;
    if (!valid_batch_config(b, *cfg, why)) return set_error(PRAY_ERR_INVALID_ARGUMENT, why);
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) return cuda_error(e, "batch sync");
    b->cfg = *cfg;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    return upload_batch(b);
}

pray_status pray_batch_tune(pray_batch *b, pray_batch_config *chosen, float *best_ms) {
    if (!b) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    const std::vector<BatchItem> full = b->items;
    for (BatchItem &it : b->items) it.L.num_samples = 1;  // one sample per pixel while timing
    static const int tiles[][2] = {{8, 4}, {4, 8}, {16, 2}, {32, 1}};
    static const int threads[] = {64, 128, 256};
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    float best = -1.f;
    pray_batch_config best_cfg = b->cfg;
    pray_status st = PRAY_OK;
    for (int stack : {32, 64}) {
        if (stack == 32 && b->max_depth >= 32) continue;
        for (const auto &tl : tiles)
            for (int bt : threads)
                for (int occ : {0, 2}) {
                    pray_batch_config c{tl[0], tl[1], bt, occ, stack};
                    b->cfg = c;
                    if ((st = upload_batch(b)) != PRAY_OK) goto done;
                    const int blocks = batch_blocks(b, c);
                    const BatchLaunch B = batch_view(b, nullptr);
                    // one untimed run (warms caches and loads the kernel), one timed
                    if ((e = launch_batch_pt(B, bt, blocks, stack, b->stream)) != cudaSuccess ||
                        (e = cudaEventRecord(t0, b->stream)) != cudaSuccess ||
                        (e = launch_batch_pt(B, bt, blocks, stack, b->stream)) != cudaSuccess ||
                        (e = cudaEventRecord(t1, b->stream)) != cudaSuccess ||
                        (e = cudaEventSynchronize(t1)) != cudaSuccess) {
                        st = cuda_error(e, "batch tuning run");
                        goto done;
                    }
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, t0, t1);
                    if (best < 0.f || ms < best) best = ms, best_cfg = c;
                }
    }
done:
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    b->items = full;
    b->cfg = best_cfg;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    pray_status up = upload_batch(b);
    if (st != PRAY_OK) return st;
    if (up != PRAY_OK) return up;
    if (chosen) *chosen = best_cfg;
    if (best_ms) *best_ms = best;
    return PRAY_OK;
}

pray_status pray_batch_render(pray_batch *b, unsigned long long *counters, void *stream) {
    if (!b) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    if (!b->exec || b->exec_counters != counters) {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
        cudaGraph_t g = nullptr;
        if ((e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
            return cuda_error(e, "batch capture");
        const cudaError_t le =
            launch_batch_pt(batch_view(b, counters), b->cfg.block_threads, batch_blocks(b, b->cfg),
                            b->cfg.stack_entries, b->stream);
        e = cudaStreamEndCapture(b->stream, &g);
        if (le != cudaSuccess || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_error(le != cudaSuccess ? le : e, "batch capture");
        }
        e = cudaGraphInstantiate(&b->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->exec = nullptr;
            return cuda_error(e, "batch graph instantiate");
        }
        b->exec_counters = counters;
    }
    cudaStream_t cs = (cudaStream_t)stream;
    if ((e = cudaEventRecord(b->ev_in, cs)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(b->stream, b->ev_in, 0)) != cudaSuccess ||
        (e = cudaGraphLaunch(b->exec, b->stream)) != cudaSuccess ||
        (e = cudaEventRecord(b->ev_out, b->stream)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(cs, b->ev_out, 0)) != cudaSuccess)
        return cuda_error(e, "batch launch");
    return PRAY_OK;
}

pray_status pray_render_features(pray_scene *s, const pray_pt_params *p, uint16_t *features, void *stream) {
    if (!s || !p || !features) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    if (p->width == 0 || p->height == 0 || p->width > 65536 || p->height > 65536)
        return set_error(PRAY_ERR_INVALID_ARGUMENT, "width and height must be in [1, 65536]");
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    const CameraConsts cam = make_camera(p->width, p->height, p->fov, p->camera_position, p->camera_look);
    e = launch_features(s->view(), cam, p->det_epsilon, reinterpret_cast<__half *>(features), (cudaStream_t)stream);
    return e == cudaSuccess ? PRAY_OK : cuda_error(e, "features launch");
}

}  // extern "C"

struct pray_denoiser {
    Denoiser net;
};

namespace {

pray_status check_dims(int32_t n, int32_t h, int32_t w) {
    if (n <= 0 || h <= 0 || w <= 0 || h % 16 || w % 16 || (int64_t)n * h * w > (1ll << 31) / 256)
        return set_error(PRAY_ERR_INVALID_ARGUMENT, "images must be non-empty, h and w multiples of 16");
    return PRAY_OK;
}

}  // namespace

extern "C" {

pray_status pray_denoiser_create(int32_t device, uint64_t seed, pray_denoiser **out) {
    if (!out) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    auto d = std::make_unique<pray_denoiser>();
    d->net.device = device;
    if ((e = d->net.init(seed)) != cudaSuccess) return cuda_error(e, "denoiser init");
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return cuda_error(e, "denoiser init");
    *out = d.release();
    return PRAY_OK;
}

pray_status pray_denoiser_destroy(pray_denoiser *d) {
    if (!d) return PRAY_OK;
    cudaSetDevice(d->net.device);
    delete d;
    return PRAY_OK;
}

pray_status pray_denoiser_num_params(const pray_denoiser *d, uint64_t *n) {
    if (!d || !n) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    *n = d->net.num_params();
    return PRAY_OK;
}

pray_status pray_denoiser_get_params(const pray_denoiser *d, float *host) {
    if (!d || !host) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    cudaSetDevice(d->net.device);
    cudaError_t e = d->net.get_params(host);
    return e == cudaSuccess ? PRAY_OK : cuda_error(e, "denoiser get_params");
}

pray_status pray_denoiser_set_params(pray_denoiser *d, const float *host) {
    if (!d || !host) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    cudaSetDevice(d->net.device);
    cudaError_t e = d->net.set_params(host);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return e == cudaSuccess ? PRAY_OK : cuda_error(e, "denoiser set_params");
}

pray_status pray_denoise(pray_denoiser *d, const float *rad, const uint16_t *feat, int32_t n, int32_t h, int32_t w,
                         float *out, void *stream) {
    if (!d || !rad || !feat || !out) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    pray_status st = check_dims(n, h, w);
    if (st != PRAY_OK) return st;
    cudaSetDevice(d->net.device);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = d->net.denoise(rad, reinterpret_cast<const __half *>(feat), n, h, w, out, s);
    return e == cudaSuccess ? PRAY_OK : cuda_error(e, "denoise");
}

pray_status pray_denoiser_train_step(pray_denoiser *d, const float *rad, const uint16_t *feat, const float *target,
                                     int32_t n, int32_t h, int32_t w, float lr, float *loss_host, void *stream) {
    if (!d || !rad || !feat || !target) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    pray_status st = check_dims(n, h, w);
    if (st != PRAY_OK) return st;
    cudaSetDevice(d->net.device);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = d->net.forward(rad, reinterpret_cast<const __half *>(feat), n, h, w, s);
    if (e == cudaSuccess) e = d->net.backward(target, s);
    if (e == cudaSuccess && loss_host)
        e = cudaMemcpyAsync(loss_host, d->net.loss_device(), 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = d->net.apply_adam(lr, s);
    if (e == cudaSuccess && loss_host) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? PRAY_OK : cuda_error(e, "denoiser train step");
}

pray_status pray_denoiser_set_tensor_cores(pray_denoiser *d, int32_t enable) {
    if (!d) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    d->net.set_tensor_cores(enable != 0);
    return PRAY_OK;
}

pray_status pray_denoiser_check(pray_denoiser *d) {
    if (!d) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    cudaSetDevice(d->net.device);
    bool ok = true;
    cudaError_t e = d->net.check(ok);
    if (e != cudaSuccess) return cuda_error(e, "denoiser check");
    if (!ok) return set_error(PRAY_ERR_CUDA, "a tensor-core convolution timed out waiting for its MMAs");
    return PRAY_OK;
}

pray_status pray_denoiser_gradients(pray_denoiser *d, const float *rad, const uint16_t *feat, const float *target,
                                    int32_t n, int32_t h, int32_t w, float *loss_host, float *grads_host) {
    if (!d || !rad || !feat || !target || !grads_host) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    pray_status st = check_dims(n, h, w);
    if (st != PRAY_OK) return st;
    cudaSetDevice(d->net.device);
    cudaError_t e = d->net.forward(rad, reinterpret_cast<const __half *>(feat), n, h, w, 0);
    if (e == cudaSuccess) e = d->net.backward(target, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess && loss_host) e = cudaMemcpy(loss_host, d->net.loss_device(), 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = d->net.get_grads(grads_host);
    return e == cudaSuccess ? PRAY_OK : cuda_error(e, "denoiser gradients");
}

pray_status pray_relmse(const double *img, double img_scale, const double *ref, double ref_scale, uint64_t n,
                        double *out, void *stream) {
    if (!img || !ref || !out) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    cudaError_t e = launch_relmse(img, img_scale, ref, ref_scale, n, out, (cudaStream_t)stream);
    return e == cudaSuccess ? PRAY_OK : cuda_error(e, "relmse launch");
}

pray_status pray_render_pt_host(pray_scene *s, const pray_pt_params *p, uint8_t *rgb_host, float *radiance_host,
                                uint64_t *rays_cast) {
    if (!s || !rgb_host) return set_error(PRAY_ERR_INVALID_ARGUMENT, "NULL argument");
    pray_status st = check_pt_params(p);
    if (st != PRAY_OK) return st;
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
    const uint64_t px = p->width * p->height;
    if ((st = ensure_frame(s, 3 * px + (radiance_host ? 12 * px : 0))) != PRAY_OK) return st;
    if ((e = cudaMemsetAsync(s->d_counters, 0, 2 * sizeof(unsigned long long), 0)) != cudaSuccess)
        return cuda_error(e, "cudaMemsetAsync");
    PtLaunch L = make_pt_launch(p);
    L.rgb = s->d_rgb;
    L.radiance = radiance_host ? reinterpret_cast<float *>(s->d_rgb + ((3 * px + 15) & ~15ull)) : nullptr;
    L.counters = s->d_counters;
    if ((st = run_pt(s, L, p->scheduler, p->wavefront_paths, 0)) != PRAY_OK) return st;
    if ((e = cudaMemcpy(rgb_host, s->d_rgb, 3 * px, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_error(e, "cudaMemcpy (frame)");
    if (radiance_host &&
        (e = cudaMemcpy(radiance_host, L.radiance, 12 * px, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_error(e, "cudaMemcpy (radiance)");
    if (rays_cast) {
        unsigned long long c[2];
        if ((e = cudaMemcpy(c, s->d_counters, sizeof(c), cudaMemcpyDeviceToHost)) != cudaSuccess)
            return cuda_error(e, "cudaMemcpy (counters)");
        rays_cast[0] = c[0];
        rays_cast[1] = c[1];
    }
    return PRAY_OK;
}

}  // extern "C"
