/*
 * nostrum_pray GB300 — C ABI of the ray-tracing hot path.
 *
 * Plain pointers and sizes only. Every function returns a pray_status; on an
 * error pray_last_error() gives a message (per calling thread). No function
 * exits the process (the reference does so inside library code:
 * src/io.cpp:33,57 and src/path_trace.cu:15).
 *
 * Threading: a pray_scene is not thread-safe; the caller serialises calls on
 * one handle. Different handles are independent. Device-pointer entry points
 * enqueue work on the given CUDA stream (NULL: the legacy default stream) and
 * do not synchronise; *_host entry points synchronise before returning.
 *
 * Reference interfaces replaced (paths in the reference project):
 *   SpatialDatabase::build / KDTree / KDTreeSAH   include/spatial.h:10-39,
 *                                                  src/kd_tree.cpp:18-84,
 *                                                  src/kd_tree_sah.cpp:25-138
 *   SpatialDatabase::intersect (per ray)           include/spatial.h:16,
 *                                                  src/kd_tree.cpp:142-279
 *   render / rayTrace                              include/pray.h:50-53,
 *                                                  src/pray.cpp:380-637
 */
#ifndef NOSTRUM_PRAY_H
#define NOSTRUM_PRAY_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PRAY_API_VERSION 1

typedef enum {
    PRAY_OK = 0,
    PRAY_ERR_INVALID_ARGUMENT = 1,
    PRAY_ERR_CUDA = 2,
    PRAY_ERR_OUT_OF_MEMORY = 3,
    PRAY_ERR_IO = 4,
    PRAY_ERR_UNSUPPORTED = 5
} pray_status;

typedef enum { PRAY_TREE_MEDIAN = 0, PRAY_TREE_SAH = 1 } pray_tree_kind;

/* Tree construction constants. The reference fixes them at compile time
 * (include/kd_tree.h:50-52, include/kd_tree_sah.h:49-50); here they are
 * arguments. pray_tree_options_default() fills the reference's values. */
typedef struct {
    int32_t tree;                  /* pray_tree_kind */
    int32_t leaf_size;             /* THRESHOLD: leaf at <= this many triangles (32) */
    int32_t max_depth;             /* MAX_DEPTH: leaf at this depth (20); at most 30 */
    float sah_traversal_cost;      /* traversalCost (5) */
    float sah_intersection_cost;   /* triangleIntersectionCost (1.5) */
    int32_t build_threads;         /* host threads for the build, 0 = all */
    int32_t leaf_refine;           /* device layout only: leaves with more references than this get a
                                      conservative sub-hierarchy (8; 0 = off). Results are unchanged. */
} pray_tree_options;

/* Ray-tracing frame parameters: the scene JSON's camera, lights and
 * background (src/io.cpp:60-101) plus the intersector's det threshold
 * (include/geometry.h:12, EPSILON = 1e-4 in the reference). */
typedef struct {
    uint64_t width, height;
    uint64_t fov;                  /* degrees, horizontal */
    float camera_position[3];
    float camera_look[3];
    float background[3];
    const float *lights;           /* host memory: n_lights x (position[3], colour[3]) */
    int32_t n_lights;              /* at most 64 */
    float det_epsilon;
} pray_rt_params;

/* Path-tracing frame parameters (scene JSON "method": "path_tracing",
 * src/io.cpp:60-63). */
typedef enum {
    PRAY_PT_KAJIYA = 0,   /* the reference's evaluatePathRecursive (src/pray.cpp:342-364) */
    PRAY_PT_NEE = 1,      /* next-event estimation + Russian roulette (no reference counterpart) */
    PRAY_PT_DIFFUSE = 2   /* the reference's branching evaluatePathRecursiveDiffuse (src/pray.cpp:315-340,
                             src/path_trace.cu:369-393): every non-emitting hit above max_depth spawns
                             num_samples bounce rays and returns albedo x their mean, so a pixel casts up to
                             1 + n + ... + n^max_depth rays; one estimate per pixel from the PCG32 stream
                             (seed, pixel, sample_offset); max_depth <= 8; PRAY_SCHED_PIXEL only. The
                             reference selects it when max_depth <= 1 (src/scene_preprocessor.cpp:34-40) */
} pray_pt_mode;

typedef enum {
    PRAY_SCHED_PIXEL = 0,      /* one thread per pixel, samples and bounces in a loop */
    PRAY_SCHED_WAVEFRONT = 1,  /* path pool + extend / shade / occlusion passes with compacted queues,
                                  one CUDA graph per frame; PRAY_PT_NEE only */
    PRAY_SCHED_AUTO = 2        /* PRAY_SCHED_WAVEFRONT for PRAY_PT_NEE frames of at least 2^19 paths
                                  (width x height x num_samples), PRAY_SCHED_PIXEL otherwise; both give
                                  the same result */
} pray_pt_scheduler;

typedef struct {
    uint64_t width, height;
    uint64_t fov;
    float camera_position[3];
    float camera_look[3];
    float background[3];
    uint32_t max_depth;            /* bounces: a hit at depth >= max_depth returns 0 */
    uint32_t num_samples;          /* paths per pixel (PRAY_PT_DIFFUSE: bounce rays per hit) */
    uint64_t seed;                 /* PCG32 streams per (seed, pixel, sample) */
    float det_epsilon;
    int32_t mode;                  /* pray_pt_mode */
    uint32_t rr_depth;             /* PRAY_PT_NEE: Russian roulette from this depth */
    int32_t scheduler;             /* pray_pt_scheduler */
    uint32_t sample_offset;        /* first sample index of this call (continues PCG streams across calls) */
    uint32_t wavefront_paths;      /* PRAY_SCHED_WAVEFRONT: paths in flight per round (0 = 2^23; at least
                                      one per pixel); a frame runs ceil(spp / (paths / pixels)) rounds */
} pray_pt_params;

typedef struct pray_scene pray_scene;
typedef struct pray_host_tree pray_host_tree;

const char *pray_last_error(void);
int32_t pray_api_version(void);
void pray_tree_options_default(pray_tree_options *opt);

/* ---- host-only tree build (no device work; for inspection and tests) ---- */

/* Precompute (initialiseTriangles, src/scene_preprocessor.cpp:74-96) and build
 * the tree. verts: n x 9 floats (a, b, c). */
pray_status pray_host_tree_build(const float *verts, uint64_t n, const pray_tree_options *opt,
                                 pray_host_tree **out);
void pray_host_tree_destroy(pray_host_tree *t);
/* out[5] = nodes, max depth, leaf nodes, empty leaf nodes, leaf references */
pray_status pray_host_tree_stats(const pray_host_tree *t, uint64_t *out);
/* Depth-first pre-order dump (left before right): per node box[6] (min, max),
 * split distance, info[4] = {is_leaf, split axis (255 for leaves), triangle
 * count, first reference}; refs = leaf triangle indices in DFS order. Array
 * sizes from pray_host_tree_stats. */
pray_status pray_host_tree_dump(const pray_host_tree *t, float *boxes, float *split, int32_t *info,
                                int64_t *refs);
/* Per triangle: box min[3], box max[3], midpoint[3], b-a[3], c-a[3], normal[3]. */
pray_status pray_host_tree_precompute(const pray_host_tree *t, float *out18);

/* The device layout this tree would be uploaded as (no device work):
 * out[4] = node records, triangle references, refined leaves, nodes added by
 * the refinement. Fails if the layout would not pass the upload checks. */
pray_status pray_host_tree_device_layout(const pray_host_tree *t, int32_t leaf_refine, uint64_t *out);

/* Camera constants the kernels use: inverse view matrix rows 0-2 (columns
 * 0-2), 1/width, 1/height, aspect, tan(fov/2) — 13 floats
 * (calculatePrimRays set-up, src/scene_preprocessor.cpp:98-120). */
pray_status pray_camera(uint64_t width, uint64_t height, uint64_t fov, const float *camera_position,
                        const float *camera_look, float *out13);

/* ---- device scenes ---- */

/* Builds the tree on the host and uploads nodes, triangle references and
 * shading data to `device`. The caller keeps its buffers. colors: n x 3
 * (albedo, or radiance when emit[i] != 0); emit may be NULL. */
pray_status pray_scene_create(const float *verts, const float *colors, const uint8_t *emit, uint64_t n,
                              const pray_tree_options *opt, int32_t device, pray_scene **out);
pray_status pray_scene_destroy(pray_scene *s);
/* out[8] = nodes, max depth, leaf nodes, empty leaf nodes, leaf references,
 *          triangles, device bytes held, device node records */
pray_status pray_scene_stats(const pray_scene *s, uint64_t *out);

/* Closest hit per ray (SpatialDatabase::intersect). rays_dev: n x 9 floats
 * (position, unit direction, 1/direction — the reference's Ray fields), all
 * device pointers. ids_dev: triangle index or -1; t_dev: distance, FLT_MAX on
 * a miss. Same triangle and distance as the reference's depth-first
 * traversal, ties included. */
pray_status pray_trace_closest(pray_scene *s, const float *rays_dev, uint64_t n, float det_epsilon,
                               int32_t *ids_dev, float *t_dev, void *stream);

/* Occlusion (shadow) rays: occluded_dev[i] = 1 iff some triangle is hit at
 * distance t > 0 with t * t < dist2_dev[i], else 0; the walk stops at the
 * first such triangle. The same answer as the reference's shadow test, the
 * closest hit followed by lightDistSq > dst * dst (src/pray.cpp:39-43);
 * dist2 <= 0 gives 0. rays_dev: n x 9 floats as for pray_trace_closest; all
 * device pointers. */
pray_status pray_trace_occluded(pray_scene *s, const float *rays_dev, const float *dist2_dev, uint64_t n,
                                float det_epsilon, uint8_t *occluded_dev, void *stream);

/* pray_trace_closest for rays in host memory, for host code that asks the
 * spatial database one ray or one batch at a time
 * (SpatialDatabase::intersect(const Ray&, Triangle&, float&),
 * include/spatial.h:16, which the reference's renderers call from many
 * OpenMP threads at once). rays_host: n x 9 floats as above; ids_host and
 * t_host receive n results. Returns when the results are in host memory.
 * Safe to call from several host threads on the same scene: calls on one
 * scene are serialised inside the library (one staging buffer per scene,
 * grown on demand, freed with the scene). Every call costs a launch and two
 * copies, so batches of thousands of rays amortise it; single rays work but
 * are slow. */
pray_status pray_trace_closest_host(pray_scene *s, const float *rays_host, uint64_t n, float det_epsilon,
                                    int32_t *ids_host, float *t_host);

/* Traversal of a scene's ray-traced frames: each lane walks its own ray
 * (LANES), or the warp walks its pixel tile's rays as one packet with a
 * mask of the lanes whose own box tests passed, for the primary and the
 * occlusion rays (PACKETS) or for the primary rays only (PRIMARY_PACKETS);
 * all return the same hits. AUTO (the default) times the three on the
 * scene's first ray-traced frame and keeps the fastest. */
typedef enum {
    PRAY_TRAVERSAL_AUTO = -1,
    PRAY_TRAVERSAL_LANES = 0,
    PRAY_TRAVERSAL_PACKETS = 1,
    PRAY_TRAVERSAL_PRIMARY_PACKETS = 2
} pray_traversal;
pray_status pray_scene_set_traversal(pray_scene *s, int32_t traversal);
/* The traversal in use (PRAY_TRAVERSAL_AUTO until the first frame chose). */
pray_status pray_scene_traversal(const pray_scene *s, int32_t *traversal);

/* One ray-traced frame into device memory: rgb_dev height x width x 3 bytes,
 * top row first (the reference's Image layout). ids_dev / t_dev (per pixel,
 * may be NULL) receive the primary hits. counters_dev (may be NULL) is
 * incremented by [primary rays, occlusion rays]. Under PRAY_TRAVERSAL_AUTO
 * the scene's first ray-traced frame (this call, pray_render_rt_host or
 * pray_render_rt_counts) renders the frame seven times to time the three
 * traversals, and synchronises. */
pray_status pray_render_rt(pray_scene *s, const pray_rt_params *p, uint8_t *rgb_dev, int32_t *ids_dev,
                           float *t_dev, unsigned long long *counters_dev, void *stream);

/* The same frame into host memory (render(Image&, const Scene&) of
 * include/pray.h:50): rgb_host height x width x 3 bytes. rays_cast (may be
 * NULL) receives [primary rays, occlusion rays]. Synchronises. */
pray_status pray_render_rt_host(pray_scene *s, const pray_rt_params *p, uint8_t *rgb_host,
                                uint64_t *rays_cast);

/* Work counts of one ray-traced frame, from an instrumented run of the same
 * kernel: out[5] = primary rays, occlusion rays, node-pair fetches (64 bytes
 * each), triangle-reference fetches (48 bytes each), shaded hits. */
pray_status pray_render_rt_counts(pray_scene *s, const pray_rt_params *p, uint64_t *out);

/* One path-traced frame (pathTrace, src/pray.cpp:592-615) into device
 * memory: rgb_dev as for pray_render_rt (may be NULL when radiance_dev is
 * given); radiance_dev (may be NULL) receives
 * the per-pixel mean radiance (height x width x 3 floats) before clamping;
 * counters_dev (may be NULL) is incremented by [paths, ray segments]. The
 * frame runs on the scene's own stream, after `stream`'s earlier work and
 * before its later work; frames of one scene run one after another. */
pray_status pray_render_pt(pray_scene *s, const pray_pt_params *p, uint8_t *rgb_dev, float *radiance_dev,
                           unsigned long long *counters_dev, void *stream);

/* The same into host memory; radiance_host and rays_cast ([paths, segments])
 * may be NULL. Synchronises. */
pray_status pray_render_pt_host(pray_scene *s, const pray_pt_params *p, uint8_t *rgb_host, float *radiance_host,
                                uint64_t *rays_cast);

/* FP64 accumulation for converged references: adds the radiance of samples
 * [sample_offset, sample_offset + num_samples) of every pixel to sum_dev
 * (height x width x 3 doubles, caller-initialised), one sample at a time in
 * sample order, so repeated calls over consecutive sample ranges give the
 * same sums as one call. Device pointers; enqueued on `stream`. Not for
 * PRAY_PT_DIFFUSE (PRAY_ERR_UNSUPPORTED). */
pray_status pray_accumulate_pt(pray_scene *s, const pray_pt_params *p, double *sum_dev,
                               unsigned long long *counters_dev, void *stream);

/* Allocation-free path tracing (no counterpart in the reference). For host
 * applications that must not have this library allocate device memory during
 * a frame: engines that reserve all GPU memory up front for their own pool
 * allocator, and frame loops that cannot afford cudaMalloc/cudaFree's
 * implicit device synchronisation. The same frame, bit for bit, as
 * pray_render_pt with PRAY_SCHED_WAVEFRONT (PRAY_PT_NEE only; p->scheduler is
 * ignored; the pool may be smaller, which changes how samples are split into
 * rounds but not the per-pixel sums, added in sample order), but the
 * path pool lives in a fixed 160 MiB static device array that every GPU
 * loading this library holds until exit; frames above 1,103,744 pixels are
 * rejected with PRAY_ERR_INVALID_ARGUMENT. Calls no cudaMalloc/cudaFree. The
 * first call on each device looks up the array's address and loads every
 * kernel a frame may launch: make it before any stream capture. All calls share the array, so
 * calls that overlap on the GPU race; order them (one stream, or events).
 * rgb_dev / radiance_dev / counters_dev as for pray_render_pt (at least one
 * of rgb_dev, radiance_dev). */
pray_status pray_render_pt_noalloc(pray_scene *s, const pray_pt_params *p, uint8_t *rgb_dev, float *radiance_dev,
                                   unsigned long long *counters_dev, void *stream);

/* ---- batches: many scenes in one persistent launch (no reference counterpart) ---- */

typedef struct pray_batch pray_batch;

/* Launch shape of a batch: 32-pixel tiles (tile_w x tile_h == 32), threads
 * per block, resident blocks per SM of the persistent grid (0 = as many as
 * fit), traversal stack entries (32 or 64; 32 only when every scene's device
 * hierarchy is shallower than 32). */
typedef struct {
    int32_t tile_w, tile_h;
    int32_t block_threads;
    int32_t blocks_per_sm;
    int32_t stack_entries;
} pray_batch_config;

/* Records n scenes (all on one device) with one path-tracing frame each:
 * params[i] as for pray_render_pt (scheduler and wavefront_paths ignored;
 * PRAY_PT_KAJIYA or PRAY_PT_NEE),
 * rgb_dev[i] / radiance_dev[i] its outputs (device pointers; each may be
 * NULL, not both). The scenes must outlive the batch. */
pray_status pray_batch_create(pray_scene *const *scenes, const pray_pt_params *params, uint8_t *const *rgb_dev,
                              float *const *radiance_dev, int32_t n, pray_batch **out);
pray_status pray_batch_destroy(pray_batch *b);
pray_status pray_batch_set_config(pray_batch *b, const pray_batch_config *cfg);
/* Autotuner: times every candidate launch shape on the batch with one sample
 * per pixel, keeps the fastest and returns it (best_ms: its time). Writes the
 * outputs (with the one-sample frames). Synchronises. */
pray_status pray_batch_tune(pray_batch *b, pray_batch_config *chosen, float *best_ms);
/* Renders every scene's frame in one persistent launch (a memset and the
 * kernel, captured once into a CUDA graph per launch shape) ordered after
 * `stream`'s earlier work and before its later work. counters_dev (may be
 * NULL): [paths, segments] accumulated; it is part of the captured graph, so
 * keep passing the same pointer (a different one re-captures). */
pray_status pray_batch_render(pray_batch *b, unsigned long long *counters_dev, void *stream);

/* ---- learned denoiser (no reference counterpart) ---- */

/* First-hit features for the denoiser (camera of p): per pixel albedo (or
 * emitted colour) 3, geometric normal 3, hit distance 1 as FP16 bits,
 * height x width x 7 (zeros on a miss). */
pray_status pray_render_features(pray_scene *s, const pray_pt_params *p, uint16_t *features_dev, void *stream);

typedef struct pray_denoiser pray_denoiser;

/* Five-level convolutional U-Net (channels 32-48-64-96-128, two 3x3
 * convolutions with ReLU per level, 2x2 average pooling, nearest 2x
 * upsampling, concatenated skips, 3x3 output convolution), BF16 weights and
 * activations, FP32 accumulation. Radiance is demodulated: divided per
 * channel by the first-hit albedo feature (clamped at 0) + 0.05 before the
 * network and multiplied by it after. Input per pixel: log(1 + demodulated
 * noisy radiance), the 7 features; output: radiance, as log(1 + demodulated
 * noisy radiance) plus the network's correction, re-modulated. Weights
 * He-initialised from seed (the output
 * convolution scaled by 0.1, so an untrained network returns its input).
 * Parameter vector: per convolution in forward order, weights
 * [cout][3][3][cin] then biases [cout]. */
pray_status pray_denoiser_create(int32_t device, uint64_t seed, pray_denoiser **out);
pray_status pray_denoiser_destroy(pray_denoiser *d);
pray_status pray_denoiser_num_params(const pray_denoiser *d, uint64_t *n);
pray_status pray_denoiser_get_params(const pray_denoiser *d, float *host);
pray_status pray_denoiser_set_params(pray_denoiser *d, const float *host);
/* Denoises n images of h x w (multiples of 16): radiance_dev n*h*w*3 floats,
 * features_dev n*h*w*7 FP16, out_dev n*h*w*3 floats (device pointers),
 * ordered after `stream`'s earlier work. The first call with a set of
 * pointers and sizes runs its kernels on the stream and records them in a
 * CUDA graph; a following call with the same pointers, sizes and kernel
 * choice launches that graph. */
pray_status pray_denoise(pray_denoiser *d, const float *radiance_dev, const uint16_t *features_dev, int32_t n,
                         int32_t h, int32_t w, float *out_dev, void *stream);
/* One Adam step (lr; betas 0.9 / 0.999) on the L1 loss between the network
 * output and log(1 + target_dev / demodulation). loss_host (may be NULL)
 * receives the loss before
 * the step (synchronises). */
pray_status pray_denoiser_train_step(pray_denoiser *d, const float *radiance_dev, const uint16_t *features_dev,
                                     const float *target_dev, int32_t n, int32_t h, int32_t w, float lr,
                                     float *loss_host, void *stream);
/* Forward convolutions on the tcgen05 tensor cores (enable != 0, the
 * default) or on the CUDA cores. The backward pass runs on the CUDA cores. */
pray_status pray_denoiser_set_tensor_cores(pray_denoiser *d, int32_t enable);
/* Synchronises and reports PRAY_ERR_CUDA if a tensor-core kernel's bounded
 * wait on its MMA completion ran out since the denoiser was created. */
pray_status pray_denoiser_check(pray_denoiser *d);
/* Loss and parameter gradients without an update (synchronises):
 * grads_host has pray_denoiser_num_params floats. */
pray_status pray_denoiser_gradients(pray_denoiser *d, const float *radiance_dev, const uint16_t *features_dev,
                                    const float *target_dev, int32_t n, int32_t h, int32_t w, float *loss_host,
                                    float *grads_host);

/* Relative mean squared error of an image against a reference, reduced in
 * FP64 on the device: mean over pixels and channels of
 * (x - r)^2 / (r^2 + 0.01), with x = img_scale * img[i], r = ref_scale * ref[i]
 * (the scales turn sums into means). n = values (pixels x 3). out_dev: one
 * double. */
pray_status pray_relmse(const double *img_dev, double img_scale, const double *ref_dev, double ref_scale,
                        uint64_t n, double *out_dev, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* NOSTRUM_PRAY_H */
