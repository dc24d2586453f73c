// `Pray <input.json> <output.bmp>`: the reference's command line
// (src/main.cpp:23-109) on the GB300 path. Same arguments, exit codes and
// output image; the phase log goes to stdout.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../../include/nostrum_pray.h"
#include "scene_io.h"

namespace {

using clk = std::chrono::steady_clock;
long ms_since(clk::time_point t) {
    return (long)std::chrono::duration_cast<std::chrono::milliseconds>(clk::now() - t).count();
}

// Tree choice of preprocessScene (src/scene_preprocessor.cpp:42-57,
// include/options.h:32-36): SAH for 20,000 <= n < 1,000,000 triangles, the
// median tree otherwise and for path-traced scenes small enough for the
// reference's GPU path (< 10,000 triangles).
int reference_tree_choice(const pray_cli::SceneDesc &s) {
    const size_t n = s.emit.size();
    if (s.path_tracing && n < 10000) return PRAY_TREE_MEDIAN;
    if (n < 20000 || n >= 1000000) return PRAY_TREE_MEDIAN;
    return PRAY_TREE_SAH;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 3) {
        std::printf("usage: %s <input.json> <output.bmp>\n", argv[0]);
        return 1;
    }
    const auto total = clk::now();
    std::printf("--------------------------------------------------------\nINPUT FILE: %s\n\n", argv[1]);
    std::printf("Reading scene description...\n");
    auto t0 = clk::now();
    pray_cli::SceneDesc scene;
    std::string err;
    if (!pray_cli::read_scene(argv[1], scene, err)) {
        std::fprintf(stderr, "%s\n", err.c_str());
        return 1;
    }
    std::printf("Finished reading scene description. (%ld ms)\n\n", ms_since(t0));
    const uint64_t n = scene.emit.size();
    std::printf("Scene information: Resolution: %llux%llu, # Lights: %zu, # Triangles: %llu",
                (unsigned long long)scene.width, (unsigned long long)scene.height, scene.lights.size() / 6,
                (unsigned long long)n);
    if (scene.path_tracing)
        std::printf(", PATH TRACING: max depth: %llu, # samples: %llu", (unsigned long long)scene.max_depth,
                    (unsigned long long)scene.num_samples);
    std::printf("\n\n");

    pray_tree_options opt;
    pray_tree_options_default(&opt);
    opt.tree = scene.tree >= 0 ? scene.tree : reference_tree_choice(scene);
    opt.leaf_size = scene.leaf_size;
    opt.max_depth = scene.max_depth_tree;
    opt.sah_traversal_cost = scene.sah_ct;
    opt.sah_intersection_cost = scene.sah_ci;

    std::printf("Preprocessing scene...\n");
    t0 = clk::now();
    pray_scene *s = nullptr;
    if (pray_scene_create(scene.verts.data(), scene.colors.data(), scene.emit.data(), n, &opt, 0, &s) != PRAY_OK) {
        std::fprintf(stderr, "scene set-up failed: %s\n", pray_last_error());
        return 1;
    }
    uint64_t st[8];
    pray_scene_stats(s, st);
    std::printf("\t# nodes: %llu, tree depth: %llu, leaf nodes: %llu (%s)\n", (unsigned long long)st[0],
                (unsigned long long)st[1], (unsigned long long)st[2], opt.tree == PRAY_TREE_SAH ? "SAH" : "median");
    std::printf("Preprocessing time: %ld ms\n", ms_since(t0));

    std::vector<uint8_t> image(3 * scene.width * scene.height);
    t0 = clk::now();
    pray_status rc;
    if (!scene.path_tracing) {
        std::printf("\nRendering scene with ray tracing on the GPU...\n");
        pray_rt_params p{};
        p.width = scene.width;
        p.height = scene.height;
        p.fov = scene.fov;
        for (int k = 0; k < 3; k++) {
            p.camera_position[k] = scene.cam_pos[k];
            p.camera_look[k] = scene.cam_look[k];
            p.background[k] = scene.background[k];
        }
        p.lights = scene.lights.data();
        p.n_lights = (int32_t)(scene.lights.size() / 6);
        p.det_epsilon = scene.det_epsilon;
        uint64_t rays[2] = {0, 0};
        rc = pray_render_rt_host(s, &p, image.data(), rays);
        if (rc == PRAY_OK)
            std::printf("\t%llu primary + %llu shadow rays\n", (unsigned long long)rays[0], (unsigned long long)rays[1]);
    } else {
        std::printf("Rendering scene with path tracing on the GPU...\n");
        pray_pt_params p{};
        p.width = scene.width;
        p.height = scene.height;
        p.fov = scene.fov;
        for (int k = 0; k < 3; k++) {
            p.camera_position[k] = scene.cam_pos[k];
            p.camera_look[k] = scene.cam_look[k];
            p.background[k] = scene.background[k];
        }
        p.max_depth = (uint32_t)scene.max_depth;
        p.num_samples = (uint32_t)scene.num_samples;
        // the reference's mode choice (src/scene_preprocessor.cpp:34-40, MAX_DEPTH_DIFFUSE = 1 in
        // include/options.h:32): branching up to depth 1, one bounce per sample above it
        if (scene.max_depth > 1) {
            std::printf("\tUsing normal path tracing.\n");
            p.mode = PRAY_PT_KAJIYA;
        } else {
            std::printf("\tUsing diffuse path tracing.\n");
            p.mode = PRAY_PT_DIFFUSE;
        }
        p.seed = scene.seed;
        p.det_epsilon = scene.det_epsilon;
        rc = pray_render_pt_host(s, &p, image.data(), nullptr, nullptr);
    }
    if (rc != PRAY_OK) {
        std::fprintf(stderr, "rendering failed: %s\n", pray_last_error());
        pray_scene_destroy(s);
        return 1;
    }
    std::printf("Finished rendering. (%ld ms)\n", ms_since(t0));
    pray_scene_destroy(s);

    std::printf("Writing result image...\n");
    t0 = clk::now();
    if (!pray_cli::write_bmp(argv[2], scene.width, scene.height, image.data())) {
        std::fprintf(stderr, "writing the BMP failed\n");
        return 1;
    }
    std::printf("Finished writing. (%ld ms)\n", ms_since(t0));
    std::printf("Total time: %ld ms\n\n", ms_since(total));
    return 0;
}
