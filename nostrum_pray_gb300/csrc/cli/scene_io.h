// Scene files of the reference's command line: JSON description
// (src/io.cpp:27-137), Wavefront OBJ/MTL geometry, 24-bit BMP output
// (src/main.cpp:93). Errors are returned, never fatal.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace pray_cli {

struct SceneDesc {
    bool path_tracing = false;
    uint64_t max_depth = 0, num_samples = 0;
    uint64_t width = 0, height = 0, fov = 0;
    float cam_pos[3] = {0, 0, 0}, cam_look[3] = {0, 0, 1};
    float background[3] = {0, 0, 0};
    std::vector<float> lights;   // n x 6
    std::vector<float> verts;    // n x 9
    std::vector<float> colors;   // n x 3
    std::vector<uint8_t> emit;   // n
    // optional keys of this framework (ignored by the reference's loader)
    int tree = -1;               // -1: the reference's choice by triangle count
    int leaf_size = 32, max_depth_tree = 20;
    float sah_ct = 5.f, sah_ci = 1.5f, det_epsilon = 1e-4f;
    uint64_t seed = 0;
};

// Reads the JSON file and the OBJ/MTL files it names. Returns false and
// sets err on failure.
bool read_scene(const std::string &json_path, SceneDesc &out, std::string &err);

// 24-bit BMP of a width x height x 3 RGB image stored top row first.
bool write_bmp(const std::string &path, uint64_t width, uint64_t height, const uint8_t *rgb);

}  // namespace pray_cli
