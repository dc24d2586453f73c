// Pinhole camera constants of calculatePrimRays (src/scene_preprocessor.cpp:98-136).
// The host computes the inverse view matrix and the per-image factors in the
// reference's operation order; the kernels generate each primary ray from
// them with the same float arithmetic.
#pragma once

#include <cstdint>

namespace pray_gpu {

struct CameraConsts {
    float m[3][3];  // rows 0-2, columns 0-2 of the inverse view matrix
    float pos[3];
    float inv_w, inv_h, aspect, angle;
    uint32_t width, height;
};

CameraConsts make_camera(uint64_t width, uint64_t height, uint64_t fov, const float pos[3], const float look[3]);

}  // namespace pray_gpu
