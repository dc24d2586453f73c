#include "camera.h"

#include <cmath>
#include <cstring>
#include <utility>

#include "geom.h"

namespace pray_gpu {

namespace {

// 4x4 inverse by Gauss-Jordan elimination with partial pivoting, in the
// order of Matrix44::inverse (include/geometry.h:322-403): the primary rays
// must match the reference's bit for bit, so the elimination steps (pivot
// choice, row operations, back substitution) follow it exactly. A singular
// matrix yields the identity, as in the reference.
void inverse4(const float in[4][4], float out[4][4]) {
    float t[4][4];
    std::memcpy(t, in, sizeof(t));
    auto set_identity = [&] {
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) out[i][j] = (i == j) ? 1.f : 0.f;
    };
    set_identity();
    for (int col = 0; col < 3; col++) {
        int pivot = col;
        float size = std::fabs(t[col][col]);
        for (int row = col + 1; row < 4; row++) {
            const float a = std::fabs(t[row][col]);
            if (a > size) pivot = row, size = a;
        }
        if (size == 0) return set_identity();
        if (pivot != col) {
            for (int k = 0; k < 4; k++) {
                std::swap(t[col][k], t[pivot][k]);
                std::swap(out[col][k], out[pivot][k]);
            }
        }
        for (int row = col + 1; row < 4; row++) {
            const float f = t[row][col] / t[col][col];
            for (int k = 0; k < 4; k++) {
                t[row][k] -= f * t[col][k];
                out[row][k] -= f * out[col][k];
            }
        }
    }
    for (int row = 3; row >= 0; --row) {
        float f = t[row][row];
        if (f == 0) return set_identity();
        for (int k = 0; k < 4; k++) {
            t[row][k] /= f;
            out[row][k] /= f;
        }
        for (int up = 0; up < row; up++) {
            f = t[up][row];
            for (int k = 0; k < 4; k++) {
                t[up][k] -= f * t[row][k];
                out[up][k] -= f * out[row][k];
            }
        }
    }
}

}  // namespace

CameraConsts make_camera(uint64_t width, uint64_t height, uint64_t fov, const float pos[3], const float look[3]) {
    CameraConsts c;
    const F3 p = f3(pos[0], pos[1], pos[2]);
    const F3 target = p + f3(look[0], look[1], look[2]);
    const F3 up = f3(0, 1, 0);
    const F3 z = unit(target - p);
    const F3 x = unit(cross3(up, z));
    const F3 y = cross3(z, x);
    const float view[4][4] = {{x[0], y[0], z[0], 0},
                              {x[1], y[1], z[1], 0},
                              {x[2], y[2], z[2], 0},
                              {-dot3(x, p), -dot3(y, p), -dot3(z, p), 1}};
    float inv[4][4];
    inverse4(view, inv);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) c.m[i][j] = inv[i][j];
    for (int k = 0; k < 3; k++) c.pos[k] = pos[k];
    c.inv_w = 1 / float(width);
    c.inv_h = 1 / float(height);
    c.aspect = width / float(height);
    const float pi = static_cast<float>(std::acos(-1));
    c.angle = std::tan(pi * 0.5f * fov / 180.f);
    c.width = (uint32_t)width;
    c.height = (uint32_t)height;
    return c;
}

}  // namespace pray_gpu
