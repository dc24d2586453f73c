// Host-side geometry for scene preparation: the per-triangle precompute and
// the box arithmetic the tree builders use. Every operation rounds exactly as
// the reference's scalar build does (this file is compiled with
// -ffp-contract=off), because the trees must come out identical to the
// reference's, split planes included.
#pragma once

#include <cmath>
#include <cstdint>
#include <limits>

namespace pray_gpu {

// std::min / std::max select semantics: the first argument on ties and NaN
// (the reference's BoundingBox code uses std::min/std::max throughout).
inline float fmin_sel(float a, float b) { return (b < a) ? b : a; }
inline float fmax_sel(float a, float b) { return (a < b) ? b : a; }

struct F3 {
    float v[3];
    float &operator[](int i) { return v[i]; }
    float operator[](int i) const { return v[i]; }
};

inline F3 f3(float x, float y, float z) { return F3{{x, y, z}}; }
inline F3 operator+(const F3 &a, const F3 &b) { return f3(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
inline F3 operator-(const F3 &a, const F3 &b) { return f3(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
inline float dot3(const F3 &a, const F3 &b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline F3 cross3(const F3 &a, const F3 &b) {
    return f3(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}
// Vec3::normalize (include/geometry.h:29-35)
inline F3 unit(F3 a) {
    float n2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    if (n2 > 0) {
        float inv = 1 / std::sqrt(n2);
        a[0] *= inv, a[1] *= inv, a[2] *= inv;
    }
    return a;
}

struct Aabb {
    F3 lo, hi;
    // BoundingBox::expand (include/geometry.h:110-117)
    Aabb grown(const Aabb &b) const {
        return Aabb{f3(fmin_sel(lo[0], b.lo[0]), fmin_sel(lo[1], b.lo[1]), fmin_sel(lo[2], b.lo[2])),
                    f3(fmax_sel(hi[0], b.hi[0]), fmax_sel(hi[1], b.hi[1]), fmax_sel(hi[2], b.hi[2]))};
    }
    // BoundingBox::clip (include/geometry.h:119-126): this = triangle box, b = voxel
    Aabb clipped(const Aabb &b) const {
        return Aabb{f3(fmax_sel(lo[0], b.lo[0]), fmax_sel(lo[1], b.lo[1]), fmax_sel(lo[2], b.lo[2])),
                    f3(fmin_sel(hi[0], b.hi[0]), fmin_sel(hi[1], b.hi[1]), fmin_sel(hi[2], b.hi[2]))};
    }
    // BoundingBox::getLongestAxis (include/geometry.h:132-149)
    int longest() const {
        float x = hi[0] - lo[0], y = hi[1] - lo[1], z = hi[2] - lo[2];
        if (x >= y && x >= z) return 0;
        if (y >= x && y >= z) return 1;
        return 2;
    }
    // BoundingBox::surfaceArea (include/geometry.h:186-192)
    float area() const {
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return 2.f * (dx * dy + dx * dz + dy * dz);
    }
};

// Per-triangle data of initialiseTriangles (src/scene_preprocessor.cpp:74-96).
struct TriPre {
    F3 a, ab, ac, normal, mid;
    Aabb box;
};

inline TriPre precompute_triangle(const float *v9) {
    TriPre t;
    F3 a = f3(v9[0], v9[1], v9[2]), b = f3(v9[3], v9[4], v9[5]), c = f3(v9[6], v9[7], v9[8]);
    t.a = a;
    for (int k = 0; k < 3; k++) {
        t.box.lo[k] = fmin_sel(a[k], fmin_sel(b[k], c[k]));
        t.box.hi[k] = fmax_sel(a[k], fmax_sel(b[k], c[k]));
    }
    F3 s = (a + b) + c;
    t.mid = f3(s[0] / 3, s[1] / 3, s[2] / 3);
    t.ab = b - a;
    t.ac = c - a;
    t.normal = unit(cross3(t.ab, t.ac));
    return t;
}

}  // namespace pray_gpu
