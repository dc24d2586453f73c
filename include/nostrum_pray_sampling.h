/*
 * Random stream and direction sampling of the GB300 path tracer, compiled
 * unchanged for the host and the device so that a path traced on the GPU and
 * the same path traced on the CPU take bit-identical directions.
 *
 * The reference's path tracers draw from a wall-clock-seeded mt19937_64 on
 * the CPU (src/pray.cpp:331,357) and curand XORWOW on the GPU
 * (src/path_trace.cu:428,449); neither stream is reproducible across the two.
 * Here every sample of every pixel owns one PCG32 stream (M. E. O'Neill, "PCG:
 * A Family of Simple Fast Space-Efficient Statistically Good Algorithms for
 * Random Number Generation", 2014; the pcg32 "XSH RR" output on a 64-bit LCG
 * with an odd per-stream increment), selected by (seed, pixel, sample).
 *
 * Hemisphere sampling follows sampleHemisphere (src/geometry.cpp:4-29): the
 * same cosine-weighted polar angle, the same tangent frame and the same sum
 * order. Its transcendentals are replaced by exact identities and a
 * polynomial: theta = acos(sqrt(1-u1)) gives cos(theta) = sqrt(1-u1) and
 * sin(theta) = sqrt(u1) (IEEE square roots), and cos/sin(2*pi*u2) come from
 * sincos_turns below (quadrant reduction on the turn count, Taylor series of
 * degree 9/10 on |x| <= pi/4; truncation error < 2e-9, total error a few
 * float ulps).
 *
 * Every operation is written with explicit round-to-nearest multiply / add so
 * that no compiler contracts them into FMAs on either side.
 */
#ifndef NOSTRUM_PRAY_SAMPLING_H
#define NOSTRUM_PRAY_SAMPLING_H

#include <stdint.h>

#if defined(__CUDACC__)
#define PRAY_HD __host__ __device__ __forceinline__
#else
#define PRAY_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define PRAY_MUL(a, b) __fmul_rn((a), (b))
#define PRAY_ADD(a, b) __fadd_rn((a), (b))
#define PRAY_SQRT(a) __fsqrt_rn(a)
#define PRAY_DIV(a, b) __fdiv_rn((a), (b))
#else
#include <math.h>
/* host: compiled with -ffp-contract=off */
#define PRAY_MUL(a, b) ((a) * (b))
#define PRAY_ADD(a, b) ((a) + (b))
#define PRAY_SQRT(a) sqrtf(a)
#define PRAY_DIV(a, b) ((a) / (b))
#endif

typedef struct {
    uint64_t state;
    uint64_t inc;
} pray_pcg32;

PRAY_HD uint32_t pray_pcg32_next(pray_pcg32 *g) {
    const uint64_t old = g->state;
    g->state = old * 6364136223846793005ULL + g->inc;
    const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
}

/* Stream of sample `sample` of pixel `pixel` (row-major index) under `seed`. */
PRAY_HD pray_pcg32 pray_pcg32_stream(uint64_t seed, uint64_t pixel, uint32_t sample) {
    pray_pcg32 g;
    g.state = 0u;
    g.inc = (((pixel << 32) ^ (uint64_t)sample) << 1u) | 1u;
    pray_pcg32_next(&g);
    g.state += seed ^ 0x853c49e6748fea9bULL;
    pray_pcg32_next(&g);
    return g;
}

/* Uniform float in [0, 1): the top 24 bits. */
PRAY_HD float pray_uniform(pray_pcg32 *g) { return (float)(pray_pcg32_next(g) >> 8) * (1.0f / 16777216.0f); }

/* cos and sin of 2*pi*u for u in [0, 1). */
PRAY_HD void pray_sincos_turns(float u, float *s_out, float *c_out) {
    /* nearest quarter turn k, remainder r in [-1/8, 1/8] (exact: u and k/4
     * are multiples of 2^-24) */
    const float q = PRAY_MUL(u, 4.0f);
    const int k = (int)(q + 0.5f);
    const float r = PRAY_ADD(u, PRAY_MUL((float)k, -0.25f));
    const float x = PRAY_MUL(r, 6.28318530717958647692f);
    const float x2 = PRAY_MUL(x, x);
    /* sin x = x (1 - x^2/3! + x^4/5! - x^6/7! + x^8/9!) */
    float ps = 2.7557319223985893e-6f;
    ps = PRAY_ADD(PRAY_MUL(ps, x2), -1.9841269841269841e-4f);
    ps = PRAY_ADD(PRAY_MUL(ps, x2), 8.3333333333333333e-3f);
    ps = PRAY_ADD(PRAY_MUL(ps, x2), -1.6666666666666667e-1f);
    ps = PRAY_ADD(PRAY_MUL(ps, x2), 1.0f);
    const float s = PRAY_MUL(ps, x);
    /* cos x = 1 - x^2/2! + x^4/4! - x^6/6! + x^8/8! - x^10/10! */
    float pc = -2.7557319223985891e-7f;
    pc = PRAY_ADD(PRAY_MUL(pc, x2), 2.4801587301587302e-5f);
    pc = PRAY_ADD(PRAY_MUL(pc, x2), -1.3888888888888889e-3f);
    pc = PRAY_ADD(PRAY_MUL(pc, x2), 4.1666666666666667e-2f);
    pc = PRAY_ADD(PRAY_MUL(pc, x2), -0.5f);
    const float c = PRAY_ADD(PRAY_MUL(pc, x2), 1.0f);
    switch (k & 3) {
        case 0: *s_out = s; *c_out = c; break;
        case 1: *s_out = c; *c_out = -s; break;
        case 2: *s_out = -s; *c_out = -c; break;
        default: *s_out = -c; *c_out = s; break;
    }
}

/* Normalise in place (Vec3::normalize, include/geometry.h:29-35). */
PRAY_HD void pray_normalize3(float *v) {
    const float n2 = PRAY_ADD(PRAY_ADD(PRAY_MUL(v[0], v[0]), PRAY_MUL(v[1], v[1])), PRAY_MUL(v[2], v[2]));
    if (n2 > 0.f) {
        const float inv = PRAY_DIV(1.0f, PRAY_SQRT(n2));
        v[0] = PRAY_MUL(v[0], inv);
        v[1] = PRAY_MUL(v[1], inv);
        v[2] = PRAY_MUL(v[2], inv);
    }
}

/* Cosine-weighted direction about the unit normal n (sampleHemisphere,
 * src/geometry.cpp:4-29). */
PRAY_HD void pray_sample_hemisphere(const float *n, float u1, float u2, float *dir) {
    const float cos_t = PRAY_SQRT(PRAY_ADD(1.0f, -u1));
    const float sin_t = PRAY_SQRT(u1);
    float sin_p, cos_p;
    pray_sincos_turns(u2, &sin_p, &cos_p);
    float h[3] = {n[0], n[1], n[2]};
    const float ax = fabsf(h[0]), ay = fabsf(h[1]), az = fabsf(h[2]);
    if (ax <= ay && ax <= az) h[0] = 1.f;
    else if (ay <= ax && ay <= az) h[1] = 1.f;
    else h[2] = 1.f;
    /* x = h x n, z = x x n */
    float x[3] = {PRAY_ADD(PRAY_MUL(h[1], n[2]), -PRAY_MUL(h[2], n[1])),
                  PRAY_ADD(PRAY_MUL(h[2], n[0]), -PRAY_MUL(h[0], n[2])),
                  PRAY_ADD(PRAY_MUL(h[0], n[1]), -PRAY_MUL(h[1], n[0]))};
    pray_normalize3(x);
    float z[3] = {PRAY_ADD(PRAY_MUL(x[1], n[2]), -PRAY_MUL(x[2], n[1])),
                  PRAY_ADD(PRAY_MUL(x[2], n[0]), -PRAY_MUL(x[0], n[2])),
                  PRAY_ADD(PRAY_MUL(x[0], n[1]), -PRAY_MUL(x[1], n[0]))};
    pray_normalize3(z);
    const float sx = PRAY_MUL(sin_t, cos_p), sy = cos_t, sz = PRAY_MUL(sin_t, sin_p);
    for (int k = 0; k < 3; k++)
        dir[k] = PRAY_ADD(PRAY_ADD(PRAY_MUL(x[k], sx), PRAY_MUL(n[k], sy)), PRAY_MUL(z[k], sz));
    pray_normalize3(dir);
}

#endif /* NOSTRUM_PRAY_SAMPLING_H */
