// ORACLE — test infrastructure, not product code.
//
// FP64 restatement of the denoiser's U-Net forward pass, L1 loss and
// backward pass (nostrum_pray_gb300/csrc/denoise_net.cpp, denoise_ops.cu),
// used only by tests to check the CUDA kernels' outputs and gradients. The
// network has no counterpart in the reference. Values the device stores in
// BF16 (packed input, convolution outputs, pooled tensors, weights) are
// rounded to BF16 at the same points here, so the comparison isolates the
// kernels' arithmetic from the storage format; everything else is double.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

using Vec = std::vector<double>;

double bf16(double x) {
    float f = (float)x;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7F800000u) == 0x7F800000u) return f;  // inf / nan unchanged
    const uint32_t lsb = (u >> 16) & 1u;
    u += 0x7FFFu + lsb;  // round to nearest even
    u &= 0xFFFF0000u;
    std::memcpy(&f, &u, 4);
    return f;
}

double half_to_double(uint16_t h) {
    const int s = h >> 15, e = (h >> 10) & 31, m = h & 1023;
    double v;
    if (e == 0) v = std::ldexp((double)m, -24);
    else if (e == 31) v = m ? NAN : INFINITY;
    else v = std::ldexp((double)(m | 1024), e - 25);
    return s ? -v : v;
}

struct T {
    int n, h, w, c;
    Vec v;
    double &at(int i, int y, int x, int ch) { return v[(((size_t)i * h + y) * w + x) * c + ch]; }
    double at(int i, int y, int x, int ch) const { return v[(((size_t)i * h + y) * w + x) * c + ch]; }
};

T make(int n, int h, int w, int c) { return T{n, h, w, c, Vec((size_t)n * h * w * c, 0.0)}; }

struct Conv {
    int cin, cout;
    bool relu;
    size_t off;
};

const int kConvs[][3] = {{10, 32, 1},  {32, 32, 1},  {32, 48, 1}, {48, 48, 1}, {48, 64, 1},
                         {64, 64, 1},  {64, 96, 1},  {96, 96, 1}, {96, 128, 1}, {128, 128, 1},
                         {224, 96, 1}, {96, 96, 1},  {160, 64, 1}, {64, 64, 1}, {112, 48, 1},
                         {48, 48, 1},  {80, 32, 1},  {32, 32, 1}, {32, 3, 0}};

// y = conv3x3(x) + b (zero padding), weights [cout][9][cin] (rounded to BF16)
T conv_fwd(const T &x, const Conv &c, const float *p, bool round_out) {
    T y = make(x.n, x.h, x.w, c.cout);
    const float *w = p + c.off, *b = p + c.off + (size_t)c.cout * 9 * c.cin;
    std::vector<double> wq((size_t)c.cout * 9 * c.cin);
    for (size_t k = 0; k < wq.size(); k++) wq[k] = bf16(w[k]);
    for (int i = 0; i < x.n; i++)
        for (int yy = 0; yy < x.h; yy++)
            for (int xx = 0; xx < x.w; xx++)
                for (int co = 0; co < c.cout; co++) {
                    double acc = 0.0;
                    for (int t = 0; t < 9; t++) {
                        const int sy = yy + t / 3 - 1, sx = xx + t % 3 - 1;
                        if (sy < 0 || sx < 0 || sy >= x.h || sx >= x.w) continue;
                        const double *wr = &wq[((size_t)co * 9 + t) * c.cin];
                        for (int ci = 0; ci < c.cin; ci++) acc += x.at(i, sy, sx, ci) * wr[ci];
                    }
                    double v = acc + (double)b[co];
                    if (c.relu && v < 0) v = 0;
                    y.at(i, yy, xx, co) = round_out ? bf16(v) : v;
                }
    return y;
}

// gradients of conv: input x, masked output gradient g; adds into dw/db,
// returns dx
T conv_bwd(const T &x, const T &g, const Conv &c, const float *p, double *dw, double *db) {
    T dx = make(x.n, x.h, x.w, c.cin);
    const float *w = p + c.off;
    for (int i = 0; i < x.n; i++)
        for (int yy = 0; yy < x.h; yy++)
            for (int xx = 0; xx < x.w; xx++)
                for (int co = 0; co < c.cout; co++) {
                    const double gv = g.at(i, yy, xx, co);
                    if (gv == 0.0) continue;
                    db[co] += gv;
                    for (int t = 0; t < 9; t++) {
                        const int sy = yy + t / 3 - 1, sx = xx + t % 3 - 1;
                        if (sy < 0 || sx < 0 || sy >= x.h || sx >= x.w) continue;
                        for (int ci = 0; ci < c.cin; ci++) {
                            dw[((size_t)co * 9 + t) * c.cin + ci] += gv * x.at(i, sy, sx, ci);
                            dx.at(i, sy, sx, ci) += gv * bf16(w[((size_t)co * 9 + t) * c.cin + ci]);
                        }
                    }
                }
    return dx;
}

T mask(const T &y, const T &g) {
    T o = g;
    for (size_t k = 0; k < o.v.size(); k++)
        if (!(y.v[k] > 0)) o.v[k] = 0;
    return o;
}

T pool(const T &x) {
    T y = make(x.n, x.h / 2, x.w / 2, x.c);
    for (int i = 0; i < x.n; i++)
        for (int yy = 0; yy < y.h; yy++)
            for (int xx = 0; xx < y.w; xx++)
                for (int ch = 0; ch < x.c; ch++)
                    y.at(i, yy, xx, ch) = bf16(0.25 * (x.at(i, 2 * yy, 2 * xx, ch) + x.at(i, 2 * yy, 2 * xx + 1, ch) +
                                                       x.at(i, 2 * yy + 1, 2 * xx, ch) +
                                                       x.at(i, 2 * yy + 1, 2 * xx + 1, ch)));
    return y;
}

void pool_bwd(const T &gy, T &gx) {
    for (int i = 0; i < gx.n; i++)
        for (int yy = 0; yy < gx.h; yy++)
            for (int xx = 0; xx < gx.w; xx++)
                for (int ch = 0; ch < gx.c; ch++) gx.at(i, yy, xx, ch) += 0.25 * gy.at(i, yy / 2, xx / 2, ch);
}

// concat(up(low), skip) along channels
T up_cat(const T &low, const T &skip) {
    T y = make(skip.n, skip.h, skip.w, low.c + skip.c);
    for (int i = 0; i < y.n; i++)
        for (int yy = 0; yy < y.h; yy++)
            for (int xx = 0; xx < y.w; xx++) {
                for (int ch = 0; ch < low.c; ch++) y.at(i, yy, xx, ch) = low.at(i, yy / 2, xx / 2, ch);
                for (int ch = 0; ch < skip.c; ch++) y.at(i, yy, xx, low.c + ch) = skip.at(i, yy, xx, ch);
            }
    return y;
}

// Demodulation divisor of radiance value i: first-hit albedo of its channel
// (feature i % 3 of pixel i / 3), clamped at 0, plus 0.05, in float as on the
// device.
float demod(const uint16_t *feat, size_t i) {
    return std::fmax((float)half_to_double(feat[7 * (i / 3) + i % 3]), 0.f) + 0.05f;
}

}  // namespace

extern "C" {

uint64_t orc_unet_num_params() {
    uint64_t t = 0;
    for (const auto &c : kConvs) t += (uint64_t)c[1] * 9 * c[0] + c[1];
    return t;
}

// One forward + backward pass of the U-Net. rad: n*h*w*3, feat: n*h*w*7 FP16
// bits, target: n*h*w*3. Radiance and target are divided by the albedo
// demodulation before log1p. out: n*h*w*3 network output (log space);
// grads: orc_unet_num_params() doubles; returns the L1 loss.
double orc_unet(const float *params, const float *rad, const uint16_t *feat, const float *target, int n, int h,
                int w, double *out, double *grads) {
    std::vector<Conv> cv;
    size_t off = 0;
    for (const auto &c : kConvs) {
        cv.push_back(Conv{c[0], c[1], c[2] != 0, off});
        off += (size_t)c[1] * 9 * c[0] + c[1];
    }
    T x0 = make(n, h, w, 10);
    const size_t px = (size_t)n * h * w;
    for (size_t p = 0; p < px; p++) {
        for (int k = 0; k < 3; k++)
            x0.v[p * 10 + k] = bf16(std::log1p((double)(std::fmax(rad[3 * p + k], 0.f) / demod(feat, 3 * p + k))));
        for (int k = 0; k < 7; k++) x0.v[p * 10 + 3 + k] = bf16(half_to_double(feat[7 * p + k]));
    }
    // forward
    std::vector<T> e(5), ea(5), pl(5);
    T cur = x0;
    for (int l = 0; l < 5; l++) {
        if (l > 0) {
            pl[l] = pool(e[l - 1]);
            cur = pl[l];
        }
        ea[l] = conv_fwd(cur, cv[2 * l], params, true);
        e[l] = conv_fwd(ea[l], cv[2 * l + 1], params, true);
    }
    std::vector<T> cat(4), da(4), d(4);  // index by level 0..3
    T low = e[4];
    for (int l = 3; l >= 0; l--) {
        const int k = 3 - l;
        cat[l] = up_cat(low, e[l]);
        da[l] = conv_fwd(cat[l], cv[10 + 2 * k], params, true);
        d[l] = conv_fwd(da[l], cv[11 + 2 * k], params, true);
        low = d[l];
    }
    T y = conv_fwd(d[0], cv[18], params, false);
    for (size_t p = 0; p < px; p++)
        for (int k = 0; k < 3; k++) y.v[p * 3 + k] += x0.v[p * 10 + k];  // residual on the input
    // loss
    const size_t nv = px * 3;
    double loss = 0.0;
    T gy = make(n, h, w, 3);
    for (size_t k = 0; k < nv; k++) {
        const double diff = y.v[k] - (double)log1pf(std::fmax(target[k], 0.f) / demod(feat, k));
        loss += std::fabs(diff);
        gy.v[k] = (diff > 0 ? 1.0 : (diff < 0 ? -1.0 : 0.0)) / (double)nv;
    }
    loss /= (double)nv;
    if (out) std::memcpy(out, y.v.data(), nv * sizeof(double));
    std::vector<double> g(off, 0.0);
    auto dw = [&](int ci) { return g.data() + cv[ci].off; };
    auto db = [&](int ci) { return g.data() + cv[ci].off + (size_t)cv[ci].cout * 9 * cv[ci].cin; };
    // backward: decoder from the output (level 0) down to level 3, whose
    // upsampled input is the bottleneck e4
    std::vector<T> ge(5);
    for (int l = 0; l < 5; l++) ge[l] = make(e[l].n, e[l].h, e[l].w, e[l].c);
    T gd = conv_bwd(d[0], gy, cv[18], params, dw(18), db(18));
    std::vector<T> gdl(4);
    gdl[0] = gd;
    for (int l = 0; l <= 3; l++) {
        const int k = 3 - l;
        T g2 = mask(d[l], gdl[l]);
        T gda = conv_bwd(da[l], g2, cv[11 + 2 * k], params, dw(11 + 2 * k), db(11 + 2 * k));
        T g1 = mask(da[l], gda);
        T gcat = conv_bwd(cat[l], g1, cv[10 + 2 * k], params, dw(10 + 2 * k), db(10 + 2 * k));
        const T &lowt = (l == 3) ? e[4] : d[l + 1];
        T glow = make(lowt.n, lowt.h, lowt.w, lowt.c);
        for (int i = 0; i < gcat.n; i++)
            for (int yy = 0; yy < gcat.h; yy++)
                for (int xx = 0; xx < gcat.w; xx++) {
                    for (int ch = 0; ch < lowt.c; ch++) glow.at(i, yy / 2, xx / 2, ch) += gcat.at(i, yy, xx, ch);
                    for (int ch = 0; ch < e[l].c; ch++) ge[l].at(i, yy, xx, ch) += gcat.at(i, yy, xx, lowt.c + ch);
                }
        if (l == 3) {
            for (size_t q = 0; q < glow.v.size(); q++) ge[4].v[q] += glow.v[q];
        } else {
            gdl[l + 1] = glow;
        }
    }
    // encoder, deepest first
    for (int l = 4; l >= 0; l--) {
        T g2 = mask(e[l], ge[l]);
        T gea = conv_bwd(ea[l], g2, cv[2 * l + 1], params, dw(2 * l + 1), db(2 * l + 1));
        T g1 = mask(ea[l], gea);
        const T &in = (l == 0) ? x0 : pl[l];
        T gin = conv_bwd(in, g1, cv[2 * l], params, dw(2 * l), db(2 * l));
        if (l > 0) pool_bwd(gin, ge[l - 1]);
    }
    std::memcpy(grads, g.data(), off * sizeof(double));
    return loss;
}

}  // extern "C"
