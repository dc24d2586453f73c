#include "scene_io.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>

namespace pray_cli {

namespace {

// ------------------------------------------------------------------ JSON
// Numbers keep the distinction the reference's JSON library makes: integer
// literals are held exactly as 64-bit integers, anything with a fraction or
// exponent is read with strtod; conversions to float / unsigned happen at
// the use site, as the reference's assignments do.

struct JValue {
    enum Kind { Null, Bool, UInt, Int, Float, Str, Arr, Obj } kind = Null;
    bool b = false;
    uint64_t u = 0;
    int64_t i = 0;
    double f = 0;
    std::string s;
    std::vector<JValue> arr;
    std::map<std::string, JValue> obj;

    bool is_number() const { return kind == UInt || kind == Int || kind == Float; }
    double as_double() const { return kind == UInt ? (double)u : kind == Int ? (double)i : f; }
    float as_float() const { return kind == UInt ? (float)u : kind == Int ? (float)i : (float)f; }
    uint64_t as_u64() const { return kind == UInt ? u : kind == Int ? (uint64_t)i : (uint64_t)f; }
    const JValue *get(const char *k) const {
        if (kind != Obj) return nullptr;
        auto it = obj.find(k);
        return it == obj.end() ? nullptr : &it->second;
    }
};

struct JParser {
    const char *p, *e;
    std::string err;

    void ws() {
        while (p < e && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++;
    }
    bool fail(const char *m) {
        if (err.empty()) err = m;
        return false;
    }
    bool lit(const char *w) {
        size_t n = std::strlen(w);
        if ((size_t)(e - p) < n || std::strncmp(p, w, n) != 0) return false;
        p += n;
        return true;
    }
    bool string(std::string &out) {
        if (p >= e || *p != '"') return fail("expected string");
        p++;
        while (p < e && *p != '"') {
            if (*p == '\\') {
                p++;
                if (p >= e) return fail("bad escape");
                switch (*p) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': {
                        if (e - p < 5) return fail("bad \\u escape");
                        unsigned cp = (unsigned)std::strtoul(std::string(p + 1, p + 5).c_str(), nullptr, 16);
                        if (cp < 0x80) {
                            out += (char)cp;
                        } else if (cp < 0x800) {
                            out += (char)(0xC0 | (cp >> 6));
                            out += (char)(0x80 | (cp & 0x3F));
                        } else {
                            out += (char)(0xE0 | (cp >> 12));
                            out += (char)(0x80 | ((cp >> 6) & 0x3F));
                            out += (char)(0x80 | (cp & 0x3F));
                        }
                        p += 4;
                        break;
                    }
                    default: out += *p;
                }
                p++;
            } else {
                out += *p++;
            }
        }
        if (p >= e) return fail("unterminated string");
        p++;
        return true;
    }
    bool number(JValue &v) {
        const char *s = p;
        bool neg = false, is_float = false, overflow = false;
        if (p < e && *p == '-') neg = true, p++;
        uint64_t acc = 0;
        const uint64_t lim = neg ? (uint64_t)INT64_MAX + 1 : UINT64_MAX;
        if (p >= e || !(*p >= '0' && *p <= '9')) return fail("bad number");
        while (p < e && *p >= '0' && *p <= '9') {
            const uint64_t d = (uint64_t)(*p - '0');
            if (acc > (lim - d) / 10) overflow = true;
            else acc = acc * 10 + d;
            p++;
        }
        if (p < e && *p == '.') {
            is_float = true;
            p++;
            while (p < e && *p >= '0' && *p <= '9') p++;
        }
        if (p < e && (*p == 'e' || *p == 'E')) {
            is_float = true;
            p++;
            if (p < e && (*p == '+' || *p == '-')) p++;
            while (p < e && *p >= '0' && *p <= '9') p++;
        }
        if (is_float || overflow) {
            v.kind = JValue::Float;
            v.f = std::strtod(std::string(s, p).c_str(), nullptr);
            if (!std::isfinite(v.f)) v.kind = JValue::Null;
        } else if (neg) {
            v.kind = JValue::Int;
            v.i = (int64_t)(0 - acc);
        } else {
            v.kind = JValue::UInt;
            v.u = acc;
        }
        return true;
    }
    bool value(JValue &v, int depth) {
        if (depth > 256) return fail("nesting too deep");
        ws();
        if (p >= e) return fail("unexpected end");
        if (*p == '{') {
            v.kind = JValue::Obj;
            p++;
            ws();
            if (p < e && *p == '}') return p++, true;
            while (true) {
                ws();
                std::string k;
                if (!string(k)) return false;
                ws();
                if (p >= e || *p != ':') return fail("expected ':'");
                p++;
                JValue item;
                if (!value(item, depth + 1)) return false;
                v.obj[k] = std::move(item);
                ws();
                if (p < e && *p == ',') { p++; continue; }
                if (p < e && *p == '}') { p++; return true; }
                return fail("expected ',' or '}'");
            }
        }
        if (*p == '[') {
            v.kind = JValue::Arr;
            p++;
            ws();
            if (p < e && *p == ']') return p++, true;
            while (true) {
                JValue item;
                if (!value(item, depth + 1)) return false;
                v.arr.push_back(std::move(item));
                ws();
                if (p < e && *p == ',') { p++; continue; }
                if (p < e && *p == ']') { p++; return true; }
                return fail("expected ',' or ']'");
            }
        }
        if (*p == '"') {
            v.kind = JValue::Str;
            return string(v.s);
        }
        if (lit("true")) { v.kind = JValue::Bool; v.b = true; return true; }
        if (lit("false")) { v.kind = JValue::Bool; v.b = false; return true; }
        if (lit("null")) { v.kind = JValue::Null; return true; }
        return number(v);
    }
};

bool read_file(const std::string &path, std::string &out) {
    std::ifstream f(path, std::ios::binary);
    if (!f.good()) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

bool vec3(const JValue *v, float out[3]) {
    if (!v || v->kind != JValue::Arr || v->arr.size() < 3) return false;
    for (int k = 0; k < 3; k++) {
        if (!v->arr[k].is_number()) return false;
        out[k] = v->arr[k].as_float();
    }
    return true;
}

// ------------------------------------------------------------------ OBJ
// Wavefront OBJ/MTL reading with the semantics of the tinyobjloader 1.0.x
// that the reference vendors (ext/tiny_obj_loader.h): its own decimal
// parser (digits accumulated in double, exponent applied as
// ldexp(m * 5^e, e), then rounded to float), polygon faces fanned into
// triangles (v0, v[k-1], v[k]), 1-based / negative-relative indices, per-face
// material ids taken when the face group is flushed, and the loader's
// shape-flushing rules (a face group moved into a shape by `usemtl` is kept
// only if more faces follow before the next `o`/`g`).

bool obj_number(const char *s, const char *end, double &out) {
    if (s >= end) return false;
    double mant = 0.0;
    int expo = 0, read = 0;
    char sign = '+', esign = '+';
    const char *c = s;
    auto digit = [](char ch) { return (unsigned)(ch - '0') < 10u; };
    if (*c == '+' || *c == '-') sign = *c++;
    else if (!digit(*c)) return false;
    bool more = c != end;
    while (more && digit(*c)) {
        mant *= 10;
        mant += (int)(*c - '0');
        c++, read++;
        more = c != end;
    }
    if (read == 0) return false;
    if (!more) goto done;
    if (*c == '.') {
        static const double tenth[8] = {1.0, 0.1, 0.01, 0.001, 0.0001, 0.00001, 0.000001, 0.0000001};
        c++;
        read = 1;
        more = c != end;
        while (more && digit(*c)) {
            mant += (int)(*c - '0') * (read < 8 ? tenth[read] : std::pow(10.0, -read));
            read++, c++;
            more = c != end;
        }
    } else if (!(*c == 'e' || *c == 'E')) {
        goto done;
    }
    if (!more) goto done;
    if (*c == 'e' || *c == 'E') {
        c++;
        more = c != end;
        if (more && (*c == '+' || *c == '-')) esign = *c++;
        else if (!digit(*c)) return false;
        read = 0;
        more = c != end;
        while (more && digit(*c)) {
            expo = expo * 10 + (int)(*c - '0');
            c++, read++;
            more = c != end;
        }
        expo *= (esign == '+' ? 1 : -1);
        if (read == 0) return false;
    }
done:
    out = (sign == '+' ? 1 : -1) * (expo ? std::ldexp(mant * std::pow(5.0, expo), expo) : mant);
    return true;
}

float obj_float(const char *&tok, double dflt = 0.0) {
    tok += std::strspn(tok, " \t");
    const char *end = tok + std::strcspn(tok, " \t\r");
    double v = dflt;
    obj_number(tok, end, v);
    tok = end;
    return (float)v;
}

std::string first_word(const char *tok) {
    tok += std::strspn(tok, " \t");
    size_t n = std::strcspn(tok, " \t\r\n");
    return std::string(tok, n);
}

bool space(char c) { return c == ' ' || c == '\t'; }

struct Material {
    std::string name;
    float kd[3] = {0, 0, 0}, ke[3] = {0, 0, 0};
};

void trim_line(std::string &l, bool trailing_space) {
    if (trailing_space && !l.empty()) l = l.substr(0, l.find_last_not_of(" \t") + 1);
    if (!l.empty() && l.back() == '\n') l.pop_back();
    if (!l.empty() && l.back() == '\r') l.pop_back();
}

// Lines end at \n, \r\n or \r (safeGetline).
bool next_line(std::istream &in, std::string &l) {
    l.clear();
    if (in.peek() == EOF) return false;
    while (true) {
        int c = in.get();
        if (c == EOF) return true;
        if (c == '\n') return true;
        if (c == '\r') {
            if (in.peek() == '\n') in.get();
            return true;
        }
        l += (char)c;
    }
}

void load_mtl(const std::string &path, std::vector<Material> &mats, std::map<std::string, int> &index) {
    std::ifstream in(path);
    Material cur;
    std::string line;
    while (in && next_line(in, line)) {
        trim_line(line, true);
        if (line.empty()) continue;
        const char *t = line.c_str();
        t += std::strspn(t, " \t");
        if (*t == '\0' || *t == '#') continue;
        if (std::strncmp(t, "newmtl", 6) == 0 && space(t[6])) {
            if (!cur.name.empty()) {
                index.insert({cur.name, (int)mats.size()});
                mats.push_back(cur);
            }
            cur = Material();
            cur.name = first_word(t + 7);
            continue;
        }
        if (t[0] == 'K' && t[1] == 'd' && space(t[2])) {
            t += 2;
            for (int k = 0; k < 3; k++) cur.kd[k] = obj_float(t);
            continue;
        }
        if (t[0] == 'K' && t[1] == 'e' && space(t[2])) {
            t += 2;
            for (int k = 0; k < 3; k++) cur.ke[k] = obj_float(t);
            continue;
        }
    }
    index.insert({cur.name, (int)mats.size()});
    mats.push_back(cur);
}

int fix_index(int idx, int n) {
    if (idx > 0) return idx - 1;
    if (idx == 0) return 0;
    return n + idx;
}

struct FaceTri {
    int v[3];
    int mat;
};

bool load_obj(const std::string &path, const std::string &mtl_dir, std::vector<float> &verts_out,
              std::vector<FaceTri> &tris, std::vector<Material> &mats, std::string &err) {
    std::ifstream in(path);
    if (!in) {
        err = "Error loading file: cannot open " + path;
        return false;
    }
    std::vector<float> v;
    std::vector<std::vector<int>> group;  // pending faces (vertex indices)
    std::vector<FaceTri> shape;           // triangles of the current shape
    std::map<std::string, int> index;
    int material = -1;
    int nvn = 0, nvt = 0;
    // exportFaceGroupToShape: fan-triangulate pending faces into `shape`
    auto flush = [&](int mat) {
        if (group.empty()) return false;
        for (const auto &f : group) {
            if (f.size() < 2) continue;
            int i0 = f[0], i2 = f[1];
            for (size_t k = 2; k < f.size(); k++) {
                int i1 = i2;
                i2 = f[k];
                shape.push_back(FaceTri{{i0, i1, i2}, mat});
            }
        }
        return true;
    };
    std::string line;
    while (next_line(in, line)) {
        trim_line(line, false);
        if (line.empty()) continue;
        const char *t = line.c_str();
        t += std::strspn(t, " \t");
        if (*t == '\0' || *t == '#') continue;
        if (t[0] == 'v' && space(t[1])) {
            t += 2;
            for (int k = 0; k < 3; k++) v.push_back(obj_float(t));
            continue;
        }
        if (t[0] == 'v' && t[1] == 'n' && space(t[2])) { nvn++; continue; }
        if (t[0] == 'v' && t[1] == 't' && space(t[2])) { nvt++; continue; }
        if (t[0] == 'f' && space(t[1])) {
            t += 2;
            t += std::strspn(t, " \t");
            std::vector<int> face;
            while (!(*t == '\r' || *t == '\n' || *t == '\0')) {
                face.push_back(fix_index(std::atoi(t), (int)(v.size() / 3)));
                // skip the rest of the i/j/k triple
                t += std::strcspn(t, " \t\r");
                t += std::strspn(t, " \t\r");
            }
            group.push_back(std::move(face));
            continue;
        }
        if (std::strncmp(t, "usemtl", 6) == 0 && space(t[6])) {
            const std::string name = first_word(t + 7);
            auto it = index.find(name);
            const int id = it == index.end() ? -1 : it->second;
            if (id != material) {
                flush(material);
                group.clear();
                material = id;
            }
            continue;
        }
        if (std::strncmp(t, "mtllib", 6) == 0 && space(t[6])) {
            load_mtl(mtl_dir + first_word(t + 7), mats, index);
            continue;
        }
        if ((t[0] == 'g' || t[0] == 'o') && space(t[1])) {
            if (flush(material)) tris.insert(tris.end(), shape.begin(), shape.end());
            shape.clear();
            group.clear();
            continue;
        }
    }
    const bool ret = flush(material);
    if (ret || !shape.empty()) tris.insert(tris.end(), shape.begin(), shape.end());
    verts_out.swap(v);
    (void)nvn, (void)nvt;
    return true;
}

std::string dir_of(const std::string &p) {
    size_t s = p.find_last_of('/');
    return s == std::string::npos ? std::string() : p.substr(0, s);
}

}  // namespace

bool read_scene(const std::string &json_path, SceneDesc &out, std::string &err) {
    std::string text;
    if (!read_file(json_path, text)) {
        err = "Error opening file: " + json_path;
        return false;
    }
    JParser jp{text.data(), text.data() + text.size(), {}};
    JValue root;
    if (!jp.value(root, 0) || root.kind != JValue::Obj) {
        err = "invalid JSON in " + json_path + ": " + jp.err;
        return false;
    }
    const JValue *obj = root.get("obj_file");
    if (!obj || obj->kind != JValue::Str) {
        err = "scene has no obj_file";
        return false;
    }
    const std::string base = dir_of(json_path);
    const std::string obj_path = base.empty() ? obj->s : base + "/" + obj->s;
    const std::string mtl_dir = base.empty() ? std::string() : base + "/";

    const JValue *m = root.get("method");
    out.path_tracing = m && m->kind == JValue::Str && m->s == "path_tracing";
    if (out.path_tracing) {
        const JValue *d = root.get("max_depth"), *n = root.get("num_samples");
        if (!d || !n || !d->is_number() || !n->is_number()) {
            err = "path tracing needs max_depth and num_samples";
            return false;
        }
        out.max_depth = d->as_u64();
        out.num_samples = n->as_u64();
    }
    const JValue *rx = root.get("resolution_x"), *ry = root.get("resolution_y"), *fov = root.get("fov");
    if (!rx || !ry || !fov || !rx->is_number() || !ry->is_number() || !fov->is_number()) {
        err = "scene needs resolution_x, resolution_y and fov";
        return false;
    }
    out.width = rx->as_u64();
    out.height = ry->as_u64();
    out.fov = fov->as_u64();
    if (!vec3(root.get("camera_position"), out.cam_pos) || !vec3(root.get("camera_look"), out.cam_look) ||
        !vec3(root.get("background"), out.background)) {
        err = "scene needs camera_position, camera_look and background";
        return false;
    }
    // lights are read for ray tracing only (src/io.cpp:91-97)
    const JValue *ls = root.get("lights");
    if (!out.path_tracing && ls && ls->kind == JValue::Arr) {
        for (const JValue &l : ls->arr) {
            float p[3], c[3];
            if (!vec3(l.get("position"), p) || !vec3(l.get("color"), c)) {
                err = "light needs position and color";
                return false;
            }
            out.lights.insert(out.lights.end(), {p[0], p[1], p[2], c[0], c[1], c[2]});
        }
    }
    // optional keys of this framework
    if (const JValue *t = root.get("tree"); t && t->kind == JValue::Str) out.tree = t->s == "sah" ? 1 : 0;
    if (const JValue *t = root.get("leaf_size"); t && t->is_number()) out.leaf_size = (int)t->as_u64();
    if (const JValue *t = root.get("tree_max_depth"); t && t->is_number()) out.max_depth_tree = (int)t->as_u64();
    if (const JValue *t = root.get("sah_traversal_cost"); t && t->is_number()) out.sah_ct = t->as_float();
    if (const JValue *t = root.get("sah_intersection_cost"); t && t->is_number()) out.sah_ci = t->as_float();
    if (const JValue *t = root.get("det_epsilon"); t && t->is_number()) out.det_epsilon = t->as_float();
    if (const JValue *t = root.get("seed"); t && t->is_number()) out.seed = t->as_u64();

    std::vector<float> v;
    std::vector<FaceTri> tris;
    std::vector<Material> mats;
    if (!load_obj(obj_path, mtl_dir, v, tris, mats, err)) return false;
    const int nv = (int)(v.size() / 3);
    out.verts.reserve(tris.size() * 9);
    for (const FaceTri &f : tris) {
        for (int k = 0; k < 3; k++) {
            const int vi = f.v[k];
            if (vi < 0 || vi >= nv) {
                err = "face references a missing vertex";
                return false;
            }
            out.verts.insert(out.verts.end(), {v[3 * vi], v[3 * vi + 1], v[3 * vi + 2]});
        }
        // per-face colour (src/io.cpp:127-134); faces without a valid
        // material (undefined in the reference) get a black diffuse colour
        Material mm;
        if (f.mat >= 0 && f.mat < (int)mats.size()) mm = mats[f.mat];
        const bool emissive = !(mm.ke[0] == 0.f && mm.ke[1] == 0.f && mm.ke[2] == 0.f);
        const float *c = emissive ? mm.ke : mm.kd;
        out.colors.insert(out.colors.end(), {c[0], c[1], c[2]});
        out.emit.push_back(emissive ? 1 : 0);
    }
    return true;
}

bool write_bmp(const std::string &path, uint64_t width, uint64_t height, const uint8_t *rgb) {
    if (width > 0x7FFFFFFF || height > 0x7FFFFFFF) return false;
    const uint32_t w = (uint32_t)width, h = (uint32_t)height;
    const uint32_t pad = (uint32_t)((-(int64_t)w * 3) & 3);
    const uint64_t file_size = 14 + 40 + (uint64_t)(w * 3 + pad) * h;
    std::FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    auto u16 = [&](uint32_t x) { uint8_t b[2] = {(uint8_t)x, (uint8_t)(x >> 8)}; std::fwrite(b, 1, 2, f); };
    auto u32 = [&](uint32_t x) {
        uint8_t b[4] = {(uint8_t)x, (uint8_t)(x >> 8), (uint8_t)(x >> 16), (uint8_t)(x >> 24)};
        std::fwrite(b, 1, 4, f);
    };
    // BITMAPFILEHEADER + BITMAPINFOHEADER (24 bpp, uncompressed, bottom-up)
    std::fputc('B', f);
    std::fputc('M', f);
    u32((uint32_t)file_size);
    u16(0);
    u16(0);
    u32(54);
    u32(40);
    u32(w);
    u32(h);
    u16(1);
    u16(24);
    for (int k = 0; k < 6; k++) u32(0);
    std::vector<uint8_t> row((size_t)w * 3 + pad, 0);
    for (uint64_t y = h; y-- > 0;) {
        const uint8_t *src = rgb + y * w * 3;
        for (uint32_t x = 0; x < w; x++) {
            row[3 * x] = src[3 * x + 2];
            row[3 * x + 1] = src[3 * x + 1];
            row[3 * x + 2] = src[3 * x];
        }
        std::fwrite(row.data(), 1, row.size(), f);
    }
    const bool ok = std::ferror(f) == 0;
    return std::fclose(f) == 0 && ok;
}

}  // namespace pray_cli
