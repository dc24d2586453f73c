// `pray_scene_dump <scene.json> <out.bin>`: reads a scene with the same loader
// as `Pray` and writes what it read, for comparing the loader with the
// reference's (readSceneDescription, src/io.cpp:27-137). Layout, little
// endian: 17 doubles (width, height, fov, mode, max_depth, num_samples,
// camera_position[3], camera_look[3], background[3], n_lights, n_triangles),
// then verts (n x 9 float), colors (n x 3 float), emit (n bytes),
// lights (n_lights x 6 float).
#include <cstdio>
#include <string>

#include "scene_io.h"

int main(int argc, char **argv) {
    if (argc != 3) {
        std::printf("usage: %s <input.json> <output.bin>\n", argv[0]);
        return 1;
    }
    pray_cli::SceneDesc s;
    std::string err;
    if (!pray_cli::read_scene(argv[1], s, err)) {
        std::fprintf(stderr, "%s\n", err.c_str());
        return 1;
    }
    const double info[17] = {(double)s.width, (double)s.height, (double)s.fov, s.path_tracing ? 1.0 : 0.0,
                             (double)s.max_depth, (double)s.num_samples, s.cam_pos[0], s.cam_pos[1], s.cam_pos[2],
                             s.cam_look[0], s.cam_look[1], s.cam_look[2], s.background[0], s.background[1],
                             s.background[2], (double)(s.lights.size() / 6), (double)s.emit.size()};
    std::FILE *f = std::fopen(argv[2], "wb");
    if (!f) return 1;
    std::fwrite(info, sizeof(double), 17, f);
    std::fwrite(s.verts.data(), sizeof(float), s.verts.size(), f);
    std::fwrite(s.colors.data(), sizeof(float), s.colors.size(), f);
    std::fwrite(s.emit.data(), 1, s.emit.size(), f);
    std::fwrite(s.lights.data(), sizeof(float), s.lights.size(), f);
    return std::fclose(f) == 0 ? 0 : 1;
}
