// Uses the C++ façade as the reference's main.cpp uses loadScene and
// RayTracer (main.cpp:74-200): a scene directory in the reference's format
// is loaded, rendered progressively, and saved as HDR.
//   load_scene <scene dir> <spp> <out.hdr>
#include <cstdio>
#include <cstdlib>
#include <memory>

#include "pgx.hpp"

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s <scene dir> <spp> <out.hdr>\n", argv[0]);
        return 2;
    }
    const int spp = std::atoi(argv[2]);
    try {
        std::unique_ptr<pgx::Scene> scene(pgx::loadScene(argv[1]));
        pgx::RayTracer rt(PGX_MODE_PLAIN, 8, 1);
        rt.init(scene.get());
        while (rt.getSPP() < spp) rt.render();
        rt.saveHDR(argv[3]);
        std::vector<float> img = rt.image();
        double sum = 0.0;
        for (float v : img) sum += v;
        std::printf("triangles=%zu width=%d height=%d spp=%d mean=%.6f\n", scene->triangleCount(),
                    scene->camera().width, scene->camera().height, rt.getSPP(), sum / (double)img.size());
    } catch (const pgx::Error& e) {
        std::printf("error %d: %s\n", e.code(), e.what());
        return 1;
    }
    try {
        std::unique_ptr<pgx::Scene> missing(pgx::loadScene("/nonexistent/scene"));
        return 1;
    } catch (const pgx::Error& e) {
        std::printf("expected error: %s\n", e.what());
    }
    return 0;
}
