// Uses the C++ façade the way the reference's main.cpp uses its classes:
// build a scene, render frames progressively, read SPP, save an HDR.  The
// scene is a closed-top box with a ceiling light, built in code.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "pgx.hpp"

static pgx_vertex vtx(float x, float y, float z, float nx, float ny, float nz) {
    pgx_vertex v{};
    v.p[0] = x; v.p[1] = y; v.p[2] = z;
    v.n[0] = nx; v.n[1] = ny; v.n[2] = nz;
    return v;
}

static void quad(std::vector<pgx_triangle>& out, const float o[3], const float u[3], const float v[3],
                 const float n[3], uint32_t mat) {
    float p[4][3];
    for (int k = 0; k < 3; k++) {
        p[0][k] = o[k];
        p[1][k] = o[k] + u[k];
        p[2][k] = o[k] + u[k] + v[k];
        p[3][k] = o[k] + v[k];
    }
    int tri[2][3] = {{0, 1, 2}, {0, 2, 3}};
    for (auto& t : tri) {
        pgx_triangle tr{};
        for (int k = 0; k < 3; k++) tr.v[k] = vtx(p[t[k]][0], p[t[k]][1], p[t[k]][2], n[0], n[1], n[2]);
        tr.material = mat;
        out.push_back(tr);
    }
}

static double image_mean(const std::vector<float>& img) {
    double m = 0;
    for (float v : img) m += v;
    return m / (double)img.size();
}

int main(int argc, char** argv) {
    const char* out = argc > 1 ? argv[1] : "box.hdr";
    const bool guided = argc > 2 && std::string(argv[2]) == "guided";
    std::vector<pgx_material> mats(2);
    for (auto& m : mats) {
        m = pgx_material{};
        m.kind = PGX_BSDF_DIFFUSE;
        m.albedo_texture = -1;
        m.albedo[0] = m.albedo[1] = m.albedo[2] = 0.7f;
        m.int_ior = 1.5f;
        m.ext_ior = 1.f;
    }
    mats[1].emission[0] = mats[1].emission[1] = mats[1].emission[2] = 17.f;
    std::vector<pgx_triangle> tris;
    float fl[3] = {-1, 0, -1}, ux[3] = {2, 0, 0}, uz[3] = {0, 0, 2}, uy[3] = {0, 2, 0};
    float up[3] = {0, 1, 0}, dn[3] = {0, -1, 0}, fw[3] = {0, 0, 1}, rt[3] = {1, 0, 0}, lf[3] = {-1, 0, 0};
    float ce[3] = {-1, 2, -1}, back[3] = {-1, 0, -1}, right[3] = {1, 0, -1};
    quad(tris, fl, ux, uz, up, 0);
    quad(tris, ce, ux, uz, dn, 0);
    quad(tris, back, ux, uy, fw, 0);
    quad(tris, back, uz, uy, rt, 0);
    quad(tris, right, uz, uy, lf, 0);
    float lo[3] = {-0.25f, 1.999f, -0.25f}, lu[3] = {0.5f, 0, 0}, lv[3] = {0, 0, 0.5f};
    quad(tris, lo, lu, lv, dn, 1);
    pgx_camera cam{};
    float from[3] = {0, 1, 3.8f}, to[3] = {0, 1, 0}, upv[3] = {0, 1, 0};
    for (int k = 0; k < 3; k++) {
        cam.from[k] = from[k];
        cam.to[k] = to[k];
        cam.up[k] = upv[k];
    }
    cam.fov_degrees = 40.f;
    cam.width = 64;
    cam.height = 64;
    try {
        pgx::Scene scene(0);
        scene.init(tris, mats, nullptr, cam);
        scene.build();
        if (guided) {
            // Plain and QuadTree-guided images of the same box at 256 spp.
            pgx::RayTracer plain(PGX_MODE_PLAIN, 8, 11);
            plain.init(&scene);
            plain.render(256);
            const double mp = image_mean(plain.image());
            pgx::RayTracer g(PGX_MODE_GUIDED_QUADTREE, 8, 12);
            g.config().guide_fraction = 0.7f;
            g.init(&scene);
            const pgx_guide_params gp = pgx::RayTracer::recommendedGuideParams();
            g.trainGuide(4, 2, &gp);  // 4 unguided + 8 guided frames, kept in the film
            g.render(256 - g.getSPP());
            std::printf("guided spp=%d mean_guided=%.6f mean_plain=%.6f\n", g.getSPP(), image_mean(g.image()), mp);
            return 0;
        }
        pgx::RayTracer tracer(PGX_MODE_PLAIN, 8, 1);
        tracer.init(&scene);
        while (tracer.getSPP() < 8) tracer.render();
        std::vector<float> img = tracer.image();
        double mean = 0;
        for (float v : img) mean += v;
        mean /= (double)img.size();
        tracer.saveHDR(out);
        pgx_render_stats st = tracer.stats();
        std::printf("spp=%d mean=%.5f bvh_nodes=%lld rays=%lld\n", tracer.getSPP(), mean,
                    (long long)scene.bvhStats().nodes, (long long)(st.extension_rays + st.shadow_rays));
        if (!(mean > 0.01 && mean < 10.0)) return 2;
        // Errors come back as exceptions.
        try {
            pgx::RayTracer bad;
            bad.render();
            return 3;
        } catch (const pgx::Error& e) {
            std::printf("expected error: %s\n", e.what());
        }
    } catch (const pgx::Error& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
