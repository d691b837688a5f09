// pgx.hpp — C++ façade over the C ABI in pgx.h, keeping the reference's class
// names and call pattern (PathGuidingDissertation/main.cpp:147-199):
//
//   pgx::Scene* scene = pgx::loadScene("Scenes/cornell-box");  // SceneLoader.h:222
//   // or: pgx::Scene scene; scene.init(triangles, materials, envmap, camera);
//   //     scene.build();             // Scene::build: BVH on the GPU, lights
//   pgx::RayTracer rt;                 // RayTracer (Renderer.h:236-752)
//   rt.init(scene);
//   while (rt.getSPP() < spp) rt.render();
//   rt.saveHDR("GI.hdr");
//
// Header-only; link with -lpgx.  Errors throw pgx::Error (the C ABI returns
// status codes; the reference printed and carried on or exited).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "pgx.h"

namespace pgx {

class Error : public std::runtime_error {
  public:
    Error(int code, const std::string& msg) : std::runtime_error(msg), code_(code) {}
    int code() const { return code_; }

  private:
    int code_;
};

inline void check(pgx_ctx* ctx, int rc) {
    if (rc != PGX_OK) throw Error(rc, std::string("pgx: ") + pgx_last_error(ctx));
}

// One device context (owns the GPU memory of a scene).
class Context {
  public:
    explicit Context(int device = 0) {
        int rc = pgx_create(device, &h_);
        if (rc != PGX_OK) throw Error(rc, std::string("pgx_create: ") + pgx_last_error(nullptr));
    }
    ~Context() { pgx_destroy(h_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    pgx_ctx* get() const { return h_; }

  private:
    pgx_ctx* h_ = nullptr;
};

// Reference `Scene`: triangles, materials, background, camera, BVH.
class Scene {
  public:
    explicit Scene(int device = 0) : ctx_(device) {}

    // Scene::init (Scene.h:121-137).  envmap may be null (black background).
    void init(const std::vector<pgx_triangle>& triangles, const std::vector<pgx_material>& materials,
              const pgx_texture* envmap, const pgx_camera& camera,
              const std::vector<pgx_texture>& textures = {}) {
        triangles_ = triangles;
        camera_ = camera;
        check(ctx_.get(), pgx_scene_upload(ctx_.get(), triangles.data(), (int64_t)triangles.size(), materials.data(),
                                           (int32_t)materials.size(), textures.empty() ? nullptr : textures.data(),
                                           (int32_t)textures.size(), envmap, &camera));
    }

    // Reads a scene directory in the reference's format (scene.json, .gem
    // meshes, textures; SceneLoader.h:104-269) and uploads it (Scene::init).
    void load(const std::string& dir) {
        pgx_scene_data* d = nullptr;
        char msg[512];
        int rc = pgx_scene_read(dir.c_str(), &d, msg, (int32_t)sizeof(msg));
        if (rc != PGX_OK) throw Error(rc, std::string("pgx: loadScene: ") + msg);
        triangles_.assign(d->triangles, d->triangles + d->ntris);
        camera_ = d->camera;
        rc = pgx_scene_upload(ctx_.get(), d->triangles, d->ntris, d->materials, d->nmats,
                              d->ntextures ? d->textures : nullptr, d->ntextures, d->has_env ? &d->env : nullptr,
                              &d->camera);
        pgx_scene_data_free(d);
        check(ctx_.get(), rc);
    }

    // Scene::build (Scene.h:84-101): binned-SAH BVH, built on the GPU.
    void build() { check(ctx_.get(), pgx_bvh_build(ctx_.get())); }

    // Scene::traverse for a batch (closest hit per ray).
    std::vector<pgx_hit> traverse(const std::vector<pgx_ray>& rays) {
        std::vector<pgx_hit> hits(rays.size());
        check(ctx_.get(), pgx_trace_closest(ctx_.get(), rays.data(), (int64_t)rays.size(), hits.data()));
        return hits;
    }

    // Scene::visible for a batch of shadow rays (1 = unoccluded).
    std::vector<uint8_t> visible(const std::vector<pgx_ray>& rays) {
        std::vector<uint8_t> vis(rays.size());
        check(ctx_.get(), pgx_trace_any(ctx_.get(), rays.data(), (int64_t)rays.size(), vis.data()));
        return vis;
    }

    // RTCamera::updateCamera (SceneLoader.h:85-89).
    void updateCamera(const pgx_camera& camera) {
        camera_ = camera;
        check(ctx_.get(), pgx_set_camera(ctx_.get(), &camera));
    }

    pgx_bvh_stats bvhStats() {
        pgx_bvh_stats s;
        check(ctx_.get(), pgx_bvh_get_stats(ctx_.get(), &s));
        return s;
    }

    const pgx_camera& camera() const { return camera_; }
    size_t triangleCount() const { return triangles_.size(); }
    pgx_ctx* context() const { return ctx_.get(); }

  private:
    Context ctx_;
    std::vector<pgx_triangle> triangles_;
    pgx_camera camera_{};
};

// `loadScene(dir)` (SceneLoader.h:222-269): the scene read, uploaded and
// built (BVH and light list), ready for RayTracer::init.
inline Scene* loadScene(const std::string& dir, int device = 0) {
    Scene* scene = new Scene(device);
    try {
        scene->load(dir);
        scene->build();
    } catch (...) {
        delete scene;
        throw;
    }
    return scene;
}

// Reference `RayTracer`: progressive film, one sample per pixel per render().
class RayTracer {
  public:
    explicit RayTracer(int mode = PGX_MODE_PLAIN, int max_depth = 8, uint64_t seed = 1) {
        cfg_.mode = mode;
        cfg_.max_depth = max_depth;
        cfg_.seed = seed;
        cfg_.guide_fraction = 0.5f;
        cfg_.record_paths = mode == PGX_MODE_GUIDED_LI ? 1 : 0;
        cfg_.flags = 0;
        cfg_.guide_depth = 0;
    }

    // RayTracer::init (Renderer.h:251-263).
    void init(Scene* scene) {
        scene_ = scene;
        clear();
    }
    // RayTracer::clear (Renderer.h:265-267).
    void clear() { check(ctx(), pgx_clear(ctx())); }
    // RayTracer::render (Renderer.h:648-747): one frame.
    void render() { check(ctx(), pgx_render(ctx(), &cfg_, 1)); }
    // Several frames in one call (same result as repeated render()).
    void render(int frames) { check(ctx(), pgx_render(ctx(), &cfg_, frames)); }
    // RayTracer::getSPP (Renderer.h:749).
    int getSPP() {
        int32_t spp = 0;
        check(ctx(), pgx_get_spp(ctx(), &spp));
        return spp;
    }
    // Film sums divided by SPP (Film::save, Imaging.h:263-272).
    std::vector<float> image() {
        const pgx_camera& c = scene_->camera();
        std::vector<float> rgb((size_t)c.width * c.height * 3);
        int32_t spp = 0;
        check(ctx(), pgx_film_read(ctx(), rgb.data(), nullptr, &spp));
        float inv = spp > 0 ? 1.f / (float)spp : 1.f;
        for (float& v : rgb) v *= inv;
        return rgb;
    }
    // RayTracer::saveHDR (Renderer.h:750): Radiance RGBE, flat scanlines.
    void saveHDR(const std::string& filename) {
        const pgx_camera& c = scene_->camera();
        std::vector<float> rgb = image();
        FILE* f = std::fopen(filename.c_str(), "wb");
        if (!f) throw Error(PGX_ERR_INVALID_ARG, "saveHDR: cannot open " + filename);
        std::fprintf(f, "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %d +X %d\n", c.height, c.width);
        for (size_t i = 0; i < (size_t)c.width * c.height; i++) {
            float r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
            float m = r > g ? (r > b ? r : b) : (g > b ? g : b);
            unsigned char px[4] = {0, 0, 0, 0};
            if (m > 1e-32f) {
                int e;
                float s = std::frexp(m, &e) * 256.f / m;
                px[0] = (unsigned char)(r * s);
                px[1] = (unsigned char)(g * s);
                px[2] = (unsigned char)(b * s);
                px[3] = (unsigned char)(e + 128);
            }
            std::fwrite(px, 1, 4, f);
        }
        std::fclose(f);
    }
    pgx_render_stats stats() {
        pgx_render_stats s;
        check(ctx(), pgx_render_get_stats(ctx(), &s));
        return s;
    }
    pgx_render_config& config() { return cfg_; }

    // Guided rendering (extension): trains the radiance-cache guide that
    // PGX_MODE_GUIDED_QUADTREE (or PGX_MODE_GUIDED_PSS) samples.  Pass k
    // renders first x 2^k frames and records their path vertices, which
    // rebuild the cache; the first pass is unguided (plain, or the PSS mode
    // without a cache), the others use the previous pass's guide.  Records
    // are weighted by Lum(Li) |cos| / pdf, so no pass inherits the guide that
    // sampled it, and the frames stay in the film (they are unbiased
    // samples).  params: as pgx_guide_configure (nullptr keeps the
    // context's).  render() then continues in this tracer's mode.
    void trainGuide(int first = 8, int passes = 2, const pgx_guide_params* params = nullptr) {
        if (params) check(ctx(), pgx_guide_configure(ctx(), params));
        const bool pss = cfg_.mode == PGX_MODE_GUIDED_PSS;
        pgx_render_config c = cfg_;
        for (int k = 0; k < passes; k++) {
            const int n = first << k;
            c.mode = pss ? PGX_MODE_GUIDED_PSS : (k == 0 ? PGX_MODE_PLAIN : PGX_MODE_GUIDED_QUADTREE);
            c.record_paths = n;
            check(ctx(), pgx_render(ctx(), &c, n));
        }
    }
    // The guide parameters measured best on the 1280x720 procedural interior
    // (with guide_fraction 0.7 and trainGuide(8, 2)): 16,384-record regions,
    // flux clamped at 20x the region's median, GGX conductors left to their
    // BSDF, the rest at their defaults.
    static pgx_guide_params recommendedGuideParams() {
        pgx_guide_params p{};
        p.region_records = 16384;
        p.refine_fraction = 0.01f;
        p.clamp_median = 20.f;
        p.uniform_share = 0.2f;
        p.compensate = 0.f;
        p.glossy_alpha = 2.f;
        return p;
    }

  private:
    pgx_ctx* ctx() const {
        if (!scene_) throw Error(PGX_ERR_STATE, "RayTracer used before init()");
        return scene_->context();
    }
    Scene* scene_ = nullptr;
    pgx_render_config cfg_{};
};

}  // namespace pgx
