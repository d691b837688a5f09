// Harness around the reference renderer compiled headless — TEST
// INFRASTRUCTURE (the checker and the CPU baseline), never linked into the
// product.
//
// It includes the reference's own headers unmodified (staged into
// oracle/_ref/src by oracle/build_ref.sh, with the platform header replaced
// by oracle/ref_shim) and exposes plain C entry points that
//  - build the reference's BVH (`BVHNode::build`, Geometry.h:419-446) and
//    export its private node and index arrays (Geometry.h:270-272);
//  - trace rays with `BVHNode::traverse` / `traverseVisible`
//    (Geometry.h:455-567), single- or multi-threaded;
//  - assemble a `Scene` like `loadScene` (SceneLoader.h:222-269) and run
//    `RayTracer::render` (Renderer.h:648-747) or the per-pixel integrators
//    with a reproducible sampler.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <functional>
#include <map>
#include <memory>
#include <random>
#include <string>
#include <thread>
#include <utility>
#include <vector>

// The BVH arrays are private members; the harness reads them for export.
#define private public
#include "Geometry.h"
#undef private

#include "Lights.h"
#include "Materials.h"
#include "Metrics.h"
#include "Scene.h"

// Count every ray the integrators trace: `Scene::traverse` and
// `Scene::visible` are the only two routes from `RayTracer` into the BVH
// (Renderer.h:293,332,415,533).  The macros wrap the first argument of those
// calls in a comma expression that bumps a per-thread counter, so the calls
// themselves are unchanged.  Each thread counts privately and adds its count
// to the total when it exits (RayTracer::render joins its threads every
// frame, Renderer.h:715-718), so the count costs one increment per ray.
static std::atomic<long long> g_rays_total{0};
struct RayCounter {
    long long n = 0;
    ~RayCounter() { g_rays_total.fetch_add(n); }
};
static thread_local RayCounter g_ray_counter;
static inline int pgx_count_ray() {
    ++g_ray_counter.n;
    return 0;
}
#define traverse(r) traverse((pgx_count_ray(), r))
#define visible(a, b) visible((pgx_count_ray(), a), b)
#define private public
#include "Renderer.h"
#undef private
#undef traverse
#undef visible
#include "SceneLoader.h"

#include "../include/pgx.h"
#include "pgx_oracle_rng.h"

namespace {

Vertex to_vertex(const pgx_vertex& v) {
    Vertex r;
    r.p = Vec4(v.p[0], v.p[1], v.p[2]);
    r.normal = Vec4(v.n[0], v.n[1], v.n[2]);
    r.u = v.u;
    r.v = v.v;
    return r;
}

std::vector<Triangle> to_triangles(const pgx_triangle* tris, int64_t n) {
    std::vector<Triangle> out((size_t)n);
    for (int64_t i = 0; i < n; i++)
        out[(size_t)i].init(to_vertex(tris[i].v[0]), to_vertex(tris[i].v[1]), to_vertex(tris[i].v[2]),
                            tris[i].material);
    return out;
}

// Sampler that replays the PCG32 stream of pgx_oracle_rng.h.
class PcgSampler : public Sampler {
  public:
    uint64_t state = 0;
    void reset(uint64_t seed, uint64_t pixel, uint64_t sample) { state = orc_pcg_init(seed, pixel, sample); }
    float next() override { return orc_pcg_next_float(&state); }
};

struct RefWorld {
    std::vector<Triangle> tris;
    BVHNode bvh;
};

Texture* make_texture(int w, int h, const float* rgb) {
    Texture* t = new Texture();
    t->width = w;
    t->height = h;
    t->channels = 3;
    t->alpha = nullptr;
    t->texels = new Colour[(size_t)w * h];
    for (size_t i = 0; i < (size_t)w * h; i++) t->texels[i] = Colour(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
    return t;
}

// Material construction as loadInstance does it (SceneLoader.h:110-176).
BSDF* make_bsdf(const pgx_material& m, std::vector<Texture*>& textures) {
    Texture* alb;
    if (m.albedo_texture >= 0) {
        alb = textures[(size_t)m.albedo_texture];
    } else {
        alb = make_texture(1, 1, m.albedo);
    }
    BSDF* b = nullptr;
    switch (m.kind) {
        case PGX_BSDF_DIFFUSE: b = new DiffuseBSDF(alb); break;
        case PGX_BSDF_MIRROR: b = new MirrorBSDF(alb); break;
        case PGX_BSDF_CONDUCTOR:
            b = new ConductorBSDF(alb, Colour(m.eta[0], m.eta[1], m.eta[2]), Colour(m.k[0], m.k[1], m.k[2]), m.roughness);
            break;
        case PGX_BSDF_GLASS: b = new GlassBSDF(alb, m.int_ior, m.ext_ior); break;
        case PGX_BSDF_DIELECTRIC: b = new DielectricBSDF(alb, m.int_ior, m.ext_ior, m.roughness); break;
        case PGX_BSDF_ORENNAYAR: b = new OrenNayarBSDF(alb, m.sigma); break;
        case PGX_BSDF_PLASTIC: b = new PlasticBSDF(alb, m.int_ior, m.ext_ior, m.roughness); break;
        default: b = new DiffuseBSDF(alb); break;
    }
    b->addLight(Colour(m.emission[0], m.emission[1], m.emission[2]));
    if (m.layered) b = new LayeredBSDF(b, Colour(0.f, 0.f, 0.f), 1.f, 1.33f, 1.f);
    return b;
}

struct RefScene {
    Scene* scene = nullptr;
    RayTracer rt;
    GamesEngineeringBase::Window canvas;
    int width = 0, height = 0;
};

}  // namespace

extern "C" {

// BVHNode::build + export of bvhBuildNode / triangleIndexes.
int64_t orcref_bvh_build(const pgx_triangle* tris, int64_t n, pgx_bvh_node* nodes, int32_t* idx) {
    std::vector<Triangle> t = to_triangles(tris, n);
    BVHNode bvh;
    bvh.build(t);
    const auto& bn = bvh.bvhBuildNode;
    for (size_t i = 0; i < bn.size(); i++) {
        nodes[i].bmin[0] = bn[i].bounds.min.x;
        nodes[i].bmin[1] = bn[i].bounds.min.y;
        nodes[i].bmin[2] = bn[i].bounds.min.z;
        nodes[i].bmax[0] = bn[i].bounds.max.x;
        nodes[i].bmax[1] = bn[i].bounds.max.y;
        nodes[i].bmax[2] = bn[i].bounds.max.z;
        nodes[i].left_first = bn[i].leftFirst;
        nodes[i].used = bn[i].used;
    }
    for (size_t i = 0; i < bvh.triangleIndexes.size(); i++) idx[i] = bvh.triangleIndexes[i];
    return (int64_t)bn.size();
}

void* orcref_world_create(const pgx_triangle* tris, int64_t n) {
    RefWorld* w = new RefWorld();
    w->tris = to_triangles(tris, n);
    w->bvh.build(w->tris);
    return w;
}

void orcref_world_destroy(void* h) { delete static_cast<RefWorld*>(h); }

// BVHNode::traverse over rays [0, n) with `threads` std::threads; returns
// the wall time in seconds of the tracing alone.
double orcref_trace_closest(void* h, const pgx_ray* rays, int64_t n, pgx_hit* hits, int32_t threads) {
    RefWorld* w = static_cast<RefWorld*>(h);
    if (threads < 1) threads = 1;
    auto work = [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) {
            Ray r(Vec4(rays[i].o[0], rays[i].o[1], rays[i].o[2]), Vec4(rays[i].d[0], rays[i].d[1], rays[i].d[2]));
            IntersectionData isect;
            isect.t = rays[i].tmax;
            w->bvh.traverse(r, w->tris, isect);
            hits[i].id = (isect.ID == UINT_MAX) ? -1 : (int32_t)isect.ID;
            hits[i].t = isect.t;
            hits[i].u = isect.beta;
            hits[i].v = isect.gamma;
        }
    };
    auto t0 = std::chrono::steady_clock::now();
    if (threads == 1) {
        work(0, n);
    } else {
        std::vector<std::thread> th;
        for (int i = 0; i < threads; i++) th.emplace_back(work, n * i / threads, n * (i + 1) / threads);
        for (auto& t : th) t.join();
    }
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

// BVHNode::traverseVisible; visible[i] = 1 when nothing is hit in (eps, tmax).
double orcref_trace_any(void* h, const pgx_ray* rays, int64_t n, uint8_t* visible, int32_t threads) {
    RefWorld* w = static_cast<RefWorld*>(h);
    if (threads < 1) threads = 1;
    auto work = [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) {
            Ray r(Vec4(rays[i].o[0], rays[i].o[1], rays[i].o[2]), Vec4(rays[i].d[0], rays[i].d[1], rays[i].d[2]));
            visible[i] = w->bvh.traverseVisible(r, w->tris, rays[i].tmax) ? 1 : 0;
        }
    };
    auto t0 = std::chrono::steady_clock::now();
    if (threads == 1) {
        work(0, n);
    } else {
        std::vector<std::thread> th;
        for (int i = 0; i < threads; i++) th.emplace_back(work, n * i / threads, n * (i + 1) / threads);
        for (auto& t : th) t.join();
    }
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

// Scene as loadScene assembles it (SceneLoader.h:222-269): triangles,
// materials, background (environment map or black), BVH + light list,
// camera from (from, to, up, fov), scene bounds.
void* orcref_scene_create(const pgx_triangle* tris, int64_t n, const pgx_material* mats, int32_t nm,
                          const pgx_texture* textures, int32_t ntex, const pgx_texture* env, const pgx_camera* cam,
                          int32_t threads) {
    RefScene* rs = new RefScene();
    rs->scene = new Scene();
    std::vector<Texture*> texs;
    for (int32_t i = 0; i < ntex; i++) texs.push_back(make_texture(textures[i].width, textures[i].height, textures[i].rgb));
    std::vector<BSDF*> bsdfs;
    for (int32_t i = 0; i < nm; i++) bsdfs.push_back(make_bsdf(mats[i], texs));
    std::vector<Triangle> t = to_triangles(tris, n);
    Light* background;
    if (env) background = new EnvironmentMap(make_texture(env->width, env->height, env->rgb));
    else background = new BackgroundColour(Colour(0.0f, 0.0f, 0.0f));
    Matrix P = Matrix::perspective(0.001f, 10000.0f, (float)cam->width / (float)cam->height, cam->fov_degrees);
    Vec4 from(cam->from[0], cam->from[1], cam->from[2]);
    Vec4 to(cam->to[0], cam->to[1], cam->to[2]);
    Vec4 up(cam->up[0], cam->up[1], cam->up[2]);
    Matrix V = Matrix::lookAt(from, to, up);
    V = V.invert();
    if (cam->flip_x == 1) P.a[0][0] = -P.a[0][0];
    rs->scene->camera.init(P, cam->width, cam->height);
    rs->scene->camera.updateView(V);
    rs->scene->init(t, bsdfs, background);
    rs->scene->build();
    use<SceneBounds>().sceneCentre = (rs->scene->bounds.max + rs->scene->bounds.min) * 0.5f;
    use<SceneBounds>().sceneRadius = (rs->scene->bounds.max - use<SceneBounds>().sceneCentre).length();
    rs->width = cam->width;
    rs->height = cam->height;
    pgx_ref_thread_count() = threads > 0 ? (unsigned)threads : 0u;
    rs->canvas.create(cam->width, cam->height, "headless");
    rs->rt.init(rs->scene, &rs->canvas);
    return rs;
}

void orcref_scene_destroy(void* h) { delete static_cast<RefScene*>(h); }

// Per-pixel loop of RayTracer::render (Renderer.h:676-706) driven by the
// PCG32 stream of (seed, pixel, sample): jitter, camera ray, then
// pathTrace (guided = 0) or guidedPath (guided = 1), NaN/Inf drop and
// Film::splat.  Samples spp0 .. spp0+nspp-1 accumulate into film_rgb (W*H*3,
// caller-zeroed); rows are split over `threads` threads with private films.
// Path vertices of sample `collect` (guided only) go to verts (capacity
// vcap); returns the number written.  rays_out gets the rays traced.
static int g_mitchell = 0;
// Selects the film filter of orcref_render_pcg: 0 box (Renderer.h:255),
// 1 MitchellNetravaliFilter (Imaging.h:153-176).
void orcref_set_filter(int32_t mitchell) { g_mitchell = mitchell; }

int64_t orcref_render_pcg(void* h, int32_t guided, uint64_t seed, int32_t spp0, int32_t nspp, float* film_rgb,
                          int32_t threads, int32_t collect, pgx_path_vertex* verts, int64_t vcap,
                          int64_t* rays_out) {
    RefScene* rs = static_cast<RefScene*>(h);
    const int W = rs->width, H = rs->height;
    if (threads < 1) threads = 1;
    std::vector<std::vector<float>> films((size_t)threads, std::vector<float>((size_t)W * H * 3, 0.f));
    std::vector<std::vector<PathVertex>> vlists((size_t)threads);
    const long long rays0 = g_rays_total.load();
    auto work = [&](int tid) {
        Film film;
        film.width = W;
        film.height = H;
        film.film = reinterpret_cast<Colour*>(films[(size_t)tid].data());
        BoxFilter box;
        MitchellNetravaliFilter mitchell;
        film.filter = g_mitchell ? static_cast<ImageFilter*>(&mitchell) : static_cast<ImageFilter*>(&box);
        film.SPP = 0;
        PcgSampler sampler;
        std::vector<PathVertex> scratch;
        for (int y = tid; y < H; y += threads) {
            for (int x = 0; x < W; x++) {
                for (int s = spp0; s < spp0 + nspp; s++) {
                    sampler.reset(seed, (uint64_t)y * W + x, (uint64_t)s);
                    float px = x + sampler.next();
                    float py = y + sampler.next();
                    Ray ray = rs->scene->camera.generateRay(px, py);
                    Colour col;
                    if (guided) {
                        scratch.clear();
                        col = rs->rt.guidedPath(ray, &sampler, scratch);
                        if (s == collect) vlists[(size_t)tid].insert(vlists[(size_t)tid].end(), scratch.begin(), scratch.end());
                    } else {
                        col = rs->rt.pathTrace(ray, &sampler);
                    }
                    if (std::isnan(col.r) || std::isnan(col.g) || std::isnan(col.b) || std::isinf(col.r) ||
                        std::isinf(col.g) || std::isinf(col.b))
                        continue;
                    film.splat(px, py, col);
                }
            }
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < threads; t++) th.emplace_back(work, t);
    for (auto& t : th) t.join();
    for (auto& f : films)
        for (size_t i = 0; i < f.size(); i++) film_rgb[i] += f[i];
    if (rays_out) *rays_out = g_rays_total.load() - rays0;
    int64_t nv = 0;
    for (auto& vl : vlists)
        for (auto& v : vl) {
            if (nv < vcap && verts) {
                pgx_path_vertex& o = verts[nv];
                o.position[0] = v.position.x; o.position[1] = v.position.y; o.position[2] = v.position.z;
                o.normal[0] = v.normal.x; o.normal[1] = v.normal.y; o.normal[2] = v.normal.z;
                o.wi[0] = v.wi.x; o.wi[1] = v.wi.y; o.wi[2] = v.wi.z;
                o.Li[0] = v.Li.r; o.Li[1] = v.Li.g; o.Li[2] = v.Li.b;
            }
            nv++;
        }
    return nv;
}

// The reference's own RayTracer::render (Renderer.h:648-747) `frames`
// times: its tile scheduler, its MTRandom samplers, its integrator (the
// GUIDED_PATH switch of the build), its film.  Returns seconds spent in
// render(); film_rgb gets Film::film, rays_out the rays traced.
double orcref_render_native(void* h, int32_t frames, float* film_rgb, int32_t* spp, int64_t* rays_out) {
    RefScene* rs = static_cast<RefScene*>(h);
    const long long rays0 = g_rays_total.load();
    double secs = 0.0;
    // The guided build prints cache statistics after every cache rebuild
    // (Renderer.h:224-231); keep stdout quiet while timing.
    std::streambuf* old = std::cout.rdbuf(nullptr);
    for (int32_t f = 0; f < frames; f++) {
        auto t0 = std::chrono::steady_clock::now();
        rs->rt.render();
        auto t1 = std::chrono::steady_clock::now();
        secs += std::chrono::duration<double>(t1 - t0).count();
    }
    std::cout.rdbuf(old);
    if (film_rgb) std::memcpy(film_rgb, rs->rt.film->film, sizeof(float) * 3 * (size_t)rs->width * rs->height);
    if (spp) *spp = rs->rt.getSPP();
    if (rays_out) *rays_out = g_rays_total.load() - rays0;
    return secs;
}

void orcref_clear(void* h) { static_cast<RefScene*>(h)->rt.clear(); }

// Camera::generateRay (Scene.h:45-57) at n film positions (px, py): ray
// origin to o3 (n x 3) and normalised direction to d3 (n x 3).
void orcref_camera_rays(void* h, const float* px, const float* py, int64_t n, float* o3, float* d3) {
    RefScene* rs = static_cast<RefScene*>(h);
    for (int64_t i = 0; i < n; i++) {
        Ray r = rs->scene->camera.generateRay(px[i], py[i]);
        o3[3 * i] = r.o.x; o3[3 * i + 1] = r.o.y; o3[3 * i + 2] = r.o.z;
        d3[3 * i] = r.dir.x; d3[3 * i + 1] = r.dir.y; d3[3 * i + 2] = r.dir.z;
    }
}

// PointBVHNode::buildPointBVHNode (Renderer.h:189-211) on given records;
// exports the tree in preorder (root first) and the records in node order.
int64_t orcref_pointbvh(const pgx_path_vertex* recs, int64_t n, pgx_cache_node* nodes, pgx_path_vertex* out) {
    std::vector<PathVertex> v((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        v[(size_t)i].position = Vec4(recs[i].position[0], recs[i].position[1], recs[i].position[2]);
        v[(size_t)i].normal = Vec4(recs[i].normal[0], recs[i].normal[1], recs[i].normal[2]);
        v[(size_t)i].wi = Vec4(recs[i].wi[0], recs[i].wi[1], recs[i].wi[2]);
        v[(size_t)i].Li = Colour(recs[i].Li[0], recs[i].Li[1], recs[i].Li[2]);
    }
    std::streambuf* old = std::cout.rdbuf(nullptr);  // silence stats()
    PointBVHNode* root = new PointBVHNode();
    root->buildPointBVHNode(std::move(v));
    std::cout.rdbuf(old);
    int64_t count = 0;
    std::function<int64_t(PointBVHNode*)> walk = [&](PointBVHNode* nd) -> int64_t {
        int64_t me = count++;
        pgx_cache_node& o = nodes[me];
        o.bmin[0] = nd->bounds.min.x; o.bmin[1] = nd->bounds.min.y; o.bmin[2] = nd->bounds.min.z;
        o.bmax[0] = nd->bounds.max.x; o.bmax[1] = nd->bounds.max.y; o.bmax[2] = nd->bounds.max.z;
        o.offset = nd->offset;
        o.used = nd->used;
        if (nd->isLeaf()) {
            o.left = o.right = -1;
        } else {
            int64_t l = walk(nd->l);
            int64_t r = walk(nd->r);
            nodes[me].left = (int32_t)l;
            nodes[me].right = (int32_t)r;
        }
        return me;
    };
    if (n > 0) walk(root);
    for (int64_t i = 0; i < n; i++) {
        const PathVertex& p = root->pathVertexRecords[(size_t)i];
        out[i].position[0] = p.position.x; out[i].position[1] = p.position.y; out[i].position[2] = p.position.z;
        out[i].normal[0] = p.normal.x; out[i].normal[1] = p.normal.y; out[i].normal[2] = p.normal.z;
        out[i].wi[0] = p.wi.x; out[i].wi[1] = p.wi.y; out[i].wi[2] = p.wi.z;
        out[i].Li[0] = p.Li.r; out[i].Li[1] = p.Li.g; out[i].Li[2] = p.Li.b;
    }
    delete root;
    return count;
}

// BSDF::sample driven by TestSampler (Sampling.h:26-48) and BSDF::invert
// for shading points with normal n[i] and outgoing direction wo[i], as
// runTest sets them up (main.cpp:301-306).
void orcref_bsdf_roundtrip(const pgx_material* mat, const float* n, const float* wo, const float* uv, int64_t count,
                           float* wi_out, float* f_out, float* pdf_out, float* uv_out) {
    std::vector<Texture*> none;
    BSDF* bsdf = make_bsdf(*mat, none);
    TestSampler ts;
    for (int64_t i = 0; i < count; i++) {
        ShadingData sd;
        sd.sNormal = Vec4(n[3 * i], n[3 * i + 1], n[3 * i + 2]);
        sd.gNormal = sd.sNormal;
        sd.wo = Vec4(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
        sd.x = Vec4(0.f, 0.f, 0.f);
        sd.tu = 0.f;
        sd.tv = 0.f;
        sd.bsdf = bsdf;
        sd.frame.fromVector(sd.sNormal);
        ts.set(uv[2 * i], uv[2 * i + 1]);
        Colour col(0.f, 0.f, 0.f);
        float pdf = 0.f;
        Vec4 wi = bsdf->sample(sd, &ts, col, pdf);
        float uo = 0.f, vo = 0.f;
        bsdf->invert(sd, wi, uo, vo);
        wi_out[3 * i] = wi.x;
        wi_out[3 * i + 1] = wi.y;
        wi_out[3 * i + 2] = wi.z;
        f_out[3 * i] = col.r;
        f_out[3 * i + 1] = col.g;
        f_out[3 * i + 2] = col.b;
        pdf_out[i] = pdf;
        uv_out[2 * i] = uo;
        uv_out[2 * i + 1] = vo;
    }
}

// Film::tonemap (Imaging.h:220-244) of a film buffer for every pixel.
void orcref_tonemap(float* film_rgb, int32_t w, int32_t h, int32_t spp, float exposure, float lmax_white,
                    uint8_t* out) {
    Film film;
    film.width = w;
    film.height = h;
    film.film = reinterpret_cast<Colour*>(film_rgb);
    film.SPP = spp;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            unsigned char r, g, b;
            film.tonemap(x, y, r, g, b, exposure, lmax_white);
            size_t i = ((size_t)y * w + x) * 3;
            out[i] = r;
            out[i + 1] = g;
            out[i + 2] = b;
        }
}

// Metrics::calculateMSE / RMSE / RRMSE (Metrics.h:8-68).
void orcref_metrics(const float* test, const float* gt, int32_t w, int32_t h, float* out3) {
    std::vector<float> t(test, test + (size_t)w * h * 3), g(gt, gt + (size_t)w * h * 3);
    Metrics m;
    out3[0] = m.calculateMSE(t, g, w, h);
    out3[1] = m.calculateRMSE(t, g, w, h);
    out3[2] = m.calculateRRMSE(t, g, w, h);
}

// ---- scene ingestion ------------------------------------------------------
// A scene as the reference holds it after loading: its triangles, BSDF
// objects, background and camera.  Built either by the reference's own
// loadScene (SceneLoader.h:222-269) from a scene directory, or from pgx's
// upload arrays with the harness's make_bsdf, so both sides export through
// the same code.
struct RefLoaded {
    Scene* scene = nullptr;
    std::vector<Texture*> textures;  // distinct albedo textures, first-use order
};

static void collect_textures(RefLoaded* rl) {
    for (BSDF* b : rl->scene->materials) {
        BSDF* base = b;
        if (auto* l = dynamic_cast<LayeredBSDF*>(b)) base = l->base;
        Texture* t = nullptr;
        if (auto* m = dynamic_cast<DiffuseBSDF*>(base)) t = m->albedo;
        else if (auto* m = dynamic_cast<MirrorBSDF*>(base)) t = m->albedo;
        else if (auto* m = dynamic_cast<ConductorBSDF*>(base)) t = m->albedo;
        else if (auto* m = dynamic_cast<GlassBSDF*>(base)) t = m->albedo;
        else if (auto* m = dynamic_cast<DielectricBSDF*>(base)) t = m->albedo;
        else if (auto* m = dynamic_cast<OrenNayarBSDF*>(base)) t = m->albedo;
        else if (auto* m = dynamic_cast<PlasticBSDF*>(base)) t = m->albedo;
        if (t && std::find(rl->textures.begin(), rl->textures.end(), t) == rl->textures.end()) rl->textures.push_back(t);
    }
}

// loadScene on `dir`; counts go to counts[0..3] = triangles, materials,
// textures, width, height (counts has 5 entries).
void* orcref_load_scene(const char* dir, int64_t* counts) {
    RefLoaded* rl = new RefLoaded();
    std::streambuf* old = std::cout.rdbuf(nullptr);
    rl->scene = loadScene(dir);
    std::cout.rdbuf(old);
    collect_textures(rl);
    counts[0] = (int64_t)rl->scene->triangles.size();
    counts[1] = (int64_t)rl->scene->materials.size();
    counts[2] = (int64_t)rl->textures.size();
    counts[3] = (int64_t)rl->scene->camera.width;
    counts[4] = (int64_t)rl->scene->camera.height;
    return rl;
}

// The same assembly from pgx arrays (orcref_scene_create's path).
void* orcref_loaded_from_arrays(const pgx_triangle* tris, int64_t n, const pgx_material* mats, int32_t nm,
                                const pgx_texture* textures, int32_t ntex, const pgx_texture* env,
                                const pgx_camera* cam, int64_t* counts) {
    RefLoaded* rl = new RefLoaded();
    rl->scene = new Scene();
    std::vector<Texture*> texs;
    for (int32_t i = 0; i < ntex; i++) texs.push_back(make_texture(textures[i].width, textures[i].height, textures[i].rgb));
    std::vector<BSDF*> bsdfs;
    for (int32_t i = 0; i < nm; i++) bsdfs.push_back(make_bsdf(mats[i], texs));
    Light* background;
    if (env) background = new EnvironmentMap(make_texture(env->width, env->height, env->rgb));
    else background = new BackgroundColour(Colour(0.0f, 0.0f, 0.0f));
    Matrix P = Matrix::perspective(0.001f, 10000.0f, (float)cam->width / (float)cam->height, cam->fov_degrees);
    Matrix V = Matrix::lookAt(Vec4(cam->from[0], cam->from[1], cam->from[2]), Vec4(cam->to[0], cam->to[1], cam->to[2]),
                              Vec4(cam->up[0], cam->up[1], cam->up[2]));
    V = V.invert();
    if (cam->flip_x == 1) P.a[0][0] = -P.a[0][0];
    rl->scene->camera.init(P, cam->width, cam->height);
    rl->scene->camera.updateView(V);
    rl->scene->init(to_triangles(tris, n), bsdfs, background);
    collect_textures(rl);
    counts[0] = (int64_t)rl->scene->triangles.size();
    counts[1] = (int64_t)rl->scene->materials.size();
    counts[2] = (int64_t)rl->textures.size();
    counts[3] = (int64_t)rl->scene->camera.width;
    counts[4] = (int64_t)rl->scene->camera.height;
    return rl;
}

void orcref_loaded_destroy(void* h) { delete static_cast<RefLoaded*>(h); }

// Triangles as pgx_triangle (vertex position, normal, uv; material index).
void orcref_loaded_triangles(void* h, pgx_triangle* out) {
    RefLoaded* rl = static_cast<RefLoaded*>(h);
    for (size_t i = 0; i < rl->scene->triangles.size(); i++) {
        const Triangle& t = rl->scene->triangles[i];
        for (int k = 0; k < 3; k++) {
            const Vertex& v = t.vertices[k];
            out[i].v[k].p[0] = v.p.x;
            out[i].v[k].p[1] = v.p.y;
            out[i].v[k].p[2] = v.p.z;
            out[i].v[k].n[0] = v.normal.x;
            out[i].v[k].n[1] = v.normal.y;
            out[i].v[k].n[2] = v.normal.z;
            out[i].v[k].u = v.u;
            out[i].v[k].v = v.v;
        }
        out[i].material = t.materialIndex;
    }
}

// Per material 20 floats: kind (pgx numbering), layered, emission rgb,
// intIOR, extIOR, alpha (the constructor's value, not the roughness),
// sigma, eta rgb, k rgb, albedo texture index, coating sigmaA rgb,
// coating thickness.
void orcref_loaded_materials(void* h, float* out) {
    RefLoaded* rl = static_cast<RefLoaded*>(h);
    for (size_t i = 0; i < rl->scene->materials.size(); i++) {
        float* p = out + 20 * i;
        for (int j = 0; j < 20; j++) p[j] = 0.f;
        BSDF* b = rl->scene->materials[i];
        BSDF* base = b;
        if (auto* l = dynamic_cast<LayeredBSDF*>(b)) {
            base = l->base;
            p[1] = 1.f;
            p[16] = l->sigmaa.r;
            p[17] = l->sigmaa.g;
            p[18] = l->sigmaa.b;
            p[19] = l->thickness;
        }
        p[2] = b->emission.r;
        p[3] = b->emission.g;
        p[4] = b->emission.b;
        Texture* t = nullptr;
        if (auto* m = dynamic_cast<DiffuseBSDF*>(base)) {
            p[0] = PGX_BSDF_DIFFUSE;
            t = m->albedo;
        } else if (auto* m = dynamic_cast<MirrorBSDF*>(base)) {
            p[0] = PGX_BSDF_MIRROR;
            t = m->albedo;
        } else if (auto* m = dynamic_cast<ConductorBSDF*>(base)) {
            p[0] = PGX_BSDF_CONDUCTOR;
            t = m->albedo;
            p[7] = m->alpha;
            p[9] = m->eta.r, p[10] = m->eta.g, p[11] = m->eta.b;
            p[12] = m->k.r, p[13] = m->k.g, p[14] = m->k.b;
        } else if (auto* m = dynamic_cast<GlassBSDF*>(base)) {
            p[0] = PGX_BSDF_GLASS;
            t = m->albedo;
            p[5] = m->intIOR, p[6] = m->extIOR;
        } else if (auto* m = dynamic_cast<DielectricBSDF*>(base)) {
            p[0] = PGX_BSDF_DIELECTRIC;
            t = m->albedo;
            p[5] = m->intIOR, p[6] = m->extIOR, p[7] = m->alpha;
        } else if (auto* m = dynamic_cast<OrenNayarBSDF*>(base)) {
            p[0] = PGX_BSDF_ORENNAYAR;
            t = m->albedo;
            p[8] = m->sigma;
        } else if (auto* m = dynamic_cast<PlasticBSDF*>(base)) {
            p[0] = PGX_BSDF_PLASTIC;
            t = m->albedo;
            p[5] = m->intIOR, p[6] = m->extIOR, p[7] = m->alpha;
        }
        p[15] = (float)(std::find(rl->textures.begin(), rl->textures.end(), t) - rl->textures.begin());
    }
}

// Size of texture i (i = -1: the environment map; 0 x 0 when there is none).
void orcref_loaded_texture_size(void* h, int32_t i, int32_t* wh) {
    RefLoaded* rl = static_cast<RefLoaded*>(h);
    Texture* t = nullptr;
    if (i < 0) {
        if (auto* e = dynamic_cast<EnvironmentMap*>(rl->scene->background)) t = e->env;
    } else {
        t = rl->textures[(size_t)i];
    }
    wh[0] = t ? t->width : 0;
    wh[1] = t ? t->height : 0;
}

void orcref_loaded_texture(void* h, int32_t i, float* rgb) {
    RefLoaded* rl = static_cast<RefLoaded*>(h);
    Texture* t = i < 0 ? dynamic_cast<EnvironmentMap*>(rl->scene->background)->env : rl->textures[(size_t)i];
    for (size_t k = 0; k < (size_t)t->width * t->height; k++) {
        rgb[3 * k] = t->texels[k].r;
        rgb[3 * k + 1] = t->texels[k].g;
        rgb[3 * k + 2] = t->texels[k].b;
    }
}

// Texture::load (Imaging.h:44-79) of one file; the texture is kept until
// orcref_texture_free.  wh gets width, height.
void* orcref_texture_load(const char* filename, int32_t* wh) {
    Texture* t = new Texture();
    t->load(filename);
    wh[0] = t->width;
    wh[1] = t->height;
    return t;
}

void orcref_texture_read(void* h, float* rgb) {
    Texture* t = static_cast<Texture*>(h);
    for (size_t k = 0; k < (size_t)t->width * t->height; k++) {
        rgb[3 * k] = t->texels[k].r;
        rgb[3 * k + 1] = t->texels[k].g;
        rgb[3 * k + 2] = t->texels[k].b;
    }
    delete t;
}

// Camera matrices: projection (16), camera-to-world (16).
void orcref_loaded_camera(void* h, float* out32) {
    RefLoaded* rl = static_cast<RefLoaded*>(h);
    memcpy(out32, rl->scene->camera.projectionMatrix.m, 16 * sizeof(float));
    memcpy(out32 + 16, rl->scene->camera.camera.m, 16 * sizeof(float));
}

void orcref_rng_floats(uint64_t seed, uint64_t pixel, uint64_t sample, int32_t count, float* out) {
    PcgSampler s;
    s.reset(seed, pixel, sample);
    for (int32_t i = 0; i < count; i++) out[i] = s.next();
}

}  // extern "C"
