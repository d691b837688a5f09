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
#include "Scene.h"

// Count every ray the integrators trace: `Scene::traverse` and
// `Scene::visible` are the only two routes from `RayTracer` into the BVH
// (Renderer.h:293,332,415,533).  The macros wrap the first argument of those
// calls in a comma expression that bumps a per-thread counter, so the calls
// themselves are unchanged.  Defined after Scene.h, before Renderer.h.
static thread_local long long g_rays_traced = 0;
static std::atomic<long long> g_rays_total{0};
static inline int pgx_count_ray() {
    ++g_rays_traced;
    return 0;
}
#define traverse(r) traverse((pgx_count_ray(), r))
#define visible(a, b) visible((pgx_count_ray(), a), b)
#include "Renderer.h"
#undef traverse
#undef visible

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

void orcref_rng_floats(uint64_t seed, uint64_t pixel, uint64_t sample, int32_t count, float* out) {
    PcgSampler s;
    s.reset(seed, pixel, sample);
    for (int32_t i = 0; i < count; i++) out[i] = s.next();
}

}  // extern "C"
