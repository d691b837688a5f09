// Wavefront path tracer: RayTracer::render (Renderer.h:648-747) with the
// integrators pathTraceRecursive (Renderer.h:531-613, PGX_MODE_PLAIN) and
// guidedPath/guidedPathRecursive (Renderer.h:368-528, PGX_MODE_GUIDED_LI),
// plus the QuadTree-guided estimator (PGX_MODE_GUIDED_QUADTREE, pgx_guide.cuh)
// and the learned-guide estimator (PGX_MODE_GUIDED_MLP, pgx_mlp.cuh), whose
// network runs on the tensor cores in k_guide_infer between traversal and
// shading at every depth.
//
// One path per (pixel, sample); a wave holds up to 2^25 of them.  The
// recursion of the reference becomes a loop over depth with queue-per-stage
// kernels:
//   camgen -> [extend -> classify -> (guide_infer) -> shade x 6 classes
//              -> shadow] x (max_depth + 1) -> finalize
// `classify` bins the depth's paths by surface class and `shade` runs once
// per class with that class's code compiled in; it compacts surviving paths
// into the next queue with warp-aggregated atomics (ballot + popc, one
// atomicAdd per warp) and appends next-event shadow rays to a shadow queue;
// `shadow` runs the any-hit traversal and adds the stored contribution of
// unoccluded rays to the path's radiance.  Queue lengths live on the device,
// so a wave needs no host round trip (batches replay their waves from a
// captured CUDA graph).
//
// Each path owns a PCG32 stream keyed by (seed, pixel, sample) and draws
// from it in the reference's order (jitter, light pick, light sample, RR,
// BSDF sample), so a CPU run of the reference's integrator driven by the same
// stream takes the same decisions.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "pgx_ctx.h"
#include <cstdarg>

#include "pgx_guide.cuh"
#include "pgx_mlp.cuh"
#include "pgx_shade.cuh"
#include "pgx_trace.cuh"

namespace {

constexpr int kThreads = 128;
constexpr int kMaxDepthCap = 16;
constexpr int kCollectionSPP = 128 / 8;  // Renderer.h:721
constexpr int kStats = 8;                 // 64-bit statistics counters
constexpr int kProfEvents = 4 * (kMaxDepthCap + 2);
// Shading classes: paths of one depth are binned by what they hit and shaded
// one class per launch, so every SM runs one class's code path at a time.
constexpr int kShadeClasses = 6;  // miss, emitter, diffuse, conductor, glass, other

// Per-path state, structure of arrays.
struct PathState {
    float4* o;    // ray origin
    float4* d;    // ray direction
    float4* T;    // throughput rgb, w = previous BSDF pdf
    float4* L;    // radiance rgb
    float4* hit;  // id bits, t, u, v
    float2* pix;  // film sample position (px, py)
    uint64_t* rng;
    int* flags;   // bit 0: previous surface pure specular
    int* nrec;    // guided-Li: records written
    int* queue[2];
    // shadow queue
    int* sh_path;
    float4* sh_o;  // w = tmax
    float4* sh_d;
    float4* sh_c;  // contribution rgb
    // guided-Li records [depth][path]
    float4* rec_pos;  // w = store flag
    float4* rec_nrm;
    float4* rec_wi;
    float4* rec_w;
    float4* rec_e;
    // counters: queue length per depth, shadow count per depth, stats
    unsigned* qcount;  // [kMaxDepthCap + 2]
    int* cqueue;       // per class [kShadeClasses][capacity]
    unsigned* ccount;  // [kMaxDepthCap + 2][kShadeClasses]
    unsigned* scount;  // [kMaxDepthCap + 2]
    unsigned* wcount;  // [2 * (kMaxDepthCap + 2)] persistent-traversal work counters
    unsigned long long* stats;  // [0] ext rays [1] shadow rays [2,3] extend nodes/tris [4,5] shadow nodes/tris
    pgx_path_vertex* vertices;
    float* vweight;   // per vertex: flux weight for the QuadTree guide (plain, QuadTree and PSS records)
    unsigned* nvertices;
    int64_t capacity;
    int64_t vcapacity;
    // learned guide: per-path mixture (10 float4), training records
    float4* guide;
    int* fallback;    // per path: QuadTree root standing in for the network (-1: the network, -2: the BSDF)
    float4* rec_wo;   // wo
    float4* rec_f;    // f |cos| / pdf of the continuation
    float* train;     // radiance samples, 13 floats each
    unsigned* ntrain;
    int64_t tcapacity;
    int* scene;       // batched rendering: scene of each path
};

struct RenderState {
    DevBuf o, d, T, L, hit, pix, rng, flags, nrec, q0, q1, sh_path, sh_o, sh_d, sh_c;
    DevBuf rec_pos, rec_nrm, rec_wi, rec_w, rec_e;
    DevBuf counters, vertices, vweight, cqueue, ccount;
    DevBuf guide, fallback, rec_wo, rec_f, train, scene;
    int64_t capacity = 0;
    int rec_depth = 0;
    int64_t guide_capacity = 0;
    int train_depth = 0;
    int64_t tcapacity = 0;
    int64_t train_last = 0;   // samples the previous batch produced
    int64_t vcapacity = 0;
    int64_t nvertices_last = 0;
    bool vweight_valid = false;  // the last recording wrote flux weights (not guided-Li)
    // captured frame graph
    cudaGraphExec_t graph = nullptr;
    int graph_mode = -1, graph_depth = -1, graph_batch = -1, graph_record = -1;
    uint64_t graph_seed = 0;
    int graph_spp0 = -1;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t prof[kProfEvents] = {};
    // differentiable rendering: evaluation parameters and scratch
    DevBuf d_mats, d_env, d_partial, d_img, d_dimg, d_genv, d_galb, d_grough, d_next, d_samples;
    bool d_params = false;
};

struct SceneView {
    BvhView bvh;
    const TriShade* __restrict__ shade;
    const unsigned char* __restrict__ tri_class;
    const DevMaterial* __restrict__ mats;
    const DevAreaLight* __restrict__ lights;
    TexView tex;
    DevEnv env;
    DevCamera cam;
    SceneBoundsDev bounds;
    int n_area_lights;
    int nlights;
    int has_env_light;
    int width, height;
};

struct FrameParams {
    int mode;
    int max_depth;
    uint64_t seed;
    int spp0;        // sample index of the batch's first sample
    int batch;       // samples per pixel in this batch
    int collect_lo;  // path vertices of samples [collect_lo, collect_hi) are recorded
    int collect_hi;
    float guide_fraction;
    int profile;     // 1: stage events; 2: stage events and node/triangle fetch counts
    int mitchell;    // Mitchell-Netravali splat instead of the box filter
    int train;       // learned guide: emit radiance samples of recorded vertices
                     // (1: indirect light only, 2: full incident radiance)
    float train_keep;  // probability of keeping one radiance sample
    int guide_depth;   // guided modes: bounces guided (max_depth + 1: all)
};

// Batched rendering: what differs between the scenes of a batch whose
// node, triangle, shading, material, texture and light arrays are merged
// into one set (pgx_batch_create).
struct BatchInfo {
    TravRoot root;        // the scene's tree in the merged node array
    int light_base;       // its area lights in the merged light array
    int n_lights;
    DevEnv env;           // its environment map (the scene context's own buffers)
    int has_env_light;    // the environment is light 0 of NEE
    DevCamera cam;
    SceneBoundsDev bounds;
    int width, height;
    float* film;
    int spp0;             // samples already in the film
    int64_t npix;
};

struct BatchWave {
    const BatchInfo* __restrict__ info;
    const int64_t* __restrict__ prefix;  // items before scene s (items = pixels x spp)
    int n;
    int64_t base, count;                 // this wave's items
    const uint64_t* seed;
};

__device__ __forceinline__ int batch_scene_of(const BatchWave& bw, int64_t item) {
    int lo = 0, hi = bw.n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (bw.prefix[mid] <= item) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Camera::generateRay (Scene.h:45-57) direction for film position (px, py).
__device__ __forceinline__ F3 camera_dir(const DevCamera& cam, float px, float py) {
    float xc = (2.f * px / cam.width) - 1.f;
    float yc = (2.f * (1.f - (py / cam.height))) - 1.f;
    const float* m = cam.inv_proj;
    float vx = ((xc * m[0] + yc * m[1]) + 0.f * m[2]) + m[3];
    float vy = ((xc * m[4] + yc * m[5]) + 0.f * m[6]) + m[7];
    float vz = ((xc * m[8] + yc * m[9]) + 0.f * m[10]) + m[11];
    float w = ((m[12] * xc + m[13] * yc) + m[14] * 0.f) + m[15];
    w = 1.f / w;
    vx = vx * w;
    vy = vy * w;
    vz = vz * w;
    const float* c = cam.cam;
    return normalize(f3((vx * c[0] + vy * c[1]) + vz * c[2], (vx * c[4] + vy * c[5]) + vz * c[6],
                        (vx * c[8] + vy * c[9]) + vz * c[10]));
}

// ---- camera rays (Camera::generateRay, Scene.h:253-265; jitter Renderer.h:679-681)
__global__ void __launch_bounds__(kThreads) k_camgen(SceneView sv, PathState ps, FrameParams fp) {
    const int64_t npix = (int64_t)sv.width * sv.height;
    const int64_t n = npix * fp.batch;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t pixel = i % npix;
        int s = (int)(i / npix);
        int xpix = (int)(pixel % sv.width), ypix = (int)(pixel / sv.width);
        uint64_t rng = pgx_rng_init(fp.seed, (uint64_t)pixel, (uint64_t)(fp.spp0 + s));
        float px = (float)xpix + pgx_rng_next(rng);
        float py = (float)ypix + pgx_rng_next(rng);
        const DevCamera& cam = sv.cam;
        F3 dir = camera_dir(cam, px, py);
        ps.o[i] = make_float4(cam.origin[0], cam.origin[1], cam.origin[2], 0.f);
        ps.d[i] = make_float4(dir.x, dir.y, dir.z, 0.f);
        ps.T[i] = make_float4(1.f, 1.f, 1.f, 0.f);
        ps.L[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        ps.pix[i] = make_float2(px, py);
        ps.rng[i] = rng;
        ps.flags[i] = 0;
        ps.nrec[i] = 0;
        ps.queue[0][i] = (int)i;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) ps.qcount[0] = (unsigned)n;
}

// Camera rays of one wave of a batch: item -> (scene, pixel, sample), the
// same PCG32 key and draws as k_camgen.
__global__ void __launch_bounds__(kThreads) k_camgen_batch(PathState ps, BatchWave bw) {
    const uint64_t seed = *bw.seed;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < bw.count; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t item = bw.base + i;
        const int sc = batch_scene_of(bw, item);
        const BatchInfo& bi = bw.info[sc];
        const int64_t local = item - bw.prefix[sc];
        const int64_t pixel = local % bi.npix;
        const int sample = bi.spp0 + (int)(local / bi.npix);
        int xpix = (int)(pixel % bi.width), ypix = (int)(pixel / bi.width);
        uint64_t rng = pgx_rng_init(seed, (uint64_t)pixel, (uint64_t)sample);
        float px = (float)xpix + pgx_rng_next(rng);
        float py = (float)ypix + pgx_rng_next(rng);
        F3 dir = camera_dir(bi.cam, px, py);
        ps.o[i] = make_float4(bi.cam.origin[0], bi.cam.origin[1], bi.cam.origin[2], 0.f);
        ps.d[i] = make_float4(dir.x, dir.y, dir.z, 0.f);
        ps.T[i] = make_float4(1.f, 1.f, 1.f, 0.f);
        ps.L[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        ps.pix[i] = make_float2(px, py);
        ps.rng[i] = rng;
        ps.flags[i] = 0;
        ps.nrec[i] = 0;
        ps.scene[i] = sc;
        ps.queue[0][i] = (int)i;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) ps.qcount[0] = (unsigned)bw.count;
}

// Root of a batched path's scene (RootOf of trace_persistent).
struct BatchRoot {
    const BatchInfo* info;
    const int* scene;
    const int* path;  // queue entry -> path index
    __device__ __forceinline__ TravRoot operator()(unsigned i, const BvhView&) const { return info[scene[path[i]]].root; }
};

// ---- closest hit for the queue of this depth ----------------------------------
__device__ __forceinline__ void add_counts(unsigned long long* dst, unsigned long long a, unsigned long long b) {
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xFFFFFFFFu, a, o);
        b += __shfl_xor_sync(0xFFFFFFFFu, b, o);
    }
    if ((threadIdx.x & 31) == 0 && (a | b)) {
        atomicAdd(dst, a);
        atomicAdd(dst + 1, b);
    }
}

constexpr int kPersistentBlocksPerSM = 8;

// Closest hit for the queue of this depth: persistent warps with lane refill
// (trace_persistent) over qcount[depth] rays.
template <bool COUNT, bool BATCH = false, int SHORT = kShortStack>
__global__ void __launch_bounds__(kThreads, kPersistentBlocksPerSM) k_extend(SceneView sv, PathState ps, int depth,
                                                                            const BatchInfo* binfo = nullptr) {
    const unsigned n = ps.qcount[depth];
    const int* __restrict__ q = ps.queue[depth & 1];
    unsigned long long ni = 0, nt = 0;
    unsigned status = 0;
    auto load = [&](unsigned i, xv3& o, xv3& d, float& tmax) {
        int p = q[i];
        float4 a = ps.o[p], b = ps.d[p];
        o = mk(a.x, a.y, a.z);
        d = mk(b.x, b.y, b.z);
        tmax = FLT_MAX;
    };
    auto store = [&](unsigned i, const TraceLane& L) {
        int p = q[i];
        int id = L.status ? -1 : L.hit_id;  // corrupt tree or stack overflow: a miss
        ps.hit[p] = make_float4(__int_as_float(id), L.tmax, L.hu, L.hv);
    };
    if (BATCH)
        trace_persistent<false, COUNT, decltype(load), decltype(store), BatchRoot, SHORT>(
            sv.bvh, n, &ps.wcount[depth], load, store, ni, nt, status, BatchRoot{binfo, ps.scene, q});
    else
        trace_persistent<false, COUNT>(sv.bvh, n, &ps.wcount[depth], load, store, ni, nt, status);
    if (COUNT) add_counts(&ps.stats[2], ni, nt);
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ps.stats[0], (unsigned long long)n);
}

// Any hit for the shadow queue of this depth; unoccluded rays add their
// contribution to the path's radiance.
template <bool COUNT, bool BATCH = false, int SHORT = kShortStack>
__global__ void __launch_bounds__(kThreads, kPersistentBlocksPerSM) k_shadow(SceneView sv, PathState ps, int depth,
                                                                            const BatchInfo* binfo = nullptr) {
    const unsigned n = ps.scount[depth];
    unsigned long long ni = 0, nt = 0;
    unsigned status = 0;
    auto load = [&](unsigned i, xv3& o, xv3& d, float& tmax) {
        float4 a = ps.sh_o[i], b = ps.sh_d[i];
        o = mk(a.x, a.y, a.z);
        d = mk(b.x, b.y, b.z);
        tmax = a.w;
    };
    auto store = [&](unsigned i, const TraceLane& L) {
        if (L.hit_id < 0 && !L.status) {
            int p = ps.sh_path[i];
            float4 c = ps.sh_c[i];
            float4 l = ps.L[p];
            ps.L[p] = make_float4(l.x + c.x, l.y + c.y, l.z + c.z, 0.f);
        }
    };
    if (BATCH)
        trace_persistent<true, COUNT, decltype(load), decltype(store), BatchRoot, SHORT>(
            sv.bvh, n, &ps.wcount[kMaxDepthCap + 2 + depth], load, store, ni, nt, status,
            BatchRoot{binfo, ps.scene, ps.sh_path});
    else
        trace_persistent<true, COUNT>(sv.bvh, n, &ps.wcount[kMaxDepthCap + 2 + depth], load, store, ni, nt, status);
    if (COUNT) add_counts(&ps.stats[4], ni, nt);
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ps.stats[1], (unsigned long long)n);
}

inline unsigned persistent_grid(int64_t n) {
    int64_t b = (n + kThreads - 1) / kThreads;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)pgx_num_sms() * kPersistentBlocksPerSM));
}

// Scene::calculateShadingData (Scene.h:152-176).
__device__ __forceinline__ void shading_data(const SceneView& sv, const float4& o, const float4& d, const float4& h,
                                             Shading& sd, DevMaterial& m, F3& tri_gn, float& tri_area) {
    int id = __float_as_int(h.x);
    float t = h.y, beta = h.z, gamma = h.w;
    float alpha = 1.f - (beta + gamma);
    const TriShade& s = sv.shade[id];
    float4 n0 = s.n0, n1 = s.n1, n2 = s.n2, vv = s.vv, gn = s.gn;
    F3 dir = f3(d);
    sd.t = t;
    sd.x = f3(o) + dir * t;
    tri_gn = f3(gn);
    tri_area = gn.w;
    F3 g = tri_gn;
    F3 sn = normalize(((f3(n0) * alpha) + (f3(n1) * beta)) + (f3(n2) * gamma));
    sd.tu = ((n0.w * alpha) + (n1.w * beta)) + (n2.w * gamma);
    sd.tv = ((vv.x * alpha) + (vv.y * beta)) + (vv.z * gamma);
    sd.mat = __float_as_int(vv.w);
    m = sv.mats[sd.mat];
    sd.wo = -dir;
    if (bsdf_two_sided(m)) {
        if (dot(sd.wo, sn) < 0.f) sn = -sn;
        if (dot(sd.wo, g) < 0.f) g = -g;
    }
    sd.sn = sn;
    sd.gn = g;
    sd.frame = frame_from(sn);
}

// RayTracer::computeDirect (Renderer.h:269-354).  Draws the light and the
// light sample; returns true with the shadow ray and the contribution it
// carries when the contribution can be non-zero.
// K is the material kind when the launch shades one kind (else -1); INL
// inlines the environment sampler as well.
template <int K, bool INL>
__device__ __forceinline__ bool next_event_t(const SceneView& sv, const DevMaterial& m, const Shading& sd, uint64_t& rng,
                                             float4& so, float4& sdir, F3& contrib, const GuideView& gv, int qroot,
                                             float frac, const float4* __restrict__ mix) {
    if (bsdf_pure_specular_k<K>(m)) return false;
    if (sv.nlights == 0) return false;
    float pmf = 1.f / (float)sv.nlights;
    unsigned nl = (unsigned)sv.nlights;
    float fu = floorf(pgx_rng_next(rng) * (float)nl);
    unsigned idx = (unsigned)fu;
    idx = (nl - 1u < idx) ? nl - 1u : idx;
    F3 target, wi, emitted;
    float pdf_light;
    if (sv.has_env_light && idx == 0) {
        F3 dir = INL ? env_sample_i(sv.env, rng, emitted, pdf_light) : env_sample(sv.env, rng, emitted, pdf_light);
        if (pdf_light <= 0.f) return false;
        wi = normalize(dir);
        float cos_t = s_max(dot(wi, sd.sn), 0.f);
        if (cos_t <= 0.f) return false;
        F3 f = bsdf_eval_k<K>(m, sv.tex, sd, wi);
        float pal = pdf_light * pmf;
        float pab = bsdf_pdf_k<K>(m, sv.tex, sd, wi);
        if (qroot >= 0) pab = gv.pss ? pss_mixture_pdf(gv, qroot, frac, sd, pab, wi) : mixture_pdf(gv, qroot, frac, pab, wi);
        if (mix) pab = frac * mlp::packed_pdf(mix, wi) + (1.f - frac) * pab;
        float wd = power_heuristic(pal, pab);
        contrib = divs(((emitted * f) * cos_t) * wd, pal);
        target = f3(sv.bounds.centre[0], sv.bounds.centre[1], sv.bounds.centre[2]) + wi * sv.bounds.radius;
    } else {
        const DevAreaLight& L = sv.lights[idx - (unsigned)sv.has_env_light];
        float r1 = pgx_rng_next(rng);
        float r2 = pgx_rng_next(rng);
        float sq = sqrtf(r1);
        float a = 1.f - sq;
        float b = r2 * sq;
        float c = (1.f - a) - b;
        float area = L.p0.w;
        pdf_light = 1.f / area;
        target = ((f3(L.p0) * a) + (f3(L.p1) * b)) + (f3(L.p2) * c);
        emitted = f3(L.emission);
        if (pdf_light <= 0.f) return false;
        F3 stl = target - sd.x;
        wi = normalize(stl);
        float den = length_sq(stl);
        if (den < PGX_EPSILON) return false;
        float cos_t = s_max(dot(wi, sd.sn), 0.f);
        float cos_tp = s_max(dot(-wi, f3(L.gn)), 0.f);
        float G = (cos_t * cos_tp) / den;
        F3 f = bsdf_eval_k<K>(m, sv.tex, sd, wi);
        float pb = bsdf_pdf_k<K>(m, sv.tex, sd, wi);
        if (qroot >= 0) pb = gv.pss ? pss_mixture_pdf(gv, qroot, frac, sd, pb, wi) : mixture_pdf(gv, qroot, frac, pb, wi);
        if (mix) pb = frac * mlp::packed_pdf(mix, wi) + (1.f - frac) * pb;
        float pal = pdf_light * pmf;
        float pab = (pb * cos_tp) / den;
        float wd = power_heuristic(pal, pab);
        contrib = divs(((emitted * f) * G) * wd, pal);
    }
    if (contrib.x == 0.f && contrib.y == 0.f && contrib.z == 0.f) return false;
    // Scene::visible (Scene.h:139-146) from the offset origin to the target.
    float sgn = (dot(wi, sd.gn) >= 0.f) ? 1.f : -1.f;
    F3 p1 = sd.x + sd.gn * (PGX_EPSILON * sgn);
    F3 dv = target - p1;
    float max_t = length(dv) - (2.f * PGX_EPSILON);
    dv = normalize(dv);
    F3 org = p1 + dv * PGX_EPSILON;
    so = make_float4(org.x, org.y, org.z, max_t);
    sdir = make_float4(dv.x, dv.y, dv.z, 0.f);
    return true;
}
__device__ __noinline__ bool next_event(const SceneView& sv, const DevMaterial& m, const Shading& sd, uint64_t& rng,
                                        float4& so, float4& sdir, F3& contrib, const GuideView& gv, int qroot, float frac,
                                        const float4* __restrict__ mix) {
    return next_event_t<-1, false>(sv, m, sd, rng, so, sdir, contrib, gv, qroot, frac, mix);
}

// Light sampling for the guided-Li estimator: the reference computes NEE
// there too (Renderer.h:463) but never uses it in the image, so only the
// random numbers are drawn.
__device__ void next_event_draws(const SceneView& sv, const DevMaterial& m, uint64_t& rng) {
    if (bsdf_pure_specular(m)) return;
    if (sv.nlights == 0) return;
    unsigned nl = (unsigned)sv.nlights;
    float fu = floorf(pgx_rng_next(rng) * (float)nl);
    unsigned idx = (unsigned)fu;
    idx = (nl - 1u < idx) ? nl - 1u : idx;
    if (sv.has_env_light && idx == 0) {
        pgx_rng_next(rng);
        pgx_rng_next(rng);
    } else {
        pgx_rng_next(rng);
        pgx_rng_next(rng);
    }
}

// Continuation direction of the learned-guide estimator: one-sample MIS
// between the network's vMF mixture (probability frac; the selection number
// is reused as the lobe choice) and the BSDF; pdf is the mixture pdf.
// K: the material kind when the caller shades a single kind, else -1.
template <int K>
__device__ __forceinline__ F3 mlp_guided_sample_t(const float4* __restrict__ mix, float frac, const DevMaterial& m,
                                                  const TexView& tv, const Shading& sd, uint64_t& rng, F3& f,
                                                  float& pdf) {
    float sel = pgx_rng_next(rng);
    F3 wi;
    if (sel < frac) {
        float u1 = pgx_rng_next(rng), u2 = pgx_rng_next(rng);
        wi = mlp::packed_sample(mix, sel / frac, u1, u2);
        f = bsdf_eval_k<K>(m, tv, sd, wi);
    } else {
        float bp;
        wi = bsdf_sample_k<K>(m, tv, sd, rng, f, bp);
        // non-specular: bsdf_sample's pdf is bsdf_pdf(wi)
        pdf = frac * mlp::packed_pdf(mix, wi) + (1.f - frac) * bp;
        return wi;
    }
    float bp = bsdf_pdf_k<K>(m, tv, sd, wi);
    pdf = frac * mlp::packed_pdf(mix, wi) + (1.f - frac) * bp;
    return wi;
}
static __device__ __noinline__ F3 mlp_guided_sample(const float4* __restrict__ mix, float frac, const DevMaterial& m,
                                                    const TexView& tv, const Shading& sd, uint64_t& rng, F3& f,
                                                    float& pdf) {
    return mlp_guided_sample_t<-1>(mix, frac, m, tv, sd, rng, f, pdf);
}

template <int K = -1>
__device__ __forceinline__ bool mlp_guided_surface(const DevMaterial& m) {
    return !m.is_light && !bsdf_pure_specular_k<K>(m) && (K >= 0 ? K : m.kind) != PGX_BSDF_GLASS;
}

// Learned guide, one depth: the network evaluated on the tensor cores for
// the paths of the depth's diffuse, conductor and other bins (classified
// first), 128 paths per tile; paths whose hit is a guided surface get their
// packed vMF mixture in ps.guide.  Each CTA runs
// kInferGroups groups of 128 threads on independent tiles (they share the
// weights in shared memory), so one group's gathers and epilogues overlap
// another's MMAs.
constexpr int kInferGroups = 3;
constexpr int kInferAct = (mlp::kIn / 8) * mlp::kChunk;
constexpr int kInferSmem = mlp::kImageBytes + mlp::kBiasFloats * 4 + kInferGroups * kInferAct;
constexpr uint32_t kInferCols = 256;  // >= 64 per group, a power of two

__global__ void __launch_bounds__(128 * kInferGroups, 2) k_guide_infer(SceneView sv, PathState ps, int depth, MlpView mv,
                                                                   int* status, GuideView gv, const int* region_count,
                                                                   int fallback_min) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mbar[kInferGroups];
    __shared__ int flag[kInferGroups];
    __shared__ uint32_t tslot;
    const int g = threadIdx.x >> 7;
    mlp::FwdSmem s;
    s.w = smem;
    s.bias = reinterpret_cast<float*>(smem + mlp::kImageBytes);
    s.act = smem + mlp::kImageBytes + mlp::kBiasFloats * 4 + g * kInferAct;
    s.mbar = &mbar[g];
    s.flag = &flag[g];
    s.bar = 1 + g;
    s.tg = threadIdx.x & 127;
    {
        const uint4* src = reinterpret_cast<const uint4*>(mv.image);
        uint4* dst = reinterpret_cast<uint4*>(s.w);
        for (int i = threadIdx.x; i < mlp::kImageBytes / 16; i += blockDim.x) dst[i] = src[i];
        const float* b = reinterpret_cast<const float*>(mv.image + mlp::kImageBytes);
        for (int i = threadIdx.x; i < mlp::kBiasFloats; i += blockDim.x) s.bias[i] = b[i];
    }
    if (threadIdx.x < kInferGroups) tc::mbar_init(&mbar[threadIdx.x], 1);
    if (threadIdx.x < 32) {
        tc::tmem_alloc(&tslot, kInferCols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    s.tmem = tslot + (uint32_t)(g * 64);
    uint32_t phase = 0;
    // Only the bins of the classes that can be guided (diffuse, conductor,
    // other; k_classify ran first) are evaluated, back to back.
    const unsigned* cc = ps.ccount + depth * kShadeClasses;
    const unsigned n2 = cc[2], n3 = cc[3], n5 = cc[5];
    const unsigned n = n2 + n3 + n5;
    const unsigned groups = gridDim.x * kInferGroups;
    for (unsigned tile = blockIdx.x * kInferGroups + g; tile * (unsigned)mlp::kRows < n; tile += groups) {
        const unsigned i = tile * mlp::kRows + s.tg;
        int p = 0;
        bool need = false;
        F3 x = zero3(), nn = zero3(), wo = zero3();
        if (i < n) {
            const size_t at = i < n2 ? 2 * ps.capacity + i
                            : (i < n2 + n3 ? 3 * ps.capacity + (i - n2) : 5 * ps.capacity + (i - n2 - n3));
            p = ps.cqueue[at];
            float4 h = ps.hit[p];
            if (__float_as_int(h.x) >= 0) {
                Shading sd;
                DevMaterial m;
                F3 tri_gn;
                float tri_area;
                shading_data(sv, ps.o[p], ps.d[p], h, sd, m, tri_gn, tri_area);
                need = mlp_guided_surface(m);
                x = sd.x;
                nn = sd.sn;
                wo = sd.wo;
            }
        }
        mlp::encode_row(s.act, s.tg, mv.bounds, x, nn, wo);
        float raw[mlp::kOut];
        if (!mlp::forward_tile(s, phase, raw)) {
            if (s.tg == 0) atomicAdd(status, 1);
            break;
        }
        // QuadTree fallback: where the network has been trained on fewer
        // than fallback_min radiance samples of the vertex's cache region,
        // that region's quadtree guides instead (as in the QuadTree mode:
        // the BSDF alone where the region recorded no flux, marked -2).
        int fb = -1;
        if (need && region_count) {
            const int r = guide_region_index(gv, x);
            if (r >= 0 && region_count[r] < fallback_min) fb = gv.region_qroot[r] >= 0 ? gv.region_qroot[r] : -2;
        }
        const unsigned nfb = __ballot_sync(0xFFFFFFFFu, fb != -1);
        if ((s.tg & 31) == 0 && nfb) atomicAdd(&ps.stats[6], (unsigned long long)__popc(nfb));
        if (need) {
            ps.fallback[p] = fb;
            if (fb == -1) {
                float4 gm[mlp::kPacked];
                mlp::pack_mixture(raw, gm);
                float4* dst = ps.guide + (size_t)p * mlp::kPacked;
#pragma unroll
                for (int j = 0; j < mlp::kPacked; j++) dst[j] = gm[j];
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_dealloc(tslot, kInferCols);
}

__device__ __forceinline__ void push_shadow(PathState& ps, int depth, int p, float4 so, float4 sdir, F3 c,
                                            bool want) {
    unsigned slot = warp_aggregated_add(&ps.scount[depth], want);
    if (want) {
        ps.sh_path[slot] = p;
        ps.sh_o[slot] = so;
        ps.sh_d[slot] = sdir;
        ps.sh_c[slot] = make_float4(c.x, c.y, c.z, 0.f);
    }
}

// Bins the paths of this depth by shading class (k_shade then runs once per
// class on its bin).  Each block takes tiles of kClassifyTile queue entries,
// kClassifyItems per thread so the hit and class gathers overlap; entries are
// ranked within their class by warp match + shared-memory counters and each
// class bin is reserved with ONE global atomic per tile (a warp-level append
// would put ~n/32 atomics on each of the six counters).
constexpr int kClassifyItems = 8;
constexpr unsigned kClassifyTile = kThreads * kClassifyItems;

__global__ void __launch_bounds__(kThreads) k_classify(SceneView sv, PathState ps, int depth) {
    __shared__ unsigned s_count[kShadeClasses];
    __shared__ unsigned s_base[kShadeClasses];
    const unsigned n = ps.qcount[depth];
    const int* __restrict__ q = ps.queue[depth & 1];
    unsigned* cc = ps.ccount + depth * kShadeClasses;
    const unsigned tiles = (n + kClassifyTile - 1) / kClassifyTile;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    for (unsigned t = blockIdx.x; t < tiles; t += gridDim.x) {  // block-uniform trip count
        if (threadIdx.x < kShadeClasses) s_count[threadIdx.x] = 0;
        int p[kClassifyItems], cls[kClassifyItems];
        unsigned rank[kClassifyItems];
#pragma unroll
        for (int j = 0; j < kClassifyItems; j++) {
            const unsigned i = t * kClassifyTile + j * kThreads + threadIdx.x;
            p[j] = i < n ? q[i] : -1;
        }
#pragma unroll
        for (int j = 0; j < kClassifyItems; j++) {
            cls[j] = -1;
            if (p[j] >= 0) {
                const int id = __float_as_int(ps.hit[p[j]].x);
                cls[j] = id >= 0 ? min((int)sv.tri_class[id], kShadeClasses - 1) : 0;
            }
        }
        __syncthreads();  // counters cleared
#pragma unroll
        for (int j = 0; j < kClassifyItems; j++) {
            const unsigned m = __match_any_sync(0xFFFFFFFFu, cls[j]);
            const int leader = __ffs(m) - 1;
            unsigned base = 0;
            if (lane == leader && cls[j] >= 0) base = atomicAdd(&s_count[cls[j]], __popc(m));
            rank[j] = __shfl_sync(0xFFFFFFFFu, base, leader) + __popc(m & below);
        }
        __syncthreads();  // tile counts complete
        if (threadIdx.x < kShadeClasses) {
            const unsigned c = s_count[threadIdx.x];
            s_base[threadIdx.x] = c ? atomicAdd(&cc[threadIdx.x], c) : 0u;
        }
        __syncthreads();  // bin bases published
#pragma unroll
        for (int j = 0; j < kClassifyItems; j++)
            if (cls[j] >= 0) ps.cqueue[(size_t)cls[j] * ps.capacity + s_base[cls[j]] + rank[j]] = p[j];
    }
}

// Resident blocks per SM the shading launches are compiled for (64
// registers).  Measured on the interior workload: the inlined diffuse and
// conductor kernels spill a little at this bound, and are still faster than
// at 5-7 blocks per SM without spills or at 10-12 with more spills.
constexpr int kShadeBlocksPerSM = 8;

// CLS >= 0 shades the bin of that surface class with everything the class
// implies known at compile time (0: misses only; 1: emitters, which end the
// path; 2, 3, 4: diffuse, conductor, glass BSDFs inlined); CLS < 0 takes the
// class from `cls` at run time (cls < 0: the whole queue of this depth).
template <int MODE, bool BATCH = false, int CLS = -1>
__global__ void __launch_bounds__(kThreads, kShadeBlocksPerSM) k_shade(SceneView sv0, PathState ps, FrameParams fp, int depth,
                                                    GuideView gv, const BatchInfo* binfo = nullptr, int cls = -1) {
    constexpr int KIND = CLS == 2 ? PGX_BSDF_DIFFUSE
                       : CLS == 3 ? PGX_BSDF_CONDUCTOR
                       : CLS == 4 ? PGX_BSDF_GLASS
                                  : -1;
    constexpr bool INL = CLS >= 0 && CLS <= 4;
    if (CLS >= 0) cls = CLS;
    const unsigned n = cls < 0 ? ps.qcount[depth] : ps.ccount[depth * kShadeClasses + cls];
    const int* __restrict__ q = cls < 0 ? ps.queue[depth & 1] : ps.cqueue + (size_t)cls * ps.capacity;
    int* __restrict__ qn = ps.queue[(depth + 1) & 1];
    const int64_t cap = ps.capacity;
    // Uniform trip count per warp so the warp-aggregated appends see whole warps.
    const unsigned stride = gridDim.x * blockDim.x;
    const unsigned first = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned rounds = (n + stride - 1) / stride;
    for (unsigned r = 0; r < rounds; r++) {
        unsigned i = first + r * stride;
        bool active = i < n;
        bool cont = false, want_shadow = false;
        float4 so = make_float4(0.f, 0.f, 0.f, 0.f), sdir = so;
        F3 sc = zero3();
        int p = active ? q[i] : 0;
        SceneView svb;
        if (BATCH) {
            // the path's scene: its lights and bounds in the merged arrays
            svb = sv0;
            if (active) {
                const BatchInfo& bi = binfo[ps.scene[p]];
                svb.lights = sv0.lights + bi.light_base;
                svb.nlights = bi.n_lights + bi.has_env_light;
                svb.n_area_lights = bi.n_lights;
                svb.env = bi.env;
                svb.has_env_light = bi.has_env_light;
                svb.bounds = bi.bounds;
                svb.width = bi.width;
                svb.height = bi.height;
            }
        }
        const SceneView& sv = BATCH ? svb : sv0;
        // Recording for the cache outside guided-Li: the radiance the path has
        // gathered up to here (after the previous vertex's NEE) is the
        // baseline from which k_finalize recovers that vertex's incident Li.
        const int sample_of_p = fp.spp0 + (int)(p / ((int64_t)sv.width * sv.height));
        const bool rec_on = MODE != PGX_MODE_GUIDED_LI && active && sample_of_p >= fp.collect_lo &&
                            sample_of_p < fp.collect_hi;
        // (written below, after this vertex's emission is known)
        if (active) {
            float4 o = ps.o[p], d = ps.d[p], h = ps.hit[p], Tw = ps.T[p];
            uint64_t rng = ps.rng[p];
            int flags = ps.flags[p];
            bool prev_spec = flags & 1;
            float prev_pdf = Tw.w;
            F3 T = f3(Tw);
            F3 add = zero3();
            F3 dir = f3(d);
            int id = __float_as_int(h.x);
            // guided-Li record of this vertex (Renderer.h:419-427)
            F3 r_pos = zero3(), r_nrm = zero3(), r_wi = zero3(), r_w = zero3(), r_e = zero3();
            F3 r_wo = zero3(), r_f = zero3();
            float r_pdf = 0.f;  // solid-angle pdf the continuation was sampled with
            bool r_store = false;
            if (CLS != 0 && id >= 0) {
                Shading sd;
                DevMaterial m;
                F3 tri_gn;
                float tri_area;
                shading_data(sv, o, d, h, sd, m, tri_gn, tri_area);
                r_pos = sd.x;
                r_nrm = sd.sn;
                r_wo = sd.wo;
                const bool is_light = CLS < 0 ? (bool)m.is_light : CLS == 1;
                if (is_light) {
                    F3 em = f3(m.emission[0], m.emission[1], m.emission[2]);
                    if (MODE == PGX_MODE_GUIDED_LI) {
                        r_e = em;
                    } else if (depth == 0 || prev_spec) {
                        add = T * em;
                    } else {
                        float pmf = 1.f / (float)sv.nlights;
                        float pdf_light = 1.f / tri_area;
                        float cos_tp = s_max(dot(-dir, tri_gn), 0.f);
                        float d2 = sd.t * sd.t;
                        if (cos_tp > 0.f && !(d2 < PGX_EPSILON)) {
                            float pal = pdf_light * pmf;
                            float pab = (prev_pdf * cos_tp) / d2;
                            float wind = power_heuristic(pab, pal);
                            add = (T * em) * wind;
                        }
                    }
                } else {
                    int qroot = -1;
                    const bool spec = bsdf_pure_specular_k<KIND>(m);
                    if (MODE == PGX_MODE_GUIDED_QUADTREE && depth < fp.guide_depth && !spec && !gv.pss &&
                        qt_guided_surface<KIND>(gv, m))
                        qroot = guide_region_root(gv, sd.x);
                    if (MODE == PGX_MODE_GUIDED_PSS && depth < fp.guide_depth && gv.pss && pss_surface<KIND>(m))
                        qroot = guide_region_root(gv, sd.x);
                    bool use_mix =
                        MODE == PGX_MODE_GUIDED_MLP && depth < fp.guide_depth && mlp_guided_surface<KIND>(m);
                    if (MODE == PGX_MODE_GUIDED_MLP && use_mix) {
                        // the region's quadtree stands in for an untrained network
                        const int fb = ps.fallback[p];
                        if (fb != -1) {
                            qroot = fb >= 0 ? fb : -1;
                            use_mix = false;
                        }
                    }
                    const float4* mix = use_mix ? ps.guide + (size_t)p * mlp::kPacked : nullptr;
                    if (MODE == PGX_MODE_GUIDED_LI) {
                        next_event_draws(sv, m, rng);
                    } else {
                        F3 c;
                        if constexpr (INL) {
                            want_shadow =
                                next_event_t<KIND, true>(sv, m, sd, rng, so, sdir, c, gv, qroot, fp.guide_fraction, mix);
                            // queued here so the shadow ray is not held through sampling
                            push_shadow(ps, depth, p, so, sdir, T * c, want_shadow);
                        } else {
                            want_shadow = next_event(sv, m, sd, rng, so, sdir, c, gv, qroot, fp.guide_fraction, mix);
                            sc = T * c;
                        }
                    }
                    bool alive = true;
                    float rrp_rec = 1.f;
                    if (depth > 3) {
                        if (MODE == PGX_MODE_GUIDED_LI) {
                            if (pgx_rng_next(rng) < 0.7f)
                                rrp_rec = 0.7f;
                            else
                                alive = false;
                        } else {
                            float rrp = s_min(s_max(PGX_EPSILON, lum(T)), 1.f);
                            if (pgx_rng_next(rng) < rrp)
                                T = divs(T, rrp);
                            else
                                alive = false;
                        }
                    }
                    if (alive && depth == fp.max_depth) alive = false;
                    if (alive) {
                        // The diffuse light sampling above reads only the frame's
                        // normal: rebuilding the frame (same input, same bits) here
                        // keeps its tangents out of registers during it.
                        if constexpr (KIND == PGX_BSDF_DIFFUSE) sd.frame = frame_from(sd.sn);
                        F3 f;
                        float pdf;
                        F3 wi;
                        if (MODE == PGX_MODE_GUIDED_QUADTREE || (MODE == PGX_MODE_GUIDED_MLP && qroot >= 0))
                            wi = guided_sample<KIND>(gv, fp.guide_fraction, m, sv.tex, sd, rng, f, pdf, qroot);
                        else if (MODE == PGX_MODE_GUIDED_PSS)
                            wi = pss_guided_sample<KIND>(gv, fp.guide_fraction, m, sv.tex, sd, rng, f, pdf, qroot);
                        else if (MODE == PGX_MODE_GUIDED_MLP && use_mix && INL)
                            wi = mlp_guided_sample_t<KIND>(mix, fp.guide_fraction, m, sv.tex, sd, rng, f, pdf);
                        else if (MODE == PGX_MODE_GUIDED_MLP && use_mix)
                            wi = mlp_guided_sample(mix, fp.guide_fraction, m, sv.tex, sd, rng, f, pdf);
                        else
                            wi = bsdf_sample_k<KIND>(m, sv.tex, sd, rng, f, pdf);
                        float cos_t = fabsf(dot(wi, sd.sn));
                        if (MODE == PGX_MODE_GUIDED_LI) {
                            if (pdf <= 0.f || cos_t <= 0.f) {
                                alive = false;
                            } else {
                                r_wi = wi;
                                r_w = divs(f * cos_t, pdf * rrp_rec);
                                r_store = !spec;
                            }
                        } else {
                            if (pdf <= 0.f || cos_t <= 0.f) {
                                alive = false;
                            } else {
                                r_f = divs(f * cos_t, pdf);
                                T = divs(T * f * cos_t, pdf);
                                if (lum(T) <= 0.f) alive = false;
                                if (isnan(T.x) || isnan(T.y) || isnan(T.z)) alive = false;
                                if (isinf(T.x) || isinf(T.y) || isinf(T.z)) alive = false;
                                if (T.x < 0.f || T.y < 0.f || T.z < 0.f) alive = false;
                            }
                        }
                        if (alive) {
                            if (rec_on) {
                                // Primary-sample guides are built over the
                                // cosine sampler's inverse: record only the
                                // surfaces that sample through it.
                                r_store = !spec && (MODE != PGX_MODE_GUIDED_PSS || pss_surface<KIND>(m));
                                r_wi = wi;
                                r_pdf = pdf;
                                r_w = T;  // throughput after this vertex
                            }
                            float sgn = (dot(wi, sd.gn) >= 0.f) ? 1.f : -1.f;
                            F3 org = sd.x + sd.gn * (PGX_EPSILON * sgn);
                            ps.o[p] = make_float4(org.x, org.y, org.z, 0.f);
                            ps.d[p] = make_float4(wi.x, wi.y, wi.z, 0.f);
                            ps.T[p] = make_float4(T.x, T.y, T.z, pdf);
                            ps.flags[p] = spec ? 1 : 0;
                            cont = true;
                        }
                    }
                }
            } else if (CLS <= 0) {
                // Miss: background (Renderer.h:501-527, 596-612).
                F3 bg = env_eval(sv.env, dir);
                if (MODE == PGX_MODE_GUIDED_LI) {
                    r_e = bg;
                } else if (depth == 0 || prev_spec) {
                    add = T * bg;
                } else if (!(lum(bg) < 1e-8f)) {
                    float pmf = 1.f / (float)sv.nlights;
                    float pdf_light = INL ? env_pdf_i(sv.env, dir) : env_pdf(sv.env, dir);
                    if (pmf > 0.f && pdf_light > 0.f) {
                        float pal = pmf * pdf_light;
                        float wind = power_heuristic(prev_pdf, pal);
                        add = (T * bg) * wind;
                    }
                }
            }
            if (MODE == PGX_MODE_GUIDED_LI) {
                size_t ri = (size_t)depth * cap + p;
                ps.rec_pos[ri] = make_float4(r_pos.x, r_pos.y, r_pos.z, r_store ? 1.f : 0.f);
                ps.rec_nrm[ri] = make_float4(r_nrm.x, r_nrm.y, r_nrm.z, 0.f);
                ps.rec_wi[ri] = make_float4(r_wi.x, r_wi.y, r_wi.z, 0.f);
                ps.rec_w[ri] = make_float4(r_w.x, r_w.y, r_w.z, 0.f);
                ps.rec_e[ri] = make_float4(r_e.x, r_e.y, r_e.z, 0.f);
                ps.nrec[p] = depth + 1;
            } else {
                const bool adds = add.x != 0.f || add.y != 0.f || add.z != 0.f || !valid(add);
                const bool snap = rec_on && depth > 0;
                if (adds || snap) {
                    float4 l = ps.L[p];
                    // Baseline of the previous vertex's incident radiance: the
                    // full Li is what the path gathers from this vertex's
                    // emission on (snapshot before it); the indirect-only
                    // target of the learned guide starts after it.
                    if (snap)
                        ps.rec_e[(size_t)(depth - 1) * cap + p] =
                            fp.train == 1 ? make_float4(l.x + add.x, l.y + add.y, l.z + add.z, 0.f) : l;
                    if (adds) ps.L[p] = make_float4(l.x + add.x, l.y + add.y, l.z + add.z, 0.f);
                }
                if (rec_on) {
                    size_t ri = (size_t)depth * cap + p;
                    ps.rec_pos[ri] = make_float4(r_pos.x, r_pos.y, r_pos.z, (cont && r_store) ? 1.f : 0.f);
                    if (cont && r_store) {
                        ps.rec_nrm[ri] = make_float4(r_nrm.x, r_nrm.y, r_nrm.z, 0.f);
                        ps.rec_wi[ri] = make_float4(r_wi.x, r_wi.y, r_wi.z, r_pdf);
                        ps.rec_w[ri] = make_float4(r_w.x, r_w.y, r_w.z, 0.f);
                        if (MODE == PGX_MODE_GUIDED_MLP && fp.train) {
                            ps.rec_wo[ri] = make_float4(r_wo.x, r_wo.y, r_wo.z, 0.f);
                            ps.rec_f[ri] = make_float4(r_f.x, r_f.y, r_f.z, 0.f);
                        }
                    }
                    ps.nrec[p] = depth + 1;
                }
            }
            ps.rng[p] = rng;
        }
        if (MODE != PGX_MODE_GUIDED_LI && !INL) push_shadow(ps, depth, p, so, sdir, sc, active && want_shadow);
        unsigned slot = warp_aggregated_add(&ps.qcount[depth + 1], active && cont);
        if (active && cont) qn[slot] = p;
    }
}

// MitchellNetravaliFilter::separable with B = C = 1/3 (Imaging.h:160-175).
__device__ __forceinline__ float mitchell_1d(float val) {
    const float B = 1.f / 3.f, C = 1.f / 3.f;
    float x = fabsf(val);
    float x2 = x * x;
    float x3 = x * x * x;
    if (x < 1.f)
        return (1.f / 6.f) * ((12.f - 9.f * B - 6.f * C) * x3 + (-18.f + 12.f * B + 6.f * C) * x2 + (6.f - 2.f * B));
    if (x < 2.f)
        return (1.f / 6.f) * ((-B - 6.f * C) * x3 + (6.f * B + 30.f * C) * x2 + (-12.f * B - 48.f * C) * x +
                              (8.f * B + 24.f * C));
    return 0.f;
}

// Film::splat (Imaging.h:186-217) with the box filter (radius 1) or the
// Mitchell-Netravali filter (radius 2): weights of the in-image pixels around
// round(x, y), normalised by their sum.
template <int R>
__device__ __forceinline__ void splat_r(float* film, float* film2, int W, int H, float x, float y, F3 c) {
    constexpr int K = (2 * R + 1) * (2 * R + 1);
    int bx = (int)floorf(x + 0.5f), by = (int)floorf(y + 0.5f);
    int idx[K];
    float wts[K];
    int used = 0;
    float total = 0.f;
    for (int i = -R; i <= R; i++)
        for (int j = -R; j <= R; j++) {
            int px = bx + j, py = by + i;
            if (px >= 0 && px < W && py >= 0 && py < H) {
                idx[used] = py * W + px;
                float dx = (float)px - x, dy = (float)py - y;
                wts[used] = (R == 1) ? ((fabsf(dx) < 0.5f && fabsf(dy) < 0.5f) ? 1.f : 0.f)
                                     : mitchell_1d(dx) * mitchell_1d(dy);
                total += wts[used];
                used++;
            }
        }
    if (used > 0 && fabsf(total) > 1e-4f) {
        for (int k = 0; k < used; k++) {
            if (wts[k] == 0.f) continue;
            F3 v = divs(c * wts[k], total);
            atomicAdd(film + 3 * idx[k] + 0, v.x);
            atomicAdd(film + 3 * idx[k] + 1, v.y);
            atomicAdd(film + 3 * idx[k] + 2, v.z);
            if (film2) {
                atomicAdd(film2 + 3 * idx[k] + 0, v.x * v.x);
                atomicAdd(film2 + 3 * idx[k] + 1, v.y * v.y);
                atomicAdd(film2 + 3 * idx[k] + 2, v.z * v.z);
            }
        }
    }
}

__device__ __forceinline__ void splat(float* film, float* film2, int W, int H, float x, float y, F3 c, bool mitchell) {
    if (mitchell)
        splat_r<2>(film, film2, W, H, x, y, c);
    else
        splat_r<1>(film, film2, W, H, x, y, c);
}

// Film::tonemap (Imaging.h:220-244) for every pixel.
__global__ void k_tonemap(const float* __restrict__ film, int64_t npix, int spp, float exposure, float lmax_white,
                          uint8_t* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    float inv_spp = (spp > 0) ? 1.f / (float)spp : 1.f;
    F3 col = (f3(film[3 * i], film[3 * i + 1], film[3 * i + 2]) * inv_spp) * exposure;
    float lin = lum(col);
    uint8_t r = 0, g = 0, b = 0;
    if (!(lin < 1e-4f)) {
        float lw2 = lmax_white * lmax_white;
        float lout = lin * (1.f + (lin / lw2)) / (1.f + lin);
        float coef = lout / lin;
        float ge = 1.f / 2.2f;
        float cr = powf(col.x * coef, ge), cg = powf(col.y * coef, ge), cb = powf(col.z * coef, ge);
        r = (uint8_t)(s_max(0.f, s_min(cr, 1.f)) * 255.f);
        g = (uint8_t)(s_max(0.f, s_min(cg, 1.f)) * 255.f);
        b = (uint8_t)(s_max(0.f, s_min(cb, 1.f)) * 255.f);
    }
    out[3 * i] = r;
    out[3 * i + 1] = g;
    out[3 * i + 2] = b;
}

// End of frame: guided-Li back-propagation (Renderer.h:376-393), NaN/Inf
// drop (Renderer.h:697-700) and the film splat.
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_finalize(SceneView sv, PathState ps, FrameParams fp, float* film,
                                                       float* film2) {
    const int64_t npix = (int64_t)sv.width * sv.height;
    const int64_t n = npix * fp.batch;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        F3 col;
        const int sample_of_p = fp.spp0 + (int)(p / npix);
        const bool collect = sample_of_p >= fp.collect_lo && sample_of_p < fp.collect_hi;
        if (MODE == PGX_MODE_GUIDED_LI) {
            int nr = ps.nrec[p];
            F3 li = zero3();
            for (int i = nr - 1; i >= 0; i--) {
                size_t ri = (size_t)i * ps.capacity + p;
                float4 pos = ps.rec_pos[ri];
                if (collect && pos.w != 0.f && valid(li) && lum(li) > 0.f) {
                    unsigned slot = atomicAdd(ps.nvertices, 1u);
                    if (slot < (unsigned)ps.vcapacity) {
                        float4 nr4 = ps.rec_nrm[ri], wi = ps.rec_wi[ri];
                        pgx_path_vertex v;
                        v.position[0] = pos.x;
                        v.position[1] = pos.y;
                        v.position[2] = pos.z;
                        v.normal[0] = nr4.x;
                        v.normal[1] = nr4.y;
                        v.normal[2] = nr4.z;
                        v.wi[0] = wi.x;
                        v.wi[1] = wi.y;
                        v.wi[2] = wi.z;
                        v.Li[0] = li.x;
                        v.Li[1] = li.y;
                        v.Li[2] = li.z;
                        ps.vertices[slot] = v;
                    }
                }
                li = f3(ps.rec_e[ri]) + (f3(ps.rec_w[ri]) * li);
            }
            col = li;
        } else {
            col = f3(ps.L[p]);
            if (collect && valid(col)) {
                // Incident radiance along each recorded wi: what the path gathered
                // after that vertex, divided by the throughput it carried.
                int nr = ps.nrec[p];
                for (int i = 0; i < nr; i++) {
                    size_t ri = (size_t)i * ps.capacity + p;
                    float4 pos = ps.rec_pos[ri];
                    if (pos.w == 0.f) continue;
                    F3 tn = f3(ps.rec_w[ri]);
                    F3 dl = col - f3(ps.rec_e[ri]);
                    F3 li = f3(tn.x > 0.f ? dl.x / tn.x : 0.f, tn.y > 0.f ? dl.y / tn.y : 0.f,
                               tn.z > 0.f ? dl.z / tn.z : 0.f);
                    if (!(valid(li) && lum(li) > 0.f)) continue;
                    if (fp.train) {
                        // radiance sample for the learned guide, weight
                        // Lum(Li f |cos| / pdf); a hash of (path, vertex,
                        // batch) keeps a uniform share fp.train_keep of them
                        uint64_t hsh = pgx_splitmix64(((uint64_t)p << 5) ^ (uint64_t)i ^ ((uint64_t)fp.spp0 << 40));
                        float u = (float)(hsh >> 40) * (1.f / 16777216.f);
                        if (u >= fp.train_keep) continue;
                        float wgt = lum(li * f3(ps.rec_f[ri]));
                        if (!(wgt > 0.f) || isinf(wgt)) continue;
                        unsigned slot = atomicAdd(ps.ntrain, 1u);
                        if (slot >= (unsigned)ps.tcapacity) continue;
                        float4 nr4 = ps.rec_nrm[ri], wi = ps.rec_wi[ri], wo = ps.rec_wo[ri];
                        float* o = ps.train + (size_t)slot * 13;
                        o[0] = pos.x, o[1] = pos.y, o[2] = pos.z;
                        o[3] = nr4.x, o[4] = nr4.y, o[5] = nr4.z;
                        o[6] = wo.x, o[7] = wo.y, o[8] = wo.z;
                        o[9] = wi.x, o[10] = wi.y, o[11] = wi.z;
                        o[12] = wgt;
                        continue;
                    }
                    unsigned slot = atomicAdd(ps.nvertices, 1u);
                    if (slot >= (unsigned)ps.vcapacity) continue;
                    float4 nr4 = ps.rec_nrm[ri], wi = ps.rec_wi[ri];
                    pgx_path_vertex v;
                    v.position[0] = pos.x;
                    v.position[1] = pos.y;
                    v.position[2] = pos.z;
                    v.normal[0] = nr4.x;
                    v.normal[1] = nr4.y;
                    v.normal[2] = nr4.z;
                    v.wi[0] = wi.x;
                    v.wi[1] = wi.y;
                    v.wi[2] = wi.z;
                    v.Li[0] = li.x;
                    v.Li[1] = li.y;
                    v.Li[2] = li.z;
                    ps.vertices[slot] = v;
                    // Flux weight for the QuadTree guide: Lum(Li) |cos| / pdf
                    // (Mueller et al. 2017 divide by the sampling pdf).  Over
                    // directions its expected density is Li |cos|, over the
                    // cosine sampler's primary samples pi Li, whichever
                    // distribution sampled wi, so training on guided paths
                    // does not compound the previous guide.
                    const float cos_n = fabsf(nr4.x * wi.x + nr4.y * wi.y + nr4.z * wi.z);
                    ps.vweight[slot] = wi.w > 0.f ? lum(li) * cos_n / wi.w : 0.f;
                }
            }
        }
        if (!valid(col)) continue;
        float2 xy = ps.pix[p];
        splat(film, film2, sv.width, sv.height, xy.x, xy.y, col, fp.mitchell != 0);
    }
}

// ---- differentiable rendering ---------------------------------------------------------
// Plain path tracing with NEE + MIS (the estimator of k_shade<PLAIN>), in
// two flavours sharing diff_path:
//  * primal: sampling decisions (directions, pdfs, MIS weights, Russian
//    roulette, the environment's sampling tables) use the uploaded scene,
//    while radiance is evaluated with the "evaluation" parameters -- the
//    environment texels, a per-material albedo offset and GGX roughness.
//    Sample values are summed per target pixel in double in sample order,
//    and a gather kernel adds the 4 neighbours' partial sums in a fixed
//    order, so the image is deterministic and a finite difference between
//    two parameter sets differs only through the samples a parameter touches;
//  * adjoint: with evaluation = uploaded parameters, one thread per sample
//    traces the path once from its seed; every vertex j keeps (in the
//    thread's registers and local memory, never in global memory) what its
//    terms need, and once the path's radiance L is known the thread adds
//      d/dtheta of the terms added at j (NEE: albedo, roughness, the
//      environment texels under the light direction; escaped rays: the
//      texels under the ray), and
//      (L - L_up_to_j) * d log beta_j / dtheta for the continuation weight
//      beta_j = f(wi) |cos| / pdf(wi) (path replay backpropagation, Vicini
//      et al. 2021, whose second replay pass the per-vertex records
//      replace), with pdf detached,
//    each weighted by dLoss/dImage at the sample's pixel / spp, into double
//    accumulators (material terms per block in shared memory).
struct DiffView {
    const DevMaterial* __restrict__ mats_e;  // evaluation materials
    DevEnv env_e;                            // evaluation environment (sampling tables of sv.env)
    int spp, max_depth;
    uint64_t seed;
    double* partial;          // primal: [npix][4][3]
    const float* dimg;        // adjoint: dLoss/dImage [npix][3]
    double* g_env;            // [env W*H*3]
    double* g_alb;            // [nmats*3]
    double* g_rough;          // [nmats]
    unsigned long long* next; // next sample to take (zeroed before each launch)
    float4* samples;          // primal: values of the chunk's samples
    int s0, ns;               // primal: the chunk's samples [s0, s0 + ns)
    int nmats;
};

// Materials whose BSDF value (and sampled weight) is proportional to the
// albedo, so d log f / d albedo_c = 1 / albedo_c.
__device__ __forceinline__ bool albedo_linear(const DevMaterial& m) {
    return !m.layered && (m.kind == PGX_BSDF_DIFFUSE || m.kind == PGX_BSDF_ORENNAYAR ||
                          m.kind == PGX_BSDF_MIRROR || m.kind == PGX_BSDF_CONDUCTOR);
}

// d log f / d roughness of a rough GGX conductor at (wil, wol): from D
// (d log D / d alpha = 2/alpha - 4 alpha c^2 / (c^2 (alpha^2 - 1) + 1)) and
// both Smith G1 factors (d log G1 / d alpha = -(d Lambda / d alpha) /
// (1 + Lambda), d Lambda / d alpha = alpha tan^2 / (2 sqrt(1 + alpha^2
// tan^2))), times d alpha / d roughness = 1.62142^2 / (2 alpha).
__device__ float conductor_dlogf_drough(const DevMaterial& m, F3 wil, F3 wol) {
    if (m.kind != PGX_BSDF_CONDUCTOR || m.layered || m.alpha < PGX_EPSILON) return 0.f;
    if (wil.z <= 0.f || wol.z <= 0.f) return 0.f;
    F3 h = wil + wol;
    if (length_sq(h) < PGX_EPSILON) return 0.f;
    h = normalize(h);
    const float a = m.alpha, a2 = a * a;
    float c2 = h.z * h.z;
    float d = 2.f / a - 4.f * a * c2 / (c2 * (a2 - 1.f) + 1.f);
    auto dlg1 = [&](F3 w) {
        float wc2 = w.z * w.z;
        float t2 = fabsf(fmaxf(1.f - wc2, 0.f) / wc2);
        float r = sqrtf(1.f + a2 * t2);
        float lam = (r - 1.f) * 0.5f;
        return -(a * t2 / (2.f * r)) / (1.f + lam);
    };
    d += dlg1(wil) + dlg1(wol);
    return d * (1.62142f * 1.62142f) / (2.f * a);
}

// Adds g (rgb) times the bilinear weights of the environment lookup of wi
// (env_eval's texel choice) to the texel gradients.
__device__ void env_scatter(const DevEnv& e, F3 wi, F3 g, double* grad) {
    if (!e.valid || !grad) return;
    float u = atan2f(wi.z, wi.x);
    u = (u < 0.f) ? u + PGX_2PI_F : u;
    u = u * PGX_INV_2PI_F;
    float v = acosf(wi.y) * PGX_INV_PI_F;
    const int W = e.width, H = e.height;
    float uu = fmaxf(0.f, fabsf(u)) * (float)W;
    float vv = fmaxf(0.f, fabsf(v)) * (float)H;
    float fu = floorf(uu), fv = floorf(vv);
    int x = (fu >= -2147483648.f && fu < 2147483648.f) ? (int)fu : 0;
    int y = (fv >= -2147483648.f && fv < 2147483648.f) ? (int)fv : 0;
    float au = uu - (float)x, av = vv - (float)y;
    float w[4] = {(1.f - au) * (1.f - av), au * (1.f - av), (1.f - au) * av, au * av};
    x = wrap_index(x, W);
    y = wrap_index(y, H);
    int x1 = wrap_index(x + 1, W), y1 = wrap_index(y + 1, H);
    long long idx[4] = {(long long)y * W + x, (long long)y * W + x1, (long long)y1 * W + x, (long long)y1 * W + x1};
    for (int k = 0; k < 4; k++) {
        if (w[k] == 0.f) continue;
        atomicAdd(grad + 3 * idx[k] + 0, (double)(g.x * w[k]));
        atomicAdd(grad + 3 * idx[k] + 1, (double)(g.y * w[k]));
        atomicAdd(grad + 3 * idx[k] + 2, (double)(g.z * w[k]));
    }
}

struct DiffAcc {
    double* alb;    // shared memory [nmats*3] or global
    double* rough;  // [nmats]
};

__device__ __forceinline__ void add_alb(const DiffAcc& acc, int mat, F3 g) {
    atomicAdd(acc.alb + 3 * mat + 0, (double)g.x);
    atomicAdd(acc.alb + 3 * mat + 1, (double)g.y);
    atomicAdd(acc.alb + 3 * mat + 2, (double)g.z);
}

// What the gradient of one path vertex needs once the path's radiance is
// known: the NEE contribution and its log-derivative factors, the radiance
// collected up to the vertex (the continuation's term is delta x (L_total -
// L_snap) x d log beta / d theta), and the environment lookup of an
// environment light sample.
struct DiffVertex {
    F3 ia;        // 1 / albedo (per channel) when the material is albedo-linear, else 0
    F3 C;         // NEE contribution T * emitted * weight (0 without one)
    F3 tcw;       // environment NEE: T * radiance weight of the sample
    F3 wi;        // environment NEE direction
    F3 l_snap;    // radiance collected up to and including this vertex's NEE
    float dr_nee, dr_cont;
    int mat;
    int flags;    // 1: NEE term, 2: environment NEE, 4: continuation term
};

__device__ __forceinline__ F3 safe_div3(F3 a, F3 b) {
    return f3(a.x / fmaxf(b.x, 1e-6f), a.y / fmaxf(b.y, 1e-6f), a.z / fmaxf(b.z, 1e-6f));
}

// State of one path of the differentiable estimator between bounces.
struct DiffPath {
    F3 o, dir;
    F3 T, Ts, L;          // evaluation and sampling throughput, radiance so far
    F3 delta;             // adjoint of the sample's value (gradient pass)
    F3 esc_dir, esc_w;    // escaped ray: direction, T x MIS weight
    uint64_t rng;
    float prev_pdf;
    int depth, nvtx;
    bool prev_spec, escaped;
};

__device__ __forceinline__ void diff_begin(DiffPath& P, uint64_t rng, F3 o, F3 dir, F3 delta) {
    P.o = o;
    P.dir = dir;
    P.T = f3(1.f, 1.f, 1.f);
    P.Ts = P.T;
    P.L = zero3();
    P.delta = delta;
    P.esc_dir = zero3();
    P.esc_w = zero3();
    P.rng = rng;
    P.prev_pdf = 0.f;
    P.depth = 0;
    P.nvtx = 0;
    P.prev_spec = false;
    P.escaped = false;
}

// One bounce of the path: trace, background or emitter, NEE, Russian
// roulette, continuation.  Returns true when the path has ended.  GRAD: the
// vertex keeps what its gradient terms need (DiffVertex) in vtx[P.nvtx].
template <bool GRAD>
__device__ bool diff_step(const SceneView& sv, const DiffView& dv, DiffPath& P, DiffVertex* vtx) {
    F3& o = P.o;
    F3& dir = P.dir;
    F3& T = P.T;
    F3& Ts = P.Ts;
    F3& L = P.L;
    uint64_t& rng = P.rng;
    bool& prev_spec = P.prev_spec;
    float& prev_pdf = P.prev_pdf;
    int& nvtx = P.nvtx;
    bool& escaped = P.escaped;
    F3& esc_dir = P.esc_dir;
    F3& esc_w = P.esc_w;
    const int depth = P.depth;
    {

        int id;
        float t, hu, hv;
        int status;
        unsigned long long ni = 0, nt = 0;
        bvh_trace<false, false>(sv.bvh, mk(o.x, o.y, o.z), mk(dir.x, dir.y, dir.z), FLT_MAX, id, t, hu, hv, status,
                                ni, nt);
        if (status) id = -1;
        if (id < 0) {
            // Background (k_shade<PLAIN>'s miss branch); decisions on the
            // sampling environment, radiance from the evaluation one.
            F3 bg_s = env_eval(sv.env, dir);
            F3 bg = env_eval(dv.env_e, dir);
            float w = 0.f;
            if (depth == 0 || prev_spec) {
                w = 1.f;
            } else if (!(lum(bg_s) < 1e-8f)) {
                float pmf = 1.f / (float)sv.nlights;
                float pdf_light = env_pdf(sv.env, dir);
                if (pmf > 0.f && pdf_light > 0.f) w = power_heuristic(prev_pdf, pmf * pdf_light);
            }
            if (w > 0.f) {
                L = L + (T * bg) * w;
                if (GRAD) {
                    escaped = true;
                    esc_dir = dir;
                    esc_w = T * w;
                }
            }
            return true;
        }
        Shading sd;
        DevMaterial ms;
        F3 tri_gn;
        float tri_area;
        shading_data(sv, make_float4(o.x, o.y, o.z, 0.f), make_float4(dir.x, dir.y, dir.z, 0.f),
                     make_float4(__int_as_float(id), t, hu, hv), sd, ms, tri_gn, tri_area);
        const DevMaterial me = dv.mats_e[sd.mat];
        DiffVertex* V = GRAD ? &vtx[nvtx] : nullptr;
        if (GRAD) {
            nvtx++;
            V->flags = 0;
            V->mat = sd.mat;
            V->ia = albedo_linear(me) ? safe_div3(f3(1.f, 1.f, 1.f), albedo_of(sv.tex, me, sd)) : zero3();
        }
        if (ms.is_light) {
            F3 em = f3(ms.emission[0], ms.emission[1], ms.emission[2]);
            if (depth == 0 || prev_spec) {
                L = L + T * em;
            } else {
                float pmf = 1.f / (float)sv.nlights;
                float cos_tp = s_max(dot(-dir, tri_gn), 0.f);
                float d2 = sd.t * sd.t;
                if (cos_tp > 0.f && !(d2 < PGX_EPSILON)) {
                    float pab = (prev_pdf * cos_tp) / d2;
                    L = L + (T * em) * power_heuristic(pab, (1.f / tri_area) * pmf);
                }
            }
            return true;
        }
        // ---- next-event estimation (next_event with detached pdfs) ----
        if (!bsdf_pure_specular(ms) && sv.nlights > 0) {
            float pmf = 1.f / (float)sv.nlights;
            unsigned nl = (unsigned)sv.nlights;
            unsigned idx = (unsigned)floorf(pgx_rng_next(rng) * (float)nl);
            idx = (nl - 1u < idx) ? nl - 1u : idx;
            F3 target, wi, emitted;
            float pal = 0.f, wd = 0.f, geo = 0.f;
            bool ok = false, env_light = false;
            if (sv.has_env_light && idx == 0) {
                F3 col_s;
                float pdf_light;
                F3 d0 = env_sample(sv.env, rng, col_s, pdf_light);
                if (pdf_light > 0.f) {
                    wi = normalize(d0);
                    float cos_t = s_max(dot(wi, sd.sn), 0.f);
                    if (cos_t > 0.f) {
                        emitted = env_eval(dv.env_e, wi);
                        pal = pdf_light * pmf;
                        wd = power_heuristic(pal, bsdf_pdf(ms, sv.tex, sd, wi));
                        geo = cos_t;
                        target = f3(sv.bounds.centre[0], sv.bounds.centre[1], sv.bounds.centre[2]) +
                                 wi * sv.bounds.radius;
                        ok = true;
                        env_light = true;
                    }
                }
            } else {
                const DevAreaLight& Lt = sv.lights[idx - (unsigned)sv.has_env_light];
                float r1 = pgx_rng_next(rng);
                float r2 = pgx_rng_next(rng);
                float sq = sqrtf(r1);
                float a = 1.f - sq, b = r2 * sq, c = (1.f - a) - b;
                float pdf_light = 1.f / Lt.p0.w;
                target = ((f3(Lt.p0) * a) + (f3(Lt.p1) * b)) + (f3(Lt.p2) * c);
                emitted = f3(Lt.emission);
                if (pdf_light > 0.f) {
                    F3 stl = target - sd.x;
                    wi = normalize(stl);
                    float den = length_sq(stl);
                    if (!(den < PGX_EPSILON)) {
                        float cos_t = s_max(dot(wi, sd.sn), 0.f);
                        float cos_tp = s_max(dot(-wi, f3(Lt.gn)), 0.f);
                        geo = (cos_t * cos_tp) / den;
                        pal = pdf_light * pmf;
                        float pab = (bsdf_pdf(ms, sv.tex, sd, wi) * cos_tp) / den;
                        wd = power_heuristic(pal, pab);
                        ok = geo > 0.f;
                    }
                }
            }
            if (ok) {
                F3 fe = bsdf_eval(me, sv.tex, sd, wi);
                F3 cw = divs(fe * (geo * wd), pal);  // radiance weight of the light sample
                F3 contrib = emitted * cw;
                if (contrib.x != 0.f || contrib.y != 0.f || contrib.z != 0.f) {
                    float sgn = (dot(wi, sd.gn) >= 0.f) ? 1.f : -1.f;
                    F3 p1 = sd.x + sd.gn * (PGX_EPSILON * sgn);
                    F3 dvv = target - p1;
                    float max_t = length(dvv) - (2.f * PGX_EPSILON);
                    dvv = normalize(dvv);
                    F3 org = p1 + dvv * PGX_EPSILON;
                    int sid, sst;
                    float st_, su, sv_;
                    bool occluded = bvh_trace<true, false>(sv.bvh, mk(org.x, org.y, org.z), mk(dvv.x, dvv.y, dvv.z),
                                                           max_t, sid, st_, su, sv_, sst, ni, nt);
                    if (!occluded && !sst) {
                        F3 C = T * contrib;
                        L = L + C;
                        if (GRAD) {
                            V->flags |= 1;
                            V->C = C;
                            V->dr_nee = conductor_dlogf_drough(me, to_local(sd.frame, wi), to_local(sd.frame, sd.wo));
                            if (env_light) {
                                V->flags |= 2;
                                V->wi = wi;
                                V->tcw = T * cw;
                            }
                        }
                    }
                }
            }
        }
        // ---- Russian roulette on the sampling throughput ----
        if (depth > 3) {
            float q = s_min(s_max(PGX_EPSILON, lum(Ts)), 1.f);
            if (pgx_rng_next(rng) < q) {
                T = divs(T, q);
                Ts = divs(Ts, q);
            } else {
                return true;
            }
        }
        if (depth == dv.max_depth) return true;
        // ---- continuation: sampled with the sampling material ----
        const bool spec = bsdf_pure_specular(ms);
        uint64_t rng0 = rng;
        F3 fs;
        float pdf;
        F3 wi = bsdf_sample(ms, sv.tex, sd, rng, fs, pdf);
        float cos_t = fabsf(dot(wi, sd.sn));
        if (pdf <= 0.f || cos_t <= 0.f) return true;
        F3 fe;
        if (spec) {
            // deterministic directions: the evaluation material's own sample
            float pe;
            uint64_t r2 = rng0;
            bsdf_sample(me, sv.tex, sd, r2, fe, pe);
        } else {
            fe = bsdf_eval(me, sv.tex, sd, wi);
        }
        if (GRAD) {
            V->flags |= 4;
            V->l_snap = L;
            V->dr_cont = spec ? 0.f : conductor_dlogf_drough(me, to_local(sd.frame, wi), to_local(sd.frame, sd.wo));
        }
        T = divs(T * fe * cos_t, pdf);
        Ts = divs(Ts * fs * cos_t, pdf);
        if (lum(Ts) <= 0.f) return true;
        if (isnan(Ts.x) || isnan(Ts.y) || isnan(Ts.z)) return true;
        if (isinf(Ts.x) || isinf(Ts.y) || isinf(Ts.z)) return true;
        if (Ts.x < 0.f || Ts.y < 0.f || Ts.z < 0.f) return true;
        float sgn = (dot(wi, sd.gn) >= 0.f) ? 1.f : -1.f;
        o = sd.x + sd.gn * (PGX_EPSILON * sgn);
        dir = wi;
        prev_spec = spec;
        prev_pdf = pdf;
    
    }
    return ++P.depth > dv.max_depth;
}

// The gradient terms of a finished path: emitted once its radiance L is
// known, and only when L is finite (the film drops the other samples).
template <bool GRAD>
__device__ void diff_finish(const DiffView& dv, const DiffPath& P, const DiffVertex* vtx, const DiffAcc& acc) {
    const F3 L = P.L, delta = P.delta;
    const int nvtx = P.nvtx;
    const bool escaped = P.escaped;
    const F3 esc_dir = P.esc_dir, esc_w = P.esc_w;
    if (GRAD && valid(L)) {  // the film drops non-finite samples: no gradient from them
        for (int j = 0; j < nvtx; j++) {
            const DiffVertex& v = vtx[j];
            const bool alb = v.ia.x != 0.f || v.ia.y != 0.f || v.ia.z != 0.f;
            if (v.flags & 1) {
                F3 g = delta * v.C;
                if (alb) add_alb(acc, v.mat, g * v.ia);
                if (v.dr_nee != 0.f) atomicAdd(acc.rough + v.mat, (double)((g.x + g.y + g.z) * v.dr_nee));
                if (v.flags & 2) env_scatter(dv.env_e, v.wi, delta * v.tcw, dv.g_env);
            }
            if (v.flags & 4) {
                F3 g = delta * (L - v.l_snap);  // radiance collected after this vertex
                if (alb) add_alb(acc, v.mat, g * v.ia);
                if (v.dr_cont != 0.f) atomicAdd(acc.rough + v.mat, (double)((g.x + g.y + g.z) * v.dr_cont));
            }
        }
        if (escaped) env_scatter(dv.env_e, esc_dir, delta * esc_w, dv.g_env);
    }
}

// One path from its seed.  Returns the path's radiance.  GRAD: delta is the
// adjoint of the sample's value; each vertex keeps what its gradient terms
// need (DiffVertex) and the terms are emitted after the last vertex, when
// the path's total radiance is known and the sample is known to be kept by
// the film (finite) — one traversal per sample (path replay
// backpropagation, Vicini et al. 2021, with the replay's second pass folded
// into per-vertex records held by the thread).
template <bool GRAD>
__device__ F3 diff_path(const SceneView& sv, const DiffView& dv, uint64_t rng, F3 o, F3 dir, F3 delta,
                        const DiffAcc& acc) {
    DiffPath P;
    DiffVertex vtx[GRAD ? kMaxDepthCap + 1 : 1];
    diff_begin(P, rng, o, dir, delta);
    while (!diff_step<GRAD>(sv, dv, P, vtx)) {
    }
    diff_finish<GRAD>(dv, P, vtx, acc);
    return P.L;
}

// Sample s of pixel (x, y): jitter, camera ray, target pixel of the box
// filter (Film::splat: the pixel round(x + U, y + U), -1 when outside).
__device__ __forceinline__ int diff_camera(const SceneView& sv, const DiffView& dv, int64_t pixel, int s, uint64_t& rng,
                                           F3& dir) {
    int x = (int)(pixel % sv.width), y = (int)(pixel / sv.width);
    rng = pgx_rng_init(dv.seed, (uint64_t)pixel, (uint64_t)s);
    float px = (float)x + pgx_rng_next(rng);
    float py = (float)y + pgx_rng_next(rng);
    dir = camera_dir(sv.cam, px, py);
    int bx = (int)floorf(px + 0.5f), by = (int)floorf(py + 0.5f);
    if (bx < 0 || bx >= sv.width || by < 0 || by >= sv.height) return -1;
    if (!(fabsf((float)bx - px) < 0.5f && fabsf((float)by - py) < 0.5f)) return -1;
    return (by - y) * 2 + (bx - x);  // 0..3: which neighbour (right, down)
}

// Primal samples [s0, s0 + ns) on persistent warps with lane refill (as the
// adjoint): sample i of the chunk (pixel-major) stores its value and the box
// filter's target neighbour k in samples[i] (w = -1 when the film drops it).
// The per-pixel sums happen afterwards in sample order (k_diff_accumulate),
// so the image does not depend on which lane traced which sample.
__global__ void __launch_bounds__(kThreads) k_diff_primal(SceneView sv, DiffView dv) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const int64_t npix = (int64_t)sv.width * sv.height;
    const unsigned long long items = (unsigned long long)npix * (unsigned long long)dv.ns;
    const F3 origin = f3(sv.cam.origin[0], sv.cam.origin[1], sv.cam.origin[2]);
    const int lane = threadIdx.x & 31;
    DiffAcc none{nullptr, nullptr};
    DiffPath P;
    DiffVertex vtx[1];
    bool active = false, exhausted = false;
    unsigned long long mine = 0;
    int k = -1;
    for (;;) {
        const bool need = !active && !exhausted;
        const unsigned m = __ballot_sync(kFull, need);
        if (m) {
            const int leader = __ffs(m) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(dv.next, (unsigned long long)__popc(m));
            base = __shfl_sync(kFull, base, leader);
            if (need) {
                mine = base + (unsigned long long)__popc(m & ((1u << lane) - 1u));
                if (mine < items) {
                    const int64_t pixel = (int64_t)(mine % (unsigned long long)npix);
                    const int smp = dv.s0 + (int)(mine / (unsigned long long)npix);
                    uint64_t rng;
                    F3 dir;
                    k = diff_camera(sv, dv, pixel, smp, rng, dir);
                    diff_begin(P, rng, origin, dir, zero3());
                    active = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (__all_sync(kFull, !active && exhausted)) break;
        if (active && diff_step<false>(sv, dv, P, vtx)) {
            const F3 c = P.L;
            const bool keep = k >= 0 && valid(c);
            dv.samples[mine] = make_float4(c.x, c.y, c.z, keep ? (float)k : -1.f);
            active = false;
        }
    }
}

// Adds each pixel's samples of a chunk to its four neighbour sums, in sample
// order (deterministic).
__global__ void k_diff_accumulate(const float4* __restrict__ samples, int64_t npix, int ns, double* __restrict__ partial) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (int64_t)gridDim.x * blockDim.x) {
        double acc[12];
        double* out = partial + p * 12;
#pragma unroll
        for (int j = 0; j < 12; j++) acc[j] = out[j];
        for (int j = 0; j < ns; j++) {
            const float4 v = samples[(int64_t)j * npix + p];
            if (v.w < 0.f) continue;
            const int k = (int)v.w;
#pragma unroll
            for (int kk = 0; kk < 4; kk++)  // constant indexes: acc stays in registers
                if (k == kk) {
                    acc[3 * kk + 0] += (double)v.x;
                    acc[3 * kk + 1] += (double)v.y;
                    acc[3 * kk + 2] += (double)v.z;
                }
        }
#pragma unroll
        for (int j = 0; j < 12; j++) out[j] = acc[j];
    }
}

// image[p] = (partials of p, of its left, upper and upper-left neighbours
// aimed at p) / spp, in a fixed order.
__global__ void k_diff_gather(const double* __restrict__ partial, int W, int H, int spp, double* __restrict__ img) {
    const int64_t npix = (int64_t)W * H;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (int64_t)gridDim.x * blockDim.x) {
        int x = (int)(p % W), y = (int)(p / W);
        double v[3] = {0.0, 0.0, 0.0};
        for (int dy = 0; dy <= 1; dy++)
            for (int dx = 0; dx <= 1; dx++) {
                int sx = x - dx, sy = y - dy;
                if (sx < 0 || sy < 0) continue;
                const double* q = partial + ((int64_t)sy * W + sx) * 12 + 3 * (dy * 2 + dx);
                for (int c = 0; c < 3; c++) v[c] += q[c];
            }
        for (int c = 0; c < 3; c++) img[p * 3 + c] = v[c] / (double)spp;
    }
}

// Persistent warps over the samples (pixel-major within each sample index):
// a lane whose path has ended takes the next sample from dv.next at once
// (warp-aggregated atomicAdd), so short and long paths share the warp's
// issue slots instead of each warp waiting for its longest path.
__global__ void __launch_bounds__(kThreads) k_diff_adjoint(SceneView sv, DiffView dv) {
    extern __shared__ double sacc[];  // [nmats*3 + nmats] when it fits
    const bool shared_acc = dv.nmats * 4 * (int)sizeof(double) <= 32 * 1024;
    DiffAcc acc;
    if (shared_acc) {
        for (int i = threadIdx.x; i < dv.nmats * 4; i += blockDim.x) sacc[i] = 0.0;
        __syncthreads();
        acc.alb = sacc;
        acc.rough = sacc + dv.nmats * 3;
    } else {
        acc.alb = dv.g_alb;
        acc.rough = dv.g_rough;
    }
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const int64_t npix = (int64_t)sv.width * sv.height;
    const unsigned long long items = (unsigned long long)npix * (unsigned long long)dv.spp;
    const F3 origin = f3(sv.cam.origin[0], sv.cam.origin[1], sv.cam.origin[2]);
    const float inv_spp = 1.f / (float)dv.spp;
    const int lane = threadIdx.x & 31;
    DiffPath P;
    DiffVertex vtx[kMaxDepthCap + 1];
    bool active = false, exhausted = false;
    for (;;) {
        const bool need = !active && !exhausted;
        const unsigned m = __ballot_sync(kFull, need);
        if (m) {
            const int leader = __ffs(m) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(dv.next, (unsigned long long)__popc(m));
            base = __shfl_sync(kFull, base, leader);
            if (need) {
                const unsigned long long item = base + (unsigned long long)__popc(m & ((1u << lane) - 1u));
                if (item < items) {
                    const int64_t pixel = (int64_t)(item % (unsigned long long)npix);
                    const int smp = (int)(item / (unsigned long long)npix);
                    const int x = (int)(pixel % sv.width), y = (int)(pixel / sv.width);
                    uint64_t rng;
                    F3 dir;
                    const int k = diff_camera(sv, dv, pixel, smp, rng, dir);
                    if (k >= 0) {
                        const int64_t tp = (int64_t)(y + k / 2) * sv.width + (x + k % 2);
                        const F3 delta = f3(dv.dimg[3 * tp], dv.dimg[3 * tp + 1], dv.dimg[3 * tp + 2]) * inv_spp;
                        if (delta.x != 0.f || delta.y != 0.f || delta.z != 0.f) {
                            diff_begin(P, rng, origin, dir, delta);
                            active = true;
                        }
                    }
                } else {
                    exhausted = true;
                }
            }
        }
        if (__all_sync(kFull, !active && exhausted)) break;
        if (active && diff_step<true>(sv, dv, P, vtx)) {
            diff_finish<true>(dv, P, vtx, acc);
            active = false;
        }
    }
    if (shared_acc) {
        __syncthreads();
        for (int i = threadIdx.x; i < dv.nmats * 3; i += blockDim.x)
            if (sacc[i] != 0.0) atomicAdd(dv.g_alb + i, sacc[i]);
        for (int i = threadIdx.x; i < dv.nmats; i += blockDim.x)
            if (sacc[dv.nmats * 3 + i] != 0.0) atomicAdd(dv.g_rough + i, sacc[dv.nmats * 3 + i]);
    }
}

// End of a batch wave: NaN/Inf drop and the box-filter splat into each
// path's scene film.
__global__ void __launch_bounds__(kThreads) k_finalize_batch(PathState ps, BatchWave bw) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < bw.count; p += (int64_t)gridDim.x * blockDim.x) {
        F3 col = f3(ps.L[p]);
        if (!valid(col)) continue;
        const BatchInfo& bi = bw.info[ps.scene[p]];
        float2 xy = ps.pix[p];
        splat(bi.film, nullptr, bi.width, bi.height, xy.x, xy.y, col, false);
    }
}

// One surface class's bin shaded by estimator MODE, with the class compiled in.
template <int MODE, bool BATCH>
void launch_shade_class(int c, unsigned grid, cudaStream_t s, const SceneView& sv, const PathState& ps,
                        const FrameParams& fp, int depth, const GuideView& gv, const BatchInfo* info) {
    switch (c) {
        case 0: k_shade<MODE, BATCH, 0><<<grid, kThreads, 0, s>>>(sv, ps, fp, depth, gv, info); break;
        case 1: k_shade<MODE, BATCH, 1><<<grid, kThreads, 0, s>>>(sv, ps, fp, depth, gv, info); break;
        case 2: k_shade<MODE, BATCH, 2><<<grid, kThreads, 0, s>>>(sv, ps, fp, depth, gv, info); break;
        case 3: k_shade<MODE, BATCH, 3><<<grid, kThreads, 0, s>>>(sv, ps, fp, depth, gv, info); break;
        case 4: k_shade<MODE, BATCH, 4><<<grid, kThreads, 0, s>>>(sv, ps, fp, depth, gv, info); break;
        default: k_shade<MODE, BATCH, 5><<<grid, kThreads, 0, s>>>(sv, ps, fp, depth, gv, info); break;
    }
}

inline unsigned grid_for(int64_t n) {
    int64_t b = (n + kThreads - 1) / kThreads;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)pgx_num_sms() * 16));
}

RenderState* state_of(pgx_ctx* ctx) {
    if (!ctx->render_state) ctx->render_state = new RenderState();
    return static_cast<RenderState*>(ctx->render_state);
}

int ensure_state(pgx_ctx* ctx, RenderState* rs, int64_t cap, int rec_depth, int64_t vcap, bool guide = false,
                 int train_depth = 0, int64_t tcap = 0, bool batch = false) {
    if (cap > rs->capacity) {
        PGX_CUDA_TRY(ctx, rs->o.reserve(sizeof(float4) * cap));
        PGX_CUDA_TRY(ctx, rs->d.reserve(sizeof(float4) * cap));
        PGX_CUDA_TRY(ctx, rs->T.reserve(sizeof(float4) * cap));
        PGX_CUDA_TRY(ctx, rs->L.reserve(sizeof(float4) * cap));
        PGX_CUDA_TRY(ctx, rs->hit.reserve(sizeof(float4) * cap));
        PGX_CUDA_TRY(ctx, rs->pix.reserve(sizeof(float2) * cap));
        PGX_CUDA_TRY(ctx, rs->rng.reserve(sizeof(uint64_t) * cap));
        PGX_CUDA_TRY(ctx, rs->flags.reserve(sizeof(int) * cap));
        PGX_CUDA_TRY(ctx, rs->nrec.reserve(sizeof(int) * cap));
        PGX_CUDA_TRY(ctx, rs->q0.reserve(sizeof(int) * cap));
        PGX_CUDA_TRY(ctx, rs->q1.reserve(sizeof(int) * cap));
        PGX_CUDA_TRY(ctx, rs->sh_path.reserve(sizeof(int) * cap));
        PGX_CUDA_TRY(ctx, rs->sh_o.reserve(sizeof(float4) * cap));
        PGX_CUDA_TRY(ctx, rs->sh_d.reserve(sizeof(float4) * cap));
        PGX_CUDA_TRY(ctx, rs->sh_c.reserve(sizeof(float4) * cap));
        rs->capacity = cap;
        rs->rec_depth = 0;
    }
    if (rec_depth > rs->rec_depth) {
        size_t nrec = (size_t)rec_depth * rs->capacity;
        PGX_CUDA_TRY(ctx, rs->rec_pos.reserve(sizeof(float4) * nrec));
        PGX_CUDA_TRY(ctx, rs->rec_nrm.reserve(sizeof(float4) * nrec));
        PGX_CUDA_TRY(ctx, rs->rec_wi.reserve(sizeof(float4) * nrec));
        PGX_CUDA_TRY(ctx, rs->rec_w.reserve(sizeof(float4) * nrec));
        PGX_CUDA_TRY(ctx, rs->rec_e.reserve(sizeof(float4) * nrec));
        rs->rec_depth = rec_depth;
    }
    if (vcap > rs->vcapacity) {
        PGX_CUDA_TRY(ctx, rs->vertices.reserve(sizeof(pgx_path_vertex) * vcap));
        PGX_CUDA_TRY(ctx, rs->vweight.reserve(sizeof(float) * vcap));
        rs->vcapacity = vcap;
    }
    if (guide && rs->guide_capacity < rs->capacity) {
        PGX_CUDA_TRY(ctx, rs->guide.reserve(sizeof(float4) * mlp::kPacked * rs->capacity));
        PGX_CUDA_TRY(ctx, rs->fallback.reserve(sizeof(int) * rs->capacity));
        rs->guide_capacity = rs->capacity;
    }
    if (train_depth > 0 && (train_depth > rs->train_depth || rs->rec_wo.bytes < sizeof(float4) * train_depth * rs->capacity)) {
        size_t nrec = (size_t)train_depth * rs->capacity;
        PGX_CUDA_TRY(ctx, rs->rec_wo.reserve(sizeof(float4) * nrec));
        PGX_CUDA_TRY(ctx, rs->rec_f.reserve(sizeof(float4) * nrec));
        rs->train_depth = train_depth;
    }
    if (tcap > rs->tcapacity) {
        PGX_CUDA_TRY(ctx, rs->train.reserve(sizeof(float) * 13 * tcap));
        rs->tcapacity = tcap;
    }
    if (batch) PGX_CUDA_TRY(ctx, rs->scene.reserve(sizeof(int) * rs->capacity));
    PGX_CUDA_TRY(ctx, rs->cqueue.reserve(sizeof(int) * kShadeClasses * rs->capacity));
    PGX_CUDA_TRY(ctx, rs->ccount.reserve(sizeof(unsigned) * kShadeClasses * (kMaxDepthCap + 2)));
    PGX_CUDA_TRY(ctx, rs->counters.reserve(sizeof(unsigned) * 4 * (kMaxDepthCap + 2) + sizeof(unsigned long long) * kStats +
                                           sizeof(unsigned) * 4));
    if (!rs->ev0) {
        PGX_CUDA_TRY(ctx, cudaEventCreate(&rs->ev0));
        PGX_CUDA_TRY(ctx, cudaEventCreate(&rs->ev1));
        for (int i = 0; i < kProfEvents; i++) PGX_CUDA_TRY(ctx, cudaEventCreate(&rs->prof[i]));
    }
    return PGX_OK;
}

PathState path_view(RenderState* rs) {
    PathState ps;
    ps.o = rs->o.as<float4>();
    ps.d = rs->d.as<float4>();
    ps.T = rs->T.as<float4>();
    ps.L = rs->L.as<float4>();
    ps.hit = rs->hit.as<float4>();
    ps.pix = rs->pix.as<float2>();
    ps.rng = rs->rng.as<uint64_t>();
    ps.flags = rs->flags.as<int>();
    ps.nrec = rs->nrec.as<int>();
    ps.queue[0] = rs->q0.as<int>();
    ps.queue[1] = rs->q1.as<int>();
    ps.sh_path = rs->sh_path.as<int>();
    ps.sh_o = rs->sh_o.as<float4>();
    ps.sh_d = rs->sh_d.as<float4>();
    ps.sh_c = rs->sh_c.as<float4>();
    ps.rec_pos = rs->rec_pos.as<float4>();
    ps.rec_nrm = rs->rec_nrm.as<float4>();
    ps.rec_wi = rs->rec_wi.as<float4>();
    ps.rec_w = rs->rec_w.as<float4>();
    ps.rec_e = rs->rec_e.as<float4>();
    unsigned* c = rs->counters.as<unsigned>();
    ps.qcount = c;
    ps.cqueue = rs->cqueue.as<int>();
    ps.ccount = rs->ccount.as<unsigned>();
    ps.scount = c + (kMaxDepthCap + 2);
    ps.wcount = c + 2 * (kMaxDepthCap + 2);
    ps.stats = reinterpret_cast<unsigned long long*>(c + 4 * (kMaxDepthCap + 2));
    ps.nvertices = c + 4 * (kMaxDepthCap + 2) + 2 * kStats;
    ps.vertices = rs->vertices.as<pgx_path_vertex>();
    ps.vweight = rs->vweight.as<float>();
    ps.capacity = rs->capacity;
    ps.vcapacity = rs->vcapacity;
    ps.guide = rs->guide.as<float4>();
    ps.fallback = rs->fallback.as<int>();
    ps.rec_wo = rs->rec_wo.as<float4>();
    ps.rec_f = rs->rec_f.as<float4>();
    ps.train = rs->train.as<float>();
    ps.ntrain = c + 4 * (kMaxDepthCap + 2) + 2 * kStats + 1;
    ps.tcapacity = rs->tcapacity;
    ps.scene = rs->scene.as<int>();
    return ps;
}

SceneView scene_view(pgx_ctx* ctx) {
    SceneView sv;
    sv.bvh = bvh_view(ctx);
    sv.shade = ctx->shade.as<TriShade>();
    sv.tri_class = ctx->tri_class.as<unsigned char>();
    sv.mats = ctx->mats.as<DevMaterial>();
    sv.lights = ctx->lights.as<DevAreaLight>();
    sv.tex.info = ctx->textures.as<DevTexture>();
    sv.tex.texels = ctx->texels.as<float>();
    sv.env = ctx->env;
    sv.cam = ctx->camera;
    sv.bounds = ctx->bounds;
    sv.n_area_lights = ctx->n_area_lights;
    sv.nlights = ctx->nlights;
    sv.has_env_light = (ctx->env.valid && ctx->env.power > 0.f) ? 1 : 0;
    sv.width = ctx->width;
    sv.height = ctx->height;
    return sv;
}

// Stage times of one profiled batch (milliseconds).
struct StageTimes {
    double extend = 0, shade = 0, shadow = 0;
};

// Enqueues one batch (fp.batch samples per pixel) on stream s; returns the
// number of kernels launched.  With fp.profile, events bracket every stage
// (read back by stage_times after the stream is synchronised).
int enqueue_frame(pgx_ctx* ctx, RenderState* rs, const FrameParams& fp, cudaStream_t s, int* mlp_status) {
    SceneView sv = scene_view(ctx);
    PathState ps = path_view(rs);
    GuideView gv = guide_view(ctx);
    MlpView mv = fp.mode == PGX_MODE_GUIDED_MLP ? mlp_view(ctx) : MlpView{};
    int fb_min = 0;
    const int* fb_counts = fp.mode == PGX_MODE_GUIDED_MLP ? mlp_region_counts(ctx, &fb_min) : nullptr;
    const int64_t n = (int64_t)ctx->width * ctx->height * fp.batch;
    const unsigned g = grid_for(n);
    const bool prof = fp.profile != 0;  // stage events
    const bool cnt = fp.profile > 1;    // counting traversal kernels
    int launches = 0;
    cudaMemsetAsync(ps.qcount, 0, sizeof(unsigned) * 4 * (kMaxDepthCap + 2), s);
    cudaMemsetAsync(ps.ccount, 0, sizeof(unsigned) * kShadeClasses * (kMaxDepthCap + 2), s);
    k_camgen<<<g, kThreads, 0, s>>>(sv, ps, fp);
    launches++;
    for (int depth = 0; depth <= fp.max_depth; depth++) {
        if (prof) cudaEventRecord(rs->prof[4 * depth + 0], s);
        const unsigned pg = persistent_grid(n);
        if (cnt)
            k_extend<true><<<pg, kThreads, 0, s>>>(sv, ps, depth);
        else
            k_extend<false><<<pg, kThreads, 0, s>>>(sv, ps, depth);
        if (prof) cudaEventRecord(rs->prof[4 * depth + 1], s);
        k_classify<<<grid_for((n + kClassifyItems - 1) / kClassifyItems), kThreads, 0, s>>>(sv, ps, depth);
        if (fp.mode == PGX_MODE_GUIDED_MLP && depth < fp.guide_depth) {
            const int64_t tiles = (n + mlp::kRows - 1) / mlp::kRows;
            const int64_t ctas = (tiles + kInferGroups - 1) / kInferGroups;
            const unsigned ig = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ctas, (int64_t)pgx_num_sms() * 2));
            k_guide_infer<<<ig, 128 * kInferGroups, kInferSmem, s>>>(sv, ps, depth, mv, mlp_status, gv, fb_counts,
                                                                      fb_min);
            launches++;
        }
        for (int c = 0; c < kShadeClasses; c++) {
            switch (fp.mode) {
                case PGX_MODE_GUIDED_LI:
                    launch_shade_class<PGX_MODE_GUIDED_LI, false>(c, g, s, sv, ps, fp, depth, gv, nullptr);
                    break;
                case PGX_MODE_GUIDED_QUADTREE:
                    launch_shade_class<PGX_MODE_GUIDED_QUADTREE, false>(c, g, s, sv, ps, fp, depth, gv, nullptr);
                    break;
                case PGX_MODE_GUIDED_PSS:
                    launch_shade_class<PGX_MODE_GUIDED_PSS, false>(c, g, s, sv, ps, fp, depth, gv, nullptr);
                    break;
                case PGX_MODE_GUIDED_MLP:
                    launch_shade_class<PGX_MODE_GUIDED_MLP, false>(c, g, s, sv, ps, fp, depth, gv, nullptr);
                    break;
                default:
                    launch_shade_class<PGX_MODE_PLAIN, false>(c, g, s, sv, ps, fp, depth, gv, nullptr);
                    break;
            }
        }
        launches += 2 + kShadeClasses;
        if (prof) cudaEventRecord(rs->prof[4 * depth + 2], s);
        if (fp.mode != PGX_MODE_GUIDED_LI) {
            if (cnt)
                k_shadow<true><<<pg, kThreads, 0, s>>>(sv, ps, depth);
            else
                k_shadow<false><<<pg, kThreads, 0, s>>>(sv, ps, depth);
            launches++;
        }
        if (prof) cudaEventRecord(rs->prof[4 * depth + 3], s);
    }
    float* film = ctx->film.as<float>();
    float* film2 = ctx->film2.as<float>();
    if (fp.mode == PGX_MODE_GUIDED_LI)
        k_finalize<PGX_MODE_GUIDED_LI><<<g, kThreads, 0, s>>>(sv, ps, fp, film, film2);
    else
        k_finalize<PGX_MODE_PLAIN><<<g, kThreads, 0, s>>>(sv, ps, fp, film, film2);
    return launches + 1;
}

void stage_times(RenderState* rs, int max_depth, StageTimes& t) {
    for (int depth = 0; depth <= max_depth; depth++) {
        float a = 0.f, b = 0.f, c = 0.f;
        cudaEventElapsedTime(&a, rs->prof[4 * depth + 0], rs->prof[4 * depth + 1]);
        cudaEventElapsedTime(&b, rs->prof[4 * depth + 1], rs->prof[4 * depth + 2]);
        cudaEventElapsedTime(&c, rs->prof[4 * depth + 2], rs->prof[4 * depth + 3]);
        t.extend += a;
        t.shade += b;
        t.shadow += c;
    }
}

int ensure_film(pgx_ctx* ctx) {
    size_t bytes = sizeof(float) * 3 * (size_t)ctx->width * ctx->height;
    if (ctx->film.bytes < bytes || !ctx->film.p) {
        PGX_CUDA_TRY(ctx, ctx->film.reserve(bytes));
        PGX_CUDA_TRY(ctx, ctx->film2.reserve(bytes));
        PGX_CUDA_TRY(ctx, cudaMemsetAsync(ctx->film.p, 0, bytes, ctx->stream));
        PGX_CUDA_TRY(ctx, cudaMemsetAsync(ctx->film2.p, 0, bytes, ctx->stream));
        ctx->spp = 0;
    }
    return PGX_OK;
}

}  // namespace

void render_state_free(pgx_ctx* ctx) {
    RenderState* rs = static_cast<RenderState*>(ctx->render_state);
    if (!rs) return;
    if (rs->graph) cudaGraphExecDestroy(rs->graph);
    if (rs->ev0) cudaEventDestroy(rs->ev0);
    if (rs->ev1) cudaEventDestroy(rs->ev1);
    for (int i = 0; i < kProfEvents; i++)
        if (rs->prof[i]) cudaEventDestroy(rs->prof[i]);
    delete rs;
    ctx->render_state = nullptr;
}

int64_t render_vertex_count(pgx_ctx* ctx) {
    RenderState* rs = static_cast<RenderState*>(ctx->render_state);
    return rs ? rs->nvertices_last : 0;
}

const pgx_path_vertex* render_vertices(pgx_ctx* ctx) {
    RenderState* rs = static_cast<RenderState*>(ctx->render_state);
    return rs ? rs->vertices.as<pgx_path_vertex>() : nullptr;
}

// Flux weights of the recorded vertices (nullptr for guided-Li records,
// which the guide weighs by Lum(Li)).
const float* render_vertex_weights(pgx_ctx* ctx) {
    RenderState* rs = static_cast<RenderState*>(ctx->render_state);
    return (rs && rs->vweight_valid) ? rs->vweight.as<float>() : nullptr;
}

extern "C" int pgx_render(pgx_ctx* ctx, const pgx_render_config* cfg, int32_t frames) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (!cfg || frames < 0) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_render: bad arguments");
    if (cfg->mode < PGX_MODE_PLAIN || cfg->mode > PGX_MODE_GUIDED_PSS)
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_render: unknown mode %d", cfg->mode);
    if (cfg->max_depth < 0 || cfg->max_depth > kMaxDepthCap)
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_render: max_depth must be in [0, %d]", kMaxDepthCap);
    if (!ctx->has_scene) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_render: no scene");
    if (!ctx->has_bvh) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_render: no BVH");
    if (cfg->mode == PGX_MODE_GUIDED_QUADTREE && !guide_ready(ctx))
        return pgx_fail(ctx, PGX_ERR_STATE, "pgx_render: guided mode needs a radiance cache (pgx_cache_build)");
    if (cfg->mode == PGX_MODE_GUIDED_QUADTREE && guide_view(ctx).pss)
        return pgx_fail(ctx, PGX_ERR_STATE,
                        "pgx_render: the radiance cache holds primary-sample trees (built by a PGX_MODE_GUIDED_PSS render)");
    if (cfg->mode == PGX_MODE_GUIDED_MLP && !mlp_view(ctx).valid)
        return pgx_fail(ctx, PGX_ERR_STATE, "pgx_render: learned-guide mode needs pgx_mlp_init");
    if ((cfg->flags & PGX_RENDER_TRAIN_GUIDE) && cfg->mode != PGX_MODE_GUIDED_MLP)
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_render: PGX_RENDER_TRAIN_GUIDE needs PGX_MODE_GUIDED_MLP");
    PGX_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    PGX_TRY(ensure_film(ctx));
    if (frames == 0) return PGX_OK;
    RenderState* rs = state_of(ctx);
    const int64_t npix = (int64_t)ctx->width * ctx->height;
    // Samples per wavefront: enough paths to fill the GPU, bounded memory.
    const bool guided_li = cfg->mode == PGX_MODE_GUIDED_LI;
    // Recorded samples [collect_lo, collect_hi).  Guided-Li keeps the vertices
    // of the last frame with SPP < 16 (Renderer.h:720-746); the other modes
    // record the last `record_paths` frames of this call.
    int collect_lo = 0, collect_hi = 0;
    if (guided_li && cfg->record_paths) {
        int last = std::min(ctx->spp + frames, kCollectionSPP - 1);
        if (last > ctx->spp) {
            collect_lo = last - 1;
            collect_hi = last;
        }
    } else if (!guided_li && cfg->record_paths > 0) {
        collect_hi = ctx->spp + frames;
        collect_lo = collect_hi - std::min(cfg->record_paths, frames);
    }
    // Online training of the learned guide records every frame's vertices
    // for radiance samples instead of path vertices.
    const bool train = (cfg->flags & PGX_RENDER_TRAIN_GUIDE) != 0;
    if (train) {
        collect_lo = ctx->spp;
        collect_hi = ctx->spp + frames;
    }
    const bool recording = collect_hi > collect_lo && !train;
    const int rec_depth = (guided_li || recording || train) ? cfg->max_depth + 1 : 0;
    // Samples per wavefront: as many as fit in 2^25 paths (~190 bytes of state
    // each, 6.4 GB): the depths where the queues have shrunk cost about the
    // same per wave whatever its size, so large waves amortise them (measured
    // on the 1280x720 interior: 1,726 Mrays/s at 4 spp per wave, 1,903 at 8,
    // 1,998 at 16, 2,041 at 32).  Recording is bounded at 2^23 paths (per-depth
    // vertex records cost 80 bytes per path and depth: 7 GB at depth 10).
    const int64_t target_paths = rec_depth ? (int64_t)(1 << 23) : (int64_t)(1 << 25);
    int batch = (int)std::max<int64_t>(1, std::min<int64_t>(frames, target_paths / std::max<int64_t>(npix, 1)));
    if (train) batch = 1;  // one round of Adam steps after every frame
    const int64_t vcap = recording ? npix * (cfg->max_depth + 1) * (collect_hi - collect_lo) : 0;
    const bool mlp_mode = cfg->mode == PGX_MODE_GUIDED_MLP;
    const int64_t tcap = train ? mlp_train_batch(ctx) : 0;
    PGX_TRY(ensure_state(ctx, rs, npix * batch, rec_depth, vcap, mlp_mode, train ? rec_depth : 0, tcap));
    if (mlp_mode)
        PGX_CUDA_TRY(ctx, cudaFuncSetAttribute(k_guide_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, kInferSmem));
    cudaStream_t s = ctx->stream;
    PathState ps = path_view(rs);
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(ps.stats, 0, sizeof(unsigned long long) * kStats + sizeof(unsigned) * 4, s));
    int* mlp_status = reinterpret_cast<int*>(ps.nvertices + 2);
    const bool count = (cfg->flags & PGX_RENDER_PROFILE) != 0;
    const bool prof = count || (cfg->flags & PGX_RENDER_TIMING) != 0;
    StageTimes times;
    int64_t launches = 0, batches = 0;
    PGX_CUDA_TRY(ctx, cudaEventRecord(rs->ev0, s));
    int done = 0;
    while (done < frames) {
        FrameParams fp;
        fp.mode = cfg->mode;
        fp.max_depth = cfg->max_depth;
        fp.seed = cfg->seed;
        fp.spp0 = ctx->spp + done;
        fp.batch = std::min(batch, frames - done);
        fp.collect_lo = collect_lo;
        fp.collect_hi = collect_hi;
        fp.guide_fraction = cfg->guide_fraction;
        fp.profile = count ? 2 : (prof ? 1 : 0);
        fp.mitchell = (cfg->flags & PGX_RENDER_FILTER_MITCHELL) ? 1 : 0;
        fp.train = train ? (mlp_train_direct(ctx) ? 2 : 1) : 0;
        fp.guide_depth = cfg->guide_depth > 0 ? cfg->guide_depth : kMaxDepthCap + 1;
        fp.train_keep = 1.f;
        if (train && rs->train_last > 0)
            fp.train_keep = (float)std::min(1.0, (double)tcap / (1.25 * (double)rs->train_last * fp.batch));
        if (train) PGX_CUDA_TRY(ctx, cudaMemsetAsync(ps.ntrain, 0, sizeof(unsigned), s));
        launches += enqueue_frame(ctx, rs, fp, s, mlp_status);
        batches++;
        PGX_CUDA_TRY(ctx, cudaGetLastError());
        if (train) {
            // one Adam step on this batch's radiance samples
            unsigned nt = 0;
            PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&nt, ps.ntrain, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
            PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
            rs->train_last = (int64_t)((double)nt / std::max(fp.train_keep, 1e-6f) / fp.batch);
            PGX_TRY(mlp_online_step(ctx, ps.train, std::min<int64_t>(nt, tcap)));
            launches += 4;
        }
        if (prof) {
            PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
            stage_times(rs, fp.max_depth, times);
        }
        done += fp.batch;
    }
    PGX_CUDA_TRY(ctx, cudaEventRecord(rs->ev1, s));
    unsigned long long st[kStats] = {};
    unsigned nv = 0;
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(st, ps.stats, sizeof(st), cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&nv, ps.nvertices, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    int mst = 0;
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&mst, mlp_status, sizeof(int), cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    if (mst != 0) return pgx_fail(ctx, PGX_ERR_TIMEOUT, "pgx_render: tensor-core wait timed out in %d CTA(s)", mst);
    float ms = 0.f;
    PGX_CUDA_TRY(ctx, cudaEventElapsedTime(&ms, rs->ev0, rs->ev1));
    ctx->spp += frames;
    pgx_render_stats& rst = ctx->rstats;
    rst = pgx_render_stats{};
    rst.paths = npix * frames;
    rst.extension_rays = (int64_t)st[0];
    rst.shadow_rays = (int64_t)st[1];
    rst.extend_interior_visits = (int64_t)st[2];
    rst.extend_tri_tests = (int64_t)st[3];
    rst.shadow_interior_visits = (int64_t)st[4];
    rst.shadow_tri_tests = (int64_t)st[5];
    rst.guide_fallbacks = (int64_t)st[6];
    rst.kernel_launches = launches;
    rst.extend_launches = batches * (cfg->max_depth + 1);
    rst.ms_total = ms;
    rst.ms_extend = times.extend;
    rst.ms_shade = times.shade;
    rst.ms_shadow = times.shadow;
    if (recording) {
        rs->nvertices_last = std::min<int64_t>(nv, rs->vcapacity);
        rs->vweight_valid = cfg->mode != PGX_MODE_GUIDED_LI;
        rst.path_vertices = rs->nvertices_last;
        // Guided-Li records (the reference's recorder) weigh by Lum(Li);
        // the others by Lum(Li) |cos| / pdf.
        PGX_TRY(cache_build_device(ctx, rs->vertices.as<pgx_path_vertex>(), rs->nvertices_last,
                                   cfg->mode == PGX_MODE_GUIDED_PSS,
                                   render_vertex_weights(ctx)));
    }
    return PGX_OK;
}

int camera_setup(pgx_ctx* ctx, const pgx_camera* camera);

extern "C" int pgx_set_camera(pgx_ctx* ctx, const pgx_camera* camera) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (!camera) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_set_camera: null camera");
    if (!ctx->has_scene) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_set_camera: no scene");
    if (camera->width != ctx->width || camera->height != ctx->height)
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_set_camera: image size differs from the scene's");
    return camera_setup(ctx, camera);
}

extern "C" int pgx_clear(pgx_ctx* ctx) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (!ctx->has_scene) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_clear: no scene");
    PGX_TRY(ensure_film(ctx));
    size_t bytes = sizeof(float) * 3 * (size_t)ctx->width * ctx->height;
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(ctx->film.p, 0, bytes, ctx->stream));
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(ctx->film2.p, 0, bytes, ctx->stream));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->spp = 0;
    return PGX_OK;
}

extern "C" int pgx_get_spp(pgx_ctx* ctx, int32_t* spp) {
    if (!ctx || !spp) return PGX_ERR_INVALID_ARG;
    *spp = ctx->spp;
    return PGX_OK;
}

extern "C" int pgx_film_read(pgx_ctx* ctx, float* rgb, float* rgb2, int32_t* spp) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (!ctx->has_scene) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_film_read: no scene");
    PGX_TRY(ensure_film(ctx));
    size_t bytes = sizeof(float) * 3 * (size_t)ctx->width * ctx->height;
    if (rgb) PGX_CUDA_TRY(ctx, cudaMemcpyAsync(rgb, ctx->film.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    if (rgb2) PGX_CUDA_TRY(ctx, cudaMemcpyAsync(rgb2, ctx->film2.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (spp) *spp = ctx->spp;
    return PGX_OK;
}

extern "C" int pgx_film_tonemap(pgx_ctx* ctx, float exposure, float lmax_white, uint8_t* rgb8) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (!rgb8) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_film_tonemap: null output");
    if (!ctx->has_scene) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_film_tonemap: no scene");
    PGX_TRY(ensure_film(ctx));
    const int64_t npix = (int64_t)ctx->width * ctx->height;
    DevBuf out;
    PGX_CUDA_TRY(ctx, out.reserve((size_t)npix * 3));
    k_tonemap<<<(unsigned)((npix + 255) / 256), 256, 0, ctx->stream>>>(ctx->film.as<float>(), npix, ctx->spp, exposure,
                                                                       lmax_white, out.as<uint8_t>());
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(rgb8, out.p, (size_t)npix * 3, cudaMemcpyDeviceToHost, ctx->stream));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return PGX_OK;
}

extern "C" int pgx_render_get_stats(pgx_ctx* ctx, pgx_render_stats* out) {
    if (!ctx || !out) return PGX_ERR_INVALID_ARG;
    *out = ctx->rstats;
    return PGX_OK;
}

// ---- differentiable rendering API ----------------------------------------------------------
namespace {

int diff_check(pgx_ctx* ctx, const char* who) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (!ctx->has_scene) return pgx_fail(ctx, PGX_ERR_STATE, "%s: no scene", who);
    if (!ctx->has_bvh) return pgx_fail(ctx, PGX_ERR_STATE, "%s: no BVH", who);
    PGX_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    return PGX_OK;
}

size_t env_floats(const pgx_ctx* ctx) {
    return ctx->env.valid ? (size_t)ctx->env.width * ctx->env.height * 3 : 0;
}

// Evaluation parameters: a copy of the uploaded materials with albedo
// offsets and roughness replaced, and of the environment texels.
int diff_params(pgx_ctx* ctx, RenderState* rs, const float* env_rgb, const float* albedo_offset,
                const float* roughness) {
    const size_t nm = (size_t)ctx->nmats;
    std::vector<DevMaterial> m(nm);
    if (nm)
        PGX_CUDA_TRY(ctx, cudaMemcpy(m.data(), ctx->mats.p, sizeof(DevMaterial) * nm, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < nm; i++) {
        for (int c = 0; c < 3; c++) m[i].alb_off[c] = albedo_offset ? albedo_offset[3 * i + c] : 0.f;
        float r = roughness ? roughness[i] : ctx->host_mats[i].roughness;
        if (!(r >= 0.f)) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_diff_set_params: roughness must be >= 0");
        m[i].alpha = 1.62142f * sqrtf(r);
    }
    PGX_CUDA_TRY(ctx, rs->d_mats.reserve(sizeof(DevMaterial) * std::max<size_t>(nm, 1)));
    if (nm)
        PGX_CUDA_TRY(ctx, cudaMemcpy(rs->d_mats.p, m.data(), sizeof(DevMaterial) * nm, cudaMemcpyHostToDevice));
    const size_t ef = env_floats(ctx);
    PGX_CUDA_TRY(ctx, rs->d_env.reserve(sizeof(float) * std::max<size_t>(ef, 1)));
    if (ef) {
        if (env_rgb)
            PGX_CUDA_TRY(ctx, cudaMemcpy(rs->d_env.p, env_rgb, sizeof(float) * ef, cudaMemcpyHostToDevice));
        else
            PGX_CUDA_TRY(ctx, cudaMemcpy(rs->d_env.p, ctx->env.texels, sizeof(float) * ef, cudaMemcpyDeviceToDevice));
    }
    rs->d_params = true;
    return PGX_OK;
}

DiffView diff_view(pgx_ctx* ctx, RenderState* rs, int spp, uint64_t seed, int max_depth) {
    DiffView dv{};
    dv.mats_e = rs->d_mats.as<DevMaterial>();
    dv.env_e = ctx->env;
    dv.env_e.texels = rs->d_env.as<float>();
    dv.spp = spp;
    dv.seed = seed;
    dv.max_depth = max_depth;
    dv.nmats = ctx->nmats;
    return dv;
}

int diff_args(pgx_ctx* ctx, int32_t spp, int32_t max_depth, const char* who) {
    if (spp <= 0 || max_depth < 0 || max_depth > kMaxDepthCap)
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "%s: spp must be > 0 and max_depth in [0, %d]", who, kMaxDepthCap);
    return PGX_OK;
}

}  // namespace

extern "C" int pgx_diff_set_params(pgx_ctx* ctx, const float* env_rgb, const float* albedo_offset,
                                   const float* roughness) {
    PGX_TRY(diff_check(ctx, "pgx_diff_set_params"));
    return diff_params(ctx, state_of(ctx), env_rgb, albedo_offset, roughness);
}

extern "C" int pgx_diff_render(pgx_ctx* ctx, int32_t spp, uint64_t seed, int32_t max_depth, double* image) {
    PGX_TRY(diff_check(ctx, "pgx_diff_render"));
    PGX_TRY(diff_args(ctx, spp, max_depth, "pgx_diff_render"));
    if (!image) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_diff_render: null image");
    RenderState* rs = state_of(ctx);
    if (!rs->d_params) PGX_TRY(diff_params(ctx, rs, nullptr, nullptr, nullptr));
    const int64_t npix = (int64_t)ctx->width * ctx->height;
    PGX_CUDA_TRY(ctx, rs->d_partial.reserve(sizeof(double) * 12 * npix));
    PGX_CUDA_TRY(ctx, rs->d_img.reserve(sizeof(double) * 3 * npix));
    // sample values of up to 1 GiB at a time
    const int chunk = (int)std::max<int64_t>(1, std::min<int64_t>(spp, ((int64_t)1 << 30) / (16 * npix)));
    PGX_CUDA_TRY(ctx, rs->d_samples.reserve(sizeof(float4) * (size_t)npix * chunk));
    PGX_CUDA_TRY(ctx, rs->d_next.reserve(sizeof(unsigned long long)));
    DiffView dv = diff_view(ctx, rs, spp, seed, max_depth);
    dv.partial = rs->d_partial.as<double>();
    dv.samples = rs->d_samples.as<float4>();
    dv.next = rs->d_next.as<unsigned long long>();
    SceneView sv = scene_view(ctx);
    cudaStream_t s = ctx->stream;
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(dv.partial, 0, sizeof(double) * 12 * npix, s));
    int per_sm = 0;
    PGX_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_diff_primal, kThreads, 0));
    for (int s0 = 0; s0 < spp; s0 += chunk) {
        dv.s0 = s0;
        dv.ns = std::min(chunk, spp - s0);
        const unsigned pg = (unsigned)std::max<int64_t>(
            1, std::min<int64_t>((npix * dv.ns + kThreads - 1) / kThreads, (int64_t)pgx_num_sms() * std::max(per_sm, 1)));
        PGX_CUDA_TRY(ctx, cudaMemsetAsync(dv.next, 0, sizeof(unsigned long long), s));
        k_diff_primal<<<pg, kThreads, 0, s>>>(sv, dv);
        k_diff_accumulate<<<grid_for(npix), kThreads, 0, s>>>(dv.samples, npix, dv.ns, dv.partial);
    }
    k_diff_gather<<<grid_for(npix), kThreads, 0, s>>>(dv.partial, ctx->width, ctx->height, spp, rs->d_img.as<double>());
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(image, rs->d_img.p, sizeof(double) * 3 * npix, cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return PGX_OK;
}

extern "C" int pgx_diff_adjoint(pgx_ctx* ctx, int32_t spp, uint64_t seed, int32_t max_depth, const float* dloss_dimage,
                                float* grad_env, float* grad_albedo, float* grad_roughness) {
    PGX_TRY(diff_check(ctx, "pgx_diff_adjoint"));
    PGX_TRY(diff_args(ctx, spp, max_depth, "pgx_diff_adjoint"));
    if (!dloss_dimage) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_diff_adjoint: null dloss_dimage");
    RenderState* rs = state_of(ctx);
    if (!rs->d_params) PGX_TRY(diff_params(ctx, rs, nullptr, nullptr, nullptr));
    const int64_t npix = (int64_t)ctx->width * ctx->height;
    const size_t ef = env_floats(ctx), nm = (size_t)ctx->nmats;
    cudaStream_t s = ctx->stream;
    PGX_CUDA_TRY(ctx, rs->d_dimg.reserve(sizeof(float) * 3 * npix));
    // Gradients are accumulated in double (millions of atomic additions
    // into the popular texels) and returned as float.
    PGX_CUDA_TRY(ctx, rs->d_genv.reserve(sizeof(double) * std::max<size_t>(ef, 1)));
    PGX_CUDA_TRY(ctx, rs->d_galb.reserve(sizeof(double) * std::max<size_t>(3 * nm, 1)));
    PGX_CUDA_TRY(ctx, rs->d_grough.reserve(sizeof(double) * std::max<size_t>(nm, 1)));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(rs->d_dimg.p, dloss_dimage, sizeof(float) * 3 * npix, cudaMemcpyHostToDevice, s));
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(rs->d_genv.p, 0, sizeof(double) * std::max<size_t>(ef, 1), s));
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(rs->d_galb.p, 0, sizeof(double) * std::max<size_t>(3 * nm, 1), s));
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(rs->d_grough.p, 0, sizeof(double) * std::max<size_t>(nm, 1), s));
    PGX_CUDA_TRY(ctx, rs->d_next.reserve(sizeof(unsigned long long)));
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(rs->d_next.p, 0, sizeof(unsigned long long), s));
    DiffView dv = diff_view(ctx, rs, spp, seed, max_depth);
    dv.dimg = rs->d_dimg.as<float>();
    dv.g_env = ef ? rs->d_genv.as<double>() : nullptr;
    dv.g_alb = rs->d_galb.as<double>();
    dv.g_rough = rs->d_grough.as<double>();
    dv.next = rs->d_next.as<unsigned long long>();
    const size_t sm = nm * 4 * sizeof(double) <= 32 * 1024 ? nm * 4 * sizeof(double) : 0;
    SceneView sv = scene_view(ctx);
    // persistent: as many blocks as are resident at once
    int per_sm = 0;
    PGX_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_diff_adjoint, kThreads, sm));
    const unsigned ag = (unsigned)std::max<int64_t>(
        1, std::min<int64_t>((npix * (int64_t)spp + kThreads - 1) / kThreads,
                             (int64_t)pgx_num_sms() * std::max(per_sm, 1)));
    k_diff_adjoint<<<ag, kThreads, sm, s>>>(sv, dv);
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    std::vector<double> he(grad_env && ef ? ef : 0), ha(grad_albedo ? 3 * nm : 0), hr(grad_roughness ? nm : 0);
    if (!he.empty())
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(he.data(), rs->d_genv.p, sizeof(double) * ef, cudaMemcpyDeviceToHost, s));
    if (!ha.empty())
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(ha.data(), rs->d_galb.p, sizeof(double) * 3 * nm, cudaMemcpyDeviceToHost, s));
    if (!hr.empty())
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(hr.data(), rs->d_grough.p, sizeof(double) * nm, cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    for (size_t i = 0; i < he.size(); i++) grad_env[i] = (float)he[i];
    for (size_t i = 0; i < ha.size(); i++) grad_albedo[i] = (float)ha[i];
    for (size_t i = 0; i < hr.size(); i++) grad_roughness[i] = (float)hr[i];
    return PGX_OK;
}

// ---- batched rendering ----------------------------------------------------------------------
// pgx_batch_create merges the scenes' traversal nodes, triangles, shading
// records, materials, textures and area lights into one set of arrays held
// by an internal context (child references, triangle ids, material,
// texture and texel indexes shifted by each scene's base) and keeps per
// scene its root, light range, camera, bounds and film (BatchInfo).  A
// render runs the wavefront pipeline over waves of (scene, pixel, sample)
// items: paths of all scenes share the queues and every launch, and each
// path finds its tree root and lights through its scene index.  The waves
// of one call are captured in one CUDA graph.
namespace {

__global__ void k_merge_nodes(TravNode* n, int64_t cnt, int rec_base, int tri_base) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (int64_t)gridDim.x * blockDim.x) {
        TravNode t = n[i];
        int lc = __float_as_int(t.lmax.w), rc = __float_as_int(t.rmax.w);
        t.lmin.w = __int_as_float(__float_as_int(t.lmin.w) + (lc > 0 ? tri_base : rec_base));
        t.rmin.w = __int_as_float(__float_as_int(t.rmin.w) + (rc > 0 ? tri_base : rec_base));
        n[i] = t;
    }
}
__global__ void k_merge_tris(TravTri* t, int64_t cnt, int tri_base) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (int64_t)gridDim.x * blockDim.x)
        t[i].v0.w = __int_as_float(__float_as_int(t[i].v0.w) + tri_base);
}
__global__ void k_merge_shade(TriShade* sh, int64_t cnt, int mat_base) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (int64_t)gridDim.x * blockDim.x)
        sh[i].vv.w = __int_as_float(__float_as_int(sh[i].vv.w) + mat_base);
}
__global__ void k_merge_mats(DevMaterial* m, int cnt, int tex_base) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) m[i].tex += tex_base;
}
__global__ void k_merge_textures(DevTexture* t, int cnt, long long texel_base) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) t[i].offset += texel_base;
}
__global__ void k_merge_lights(DevAreaLight* l, int cnt, int tri_base) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
        l[i].p1.w = __int_as_float(__float_as_int(l[i].p1.w) + tri_base);
}

}  // namespace

struct pgx_batch {
    std::vector<pgx_ctx*> ctx;
    pgx_ctx* host = nullptr;        // merged arrays, stream, error text, path state
    std::vector<BatchInfo> info;    // per scene (roots and bases fixed at creation)
    DevBuf d_info, d_prefix, d_seed;
    pgx_batch_tuning tuning{1 << 24, 8, 16, kShortStack};
    pgx_batch_stats stats{};
    cudaGraphExec_t graph = nullptr;
    int g_spp = -1, g_depth = -1;
    pgx_batch_tuning g_tuning{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int sms = 0;
};

namespace {

int batch_fail(pgx_batch* b, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    b->host->err = buf;
    return code;
}

bool tuning_ok(const pgx_batch_tuning& t) {
    bool stack_ok = false;
    for (int c : kShortStackChoices) stack_ok |= t.stack_shared == c;
    return t.wave_paths >= (1 << 16) && t.wave_paths <= (1LL << 25) && t.trace_blocks_per_sm >= 1 &&
           t.trace_blocks_per_sm <= kPersistentBlocksPerSM && t.shade_blocks_per_sm >= 1 && t.shade_blocks_per_sm <= 16 &&
           stack_ok;
}

// Per-scene tables for `spp` samples; films of the scenes, or one scratch
// film for all (autotuning).
int batch_tables(pgx_batch* b, int spp, float* scratch) {
    const int n = (int)b->ctx.size();
    std::vector<BatchInfo> t = b->info;
    std::vector<int64_t> prefix((size_t)n + 1, 0);
    for (int i = 0; i < n; i++) {
        pgx_ctx* c = b->ctx[(size_t)i];
        if (ensure_film(c) != PGX_OK) return batch_fail(b, PGX_ERR_CUDA, "%s", c->err.c_str());
        t[(size_t)i].film = scratch ? scratch : c->film.as<float>();
        t[(size_t)i].spp0 = c->spp;
        prefix[(size_t)i + 1] = prefix[(size_t)i] + t[(size_t)i].npix * spp;
    }
    cudaStream_t s = b->host->stream;
    PGX_CUDA_TRY(b->host, cudaMemcpyAsync(b->d_info.p, t.data(), sizeof(BatchInfo) * (size_t)n, cudaMemcpyHostToDevice, s));
    PGX_CUDA_TRY(b->host, cudaMemcpyAsync(b->d_prefix.p, prefix.data(), sizeof(int64_t) * (size_t)(n + 1),
                                          cudaMemcpyHostToDevice, s));
    PGX_CUDA_TRY(b->host, cudaStreamSynchronize(s));
    b->stats.paths = prefix[(size_t)n];
    return PGX_OK;
}

// Enqueues every wave of one call: camera rays, (extend, shade, shadow) per
// depth, splat.
int batch_enqueue(pgx_batch* b, int64_t total, int depth, const pgx_batch_tuning& tu) {
    pgx_ctx* h = b->host;
    RenderState* rs = state_of(h);
    SceneView sv = scene_view(h);
    PathState ps = path_view(rs);
    GuideView gv{};
    const BatchInfo* info = b->d_info.as<BatchInfo>();
    cudaStream_t s = h->stream;
    FrameParams fp{};
    fp.mode = PGX_MODE_PLAIN;
    fp.max_depth = depth;
    fp.batch = 1;
    const unsigned tg = (unsigned)(b->sms * tu.trace_blocks_per_sm);
    const unsigned sg = (unsigned)(b->sms * tu.shade_blocks_per_sm);
    for (int64_t base = 0; base < total; base += tu.wave_paths) {
        BatchWave bw{info, b->d_prefix.as<int64_t>(), (int)b->ctx.size(), base, std::min<int64_t>(tu.wave_paths, total - base),
                     b->d_seed.as<uint64_t>()};
        cudaMemsetAsync(ps.qcount, 0, sizeof(unsigned) * 4 * (kMaxDepthCap + 2), s);
        cudaMemsetAsync(ps.ccount, 0, sizeof(unsigned) * kShadeClasses * (kMaxDepthCap + 2), s);
        k_camgen_batch<<<sg, kThreads, 0, s>>>(ps, bw);
        for (int d = 0; d <= depth; d++) {
            switch (tu.stack_shared) {
                case 4: k_extend<false, true, 4><<<tg, kThreads, 0, s>>>(sv, ps, d, info); break;
                case 16: k_extend<false, true, 16><<<tg, kThreads, 0, s>>>(sv, ps, d, info); break;
                default: k_extend<false, true, 8><<<tg, kThreads, 0, s>>>(sv, ps, d, info); break;
            }
            k_classify<<<grid_for((bw.count + kClassifyItems - 1) / kClassifyItems), kThreads, 0, s>>>(sv, ps, d);
            for (int c = 0; c < kShadeClasses; c++)
                launch_shade_class<PGX_MODE_PLAIN, true>(c, sg, s, sv, ps, fp, d, gv, info);
            switch (tu.stack_shared) {
                case 4: k_shadow<false, true, 4><<<tg, kThreads, 0, s>>>(sv, ps, d, info); break;
                case 16: k_shadow<false, true, 16><<<tg, kThreads, 0, s>>>(sv, ps, d, info); break;
                default: k_shadow<false, true, 8><<<tg, kThreads, 0, s>>>(sv, ps, d, info); break;
            }
        }
        k_finalize_batch<<<sg, kThreads, 0, s>>>(ps, bw);
    }
    PGX_CUDA_TRY(h, cudaGetLastError());
    return PGX_OK;
}

int batch_state(pgx_batch* b, const pgx_batch_tuning& tu) {
    return ensure_state(b->host, state_of(b->host), tu.wave_paths, 0, 0, false, 0, 0, true);
}

}  // namespace

extern "C" int pgx_batch_create(pgx_ctx* const* scenes, int32_t n, pgx_batch** out) {
    if (!out) return PGX_ERR_INVALID_ARG;
    *out = nullptr;
    if (!scenes || n <= 0) return PGX_ERR_INVALID_ARG;
    int64_t recs = 0, tris = 0, texels = 0;
    int64_t mats = 0, texs = 0, lights = 0;
    for (int32_t i = 0; i < n; i++) {
        pgx_ctx* c = scenes[i];
        if (!c || c->device != scenes[0]->device) return PGX_ERR_INVALID_ARG;
        if (!c->has_scene || !c->has_bvh) return PGX_ERR_STATE;
        recs += c->n_records;
        tris += c->ntris;
        mats += c->nmats;
        texs += c->ntex;
        texels += c->ntexels;
        lights += c->n_area_lights;
    }
    if (recs >= INT32_MAX || tris >= INT32_MAX || texs >= INT32_MAX) return PGX_ERR_OVERFLOW;
    pgx_batch* b = new pgx_batch();
    b->ctx.assign(scenes, scenes + n);
    b->host = new pgx_ctx();
    pgx_ctx* h = b->host;
    h->device = scenes[0]->device;
    auto fail = [&](int code) {
        pgx_batch_destroy(b);
        return code;
    };
    if (cudaSetDevice(h->device) != cudaSuccess || cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
        cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess)
        return fail(PGX_ERR_CUDA);
    if (h->trav_nodes.reserve(sizeof(TravNode) * std::max<int64_t>(recs, 1)) != cudaSuccess ||
        h->trav_tris.reserve(sizeof(TravTri) * tris) != cudaSuccess || h->shade.reserve(sizeof(TriShade) * tris) != cudaSuccess ||
        h->mats.reserve(sizeof(DevMaterial) * mats) != cudaSuccess ||
        h->textures.reserve(sizeof(DevTexture) * std::max<int64_t>(texs, 1)) != cudaSuccess ||
        h->texels.reserve(sizeof(float) * 3 * std::max<int64_t>(texels, 1)) != cudaSuccess ||
        h->lights.reserve(sizeof(DevAreaLight) * lights) != cudaSuccess || h->tri_class.reserve(tris) != cudaSuccess ||
        b->d_info.reserve(sizeof(BatchInfo) * n) != cudaSuccess ||
        b->d_prefix.reserve(sizeof(int64_t) * (n + 1)) != cudaSuccess || b->d_seed.reserve(sizeof(uint64_t)) != cudaSuccess)
        return fail(PGX_ERR_OOM);
    cudaStream_t s = h->stream;
    int64_t rb = 0, tb = 0, mb = 0, xb = 0, eb = 0, lb = 0;
    b->info.resize((size_t)n);
    for (int32_t i = 0; i < n; i++) {
        pgx_ctx* c = scenes[i];
        cudaStreamSynchronize(c->stream);
        bool ok = cudaMemcpyAsync(h->trav_nodes.as<TravNode>() + rb, c->trav_nodes.p, sizeof(TravNode) * c->n_records,
                                  cudaMemcpyDeviceToDevice, s) == cudaSuccess &&
                  cudaMemcpyAsync(h->trav_tris.as<TravTri>() + tb, c->trav_tris.p, sizeof(TravTri) * c->ntris,
                                  cudaMemcpyDeviceToDevice, s) == cudaSuccess &&
                  cudaMemcpyAsync(h->shade.as<TriShade>() + tb, c->shade.p, sizeof(TriShade) * c->ntris,
                                  cudaMemcpyDeviceToDevice, s) == cudaSuccess &&
                  cudaMemcpyAsync(h->mats.as<DevMaterial>() + mb, c->mats.p, sizeof(DevMaterial) * c->nmats,
                                  cudaMemcpyDeviceToDevice, s) == cudaSuccess &&
                  cudaMemcpyAsync(h->textures.as<DevTexture>() + xb, c->textures.p, sizeof(DevTexture) * c->ntex,
                                  cudaMemcpyDeviceToDevice, s) == cudaSuccess &&
                  cudaMemcpyAsync(h->texels.as<float>() + 3 * eb, c->texels.p, sizeof(float) * 3 * c->ntexels,
                                  cudaMemcpyDeviceToDevice, s) == cudaSuccess &&
                  cudaMemcpyAsync(h->lights.as<DevAreaLight>() + lb, c->lights.p, sizeof(DevAreaLight) * c->n_area_lights,
                                  cudaMemcpyDeviceToDevice, s) == cudaSuccess &&
                  cudaMemcpyAsync(h->tri_class.as<unsigned char>() + tb, c->tri_class.p, (size_t)c->ntris,
                                  cudaMemcpyDeviceToDevice, s) == cudaSuccess;
        if (!ok) return fail(PGX_ERR_CUDA);
        const unsigned g = 256;
        if (c->n_records) k_merge_nodes<<<g, 256, 0, s>>>(h->trav_nodes.as<TravNode>() + rb, c->n_records, (int)rb, (int)tb);
        k_merge_tris<<<g, 256, 0, s>>>(h->trav_tris.as<TravTri>() + tb, c->ntris, (int)tb);
        k_merge_shade<<<g, 256, 0, s>>>(h->shade.as<TriShade>() + tb, c->ntris, (int)mb);
        k_merge_mats<<<g, 256, 0, s>>>(h->mats.as<DevMaterial>() + mb, c->nmats, (int)xb);
        k_merge_textures<<<g, 256, 0, s>>>(h->textures.as<DevTexture>() + xb, c->ntex, (long long)eb);
        k_merge_lights<<<g, 256, 0, s>>>(h->lights.as<DevAreaLight>() + lb, c->n_area_lights, (int)tb);
        BatchInfo& bi = b->info[(size_t)i];
        bi = BatchInfo{};
        bi.root = c->root;
        bi.root.ref += (c->root.count > 0) ? (int)tb : (int)rb;
        bi.light_base = (int)lb;
        bi.n_lights = c->n_area_lights;
        bi.env = c->env;
        bi.has_env_light = (c->env.valid && c->env.power > 0.f) ? 1 : 0;
        bi.cam = c->camera;
        bi.bounds = c->bounds;
        bi.width = c->width;
        bi.height = c->height;
        bi.npix = (int64_t)c->width * c->height;
        rb += c->n_records;
        tb += c->ntris;
        mb += c->nmats;
        xb += c->ntex;
        eb += c->ntexels;
        lb += c->n_area_lights;
    }
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) return fail(PGX_ERR_CUDA);
    h->n_records = recs;
    h->ntris = tris;
    h->nmats = (int32_t)mats;
    h->ntex = (int32_t)texs;
    h->ntexels = texels;
    h->n_area_lights = (int32_t)lights;
    h->nlights = (int32_t)lights;
    h->has_scene = true;
    h->has_bvh = true;
    h->root.valid = 0;  // every path starts from its scene's root
    h->env.valid = 0;
    h->width = h->height = 1;  // per-path sizes come from BatchInfo
    *out = b;
    return PGX_OK;
}

extern "C" int pgx_batch_destroy(pgx_batch* b) {
    if (!b) return PGX_OK;
    if (b->host) {
        cudaSetDevice(b->host->device);
        if (b->host->stream) cudaStreamSynchronize(b->host->stream);
        if (b->graph) cudaGraphExecDestroy(b->graph);
        if (b->ev0) cudaEventDestroy(b->ev0);
        if (b->ev1) cudaEventDestroy(b->ev1);
        b->d_info.release();
        b->d_prefix.release();
        b->d_seed.release();
        render_state_free(b->host);
        if (b->host->stream) cudaStreamDestroy(b->host->stream);
        delete b->host;
    }
    delete b;
    return PGX_OK;
}

extern "C" const char* pgx_batch_last_error(pgx_batch* b) { return (b && b->host) ? b->host->err.c_str() : "null batch"; }

extern "C" int pgx_batch_set_tuning(pgx_batch* b, const pgx_batch_tuning* t) {
    if (!b || !t) return PGX_ERR_INVALID_ARG;
    if (!tuning_ok(*t)) return batch_fail(b, PGX_ERR_INVALID_ARG, "pgx_batch_set_tuning: out of range");
    b->tuning = *t;
    return PGX_OK;
}

extern "C" int pgx_batch_get_stats(pgx_batch* b, pgx_batch_stats* st) {
    if (!b || !st) return PGX_ERR_INVALID_ARG;
    *st = b->stats;
    return PGX_OK;
}

extern "C" int pgx_batch_render(pgx_batch* b, int32_t spp, uint64_t seed, int32_t max_depth) {
    if (!b) return PGX_ERR_INVALID_ARG;
    pgx_ctx* h = b->host;
    h->err.clear();
    if (spp <= 0 || max_depth < 0 || max_depth > kMaxDepthCap)
        return batch_fail(b, PGX_ERR_INVALID_ARG, "pgx_batch_render: bad spp or max_depth");
    PGX_CUDA_TRY(h, cudaSetDevice(h->device));
    for (pgx_ctx* c : b->ctx) PGX_CUDA_TRY(h, cudaStreamSynchronize(c->stream));
    PGX_TRY(batch_state(b, b->tuning));
    PGX_TRY(batch_tables(b, spp, nullptr));
    PGX_CUDA_TRY(h, cudaMemcpyAsync(b->d_seed.p, &seed, sizeof(uint64_t), cudaMemcpyHostToDevice, h->stream));
    const bool replay = b->graph && b->g_spp == spp && b->g_depth == max_depth &&
                        b->g_tuning.wave_paths == b->tuning.wave_paths &&
                        b->g_tuning.trace_blocks_per_sm == b->tuning.trace_blocks_per_sm &&
                        b->g_tuning.shade_blocks_per_sm == b->tuning.shade_blocks_per_sm;
    if (!replay) {
        if (b->graph) cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        cudaGraph_t g;
        PGX_CUDA_TRY(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        int rc = batch_enqueue(b, b->stats.paths, max_depth, b->tuning);
        cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
        if (rc != PGX_OK) return rc;
        PGX_CUDA_TRY(h, ec);
        cudaError_t e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->graph = nullptr;
            return batch_fail(b, PGX_ERR_CUDA, "pgx_batch_render: graph instantiation: %s", cudaGetErrorString(e));
        }
        b->g_spp = spp;
        b->g_depth = max_depth;
        b->g_tuning = b->tuning;
    }
    PGX_CUDA_TRY(h, cudaEventRecord(b->ev0, h->stream));
    PGX_CUDA_TRY(h, cudaGraphLaunch(b->graph, h->stream));
    PGX_CUDA_TRY(h, cudaEventRecord(b->ev1, h->stream));
    PGX_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    float ms = 0.f;
    PGX_CUDA_TRY(h, cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->stats.ms = ms;
    b->stats.graph_replayed = replay ? 1 : 0;
    for (pgx_ctx* c : b->ctx) c->spp += spp;
    return PGX_OK;
}

extern "C" int pgx_batch_autotune(pgx_batch* b, int32_t spp, int32_t max_depth, pgx_batch_tuning* best) {
    if (!b) return PGX_ERR_INVALID_ARG;
    pgx_ctx* h = b->host;
    h->err.clear();
    if (spp <= 0 || max_depth < 0 || max_depth > kMaxDepthCap)
        return batch_fail(b, PGX_ERR_INVALID_ARG, "pgx_batch_autotune: bad spp or max_depth");
    PGX_CUDA_TRY(h, cudaSetDevice(h->device));
    int64_t max_film = 0;
    for (const BatchInfo& bi : b->info) max_film = std::max(max_film, bi.npix * 3);
    DevBuf scratch;
    PGX_CUDA_TRY(h, scratch.reserve(sizeof(float) * (size_t)max_film));
    PGX_TRY(batch_tables(b, spp, scratch.as<float>()));
    uint64_t seed = 0x5eedULL;
    PGX_CUDA_TRY(h, cudaMemcpyAsync(b->d_seed.p, &seed, sizeof(uint64_t), cudaMemcpyHostToDevice, h->stream));
    const int64_t total = b->stats.paths;
    const int64_t waves[] = {1 << 20, 1 << 21, 1 << 22, 1 << 23, 1 << 24, 1 << 25};
    const int trace_bps[] = {4, 8};
    const int shade_bps[] = {8, 16};
    float best_ms = 1e30f;
    pgx_batch_tuning pick = b->tuning;
    auto trial = [&](const pgx_batch_tuning& t) -> int {
        PGX_TRY(batch_state(b, t));
        PGX_TRY(batch_enqueue(b, total, max_depth, t));  // warm-up
        PGX_CUDA_TRY(h, cudaEventRecord(b->ev0, h->stream));
        PGX_TRY(batch_enqueue(b, total, max_depth, t));
        PGX_CUDA_TRY(h, cudaEventRecord(b->ev1, h->stream));
        PGX_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        float ms = 0.f;
        PGX_CUDA_TRY(h, cudaEventElapsedTime(&ms, b->ev0, b->ev1));
        if (ms < best_ms) {
            best_ms = ms;
            pick = t;
        }
        return PGX_OK;
    };
    // Queue capacity and block shapes at the default stack split, then the
    // stack's shared-memory depth at the best of those.
    for (int64_t w : waves) {
        if (w > 2 * total && w != waves[0]) continue;  // larger waves than the work change nothing
        for (int tbp : trace_bps)
            for (int sbp : shade_bps) PGX_TRY(trial(pgx_batch_tuning{w, tbp, sbp, kShortStack}));
    }
    const pgx_batch_tuning shape = pick;
    for (int sh : kShortStackChoices)
        if (sh != kShortStack) PGX_TRY(trial(pgx_batch_tuning{shape.wave_paths, shape.trace_blocks_per_sm,
                                                              shape.shade_blocks_per_sm, sh}));
    b->tuning = pick;
    if (best) *best = pick;
    return PGX_OK;
}
