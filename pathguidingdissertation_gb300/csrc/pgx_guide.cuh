// QuadTree directional guide over the point-BVH radiance cache (extension;
// the reference sketches it in Renderer.h:398-414 and ships only an unused
// point quadtree, QuadTree.h).
//
// Spatial side: the cache's point BVH is cut into regions — the subtrees
// whose record count first drops to pgx_guide_params.region_records.
// Directional side: each region owns a quadtree over the cylindrical
// equal-area map of world directions, (u, v) = ((cos(theta) + 1) / 2,
// (phi + pi) / 2pi) with theta measured from +z (solid angle = 4*pi * area
// in (u, v)).  Cells are refined while they hold more than refine_fraction
// (1 %) of the region's flux (Mueller et al. 2017, "Practical Path
// Guiding").  A record's flux is its weight: Lum(Li) |cos| / pdf for the
// records of plain and guided renders (an estimate of Li |cos| whichever
// distribution sampled wi), Lum(Li) for host and guided-Li records; weights
// are clamped at clamp_median x the region's median (10 by default).
//
// At a shading point the region is found by descending the point BVH; the
// guide is the region's quadtree mixed with a uniform share (20 % by
// default), and the continuation direction is drawn by one-sample MIS
// between the guide and the BSDF (probability `guide_fraction` for the
// guide); the combined pdf is used both for the throughput and for the MIS
// weights of NEE and of emitter hits, so the estimator stays unbiased.
// Pure-specular BSDFs, glass, conductors narrower than glossy_alpha and
// regions without flux sample the BSDF alone.
#pragma once

#include "pgx_ctx.h"
#include "pgx_shade.cuh"

#define PGX_QT_MAX_DEPTH 10
#define PGX_QT_MAX_NODES 256

// Interior quadtree cell: flux of its four children (index = 2*yhalf + xhalf
// in (u, v)) and their node indices within the region (-1 = leaf).
struct __align__(16) QuadNode {
    float flux[4];
    int child[4];
};

// Point-BVH node for nearest-record queries: bmin.w = left child (or
// -(offset + 1) for a leaf), bmax.w = right child (or record count).
struct __align__(16) CacheTravNode {
    float4 bmin;
    float4 bmax;
};

struct GuideView {
    int valid;
    int n_nodes;
    int n_records;
    const CacheTravNode* __restrict__ nodes;
    const float4* __restrict__ rec_pos;   // xyz, w = region id bits
    const int* __restrict__ region_qroot; // first QuadNode of each region (-1: no flux)
    const QuadNode* __restrict__ qnodes;
    const int* __restrict__ node_region;  // region index of region-root nodes, else -1
    int pss;  // 1: the quadtrees are over the diffuse BSDF's primary samples, 0: over directions
    float uniform;  // share of the guide's samples drawn uniformly (defensive)
    float min_alpha;  // conductors with a smaller GGX alpha sample the BSDF alone
};

GuideView guide_view(const pgx_ctx* ctx);
bool guide_ready(const pgx_ctx* ctx);
// Number of the cache build (changes whenever the cache is rebuilt) and its
// region count; 0 regions when there is no cache.
uint64_t guide_generation(const pgx_ctx* ctx);
int guide_regions(const pgx_ctx* ctx);
// d_weights: flux weight per record (nullptr: the luminance of its Li).
int cache_build_device(pgx_ctx* ctx, const pgx_path_vertex* d_records, int64_t n, bool pss = false,
                       const float* d_weights = nullptr);

__device__ __forceinline__ void dir_to_uv(F3 w, float& u, float& v) {
    float c = fminf(fmaxf(w.z, -1.f), 1.f);
    u = (c + 1.f) * 0.5f;
    float phi = atan2f(w.y, w.x);
    v = (phi + 3.14159265f) * (1.f / (2.f * 3.14159265f));
    u = fminf(fmaxf(u, 0.f), 0.99999994f);
    v = fminf(fmaxf(v, 0.f), 0.99999994f);
}
__device__ __forceinline__ F3 uv_to_dir(float u, float v) {
    float c = 2.f * u - 1.f;
    float s = sqrtf(fmaxf(0.f, 1.f - c * c));
    float phi = 2.f * 3.14159265f * v - 3.14159265f;
    return f3(s * cosf(phi), s * sinf(phi), c);
}

// Nearest cached record to x (squared distance, ties to the lower index).
static __device__ int guide_nearest(const GuideView& g, F3 x) {
    if (g.n_nodes <= 0) return -1;
    int stack[64];
    int sp = 0;
    int best = -1;
    float bestd = FLT_MAX;
    int node = 0;
    for (;;) {
        CacheTravNode n = g.nodes[node];
        int l = __float_as_int(n.bmin.w), r = __float_as_int(n.bmax.w);
        if (l < 0) {
            int off = -l - 1;
            for (int k = 0; k < r; k++) {
                float4 p = g.rec_pos[off + k];
                float dx = p.x - x.x, dy = p.y - x.y, dz = p.z - x.z;
                float d = dx * dx + dy * dy + dz * dz;
                if (d < bestd || (d == bestd && off + k < best)) {
                    bestd = d;
                    best = off + k;
                }
            }
        } else {
            CacheTravNode a = g.nodes[l], b = g.nodes[r];
            auto box_d = [&](const CacheTravNode& c) {
                float dx = fmaxf(fmaxf(c.bmin.x - x.x, x.x - c.bmax.x), 0.f);
                float dy = fmaxf(fmaxf(c.bmin.y - x.y, x.y - c.bmax.y), 0.f);
                float dz = fmaxf(fmaxf(c.bmin.z - x.z, x.z - c.bmax.z), 0.f);
                return dx * dx + dy * dy + dz * dz;
            };
            float da = box_d(a), db = box_d(b);
            int first = l, second = r;
            if (db < da) {
                float t = da;
                da = db;
                db = t;
                first = r;
                second = l;
            }
            if (da <= bestd) {
                if (db <= bestd && sp < 64) stack[sp++] = second;
                node = first;
                continue;
            }
        }
        // pop the next node that can still hold a closer record
        bool found = false;
        while (sp > 0) {
            int c = stack[--sp];
            CacheTravNode n2 = g.nodes[c];
            float dx = fmaxf(fmaxf(n2.bmin.x - x.x, x.x - n2.bmax.x), 0.f);
            float dy = fmaxf(fmaxf(n2.bmin.y - x.y, x.y - n2.bmax.y), 0.f);
            float dz = fmaxf(fmaxf(n2.bmin.z - x.z, x.z - n2.bmax.z), 0.f);
            if (dx * dx + dy * dy + dz * dz <= bestd) {
                node = c;
                found = true;
                break;
            }
        }
        if (!found) break;
    }
    return best;
}

// Quadtree pdf in (u, v) space (density w.r.t. area; 1 = uniform).
static __device__ float quad_pdf(const QuadNode* qn, int root, float u, float v) {
    float pdf = 1.f;
    int node = root;
    for (int d = 0; d < PGX_QT_MAX_DEPTH + 1; d++) {
        QuadNode n = qn[node];
        float total = n.flux[0] + n.flux[1] + n.flux[2] + n.flux[3];
        if (!(total > 0.f)) return 0.f;
        int xi = u >= 0.5f ? 1 : 0, yi = v >= 0.5f ? 1 : 0;
        int c = 2 * yi + xi;
        pdf *= 4.f * n.flux[c] / total;
        if (n.child[c] < 0 || pdf == 0.f) return pdf;
        u = u * 2.f - (float)xi;
        v = v * 2.f - (float)yi;
        node = n.child[c];
    }
    return pdf;
}

static __device__ void quad_sample(const QuadNode* qn, int root, float r1, float r2, float& u, float& v) {
    float u0 = 0.f, v0 = 0.f, size = 1.f;
    int node = root;
    for (int d = 0; d < PGX_QT_MAX_DEPTH + 1; d++) {
        QuadNode n = qn[node];
        float left = n.flux[0] + n.flux[2], right = n.flux[1] + n.flux[3];
        float total = left + right;
        int xi;
        float pl = total > 0.f ? left / total : 0.5f;
        if (r1 < pl) {
            xi = 0;
            r1 = pl > 0.f ? r1 / pl : 0.f;
        } else {
            xi = 1;
            r1 = (1.f - pl) > 0.f ? (r1 - pl) / (1.f - pl) : 0.f;
        }
        float top = n.flux[xi], bot = n.flux[2 + xi];
        float pt = (top + bot) > 0.f ? top / (top + bot) : 0.5f;
        int yi;
        if (r2 < pt) {
            yi = 0;
            r2 = pt > 0.f ? r2 / pt : 0.f;
        } else {
            yi = 1;
            r2 = (1.f - pt) > 0.f ? (r2 - pt) / (1.f - pt) : 0.f;
        }
        r1 = fminf(r1, 0.99999994f);
        r2 = fminf(r2, 0.99999994f);
        size *= 0.5f;
        u0 += size * (float)xi;
        v0 += size * (float)yi;
        int c = 2 * yi + xi;
        if (n.child[c] < 0) break;
        node = n.child[c];
    }
    u = u0 + size * r1;
    v = v0 + size * r2;
}

// Region of x: descend the point BVH from the root, entering the child whose
// box is nearer to x (0 when inside; ties to the left), until a region root;
// returns the region's index (-1 when a leaf comes first).
__device__ __forceinline__ int guide_region_index(const GuideView& g, F3 x) {
    if (!g.valid || g.n_nodes <= 0) return -1;
    int node = 0;
    for (int d = 0; d < 64; d++) {
        int r = g.node_region[node];
        if (r >= 0) return r;
        CacheTravNode n = g.nodes[node];
        int l = __float_as_int(n.bmin.w), rt = __float_as_int(n.bmax.w);
        if (l < 0) return -1;
        CacheTravNode a = g.nodes[l], b = g.nodes[rt];
        auto box_d = [&](const CacheTravNode& c) {
            float dx = fmaxf(fmaxf(c.bmin.x - x.x, x.x - c.bmax.x), 0.f);
            float dy = fmaxf(fmaxf(c.bmin.y - x.y, x.y - c.bmax.y), 0.f);
            float dz = fmaxf(fmaxf(c.bmin.z - x.z, x.z - c.bmax.z), 0.f);
            return dx * dx + dy * dy + dz * dz;
        };
        node = (box_d(b) < box_d(a)) ? rt : l;
    }
    return -1;
}

// The quadtree root of x's region (-1: no region or no flux).
__device__ __forceinline__ int guide_region_root(const GuideView& g, F3 x) {
    const int r = guide_region_index(g, x);
    return r >= 0 ? g.region_qroot[r] : -1;
}

// Surfaces the direction-space QuadTree guides: every non-specular one
// except conductors narrower than min_alpha.  K: the kind when known.
template <int K = -1>
__device__ __forceinline__ bool qt_guided_surface(const GuideView& g, const DevMaterial& m) {
    return (K >= 0 ? K : m.kind) != PGX_BSDF_CONDUCTOR || m.alpha >= g.min_alpha;
}

// Solid-angle pdf of the guide (quadtree mixed with a uniform share).
__device__ __forceinline__ float guide_pdf_dir(const GuideView& g, int qroot, F3 wi) {
    float u, v;
    dir_to_uv(wi, u, v);
    return ((1.f - g.uniform) * quad_pdf(g.qnodes, qroot, u, v) + g.uniform) *
           (1.f / (4.f * 3.14159265f));
}

// Primary sample of the diffuse BSDFs' sampler mapping to wi at a record or
// shading point with shading normal n (the frame the shading code builds),
// clamped into the quadtree's half-open square; false below the hemisphere.
__device__ __forceinline__ bool pss_uv(F3 n, F3 wi, float& u, float& v) {
    const Frame fr = frame_from(n);
    if (dot(wi, fr.w) <= 0.f) return false;
    cosine_invert(fr, wi, u, v);
    u = fminf(fmaxf(u, 0.f), 0.99999994f);
    v = fminf(fmaxf(v, 0.f), 0.99999994f);
    return true;
}

// Density over the primary-sample square of the PSS guide at (u, v): the
// quadtree mixed with a uniform share.
__device__ __forceinline__ float guide_pdf_uv(const GuideView& g, int qroot, float u, float v) {
    u = fminf(fmaxf(u, 0.f), 0.99999994f);
    v = fminf(fmaxf(v, 0.f), 0.99999994f);
    return (1.f - g.uniform) * quad_pdf(g.qnodes, qroot, u, v) + g.uniform;
}

// Solid-angle pdf of the one-sample mixture at wi.
__device__ __forceinline__ float mixture_pdf(const GuideView& g, int qroot, float frac, float bsdf_p, F3 wi) {
    if (qroot < 0) return bsdf_p;
    return frac * guide_pdf_dir(g, qroot, wi) + (1.f - frac) * bsdf_p;
}

// Continuation direction for the guided estimator: pdf is the mixture pdf.
// K: the material kind when the caller shades a single kind, else -1.
template <int K = -1>
__device__ __forceinline__ F3 guided_sample(const GuideView& g, float frac, const DevMaterial& m, const TexView& tv,
                                            const Shading& sd, uint64_t& rng, F3& f, float& pdf, int qroot) {
    if (qroot < 0 || bsdf_pure_specular_k<K>(m) || (K >= 0 ? K : m.kind) == PGX_BSDF_GLASS) {
        return bsdf_sample_k<K>(m, tv, sd, rng, f, pdf);
    }
    float sel = pgx_rng_next(rng);
    F3 wi;
    if (sel < frac) {
        float r1 = pgx_rng_next(rng), r2 = pgx_rng_next(rng);
        float u, v;
        float pick = sel / frac;  // reuse the selection number for the uniform share
        if (pick < g.uniform) {
            u = r1;
            v = r2;
        } else {
            quad_sample(g.qnodes, qroot, r1, r2, u, v);
        }
        wi = uv_to_dir(u, v);
        f = bsdf_eval_k<K>(m, tv, sd, wi);
    } else {
        float bp;
        wi = bsdf_sample_k<K>(m, tv, sd, rng, f, bp);
    }
    float bp = bsdf_pdf_k<K>(m, tv, sd, wi);
    pdf = mixture_pdf(g, qroot, frac, bp, wi);
    return wi;
}

// ---- guiding in the BSDF's primary sample space (PGX_MODE_GUIDED_PSS) ----------------
// Surfaces guided: the diffuse BSDFs, whose cosine sampler the cache's
// primary-sample quadtrees were built with.  K: the kind when known.
template <int K = -1>
__device__ __forceinline__ bool pss_surface(const DevMaterial& m) {
    const int kind = K >= 0 ? K : m.kind;
    return !m.is_light && (kind == PGX_BSDF_DIFFUSE || kind == PGX_BSDF_ORENNAYAR);
}

// Solid-angle pdf at wi of the mixture that draws the primary sample from
// the guide with probability frac (else uniformly) and maps it through the
// cosine sampler: (frac q(u, v) + 1 - frac) x the BSDF pdf, (u, v) the
// sampler's inverse at wi.
__device__ __forceinline__ float pss_mixture_pdf(const GuideView& g, int qroot, float frac, const Shading& sd,
                                                 float bsdf_p, F3 wi) {
    if (qroot < 0) return bsdf_p;
    if (dot(wi, sd.frame.w) <= 0.f) return (1.f - frac) * bsdf_p;  // the cosine sampler never goes there
    float u, v;
    cosine_invert(sd.frame, wi, u, v);
    return (frac * guide_pdf_uv(g, qroot, u, v) + (1.f - frac)) * bsdf_p;
}

// Continuation direction of the PSS-guided estimator: a primary sample from
// the region's quadtree (probability frac; the selection number is reused
// for the uniform share) or uniform, through BSDF::sample; pdf is the
// mixture's solid-angle density.
template <int K = -1>
__device__ __forceinline__ F3 pss_guided_sample(const GuideView& g, float frac, const DevMaterial& m,
                                                const TexView& tv, const Shading& sd, uint64_t& rng, F3& f,
                                                float& pdf, int qroot) {
    if (qroot < 0) return bsdf_sample_k<K>(m, tv, sd, rng, f, pdf);
    const float sel = pgx_rng_next(rng);
    const float r1 = pgx_rng_next(rng), r2 = pgx_rng_next(rng);
    float u = r1, v = r2;
    if (sel < frac && sel / frac >= g.uniform) quad_sample(g.qnodes, qroot, r1, r2, u, v);
    FixedSampler fs{u, v, 0};
    float bp;
    F3 wi;
    if constexpr (K >= 0)
        wi = bsdf_sample_i<K>(m, tv, sd, fs, f, bp);
    else
        wi = bsdf_sample_s(m, tv, sd, fs, f, bp);
    pdf = (frac * guide_pdf_uv(g, qroot, u, v) + (1.f - frac)) * bp;
    return wi;
}

// Overload used by render.cu's shade kernel (region looked up here).
__device__ __forceinline__ F3 guided_sample(const GuideView& g, float frac, const DevMaterial& m, const TexView& tv,
                                            const Shading& sd, uint64_t& rng, F3& f, float& pdf) {
    int qroot = guide_region_root(g, sd.x);
    return guided_sample(g, frac, m, tv, sd, rng, f, pdf, qroot);
}
