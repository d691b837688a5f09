// Host-side context of libpgx: device buffers, the stream, error state.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pgx.h"
#include "pgx_device.cuh"
#include "pgx_trace.cuh"

// Owning device allocation.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    // Grows (never shrinks) to at least n bytes; contents are not kept.
    cudaError_t reserve(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        release();
        if (n == 0) n = 16;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        bytes = n;
        return cudaSuccess;
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

// Per-material parameters on the device (reference BSDF constructor
// arguments, Materials.h:136-897).
struct DevMaterial {
    int kind;
    int tex;          // texture index (always valid; constant albedo = 1x1 texture)
    int layered;
    int is_light;     // emission.Lum() > 0 (BSDF::isLight, Materials.h:130)
    float eta[3], k[3];
    float int_ior, ext_ior;
    float alpha;      // 1.62142 * sqrt(roughness)
    float sigma;
    float emission[3];
    float alb_off[3];  // added to the sampled albedo (0 except in differentiable renders)
};

// Shading class of a surface (the wavefront shades one class per launch):
// 1 emitter, 2 diffuse, 3 conductor, 4 glass, 5 other; 0 is a miss.
__host__ __device__ inline unsigned char shade_class(const DevMaterial& m) {
    return m.is_light ? 1 : (m.kind == PGX_BSDF_DIFFUSE ? 2 : (m.kind == PGX_BSDF_CONDUCTOR ? 3 : (m.kind == PGX_BSDF_GLASS ? 4 : 5)));
}

struct DevTexture {
    int width, height;
    long long offset;  // first texel in the texel pool (float3 units)
};

// Per-triangle shading data in original triangle order (Triangle::init,
// Geometry.h:76-94): vertex normals with uv, geometric normal with area.
struct __align__(16) TriShade {
    float4 n0;  // xyz normal, w = u0
    float4 n1;  // w = u1
    float4 n2;  // w = u2
    float4 vv;  // v0, v1, v2 texture v; w = material index bits
    float4 gn;  // gNormal (Geometry.h:153) xyz, w = area
};

// Emitting triangle (AreaLight, Lights.h:28-73).
struct __align__(16) DevAreaLight {
    float4 p0;   // w = area
    float4 p1;   // w = triangle id bits
    float4 p2;
    float4 gn;   // gNormal
    float4 emission;
};

struct DevCamera {
    float inv_proj[16];  // Camera::inverseProjectionMatrix
    float cam[16];       // Camera::camera (camera -> world)
    float origin[3];
    float width, height;
};

struct DevEnv {
    int valid;       // 0: black BackgroundColour
    int width, height;
    const float* texels;       // W*H*3
    const float* cond_func;    // H x W  (Distribution1D::function per row)
    const float* cond_cdf;     // H x (W+1)
    const float* cond_int;     // H      (functionIntegral per row)
    const float* marg_func;    // H
    const float* marg_cdf;     // H+1
    float marg_int;            // pMarginal->functionIntegral
    float power;               // totalIntegratedPower (Lights.h:200-210)
    // Guide tables of the CDFs (nullptr: plain binary search): for bucket k
    // of cdf_bucket(), the first CDF index in that bucket; H x (W + 1) and
    // H + 1 entries.
    const int* cond_guide;
    const int* marg_guide;
};

struct SceneBoundsDev {
    float centre[3];
    float radius;
    float bmin[3], bmax[3];
};

struct pgx_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;

    // ---- scene ----
    int64_t ntris = 0;
    int32_t nmats = 0;
    int32_t nlights = 0;       // area lights (+1 for the env map when present)
    int32_t n_area_lights = 0;
    DevBuf tris_in;            // pgx_triangle[ntris]
    DevBuf shade;              // TriShade[ntris]
    DevBuf tri_class;          // shade_class of each triangle's material (uint8)
    DevBuf mats;               // DevMaterial[nmats]
    DevBuf textures;           // DevTexture[ntex]
    DevBuf texels;             // float3 pool
    int32_t ntex = 0;
    int64_t ntexels = 0;       // float3 entries of the pool
    DevBuf lights;             // DevAreaLight[n_area_lights]
    std::vector<pgx_material> host_mats;
    DevCamera camera{};
    pgx_camera host_camera{};
    SceneBoundsDev bounds{};
    bool has_scene = false;

    // environment map
    DevBuf env_texels, env_cond_func, env_cond_cdf, env_cond_int, env_marg_func, env_marg_cdf;
    DevBuf env_cond_guide, env_marg_guide;
    DevEnv env{};

    // ---- BVH ----
    DevBuf bvh_nodes_ref;  // pgx_bvh_node[n_nodes] (reference layout)
    DevBuf bvh_idx;        // int32[ntris]
    DevBuf trav_nodes;     // TravNode[n_records]
    DevBuf trav_tris;      // TravTri[ntris]
    TravRoot root{};
    int64_t n_nodes = 0;
    int64_t n_records = 0;
    bool has_bvh = false;
    double bvh_build_ms = 0.0;

    // ---- trace scratch ----
    DevBuf trace_rays, trace_out, counters;
    unsigned long long last_interior = 0, last_tris = 0;

    // ---- build scratch ----
    DevBuf b_cent, b_tmin, b_tmax, b_idx2, b_items, b_items2, b_bins, b_chunks, b_small, b_misc, b_noderec;

    // ---- film / render ----
    int32_t width = 0, height = 0;
    int32_t spp = 0;
    DevBuf film, film2;
    pgx_render_stats rstats{};
    void* render_state = nullptr;  // owned by render.cu
    void* cache_state = nullptr;   // owned by cache.cu
    pgx_guide_params guide{1024, 0.01f, 10.f, 0.2f, 0.f, 0.f};  // QuadTree guide parameters (pgx_guide_configure)
    void* mlp_state = nullptr;     // owned by mlp.cu

    pgx_ctx() = default;
    pgx_ctx(const pgx_ctx&) = delete;
    pgx_ctx& operator=(const pgx_ctx&) = delete;
};

// Error helpers: record a message and return a status.
int pgx_fail(pgx_ctx* ctx, int code, const char* fmt, ...);
#define PGX_CUDA_TRY(ctx, call)                                                                     \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return pgx_fail((ctx), PGX_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,         \
                            cudaGetErrorString(e_));                                                \
    } while (0)
#define PGX_TRY(call)                 \
    do {                              \
        int s_ = (call);              \
        if (s_ != PGX_OK) return s_;  \
    } while (0)

// Streaming multiprocessors of the current device (queried once per device
// ordinal and cached); grids of persistent and grid-stride kernels are sized
// in multiples of it.
int pgx_num_sms();

// Internal entry points implemented across the .cu files.
int bvh_build_gpu(pgx_ctx* ctx);
int bvh_import_ref(pgx_ctx* ctx, const pgx_bvh_node* nodes, int64_t nnodes, const int32_t* idx);
int bvh_layout_from_ref(pgx_ctx* ctx, const int32_t* node_rec_host);
BvhView bvh_view(const pgx_ctx* ctx);
void render_state_free(pgx_ctx* ctx);
void cache_state_free(pgx_ctx* ctx);
void mlp_state_free(pgx_ctx* ctx);
