// Device-side building blocks shared by the kernels of libpgx.
//
// Two kinds of arithmetic live here:
//  * "exact" helpers (x_add, x_mul, ...) use the _rn intrinsics, which the
//    compiler never fuses into FMA, so ray/box and ray/triangle tests and the
//    BVH build round exactly like the reference's scalar code (Geometry.h);
//  * ordinary float math for shading, where the reference's results are
//    matched to a tolerance (transcendentals differ between libm and CUDA).
#pragma once

#include <cfloat>
#include <cstdint>

#include <cuda_runtime.h>

#define PGX_EPSILON 1e-4f        // Geometry.h:13
#define PGX_MT_EPSILON 1e-8f     // Geometry.h:14
#define PGX_STACK_SIZE 64        // Geometry.h:461

// ---- exact scalar ops (never contracted) ---------------------------------
__device__ __forceinline__ float x_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float x_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float x_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float x_div(float a, float b) { return __fdiv_rn(a, b); }
// std::min(a, b) / std::max(a, b): which operand wins decides NaN behaviour.
// Bucket of a value in [0, 1] among K equal buckets, for the guide tables of
// the environment's CDFs: built and read with this one function, so it only
// needs to be monotone (a rounded product, truncated and clamped, is).
__device__ __forceinline__ int cdf_bucket(float x, int K) {
    const int k = (int)x_mul(x, (float)K);
    return k < 0 ? 0 : (k > K - 1 ? K - 1 : k);
}

__host__ __device__ __forceinline__ float s_min(float a, float b) { return (b < a) ? b : a; }
__host__ __device__ __forceinline__ float s_max(float a, float b) { return (a < b) ? b : a; }

struct xv3 {
    float x, y, z;
};
__device__ __forceinline__ xv3 mk(float x, float y, float z) { return xv3{x, y, z}; }
__device__ __forceinline__ xv3 mk(float4 v) { return xv3{v.x, v.y, v.z}; }
__device__ __forceinline__ xv3 x_sub(xv3 a, xv3 b) { return mk(x_sub(a.x, b.x), x_sub(a.y, b.y), x_sub(a.z, b.z)); }
__device__ __forceinline__ xv3 x_add(xv3 a, xv3 b) { return mk(x_add(a.x, b.x), x_add(a.y, b.y), x_add(a.z, b.z)); }
__device__ __forceinline__ xv3 x_scale(xv3 a, float s) { return mk(x_mul(a.x, s), x_mul(a.y, s), x_mul(a.z, s)); }
// Vec4::dot / Dot: (x*x' + y*y') + z*z'  (MyMath.h:118,142)
__device__ __forceinline__ float x_dot(xv3 a, xv3 b) {
    return x_add(x_add(x_mul(a.x, b.x), x_mul(a.y, b.y)), x_mul(a.z, b.z));
}
// Cross, MyMath.h:134-140
__device__ __forceinline__ xv3 x_cross(xv3 a, xv3 b) {
    return mk(x_sub(x_mul(a.y, b.z), x_mul(a.z, b.y)), x_sub(x_mul(a.z, b.x), x_mul(a.x, b.z)),
              x_sub(x_mul(a.x, b.y), x_mul(a.y, b.x)));
}
__device__ __forceinline__ float comp(xv3 a, int ax) { return ax == 0 ? a.x : (ax == 1 ? a.y : a.z); }

// Ordered-int encoding of floats so atomicMin/atomicMax order them like
// floats (non-NaN inputs).
__device__ __forceinline__ int f2o(float f) {
    int i = __float_as_int(f);
    return i ^ ((i >> 31) & 0x7FFFFFFF);
}
__device__ __forceinline__ float o2f(int i) { return __int_as_float(i ^ ((i >> 31) & 0x7FFFFFFF)); }

// ---- slab test, AABB::rayAABB (Geometry.h:175-192), exact ---------------
__device__ __forceinline__ bool ray_box(float bminx, float bminy, float bminz, float bmaxx, float bmaxy,
                                        float bmaxz, const xv3& o, const xv3& inv, float& t) {
    float t0x = x_mul(x_sub(bminx, o.x), inv.x);
    float t0y = x_mul(x_sub(bminy, o.y), inv.y);
    float t0z = x_mul(x_sub(bminz, o.z), inv.z);
    float t1x = x_mul(x_sub(bmaxx, o.x), inv.x);
    float t1y = x_mul(x_sub(bmaxy, o.y), inv.y);
    float t1z = x_mul(x_sub(bmaxz, o.z), inv.z);
    float enx = s_min(t0x, t1x), eny = s_min(t0y, t1y), enz = s_min(t0z, t1z);
    float exx = s_max(t0x, t1x), exy = s_max(t0y, t1y), exz = s_max(t0z, t1z);
    float fen = s_max(enx, s_max(eny, enz));
    float fex = s_min(exx, s_min(exy, exz));
    if (fen > fex || fex < 0.f) return false;
    t = s_max(0.f, fen);
    return true;
}

// Same test for rays whose inverse direction is finite in every component.
// Then no slab bound is NaN (a finite difference times a finite inverse), so
// the hardware min/max (which differ from std::min/std::max only for NaN
// operands and in the sign of a zero result) give the same accept/reject
// decision; the entry distance may differ from the exact version only in the
// sign of a zero, which compares equal everywhere it is used.
__device__ __forceinline__ bool ray_box_finite(float bminx, float bminy, float bminz, float bmaxx, float bmaxy,
                                               float bmaxz, const xv3& o, const xv3& inv, float& t) {
    float t0x = x_mul(x_sub(bminx, o.x), inv.x);
    float t0y = x_mul(x_sub(bminy, o.y), inv.y);
    float t0z = x_mul(x_sub(bminz, o.z), inv.z);
    float t1x = x_mul(x_sub(bmaxx, o.x), inv.x);
    float t1y = x_mul(x_sub(bmaxy, o.y), inv.y);
    float t1z = x_mul(x_sub(bmaxz, o.z), inv.z);
    float fen = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z));
    float fex = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
    if (fen > fex || fex < 0.f) return false;
    t = fmaxf(0.f, fen);
    return true;
}

// ---- Möller–Trumbore, Triangle::rayIntersect (Geometry.h:101-130), exact --
// e0 = v1 - v0 and e1 = v2 - v0 are precomputed with the same subtraction the
// reference performs per call.
__device__ __forceinline__ bool ray_tri(const xv3& v0, const xv3& e0, const xv3& e1, const xv3& o, const xv3& d,
                                        float& t, float& u, float& v) {
    xv3 p = x_cross(d, e1);
    float det = x_dot(e0, p);
    if (fabsf(det) < PGX_MT_EPSILON) return false;
    float inv_det = x_div(1.f, det);
    xv3 T = x_sub(o, v0);
    u = x_mul(x_dot(T, p), inv_det);
    if (u < 0.f || u > 1.f) return false;
    xv3 q = x_cross(T, e0);
    v = x_mul(x_dot(d, q), inv_det);
    if (v < 0.f || v > 1.f || (x_add(u, v) > 1.f)) return false;
    t = x_mul(x_dot(e1, q), inv_det);
    return t >= 0.f;
}

// ---- traversal layout ----------------------------------------------------
// One 64-byte record per interior node of the binary tree, holding both
// children's boxes so one visit costs four 16-byte loads:
//   lmin.xyz/lmax.xyz  left child box,  lmin.w = ref, lmax.w = count
//   rmin.xyz/rmax.xyz  right child box, rmin.w = ref, rmax.w = count
// count > 0: leaf with `count` triangles at positions [ref, ref+count) of
// the leaf-ordered triangle array; count == 0: interior, ref = record index.
struct __align__(16) TravNode {
    float4 lmin, lmax, rmin, rmax;
};
// Leaf-ordered triangle: v0 (w = original triangle id bits), e0, e1, padded
// to 64 bytes so that v0 and e0 arrive in one 32-byte aligned 256-bit load
// (two load instructions per triangle test instead of three; the padding is
// never read).
struct __align__(16) TravTri {
    float4 v0, e0, e1, pad;
};
struct TravRoot {
    float bmin[3], bmax[3];
    int ref, count;  // as a child reference
    int valid;
};

struct TraceCounters {
    unsigned long long interior_visits;
    unsigned long long tri_tests;
    unsigned int overflow;
    unsigned int next;  // work counter of the persistent traversal
};

// ---- PCG32 stream (same definition as the oracle's pgx_oracle_rng.h) ------
#define PGX_PCG_MULT 6364136223846793005ULL
#define PGX_PCG_INC 1442695040888963407ULL

__host__ __device__ __forceinline__ uint64_t pgx_splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}
__host__ __device__ __forceinline__ uint64_t pgx_rng_init(uint64_t seed, uint64_t pixel, uint64_t sample) {
    uint64_t key = pgx_splitmix64(pgx_splitmix64(pgx_splitmix64(seed) ^ pixel) ^ sample);
    uint64_t state = PGX_PCG_INC + key;
    return state * PGX_PCG_MULT + PGX_PCG_INC;
}
__host__ __device__ __forceinline__ float pgx_rng_next(uint64_t& state) {
    uint64_t old = state;
    state = old * PGX_PCG_MULT + PGX_PCG_INC;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    uint32_t r = (xs >> rot) | (xs << ((0u - rot) & 31u));
    return (float)(r >> 8) * (1.0f / 16777216.0f);
}

// ---- generic helpers -------------------------------------------------------
__device__ __forceinline__ unsigned warp_aggregated_add(unsigned* counter, bool pred) {
    unsigned mask = __ballot_sync(__activemask(), pred);
    if (!pred) return 0xFFFFFFFFu;
    int leader = __ffs(mask) - 1;
    unsigned base = 0;
    int lane = threadIdx.x & 31;
    if (lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}
