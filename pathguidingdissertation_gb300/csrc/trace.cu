// Batch ray queries: pgx_trace_closest / pgx_trace_any (BVHNode::traverse and
// BVHNode::traverseVisible, Geometry.h:448-567) and camera rays
// (Camera::generateRay, Scene.h:253-265).
#include <algorithm>
#include <mutex>

#include "pgx_ctx.h"
#include "pgx_trace.cuh"

namespace {

constexpr int kTraceThreads = 128;

constexpr int kPersistentBlocksPerSM = 8;

// Persistent traversal of a ray batch: whole warps loop, refilling lanes
// from counters->next (see trace_persistent).
template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(kTraceThreads, kPersistentBlocksPerSM)
    k_trace(BvhView bvh, const pgx_ray* __restrict__ rays, int64_t n, pgx_hit* __restrict__ hits,
            uint8_t* __restrict__ visible, TraceCounters* __restrict__ counters) {
    unsigned long long ni = 0, nt = 0;
    unsigned status = 0;
    auto load = [&](unsigned i, xv3& o, xv3& d, float& tmax) {
        const float4* rp = reinterpret_cast<const float4*>(rays + i);
        float4 a = __ldg(rp), b = __ldg(rp + 1);
        o = mk(a.x, a.y, a.z);
        d = mk(b.x, b.y, b.z);
        tmax = a.w;
    };
    auto store = [&](unsigned i, const TraceLane& L) {
        if (ANY)
            visible[i] = (L.hit_id >= 0) ? 0 : 1;
        else
            reinterpret_cast<float4*>(hits)[i] = make_float4(__int_as_float(L.hit_id), L.tmax, L.hu, L.hv);
    };
    trace_persistent<ANY, COUNT>(bvh, (unsigned)n, &counters->next, load, store, ni, nt, status);
    if (COUNT) {
        for (int o = 16; o > 0; o >>= 1) {
            ni += __shfl_xor_sync(0xFFFFFFFFu, ni, o);
            nt += __shfl_xor_sync(0xFFFFFFFFu, nt, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&counters->interior_visits, ni);
            atomicAdd(&counters->tri_tests, nt);
        }
    }
    if (status) atomicOr(&counters->overflow, status);
}

unsigned persistent_grid(int64_t n) {
    int64_t blocks = (n + kTraceThreads - 1) / kTraceThreads;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)pgx_num_sms() * kPersistentBlocksPerSM));
}

// Camera::generateRay with exact arithmetic.
__global__ void k_camera_rays(DevCamera cam, const float* __restrict__ px, const float* __restrict__ py, int64_t n,
                              pgx_ray* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float x = px[i], y = py[i];
    float xc = x_sub(x_div(x_mul(2.f, x), cam.width), 1.f);
    float yc = x_sub(x_mul(2.f, x_sub(1.f, x_div(y, cam.height))), 1.f);
    const float* m = cam.inv_proj;
    float vx = x_add(x_add(x_add(x_mul(xc, m[0]), x_mul(yc, m[1])), x_mul(0.f, m[2])), m[3]);
    float vy = x_add(x_add(x_add(x_mul(xc, m[4]), x_mul(yc, m[5])), x_mul(0.f, m[6])), m[7]);
    float vz = x_add(x_add(x_add(x_mul(xc, m[8]), x_mul(yc, m[9])), x_mul(0.f, m[10])), m[11]);
    float w = x_add(x_add(x_add(x_mul(m[12], xc), x_mul(m[13], yc)), x_mul(m[14], 0.f)), m[15]);
    w = x_div(1.f, w);
    vx = x_mul(vx, w);
    vy = x_mul(vy, w);
    vz = x_mul(vz, w);
    const float* c = cam.cam;
    float dx = x_add(x_add(x_mul(vx, c[0]), x_mul(vy, c[1])), x_mul(vz, c[2]));
    float dy = x_add(x_add(x_mul(vx, c[4]), x_mul(vy, c[5])), x_mul(vz, c[6]));
    float dz = x_add(x_add(x_mul(vx, c[8]), x_mul(vy, c[9])), x_mul(vz, c[10]));
    float l = x_div(1.f, __fsqrt_rn(x_add(x_add(x_mul(dx, dx), x_mul(dy, dy)), x_mul(dz, dz))));
    pgx_ray r;
    r.o[0] = cam.origin[0];
    r.o[1] = cam.origin[1];
    r.o[2] = cam.origin[2];
    r.tmax = FLT_MAX;
    r.d[0] = x_mul(dx, l);
    r.d[1] = x_mul(dy, l);
    r.d[2] = x_mul(dz, l);
    r.pad = 0.f;
    out[i] = r;
}

int launch_trace(pgx_ctx* ctx, const pgx_ray* d_rays, int64_t n, pgx_hit* d_hits, uint8_t* d_vis, bool any,
                 cudaStream_t s) {
    PGX_CUDA_TRY(ctx, ctx->counters.reserve(sizeof(TraceCounters)));
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(ctx->counters.p, 0, sizeof(TraceCounters), s));
    if (n > 0) {
        if (n > (int64_t)UINT32_MAX) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "too many rays in one call");
        unsigned grid = persistent_grid(n);
        BvhView v = bvh_view(ctx);
        TraceCounters* c = ctx->counters.as<TraceCounters>();
        if (any)
            k_trace<true, true><<<grid, kTraceThreads, 0, s>>>(v, d_rays, n, nullptr, d_vis, c);
        else
            k_trace<false, true><<<grid, kTraceThreads, 0, s>>>(v, d_rays, n, d_hits, nullptr, c);
        PGX_CUDA_TRY(ctx, cudaGetLastError());
    }
    TraceCounters hc{};
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&hc, ctx->counters.p, sizeof(hc), cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    ctx->last_interior = hc.interior_visits;
    ctx->last_tris = hc.tri_tests;
    if (hc.overflow & 2u) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "traversal met a reference outside the BVH");
    if (hc.overflow) return pgx_fail(ctx, PGX_ERR_OVERFLOW, "traversal stack overflow (depth > %d)", PGX_STACK_SIZE);
    return PGX_OK;
}

int check_trace_args(pgx_ctx* ctx, const void* rays, int64_t n, const void* out) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (n < 0) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "negative ray count");
    if (n > 0 && (!rays || !out)) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "null ray or output pointer");
    if (!ctx->has_bvh) return pgx_fail(ctx, PGX_ERR_STATE, "no BVH: call pgx_bvh_build or pgx_bvh_import first");
    return PGX_OK;
}

int trace_host(pgx_ctx* ctx, const pgx_ray* rays, int64_t n, void* out, bool any) {
    PGX_TRY(check_trace_args(ctx, rays, n, out));
    if (n == 0) return launch_trace(ctx, nullptr, 0, nullptr, nullptr, any, ctx->stream);
    cudaStream_t s = ctx->stream;
    size_t out_bytes = any ? sizeof(uint8_t) * n : sizeof(pgx_hit) * n;
    PGX_CUDA_TRY(ctx, ctx->trace_rays.reserve(sizeof(pgx_ray) * n));
    PGX_CUDA_TRY(ctx, ctx->trace_out.reserve(out_bytes));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->trace_rays.p, rays, sizeof(pgx_ray) * n, cudaMemcpyHostToDevice, s));
    int st = launch_trace(ctx, ctx->trace_rays.as<pgx_ray>(), n, any ? nullptr : ctx->trace_out.as<pgx_hit>(),
                          any ? ctx->trace_out.as<uint8_t>() : nullptr, any, s);
    if (st != PGX_OK) return st;
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(out, ctx->trace_out.p, out_bytes, cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return PGX_OK;
}

}  // namespace

// ---- allocation-free batch query -------------------------------------------
// Fixed device scratch for pgx_trace_closest_noalloc: trace counters, then
// room for PGX_NOALLOC_MAX_RAYS rays and as many hits (3 MiB + 256 B).  It is
// a file-scope device array, so every GPU that loads libpgx holds it until
// the process exits, and all calls share it.
constexpr size_t kNoAllocCounterBytes = 256;
constexpr size_t kNoAllocRayBytes = sizeof(pgx_ray) * (size_t)PGX_NOALLOC_MAX_RAYS;
constexpr size_t kNoAllocHitBytes = sizeof(pgx_hit) * (size_t)PGX_NOALLOC_MAX_RAYS;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocCounterBytes + kNoAllocRayBytes +
                                                                 kNoAllocHitBytes];
static_assert(sizeof(TraceCounters) <= kNoAllocCounterBytes, "counters must fit their slot");

namespace {
constexpr int kMaxDevices = 256;
std::mutex g_noalloc_mutex;
unsigned char* g_noalloc_base[kMaxDevices] = {};

// Device address of the scratch on ctx's device.  In host code the array's
// name only stands in for the symbol, so its address must be asked for with
// the device current; it is looked up once per device and cached.
int noalloc_scratch(pgx_ctx* ctx, unsigned char** out) {
    if (ctx->device < 0 || ctx->device >= kMaxDevices)
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_trace_closest_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_base[ctx->device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return pgx_fail(ctx, PGX_ERR_CUDA, "pgx_trace_closest_noalloc: cudaGetSymbolAddress failed: %s",
                            cudaGetErrorString(e));
        g_noalloc_base[ctx->device] = static_cast<unsigned char*>(p);
    }
    *out = g_noalloc_base[ctx->device];
    return PGX_OK;
}
}  // namespace

extern "C" int pgx_trace_closest_noalloc(pgx_ctx* ctx, const pgx_ray* rays, int64_t n, pgx_hit* hits) {
    PGX_TRY(check_trace_args(ctx, rays, n, hits));
    if (n > PGX_NOALLOC_MAX_RAYS)
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG,
                        "pgx_trace_closest_noalloc: %lld rays exceed the fixed scratch of %d rays; split the batch",
                        (long long)n, PGX_NOALLOC_MAX_RAYS);
    PGX_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    unsigned char* base = nullptr;
    PGX_TRY(noalloc_scratch(ctx, &base));
    TraceCounters* counters = reinterpret_cast<TraceCounters*>(base);
    pgx_ray* d_rays = reinterpret_cast<pgx_ray*>(base + kNoAllocCounterBytes);
    pgx_hit* d_hits = reinterpret_cast<pgx_hit*>(base + kNoAllocCounterBytes + kNoAllocRayBytes);
    cudaStream_t s = ctx->stream;
    // The array keeps the previous call's contents: the counters must start at zero.
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(counters, 0, sizeof(TraceCounters), s));
    if (n > 0) {
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(d_rays, rays, sizeof(pgx_ray) * n, cudaMemcpyHostToDevice, s));
        k_trace<false, true><<<persistent_grid(n), kTraceThreads, 0, s>>>(bvh_view(ctx), d_rays, n, d_hits, nullptr,
                                                                          counters);
        PGX_CUDA_TRY(ctx, cudaGetLastError());
    }
    TraceCounters hc{};
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&hc, counters, sizeof(hc), cudaMemcpyDeviceToHost, s));
    if (n > 0) PGX_CUDA_TRY(ctx, cudaMemcpyAsync(hits, d_hits, sizeof(pgx_hit) * n, cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    ctx->last_interior = hc.interior_visits;
    ctx->last_tris = hc.tri_tests;
    if (hc.overflow & 2u) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "traversal met a reference outside the BVH");
    if (hc.overflow) return pgx_fail(ctx, PGX_ERR_OVERFLOW, "traversal stack overflow (depth > %d)", PGX_STACK_SIZE);
    return PGX_OK;
}

extern "C" int pgx_trace_closest(pgx_ctx* ctx, const pgx_ray* rays, int64_t n, pgx_hit* hits) {
    return trace_host(ctx, rays, n, hits, false);
}

extern "C" int pgx_trace_any(pgx_ctx* ctx, const pgx_ray* rays, int64_t n, uint8_t* visible) {
    return trace_host(ctx, rays, n, visible, true);
}

extern "C" int pgx_trace_closest_device(pgx_ctx* ctx, const pgx_ray* d_rays, int64_t n, pgx_hit* d_hits,
                                        void* stream) {
    PGX_TRY(check_trace_args(ctx, d_rays, n, d_hits));
    return launch_trace(ctx, d_rays, n, d_hits, nullptr, false, stream ? (cudaStream_t)stream : ctx->stream);
}

extern "C" int pgx_trace_any_device(pgx_ctx* ctx, const pgx_ray* d_rays, int64_t n, uint8_t* d_visible,
                                    void* stream) {
    PGX_TRY(check_trace_args(ctx, d_rays, n, d_visible));
    return launch_trace(ctx, d_rays, n, nullptr, d_visible, true, stream ? (cudaStream_t)stream : ctx->stream);
}

extern "C" int pgx_trace_counters(pgx_ctx* ctx, int64_t* nodes_visited, int64_t* tris_tested) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    if (nodes_visited) *nodes_visited = (int64_t)ctx->last_interior;
    if (tris_tested) *tris_tested = (int64_t)ctx->last_tris;
    return PGX_OK;
}

extern "C" int pgx_camera_rays(pgx_ctx* ctx, const float* px, const float* py, int64_t n, pgx_ray* rays) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (n < 0 || (n > 0 && (!px || !py || !rays))) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_camera_rays: bad args");
    if (!ctx->has_scene) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_camera_rays: no scene");
    if (n == 0) return PGX_OK;
    cudaStream_t s = ctx->stream;
    DevBuf dpx, dpy, dr;
    PGX_CUDA_TRY(ctx, dpx.reserve(sizeof(float) * n));
    PGX_CUDA_TRY(ctx, dpy.reserve(sizeof(float) * n));
    PGX_CUDA_TRY(ctx, dr.reserve(sizeof(pgx_ray) * n));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(dpx.p, px, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(dpy.p, py, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    k_camera_rays<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(ctx->camera, dpx.as<float>(), dpy.as<float>(), n,
                                                             dr.as<pgx_ray>());
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(rays, dr.p, sizeof(pgx_ray) * n, cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return PGX_OK;
}
