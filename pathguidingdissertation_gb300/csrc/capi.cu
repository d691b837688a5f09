// Context management, error reporting and the BVH entry points of the C ABI.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <functional>
#include <vector>

#include "pgx_ctx.h"

int pgx_fail(pgx_ctx* ctx, int code, const char* fmt, ...) {
    if (ctx) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->err = buf;
    }
    return code;
}

static thread_local std::string g_create_error;

extern "C" const char* pgx_version(void) { return "pgx 0.1 (sm_103a)"; }

extern "C" const char* pgx_last_error(const pgx_ctx* ctx) {
    if (!ctx) return g_create_error.c_str();
    return ctx->err.c_str();
}

int pgx_num_sms() {
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    if (dev >= 0 && dev < 64) {
        int v = cache[dev].load(std::memory_order_relaxed);
        if (v > 0) return v;
    }
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 1;
    if (dev >= 0 && dev < 64) cache[dev].store(v, std::memory_order_relaxed);
    return v;
}

extern "C" int pgx_create(int32_t device, pgx_ctx** out) {
    if (!out) return PGX_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        g_create_error = std::string("no CUDA device: ") + cudaGetErrorString(e);
        return PGX_ERR_CUDA;
    }
    if (device < 0 || device >= count) {
        g_create_error = "device ordinal out of range";
        return PGX_ERR_INVALID_ARG;
    }
    e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        g_create_error = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
        return PGX_ERR_CUDA;
    }
    pgx_ctx* ctx = new pgx_ctx();
    ctx->device = device;
    e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        g_create_error = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
        delete ctx;
        return PGX_ERR_CUDA;
    }
    *out = ctx;
    return PGX_OK;
}

extern "C" int pgx_destroy(pgx_ctx* ctx) {
    if (!ctx) return PGX_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    render_state_free(ctx);
    cache_state_free(ctx);
    mlp_state_free(ctx);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return PGX_OK;
}

extern "C" int pgx_bvh_build(pgx_ctx* ctx) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    PGX_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    return bvh_build_gpu(ctx);
}

extern "C" int pgx_bvh_import(pgx_ctx* ctx, const pgx_bvh_node* nodes, int64_t nnodes, const int32_t* tri_index) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    PGX_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    return bvh_import_ref(ctx, nodes, nnodes, tri_index);
}

extern "C" int pgx_bvh_export(pgx_ctx* ctx, pgx_bvh_node* nodes, int64_t* nnodes, int32_t* tri_index,
                              int64_t* ntri_index) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (!ctx->has_bvh) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_bvh_export: no BVH");
    if (nnodes) *nnodes = ctx->n_nodes;
    if (ntri_index) *ntri_index = ctx->ntris;
    cudaStream_t s = ctx->stream;
    if (nodes && ctx->n_nodes > 0)
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(nodes, ctx->bvh_nodes_ref.p, sizeof(pgx_bvh_node) * ctx->n_nodes,
                                          cudaMemcpyDeviceToHost, s));
    if (tri_index && ctx->ntris > 0)
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(tri_index, ctx->bvh_idx.p, sizeof(int32_t) * ctx->ntris,
                                          cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return PGX_OK;
}

extern "C" int pgx_bvh_get_stats(pgx_ctx* ctx, pgx_bvh_stats* out) {
    if (!ctx || !out) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (!ctx->has_bvh) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_bvh_get_stats: no BVH");
    *out = pgx_bvh_stats{};
    out->build_ms = ctx->bvh_build_ms;
    if (ctx->n_nodes == 0) return PGX_OK;
    std::vector<pgx_bvh_node> nodes((size_t)ctx->n_nodes);
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(nodes.data(), ctx->bvh_nodes_ref.p, sizeof(pgx_bvh_node) * nodes.size(),
                                      cudaMemcpyDeviceToHost, ctx->stream));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    auto area = [](const pgx_bvh_node& n) {
        double sx = (double)n.bmax[0] - n.bmin[0], sy = (double)n.bmax[1] - n.bmin[1], sz = (double)n.bmax[2] - n.bmin[2];
        return 2.0 * (sx * sy + sy * sz + sx * sz);
    };
    double root = area(nodes[0]);
    // Iterative walk from the root: only reachable nodes count.
    std::vector<std::pair<int64_t, int>> st;
    st.push_back({0, 0});
    double cost = 0.0;
    while (!st.empty()) {
        auto [i, depth] = st.back();
        st.pop_back();
        const pgx_bvh_node& n = nodes[(size_t)i];
        out->nodes++;
        if (depth > out->max_depth) out->max_depth = depth;
        double a = root > 0 ? area(n) / root : 0.0;
        if (n.used > 0) {
            out->leaves++;
            if (n.used > out->max_leaf_size) out->max_leaf_size = n.used;
            cost += a * n.used * 1.5;
        } else {
            cost += a * 1.0;
            st.push_back({n.left_first + 1, depth + 1});
            st.push_back({n.left_first, depth + 1});
        }
    }
    out->sah_cost = cost;
    return PGX_OK;
}
