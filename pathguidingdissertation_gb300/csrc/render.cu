// Wavefront renderer (placeholder until the integrator lands).
#include "pgx_ctx.h"

void render_state_free(pgx_ctx* ctx) { (void)ctx; }
void cache_state_free(pgx_ctx* ctx) { (void)ctx; }

extern "C" int pgx_render(pgx_ctx* ctx, const pgx_render_config* cfg, int32_t frames) {
    (void)cfg;
    (void)frames;
    return pgx_fail(ctx, PGX_ERR_STATE, "pgx_render: not built yet");
}
extern "C" int pgx_clear(pgx_ctx* ctx) { return pgx_fail(ctx, PGX_ERR_STATE, "not built yet"); }
extern "C" int pgx_get_spp(pgx_ctx* ctx, int32_t* spp) {
    (void)spp;
    return pgx_fail(ctx, PGX_ERR_STATE, "not built yet");
}
extern "C" int pgx_film_read(pgx_ctx* ctx, float* rgb, float* rgb2, int32_t* spp) {
    (void)rgb;
    (void)rgb2;
    (void)spp;
    return pgx_fail(ctx, PGX_ERR_STATE, "not built yet");
}
extern "C" int pgx_render_get_stats(pgx_ctx* ctx, pgx_render_stats* out) {
    (void)out;
    return pgx_fail(ctx, PGX_ERR_STATE, "not built yet");
}
extern "C" int pgx_cache_build(pgx_ctx* ctx, const pgx_path_vertex* r, int64_t n) {
    (void)r;
    (void)n;
    return pgx_fail(ctx, PGX_ERR_STATE, "not built yet");
}
extern "C" int pgx_cache_build_from_render(pgx_ctx* ctx) { return pgx_fail(ctx, PGX_ERR_STATE, "not built yet"); }
extern "C" int pgx_cache_get_stats(pgx_ctx* ctx, pgx_cache_stats* out) {
    (void)out;
    return pgx_fail(ctx, PGX_ERR_STATE, "not built yet");
}
extern "C" int pgx_cache_export(pgx_ctx* ctx, pgx_cache_node* nodes, int64_t* nn, pgx_path_vertex* r, int64_t* nr) {
    (void)nodes;
    (void)nn;
    (void)r;
    (void)nr;
    return pgx_fail(ctx, PGX_ERR_STATE, "not built yet");
}
extern "C" int pgx_cache_knn(pgx_ctx* ctx, const float* q, int64_t nq, int32_t k, int32_t* idx, float* d2) {
    (void)q;
    (void)nq;
    (void)k;
    (void)idx;
    (void)d2;
    return pgx_fail(ctx, PGX_ERR_STATE, "not built yet");
}
