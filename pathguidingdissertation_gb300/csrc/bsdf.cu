// Batch BSDF queries: BSDF::sample with a fixed primary sample and
// BSDF::invert (Materials.h:121-134) for shading points given by a normal and
// an outgoing direction — the operations of primary-sample-space guiding and
// of the reference's inversion test (main.cpp:13-72).
#include <cmath>

#include "pgx_ctx.h"
#include "pgx_shade.cuh"

namespace {

struct BsdfBatch {
    DevMaterial m;
    float albedo[3];
};

// ShadingData for a test point: x = 0, sNormal = gNormal = n, frame from n.
__device__ Shading test_shading(const float* n, const float* wo) {
    Shading sd;
    sd.x = f3(0.f, 0.f, 0.f);
    sd.sn = f3(n[0], n[1], n[2]);
    sd.gn = sd.sn;
    sd.wo = f3(wo[0], wo[1], wo[2]);
    sd.tu = 0.f;
    sd.tv = 0.f;
    sd.t = 0.f;
    sd.mat = 0;
    sd.frame = frame_from(sd.sn);
    return sd;
}

__global__ void k_bsdf_sample(BsdfBatch b, const float* __restrict__ n, const float* __restrict__ wo,
                              const float* __restrict__ uv, int64_t count, float* __restrict__ wi_out,
                              float* __restrict__ f_out, float* __restrict__ pdf_out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    DevTexture tex{1, 1, 0};
    TexView tv{&tex, b.albedo};
    Shading sd = test_shading(n + 3 * i, wo + 3 * i);
    FixedSampler smp{uv[2 * i], uv[2 * i + 1], 0};
    F3 f;
    float pdf;
    F3 wi = bsdf_sample_s(b.m, tv, sd, smp, f, pdf);
    wi_out[3 * i] = wi.x;
    wi_out[3 * i + 1] = wi.y;
    wi_out[3 * i + 2] = wi.z;
    if (f_out) {
        f_out[3 * i] = f.x;
        f_out[3 * i + 1] = f.y;
        f_out[3 * i + 2] = f.z;
    }
    if (pdf_out) pdf_out[i] = pdf;
}

__global__ void k_bsdf_invert(BsdfBatch b, const float* __restrict__ n, const float* __restrict__ wo,
                              const float* __restrict__ wi, int64_t count, float* __restrict__ uv_out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    Shading sd = test_shading(n + 3 * i, wo + 3 * i);
    float u = 0.f, v = 0.f;
    bsdf_invert(b.m, sd, f3(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]), u, v);
    uv_out[2 * i] = u;
    uv_out[2 * i + 1] = v;
}

int make_batch(pgx_ctx* ctx, const pgx_material* mat, BsdfBatch& b) {
    if (!mat) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_bsdf_*: null material");
    if (mat->kind < PGX_BSDF_DIFFUSE || mat->kind > PGX_BSDF_PLASTIC)
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_bsdf_*: unknown BSDF kind %d", mat->kind);
    if (mat->albedo_texture != -1)
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_bsdf_*: only constant albedos (albedo_texture = -1)");
    DevMaterial& d = b.m;
    d.kind = mat->kind;
    d.tex = 0;
    d.layered = mat->layered;
    d.is_light = 0;
    for (int k = 0; k < 3; k++) {
        d.eta[k] = mat->eta[k];
        d.k[k] = mat->k[k];
        d.emission[k] = mat->emission[k];
        d.alb_off[k] = 0.f;
        b.albedo[k] = mat->albedo[k];
    }
    d.int_ior = mat->int_ior;
    d.ext_ior = mat->ext_ior;
    d.alpha = 1.62142f * sqrtf(mat->roughness);
    d.sigma = mat->sigma;
    return PGX_OK;
}

}  // namespace

extern "C" int pgx_bsdf_sample_batch(pgx_ctx* ctx, const pgx_material* mat, const float* normals, const float* wo,
                                     const float* uv, int64_t count, float* wi, float* f, float* pdf) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (count < 0 || (count > 0 && (!normals || !wo || !uv || !wi)))
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_bsdf_sample_batch: bad arguments");
    BsdfBatch b{};
    PGX_TRY(make_batch(ctx, mat, b));
    if (count == 0) return PGX_OK;
    cudaStream_t s = ctx->stream;
    DevBuf dn, dwo, duv, dwi, df, dp;
    PGX_CUDA_TRY(ctx, dn.reserve(sizeof(float) * 3 * count));
    PGX_CUDA_TRY(ctx, dwo.reserve(sizeof(float) * 3 * count));
    PGX_CUDA_TRY(ctx, duv.reserve(sizeof(float) * 2 * count));
    PGX_CUDA_TRY(ctx, dwi.reserve(sizeof(float) * 3 * count));
    PGX_CUDA_TRY(ctx, df.reserve(sizeof(float) * 3 * count));
    PGX_CUDA_TRY(ctx, dp.reserve(sizeof(float) * count));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(dn.p, normals, sizeof(float) * 3 * count, cudaMemcpyHostToDevice, s));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(dwo.p, wo, sizeof(float) * 3 * count, cudaMemcpyHostToDevice, s));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(duv.p, uv, sizeof(float) * 2 * count, cudaMemcpyHostToDevice, s));
    k_bsdf_sample<<<(unsigned)((count + 127) / 128), 128, 0, s>>>(b, dn.as<float>(), dwo.as<float>(), duv.as<float>(),
                                                                   count, dwi.as<float>(), df.as<float>(),
                                                                   dp.as<float>());
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(wi, dwi.p, sizeof(float) * 3 * count, cudaMemcpyDeviceToHost, s));
    if (f) PGX_CUDA_TRY(ctx, cudaMemcpyAsync(f, df.p, sizeof(float) * 3 * count, cudaMemcpyDeviceToHost, s));
    if (pdf) PGX_CUDA_TRY(ctx, cudaMemcpyAsync(pdf, dp.p, sizeof(float) * count, cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return PGX_OK;
}

extern "C" int pgx_bsdf_invert_batch(pgx_ctx* ctx, const pgx_material* mat, const float* normals, const float* wo,
                                     const float* wi, int64_t count, float* uv) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (count < 0 || (count > 0 && (!normals || !wo || !wi || !uv)))
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_bsdf_invert_batch: bad arguments");
    BsdfBatch b{};
    PGX_TRY(make_batch(ctx, mat, b));
    if (count == 0) return PGX_OK;
    cudaStream_t s = ctx->stream;
    DevBuf dn, dwo, dwi, duv;
    PGX_CUDA_TRY(ctx, dn.reserve(sizeof(float) * 3 * count));
    PGX_CUDA_TRY(ctx, dwo.reserve(sizeof(float) * 3 * count));
    PGX_CUDA_TRY(ctx, dwi.reserve(sizeof(float) * 3 * count));
    PGX_CUDA_TRY(ctx, duv.reserve(sizeof(float) * 2 * count));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(dn.p, normals, sizeof(float) * 3 * count, cudaMemcpyHostToDevice, s));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(dwo.p, wo, sizeof(float) * 3 * count, cudaMemcpyHostToDevice, s));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(dwi.p, wi, sizeof(float) * 3 * count, cudaMemcpyHostToDevice, s));
    k_bsdf_invert<<<(unsigned)((count + 127) / 128), 128, 0, s>>>(b, dn.as<float>(), dwo.as<float>(), dwi.as<float>(),
                                                                   count, duv.as<float>());
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(uv, duv.p, sizeof(float) * 2 * count, cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return PGX_OK;
}
