// Scene upload: Scene::init + the non-BVH half of Scene::build (Scene.h:84-137),
// the camera set-up of loadScene (SceneLoader.h:226-243) and the
// environment-map sampling tables (Distribution2D, Sampling.h:166-189).
#include <cmath>
#include <cstring>
#include <vector>

#include "pgx_ctx.h"

namespace {

// ---- host 4x4 matrix, restating Matrix (MyMath.h:151-404) ------------------
struct HMat {
    float m[16];
};
HMat hm_identity() {
    HMat r;
    std::memset(r.m, 0, sizeof(r.m));
    r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.f;
    return r;
}
struct HV {
    float x, y, z;
};
float hv_len(HV a) { return sqrtf(((a.x * a.x) + (a.y * a.y)) + (a.z * a.z)); }
HV hv_norm(HV a) {
    float l = 1.f / hv_len(a);
    return HV{a.x * l, a.y * l, a.z * l};
}
HV hv_cross(HV a, HV b) {
    return HV{(a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x)};
}
float hv_dot(HV a, HV b) { return ((a.x * b.x) + (a.y * b.y)) + (a.z * b.z); }

// Matrix::invert (MESA unrolled inverse), MyMath.h:286-323.
HMat hm_invert(const HMat& M) {
    const float* m = M.m;
    HMat r;
    float* inv = r.m;
    inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] +
             m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
    inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] -
             m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
    inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] +
             m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
    inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] -
              m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
    inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] -
             m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
    inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] +
             m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
    inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] -
             m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
    inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] +
              m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
    inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] +
             m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
    inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] -
             m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
    inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] +
              m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
    inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] -
              m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
    inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] -
             m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
    inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] +
             m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
    inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] -
              m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
    inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] +
              m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
    float det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
    if (det == 0.f) det = 1.f;
    det = 1.f / det;
    for (int i = 0; i < 16; i++) inv[i] = inv[i] * det;
    return r;
}

// Matrix::lookAt, MyMath.h:325-348.
HMat hm_lookat(HV from, HV to, HV up) {
    HV dir = hv_norm(HV{from.x - to.x, from.y - to.y, from.z - to.z});
    HV left = hv_norm(hv_cross(up, dir));
    HV nup = hv_cross(dir, left);
    HMat r = hm_identity();
    r.m[0] = left.x;
    r.m[1] = left.y;
    r.m[2] = left.z;
    r.m[4] = nup.x;
    r.m[5] = nup.y;
    r.m[6] = nup.z;
    r.m[8] = dir.x;
    r.m[9] = dir.y;
    r.m[10] = dir.z;
    r.m[3] = -hv_dot(from, left);
    r.m[7] = -hv_dot(from, nup);
    r.m[11] = -hv_dot(from, dir);
    r.m[15] = 1.f;
    return r;
}

// Matrix::perspective, MyMath.h:350-364.
HMat hm_perspective(float n, float f, float aspect, float fov) {
    HMat r;
    std::memset(r.m, 0, sizeof(r.m));
    float t = 1.f / (tanf(fov * 0.5f * 3.141592654f / 180.f));
    float inv_fmn = 1.f / (f - n);
    r.m[0] = t / aspect;
    r.m[5] = t;
    r.m[10] = -f * inv_fmn;
    r.m[11] = -(f * n) * inv_fmn;
    r.m[14] = -1.f;
    return r;
}

float lum(float r, float g, float b) { return ((0.2126f * r) + (0.7152f * g)) + (0.0722f * b); }

// Triangle::init (Geometry.h:76-94) and gNormal (Geometry.h:153) per triangle.
__global__ void k_tri_setup(const pgx_triangle* __restrict__ tris, int64_t n, TriShade* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const pgx_triangle& t = tris[i];
    xv3 p0 = mk(t.v[0].p[0], t.v[0].p[1], t.v[0].p[2]);
    xv3 p1 = mk(t.v[1].p[0], t.v[1].p[1], t.v[1].p[2]);
    xv3 p2 = mk(t.v[2].p[0], t.v[2].p[1], t.v[2].p[2]);
    xv3 e1 = x_sub(p2, p1);
    xv3 e2 = x_sub(p0, p2);
    xv3 c = x_cross(e1, e2);
    float len = __fsqrt_rn(x_dot(c, c));
    float il = x_div(1.f, len);
    xv3 nrm = x_scale(c, il);
    float area = x_mul(len, 0.5f);
    xv3 vn0 = mk(t.v[0].n[0], t.v[0].n[1], t.v[0].n[2]);
    float sgn = (x_dot(vn0, nrm) > 0.f) ? 1.f : -1.f;
    TriShade s;
    s.n0 = make_float4(t.v[0].n[0], t.v[0].n[1], t.v[0].n[2], t.v[0].u);
    s.n1 = make_float4(t.v[1].n[0], t.v[1].n[1], t.v[1].n[2], t.v[1].u);
    s.n2 = make_float4(t.v[2].n[0], t.v[2].n[1], t.v[2].n[2], t.v[2].u);
    s.vv = make_float4(t.v[0].v, t.v[1].v, t.v[2].v, __int_as_float((int)t.material));
    s.gn = make_float4(x_mul(nrm.x, sgn), x_mul(nrm.y, sgn), x_mul(nrm.z, sgn), area);
    out[i] = s;
}

// Area-light table (Scene::build, Scene.h:92-100): emitting triangles in
// triangle order.
__global__ void k_lights(const pgx_triangle* __restrict__ tris, const TriShade* __restrict__ shade,
                         const int* __restrict__ light_tris, int nl, const DevMaterial* __restrict__ mats,
                         DevAreaLight* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nl) return;
    int ti = light_tris[i];
    const pgx_triangle& t = tris[ti];
    const TriShade& s = shade[ti];
    const DevMaterial& m = mats[t.material];
    DevAreaLight L;
    L.p0 = make_float4(t.v[0].p[0], t.v[0].p[1], t.v[0].p[2], s.gn.w);
    L.p1 = make_float4(t.v[1].p[0], t.v[1].p[1], t.v[1].p[2], __int_as_float(ti));
    L.p2 = make_float4(t.v[2].p[0], t.v[2].p[1], t.v[2].p[2], 0.f);
    L.gn = make_float4(s.gn.x, s.gn.y, s.gn.z, 0.f);
    L.emission = make_float4(m.emission[0], m.emission[1], m.emission[2], 0.f);
    out[i] = L;
}

// Distribution2D constructor (Sampling.h:171-189): one thread per row scans
// its conditional CDF sequentially, as Distribution1D's constructor does
// (Sampling.h:130-148), so the sums round identically.
__global__ void k_env_rows(const float* __restrict__ tex, int W, int H, float* __restrict__ func,
                           float* __restrict__ cdf, float* __restrict__ integ) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= H) return;
    float st = (float)sin(3.14159265358979323846 * (double)x_div(x_add((float)v, 0.5f), (float)H));
    const float* row = tex + (size_t)v * W * 3;
    float* f = func + (size_t)v * W;
    float* c = cdf + (size_t)v * (W + 1);
    for (int u = 0; u < W; u++) {
        float l = x_add(x_add(x_mul(0.2126f, row[3 * u]), x_mul(0.7152f, row[3 * u + 1])), x_mul(0.0722f, row[3 * u + 2]));
        f[u] = x_mul(l, st);
    }
    c[0] = 0.f;
    for (int i = 1; i < W + 1; i++) c[i] = x_add(c[i - 1], x_div(f[i - 1], (float)W));
    float total = c[W];
    integ[v] = total;
    if (total == 0.f) {
        for (int i = 1; i < W + 1; i++) c[i] = x_div((float)i, (float)W);
    } else {
        for (int i = 1; i < W + 1; i++) c[i] = x_div(c[i], total);
    }
}

__global__ void k_env_marginal(const float* __restrict__ integ, int H, float* __restrict__ func,
                               float* __restrict__ cdf, float* __restrict__ total_out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int v = 0; v < H; v++) func[v] = integ[v];
    cdf[0] = 0.f;
    for (int i = 1; i < H + 1; i++) cdf[i] = x_add(cdf[i - 1], x_div(func[i - 1], (float)H));
    float total = cdf[H];
    *total_out = total;
    if (total == 0.f) {
        for (int i = 1; i < H + 1; i++) cdf[i] = x_div((float)i, (float)H);
    } else {
        for (int i = 1; i < H + 1; i++) cdf[i] = x_div(cdf[i], total);
    }
}

// Guide table of one CDF (`size` entries, K buckets of cdf_bucket):
// g[k] = the first index whose bucket is >= k, g[K] = size.  *unsorted is
// set when the CDF decreases or holds a NaN (negative texels): the sampler
// then keeps the full binary search.
__device__ void build_cdf_guide(const float* __restrict__ cdf, int size, int K, int* __restrict__ g, int* unsorted) {
    int last = -1;
    float prev = -FLT_MAX;
    for (int i = 0; i < size; i++) {
        const float c = cdf[i];
        if (!(c >= prev)) *unsorted = 1;
        prev = c;
        const int b = cdf_bucket(c, K);
        for (int k = last + 1; k <= b; k++) g[k] = i;
        last = b > last ? b : last;
    }
    for (int k = last + 1; k <= K; k++) g[k] = size;
}

__global__ void k_env_row_guides(const float* __restrict__ cdf, int W, int H, int* __restrict__ guide, int* unsorted) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= H) return;
    build_cdf_guide(cdf + (size_t)v * (W + 1), W + 1, W, guide + (size_t)v * (W + 1), unsorted);
}

__global__ void k_env_marginal_guide(const float* __restrict__ cdf, int H, int* __restrict__ guide, int* unsorted) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    build_cdf_guide(cdf, H + 1, H, guide, unsorted);
}

inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

int camera_setup(pgx_ctx* ctx, const pgx_camera* camera);

extern "C" int pgx_scene_upload(pgx_ctx* ctx, const pgx_triangle* tris, int64_t ntris, const pgx_material* mats,
                                int32_t nmats, const pgx_texture* textures, int32_t ntextures,
                                const pgx_texture* envmap, const pgx_camera* camera) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (ntris < 0 || nmats < 0 || ntextures < 0)
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_scene_upload: negative count");
    if ((ntris > 0 && !tris) || (nmats > 0 && !mats) || (ntextures > 0 && !textures) || !camera)
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_scene_upload: null pointer");
    if (ntris > (int64_t)INT32_MAX / 2) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_scene_upload: too many triangles");
    if (camera->width <= 0 || camera->height <= 0)
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_scene_upload: bad image size");
    for (int64_t i = 0; i < ntris; i++)
        if (tris[i].material >= (uint32_t)nmats)
            return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_scene_upload: triangle %lld has material %u of %d",
                            (long long)i, tris[i].material, nmats);
    for (int32_t t = 0; t < ntextures; t++)
        if (textures[t].width <= 0 || textures[t].height <= 0 || !textures[t].rgb)
            return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_scene_upload: texture %d invalid", t);
    for (int32_t i = 0; i < nmats; i++) {
        if (mats[i].kind < PGX_BSDF_DIFFUSE || mats[i].kind > PGX_BSDF_PLASTIC)
            return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_scene_upload: material %d has unknown kind %d", i,
                            mats[i].kind);
        if (mats[i].albedo_texture >= ntextures || mats[i].albedo_texture < -1)
            return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_scene_upload: material %d texture out of range", i);
    }
    if (envmap && (envmap->width <= 0 || envmap->height <= 0 || !envmap->rgb))
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_scene_upload: invalid environment map");

    cudaStream_t s = ctx->stream;
    ctx->has_scene = false;
    ctx->has_bvh = false;
    ctx->ntris = ntris;
    ctx->nmats = nmats;
    ctx->host_mats.assign(mats, mats + nmats);

    // Texture pool: uploaded textures first, then one 1x1 texture per
    // material with a constant albedo.
    std::vector<DevTexture> tex_info;
    std::vector<float> pool;
    for (int32_t t = 0; t < ntextures; t++) {
        DevTexture d{textures[t].width, textures[t].height, (long long)(pool.size() / 3)};
        pool.insert(pool.end(), textures[t].rgb, textures[t].rgb + (size_t)textures[t].width * textures[t].height * 3);
        tex_info.push_back(d);
    }
    std::vector<DevMaterial> dm((size_t)nmats);
    for (int32_t i = 0; i < nmats; i++) {
        const pgx_material& m = mats[i];
        DevMaterial& d = dm[(size_t)i];
        d.kind = m.kind;
        d.layered = m.layered;
        if (m.albedo_texture >= 0) {
            d.tex = m.albedo_texture;
        } else {
            d.tex = (int)tex_info.size();
            tex_info.push_back(DevTexture{1, 1, (long long)(pool.size() / 3)});
            pool.push_back(m.albedo[0]);
            pool.push_back(m.albedo[1]);
            pool.push_back(m.albedo[2]);
        }
        for (int k = 0; k < 3; k++) {
            d.eta[k] = m.eta[k];
            d.k[k] = m.k[k];
            d.emission[k] = m.emission[k];
        }
        d.int_ior = m.int_ior;
        d.ext_ior = m.ext_ior;
        d.alpha = 1.62142f * sqrtf(m.roughness);
        d.sigma = m.sigma;
        d.is_light = lum(m.emission[0], m.emission[1], m.emission[2]) > 0.f ? 1 : 0;
    }
    if (tex_info.empty()) {
        tex_info.push_back(DevTexture{1, 1, 0});
        pool.assign({1.f, 1.f, 1.f});
    }
    PGX_CUDA_TRY(ctx, ctx->textures.reserve(sizeof(DevTexture) * tex_info.size()));
    PGX_CUDA_TRY(ctx, ctx->texels.reserve(sizeof(float) * pool.size()));
    ctx->ntex = (int32_t)tex_info.size();
    ctx->ntexels = (int64_t)(pool.size() / 3);
    PGX_CUDA_TRY(ctx, ctx->mats.reserve(sizeof(DevMaterial) * std::max<size_t>(dm.size(), 1)));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->textures.p, tex_info.data(), sizeof(DevTexture) * tex_info.size(),
                                      cudaMemcpyHostToDevice, s));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->texels.p, pool.data(), sizeof(float) * pool.size(), cudaMemcpyHostToDevice, s));
    if (!dm.empty())
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->mats.p, dm.data(), sizeof(DevMaterial) * dm.size(),
                                          cudaMemcpyHostToDevice, s));

    // Triangles and per-triangle shading data.
    PGX_CUDA_TRY(ctx, ctx->tris_in.reserve(sizeof(pgx_triangle) * std::max<int64_t>(ntris, 1)));
    PGX_CUDA_TRY(ctx, ctx->shade.reserve(sizeof(TriShade) * std::max<int64_t>(ntris, 1)));
    if (ntris > 0) {
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->tris_in.p, tris, sizeof(pgx_triangle) * ntris, cudaMemcpyHostToDevice, s));
        k_tri_setup<<<blocks_for(ntris, 256), 256, 0, s>>>(ctx->tris_in.as<pgx_triangle>(), ntris,
                                                           ctx->shade.as<TriShade>());
        PGX_CUDA_TRY(ctx, cudaGetLastError());
    }
    PGX_CUDA_TRY(ctx, ctx->tri_class.reserve(std::max<int64_t>(ntris, 1)));
    if (ntris > 0) {
        std::vector<unsigned char> cls((size_t)ntris);
        for (int64_t i = 0; i < ntris; i++) cls[(size_t)i] = shade_class(dm[tris[i].material]);
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->tri_class.p, cls.data(), (size_t)ntris, cudaMemcpyHostToDevice, s));
        PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    }

    // Scene bounds (Scene::init Scene.h:130-135; SceneLoader.h:267-268).
    float bmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, bmx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int64_t i = 0; i < ntris; i++)
        for (int v = 0; v < 3; v++)
            for (int k = 0; k < 3; k++) {
                float p = tris[i].v[v].p[k];
                bmx[k] = s_max(bmx[k], p);
                bmn[k] = s_min(bmn[k], p);
            }
    SceneBoundsDev& sb = ctx->bounds;
    for (int k = 0; k < 3; k++) {
        sb.bmin[k] = bmn[k];
        sb.bmax[k] = bmx[k];
        sb.centre[k] = (bmx[k] + bmn[k]) * 0.5f;
    }
    sb.radius = hv_len(HV{bmx[0] - sb.centre[0], bmx[1] - sb.centre[1], bmx[2] - sb.centre[2]});

    // Environment map and its sampling tables.
    ctx->env = DevEnv{};
    if (envmap) {
        int W = envmap->width, H = envmap->height;
        size_t nt = (size_t)W * H;
        PGX_CUDA_TRY(ctx, ctx->env_texels.reserve(sizeof(float) * nt * 3));
        PGX_CUDA_TRY(ctx, ctx->env_cond_func.reserve(sizeof(float) * nt));
        PGX_CUDA_TRY(ctx, ctx->env_cond_cdf.reserve(sizeof(float) * (size_t)H * (W + 1)));
        PGX_CUDA_TRY(ctx, ctx->env_cond_int.reserve(sizeof(float) * H));
        PGX_CUDA_TRY(ctx, ctx->env_marg_func.reserve(sizeof(float) * H));
        PGX_CUDA_TRY(ctx, ctx->env_marg_cdf.reserve(sizeof(float) * (H + 1) + sizeof(float)));
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->env_texels.p, envmap->rgb, sizeof(float) * nt * 3,
                                          cudaMemcpyHostToDevice, s));
        k_env_rows<<<blocks_for(H, 64), 64, 0, s>>>(ctx->env_texels.as<float>(), W, H, ctx->env_cond_func.as<float>(),
                                                     ctx->env_cond_cdf.as<float>(), ctx->env_cond_int.as<float>());
        float* total_dev = ctx->env_marg_cdf.as<float>() + (H + 1);
        k_env_marginal<<<1, 32, 0, s>>>(ctx->env_cond_int.as<float>(), H, ctx->env_marg_func.as<float>(),
                                        ctx->env_marg_cdf.as<float>(), total_dev);
        // Guide tables of the row and marginal CDFs (sampling only; the
        // indices they give are the binary search's).
        PGX_CUDA_TRY(ctx, ctx->env_cond_guide.reserve(sizeof(int) * (size_t)H * (W + 1)));
        PGX_CUDA_TRY(ctx, ctx->env_marg_guide.reserve(sizeof(int) * (H + 2)));
        int* unsorted_dev = ctx->env_marg_guide.as<int>() + (H + 1);
        PGX_CUDA_TRY(ctx, cudaMemsetAsync(unsorted_dev, 0, sizeof(int), s));
        k_env_row_guides<<<blocks_for(H, 64), 64, 0, s>>>(ctx->env_cond_cdf.as<float>(), W, H,
                                                          ctx->env_cond_guide.as<int>(), unsorted_dev);
        k_env_marginal_guide<<<1, 32, 0, s>>>(ctx->env_marg_cdf.as<float>(), H, ctx->env_marg_guide.as<int>(),
                                              unsorted_dev);
        PGX_CUDA_TRY(ctx, cudaGetLastError());
        float marg_int = 0.f;
        int unsorted = 0;
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&marg_int, total_dev, sizeof(float), cudaMemcpyDeviceToHost, s));
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&unsorted, unsorted_dev, sizeof(int), cudaMemcpyDeviceToHost, s));
        PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
        // EnvironmentMap::totalIntegratedPower, Lights.h:200-210 (sequential sum).
        float total = 0.f;
        for (int i = 0; i < H; i++) {
            float st = sinf((float)(((double)((float)i / (float)H)) * 3.14159265358979323846));
            for (int nn = 0; nn < W; nn++) {
                const float* t = envmap->rgb + ((size_t)i * W + nn) * 3;
                total += (lum(t[0], t[1], t[2]) * st);
            }
        }
        total = total / (float)(W * H);
        total = (float)((double)total * 4.0 * 3.14159265358979323846);
        DevEnv& e = ctx->env;
        e.valid = 1;
        e.width = W;
        e.height = H;
        e.texels = ctx->env_texels.as<float>();
        e.cond_func = ctx->env_cond_func.as<float>();
        e.cond_cdf = ctx->env_cond_cdf.as<float>();
        e.cond_int = ctx->env_cond_int.as<float>();
        e.marg_func = ctx->env_marg_func.as<float>();
        e.marg_cdf = ctx->env_marg_cdf.as<float>();
        e.marg_int = marg_int;
        e.power = total;
        e.cond_guide = unsorted ? nullptr : ctx->env_cond_guide.as<int>();
        e.marg_guide = unsorted ? nullptr : ctx->env_marg_guide.as<int>();
    }

    // Light list: the environment first when it has power (Scene::init,
    // Scene.h:133-136), then emitting triangles in order (Scene::build).
    std::vector<int> light_tris;
    for (int64_t i = 0; i < ntris; i++)
        if (dm[tris[i].material].is_light) light_tris.push_back((int)i);
    ctx->n_area_lights = (int32_t)light_tris.size();
    ctx->nlights = ctx->n_area_lights + ((ctx->env.valid && ctx->env.power > 0.f) ? 1 : 0);
    PGX_CUDA_TRY(ctx, ctx->lights.reserve(sizeof(DevAreaLight) * std::max<size_t>(light_tris.size(), 1)));
    if (!light_tris.empty()) {
        DevBuf lt;
        PGX_CUDA_TRY(ctx, lt.reserve(sizeof(int) * light_tris.size()));
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(lt.p, light_tris.data(), sizeof(int) * light_tris.size(),
                                          cudaMemcpyHostToDevice, s));
        k_lights<<<blocks_for((int64_t)light_tris.size(), 128), 128, 0, s>>>(
            ctx->tris_in.as<pgx_triangle>(), ctx->shade.as<TriShade>(), lt.as<int>(), (int)light_tris.size(),
            ctx->mats.as<DevMaterial>(), ctx->lights.as<DevAreaLight>());
        PGX_CUDA_TRY(ctx, cudaGetLastError());
        PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    }

    PGX_TRY(camera_setup(ctx, camera));
    ctx->has_scene = true;
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return PGX_OK;
}

// Camera (loadScene, SceneLoader.h:226-243; Camera::init/updateView,
// Scene.h:25-43).
int camera_setup(pgx_ctx* ctx, const pgx_camera* camera) {
    const pgx_camera& c = *camera;
    if (c.width <= 0 || c.height <= 0) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "camera: bad image size");
    ctx->host_camera = c;
    HMat P = hm_perspective(0.001f, 10000.0f, (float)c.width / (float)c.height, c.fov_degrees);
    HMat V = hm_invert(hm_lookat(HV{c.from[0], c.from[1], c.from[2]}, HV{c.to[0], c.to[1], c.to[2]},
                                 HV{c.up[0], c.up[1], c.up[2]}));
    if (c.flip_x == 1) P.m[0] = -P.m[0];
    HMat IP = hm_invert(P);
    DevCamera& dc = ctx->camera;
    std::memcpy(dc.inv_proj, IP.m, sizeof(dc.inv_proj));
    std::memcpy(dc.cam, V.m, sizeof(dc.cam));
    dc.origin[0] = ((0.f * V.m[0] + 0.f * V.m[1]) + 0.f * V.m[2]) + V.m[3];
    dc.origin[1] = ((0.f * V.m[4] + 0.f * V.m[5]) + 0.f * V.m[6]) + V.m[7];
    dc.origin[2] = ((0.f * V.m[8] + 0.f * V.m[9]) + 0.f * V.m[10]) + V.m[11];
    dc.width = (float)c.width;
    dc.height = (float)c.height;
    ctx->width = c.width;
    ctx->height = c.height;
    return PGX_OK;
}
