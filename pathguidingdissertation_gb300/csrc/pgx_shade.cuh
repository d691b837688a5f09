// Device restatement of the reference's shading: textures (Imaging.h:82-108),
// shading frames (MyMath.h:406-433), the BSDFs (Materials.h:34-897), area and
// environment lights (Lights.h:28-228) and the MIS power heuristic
// (MyMath.h:23-28).
//
// render.cu is compiled with -fmad=false, so every a*b+c below rounds twice
// like the reference's scalar code; where the reference promotes to double
// (M_PI and long literals) the expression is computed in float (see
// PGX_PI_F), within an ulp or two of the reference.  Random numbers
// are drawn in exactly the reference's order so a path driven by the same
// stream follows the same decisions.
#pragma once

#include "pgx_ctx.h"

#define PGX_PI_D 3.14159265358979323846
#define PGX_INV_PI_F 0.318309886183790671538f
// Single-precision forms of the reference's double-promoted pi expressions
// (M_PI * x, x / (2 M_PI), ...): the hot path computes them in float, within
// an ulp or two of the reference's double-then-float rounding, because FP64
// runs at a small fraction of the FP32 rate on this GPU.
#define PGX_PI_F 3.14159265358979323846f
#define PGX_2PI_F 6.28318530717958647692f
#define PGX_INV_2PI_F 0.159154943091895335769f
#define PGX_2PI2_F 19.7392088021787172376f

struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 f3(float4 v) { return F3{v.x, v.y, v.z}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ F3 operator*(F3 a, F3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ F3 operator*(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ F3 operator-(F3 a) { return f3(-a.x, -a.y, -a.z); }
// Vec4/Colour operator/(float): multiply by the reciprocal (MyMath.h:54-57,95-98).
__device__ __forceinline__ F3 divs(F3 a, float s) {
    float inv = 1.f / s;
    return f3(a.x * inv, a.y * inv, a.z * inv);
}
__device__ __forceinline__ F3 divc(F3 a, F3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
__device__ __forceinline__ float dot(F3 a, F3 b) { return ((a.x * b.x) + (a.y * b.y)) + (a.z * b.z); }
__device__ __forceinline__ F3 cross(F3 a, F3 b) {
    return f3((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x));
}
__device__ __forceinline__ float length_sq(F3 a) { return ((a.x * a.x) + (a.y * a.y)) + (a.z * a.z); }
__device__ __forceinline__ float length(F3 a) { return sqrtf(length_sq(a)); }
__device__ __forceinline__ F3 normalize(F3 a) {
    float l = 1.f / length(a);
    return f3(a.x * l, a.y * l, a.z * l);
}
__device__ __forceinline__ float lum(F3 c) { return ((0.2126f * c.x) + (0.7152f * c.y)) + (0.0722f * c.z); }
__device__ __forceinline__ bool valid(F3 c) {
    return !(isnan(c.x) || isnan(c.y) || isnan(c.z)) && !(isinf(c.x) || isinf(c.y) || isinf(c.z));
}
__device__ __forceinline__ F3 zero3() { return f3(0.f, 0.f, 0.f); }

// MIS power heuristic with beta = 2 (MyMath.h:23-28).
__device__ __forceinline__ float power_heuristic(float a, float b) {
    float a2 = a * a, b2 = b * b;
    if (a2 + b2 <= 0.f) return 0.f;
    return a2 / (a2 + b2);
}

// ---- Frame (MyMath.h:406-433) ------------------------------------------------
struct Frame {
    F3 u, v, w;
};
__device__ __forceinline__ Frame frame_from(F3 n) {
    Frame f;
    f.w = normalize(n);
    if (fabsf(f.w.x) > fabsf(f.w.y)) {
        float l = 1.f / sqrtf(f.w.x * f.w.x + f.w.z * f.w.z);
        f.u = f3(f.w.z * l, 0.f, -f.w.x * l);
    } else {
        float l = 1.f / sqrtf(f.w.y * f.w.y + f.w.z * f.w.z);
        f.u = f3(0.f, f.w.z * l, -f.w.y * l);
    }
    f.v = cross(f.w, f.u);
    return f;
}
__device__ __forceinline__ F3 to_local(const Frame& f, F3 a) { return f3(dot(a, f.u), dot(a, f.v), dot(a, f.w)); }
__device__ __forceinline__ F3 to_world(const Frame& f, F3 a) { return ((f.u * a.x) + (f.v * a.y)) + (f.w * a.z); }

// SphericalCoordinates (MyMath.h:435-449).
__device__ __forceinline__ F3 spherical_to_world(float theta, float phi) {
    return f3(cosf(phi) * sinf(theta), sinf(phi) * sinf(theta), cosf(theta));
}
__device__ __forceinline__ float spherical_phi(F3 w) {
    float p = atan2f(w.y, w.x);
    return (p < 0.f) ? p + PGX_2PI_F : p;
}

// ---- shading data (ShadingData, Materials.h:12-32) -----------------------------
struct Shading {
    F3 x, wo, sn, gn;
    float tu, tv, t;
    Frame frame;
    int mat;
};

// ---- textures (Texture::sample, Imaging.h:82-108) ---------------------------
struct TexView {
    const DevTexture* info;
    const float* texels;
};
__device__ __forceinline__ F3 texel(const float* p, long long i) { return f3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
__device__ __forceinline__ int wrap_index(int a, int n) {
    int r = a % n;
    return (r < 0 || r >= n) ? 0 : r;  // the reference relies on in-range values; keep reads in bounds
}
static __device__ F3 tex_sample_raw(const float* texels, long long offset, int W, int H, float tu, float tv) {
    float u = fmaxf(0.f, fabsf(tu)) * (float)W;
    float v = fmaxf(0.f, fabsf(tv)) * (float)H;
    float fu = floorf(u), fv = floorf(v);
    int x = (fu >= -2147483648.f && fu < 2147483648.f) ? (int)fu : 0;
    int y = (fv >= -2147483648.f && fv < 2147483648.f) ? (int)fv : 0;
    float frac_u = u - (float)x;
    float frac_v = v - (float)y;
    float w0 = (1.f - frac_u) * (1.f - frac_v);
    float w1 = frac_u * (1.f - frac_v);
    float w2 = (1.f - frac_u) * frac_v;
    float w3 = frac_u * frac_v;
    x = wrap_index(x, W);
    y = wrap_index(y, H);
    int x1 = wrap_index(x + 1, W), y1 = wrap_index(y + 1, H);
    const float* p = texels + 3 * offset;
    F3 s0 = texel(p, (long long)y * W + x);
    F3 s1 = texel(p, (long long)y * W + x1);
    F3 s2 = texel(p, (long long)y1 * W + x);
    F3 s3 = texel(p, (long long)y1 * W + x1);
    return (((s0 * w0) + (s1 * w1)) + (s2 * w2)) + (s3 * w3);
}
__device__ __forceinline__ F3 albedo_of(const TexView& tv, const DevMaterial& m, const Shading& sd) {
    DevTexture t = tv.info[m.tex];
    F3 a = tex_sample_raw(tv.texels, t.offset, t.width, t.height, sd.tu, sd.tv);
    return f3(a.x + m.alb_off[0], a.y + m.alb_off[1], a.z + m.alb_off[2]);
}

// ---- Fresnel and GGX (ShadingHelper, Materials.h:34-119) ---------------------
static __device__ float fresnel_dielectric(float cos_theta, float ior_int, float ior_ext) {
    float ci = s_max(s_min(cos_theta, 1.f), -1.f);
    float eta = (ci < 0.f) ? (ior_int / ior_ext) : (ior_ext / ior_int);
    if (ci < 0.f) ci = fabsf(ci);
    float eta_sq = eta * eta;
    float ci_sq = s_max(ci * ci, 0.f);
    float si_sq = s_max(1.f - ci_sq, 0.f);
    float st_sq = eta_sq * si_sq;
    if (st_sq > 1.f) return 1.f;
    float ct = sqrtf(s_max(1.f - st_sq, 0.f));
    float par = (ci - eta * ct) / (ci + eta * ct);
    float perp = (eta * ci - ct) / (eta * ci + ct);
    return (par * par + perp * perp) * 0.5f;
}

// Each BSDF routine below has a force-inlined core (suffix _i, or a template
// on the material kind K) and an out-of-line entry point of the original name
// for the generic shading path.  A wavefront launch that shades a single
// surface class instantiates the cores with its kind known at compile time:
// the other kinds' code disappears and no material, shading frame or scene
// view has to be spilled to local memory to be passed by reference.
__device__ __forceinline__ F3 fresnel_conductor_i(float cos_theta, const float* ior, const float* k) {
    float ci = s_max(s_min(cos_theta, 1.f), -1.f);
    float ci_sq = s_max(ci * ci, 0.f);
    float si_sq = s_max(1.f - ci_sq, 0.f);
    F3 out;
    float* o = &out.x;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float n2 = ior[c] * ior[c];
        float k2 = k[c] * k[c];
        float two_n_ci = (ior[c] * ci) * 2.f;
        float par = ((((n2 + k2) * ci_sq) - two_n_ci) + si_sq) / ((((n2 + k2) * ci_sq) + two_n_ci) + si_sq);
        float perp = (((n2 + k2) - two_n_ci) + ci_sq) / (((n2 + k2) + two_n_ci) + ci_sq);
        o[c] = (par + perp) * 0.5f;
    }
    return out;
}
static __device__ __noinline__ F3 fresnel_conductor(float cos_theta, const float* ior, const float* k) {
    return fresnel_conductor_i(cos_theta, ior, k);
}
template <int K>
__device__ __forceinline__ F3 fresnel_conductor_k(float cos_theta, const float* ior, const float* k) {
    if constexpr (K < 0)
        return fresnel_conductor(cos_theta, ior, k);
    else
        return fresnel_conductor_i(cos_theta, ior, k);
}

__device__ __forceinline__ float lambda_ggx(F3 wi, float alpha) {
    if (wi.z <= 0.f) return 0.f;
    float a2 = alpha * alpha;
    float c2 = wi.z * wi.z;
    float s2 = s_max(1.f - c2, 0.f);
    float t2 = fabsf(s2 / c2);
    return (sqrtf(1.f + a2 * t2) - 1.f) * 0.5f;
}
__device__ __forceinline__ float g_ggx(F3 wi, F3 wo, float alpha) {
    float g1o = 1.f / (1.f + lambda_ggx(wo, alpha));
    float g1i = 1.f / (1.f + lambda_ggx(wi, alpha));
    return g1o * g1i;
}
__device__ __forceinline__ float d_ggx(F3 h, float alpha) {
    if (h.z <= 0.f) return 0.f;
    float a2 = alpha * alpha;
    float c2 = h.z * h.z;
    float t = c2 * (a2 - 1.f) + 1.f;
    float den = (PGX_PI_F * t) * t;
    if (den <= 0.f) return 0.f;
    return a2 / den;
}

// GGX half-vector sample (Materials.h:274-278).
__device__ __forceinline__ F3 ggx_sample_h(float alpha, float r1, float r2) {
    float a2 = alpha * alpha;
    float theta = acosf(sqrtf((1.f - r1) / (r1 * (a2 - 1.f) + 1.f)));
    float phi = PGX_2PI_F * r2;
    return spherical_to_world(theta, phi);
}

// Cosine hemisphere sample / pdf (Sampling.h:92-101).
__device__ __forceinline__ F3 cosine_sample(float r1, float r2) {
    float theta = acosf(sqrtf(r1));
    float phi = PGX_2PI_F * r2;
    return spherical_to_world(theta, phi);
}
__device__ __forceinline__ float cosine_pdf(F3 wl) {
    float theta = acosf(wl.z);
    float c = cosf(theta);
    return (c > 0.f) ? c * PGX_INV_PI_F : 0.f;
}

// ---- BSDF dispatch ------------------------------------------------------------
template <int K>
__device__ __forceinline__ bool bsdf_pure_specular_k(const DevMaterial& m) {
    switch (K >= 0 ? K : m.kind) {
        case PGX_BSDF_MIRROR:
        case PGX_BSDF_GLASS:
            return true;
        case PGX_BSDF_CONDUCTOR:
        case PGX_BSDF_DIELECTRIC:
            return m.alpha < PGX_EPSILON;
        default:
            return false;
    }
}
__device__ __forceinline__ bool bsdf_pure_specular(const DevMaterial& m) { return bsdf_pure_specular_k<-1>(m); }
__device__ __forceinline__ bool bsdf_two_sided(const DevMaterial& m) {
    if (m.layered) return true;  // LayeredBSDF::isTwoSided, Materials.h:895
    return !(m.kind == PGX_BSDF_GLASS || m.kind == PGX_BSDF_DIELECTRIC);
}

template <int K>
__device__ __forceinline__ F3 conductor_eval_i(const DevMaterial& m, F3 alb, F3 wil, F3 wol) {
    if (wil.z <= 0.f || wol.z <= 0.f) return zero3();
    if (m.alpha < PGX_EPSILON) return zero3();
    F3 h = wil + wol;
    if (length_sq(h) < PGX_EPSILON) return zero3();
    h = normalize(h);
    if (dot(wol, h) <= 0.f) return zero3();
    if (wil.z * wol.z <= 0.f) return zero3();
    float G = g_ggx(wil, wol, m.alpha);
    float D = d_ggx(h, m.alpha);
    F3 F = fresnel_conductor_k<K>(dot(wol, h), m.eta, m.k);
    return alb * divs((F * G) * D, (4.f * wil.z) * wol.z);
}
static __device__ __noinline__ F3 conductor_eval(const DevMaterial& m, F3 alb, F3 wil, F3 wol) {
    return conductor_eval_i<-1>(m, alb, wil, wol);
}
template <int K>
__device__ __forceinline__ F3 conductor_eval_k(const DevMaterial& m, F3 alb, F3 wil, F3 wol) {
    if constexpr (K < 0)
        return conductor_eval(m, alb, wil, wol);
    else
        return conductor_eval_i<K>(m, alb, wil, wol);
}
static __device__ float conductor_pdf(const DevMaterial& m, F3 wil, F3 wol) {
    if (wil.z <= 0.f || wol.z <= 0.f) return 0.f;
    if (m.alpha < PGX_EPSILON) return 0.f;
    F3 h = wil + wol;
    if (length_sq(h) < PGX_EPSILON) return 0.f;
    h = normalize(h);
    if (dot(wol, h) <= 0.f) return 0.f;
    if (wil.z * wol.z <= 0.f) return 0.f;
    float D = d_ggx(h, m.alpha);
    return (D * h.z) / (4.f * dot(wol, h));
}

// Rough dielectric eval/pdf (Materials.h:545-634).
__device__ __forceinline__ void dielectric_eval_pdf_i(const DevMaterial& m, F3 alb, F3 wol, F3 wil, F3* f, float* pdf) {
    if (f) *f = zero3();
    if (pdf) *pdf = 0.f;
    if (wol.z == 0.f || wil.z == 0.f) return;
    float eta = wol.z > 0.f ? m.ext_ior / m.int_ior : m.int_ior / m.ext_ior;
    if (eta == 1.f || m.alpha < PGX_EPSILON) return;
    bool reflect = wol.z * wil.z > 0.f;
    float etap = 1.f;
    if (!reflect) etap = wol.z > 0.f ? eta : 1.f / eta;
    F3 h = (wil * etap) + wol;
    if (length_sq(h) < PGX_EPSILON) return;
    h = normalize(h);
    if (dot(h, wil) * wil.z < 0.f || dot(h, wol) * wol.z < 0.f) return;
    float F = fresnel_dielectric(dot(wol, h), m.int_ior, m.ext_ior);
    if (reflect) {
        if (dot(wol, h) <= 0.f) return;
        if (wil.z * wol.z == 0.f) return;
        float D = d_ggx(h, m.alpha);
        if (f) {
            float G = g_ggx(wil, wol, m.alpha);
            *f = alb * (((F * G) * D) / ((4.f * wil.z) * wol.z));
        }
        if (pdf) *pdf = F * ((D * h.z) / (4.f * dot(wol, h)));
    } else {
        float a = dot(wil, h) + dot(wol, h) / etap;
        float den = a * a;
        if (den <= 0.f) return;
        float D = d_ggx(h, m.alpha);
        if (f) {
            float G = g_ggx(wil, wol, m.alpha);
            *f = ((alb * ((((1.f - F) * G) * D) / den)) * (fabsf(dot(wil, h)) / fabsf(wil.z))) *
                 (fabsf(dot(wol, h)) / fabsf(wol.z));
        }
        if (pdf) *pdf = (1.f - F) * ((D * fabsf(dot(wol, h))) / den);
    }
}
static __device__ __noinline__ void dielectric_eval_pdf(const DevMaterial& m, F3 alb, F3 wol, F3 wil, F3* f, float* pdf) {
    dielectric_eval_pdf_i(m, alb, wol, wil, f, pdf);
}
template <int K>
__device__ __forceinline__ void dielectric_eval_pdf_k(const DevMaterial& m, F3 alb, F3 wol, F3 wil, F3* f, float* pdf) {
    if constexpr (K < 0)
        dielectric_eval_pdf(m, alb, wol, wil, f, pdf);
    else
        dielectric_eval_pdf_i(m, alb, wol, wil, f, pdf);
}

__device__ __forceinline__ float plastic_exponent(float alpha) {
    float a = s_max(alpha, 0.001f);
    return (2.f / (a * a)) - 2.f;
}

// BSDF::evaluate for all kinds.
template <int K>
__device__ __forceinline__ F3 bsdf_eval_i(const DevMaterial& m, const TexView& tv, const Shading& sd, F3 wi) {
    switch (K >= 0 ? K : m.kind) {
        case PGX_BSDF_DIFFUSE: {
            F3 wl = to_local(sd.frame, wi);
            if (wl.z <= 0.f) return zero3();
            return albedo_of(tv, m, sd) * PGX_INV_PI_F;
        }
        case PGX_BSDF_CONDUCTOR:
            return conductor_eval_k<K>(m, albedo_of(tv, m, sd), to_local(sd.frame, wi), to_local(sd.frame, sd.wo));
        case PGX_BSDF_DIELECTRIC: {
            F3 f;
            dielectric_eval_pdf_k<K>(m, albedo_of(tv, m, sd), to_local(sd.frame, sd.wo), to_local(sd.frame, wi), &f,
                                     nullptr);
            return f;
        }
        case PGX_BSDF_ORENNAYAR: {
            F3 wol = to_local(sd.frame, sd.wo), wil = to_local(sd.frame, wi);
            float s2 = m.sigma * m.sigma;
            float A = 1.f - (s2 / (2.f * (s2 + 0.33f)));
            float B = (0.45f * s2) / (s2 + 0.09f);
            float phi_i = spherical_phi(wil), phi_o = spherical_phi(wol);
            float th_i = acosf(wil.z), th_o = acosf(wol.z);
            float c = cosf(phi_i - phi_o);
            float sa = sinf(s_max(th_i, th_o));
            float tb = tanf(s_min(th_i, th_o));
            float on = A + (((B * s_max(0.f, c)) * sa) * tb);
            return (albedo_of(tv, m, sd) * PGX_INV_PI_F) * on;
        }
        case PGX_BSDF_PLASTIC: {
            F3 wil = to_local(sd.frame, wi), wol = to_local(sd.frame, sd.wo);
            if (wil.z <= 0.f || wol.z <= 0.f) return zero3();
            F3 h = wil + wol;
            if (length_sq(h) < PGX_EPSILON) return zero3();
            h = normalize(h);
            float e = plastic_exponent(m.alpha);
            float ks = fresnel_dielectric(dot(wol, h), m.int_ior, m.ext_ior);
            float kd = 1.f - ks;
            float norm = (e + 2.f) / ((4.f * PGX_PI_F) * (2.f - powf(2.f, -e * 0.5f)));
            float lo = (e + 2.f) * (1.f / (8.f * PGX_PI_F));
            float hi = (e + 4.f) * (1.f / (8.f * PGX_PI_F));
            norm = s_min(s_max(lo, norm), hi);
            float glossy = powf(s_max(h.z, 0.f), e);
            F3 diffuse = albedo_of(tv, m, sd) * PGX_INV_PI_F;
            F3 gl = dot(wol, h) <= 0.f ? zero3() : f3(1.f, 1.f, 1.f) * glossy;
            return (diffuse * kd) + ((gl * norm) * ks);
        }
        default:  // Mirror, Glass: delta lobes evaluate to zero
            return zero3();
    }
}
static __device__ __noinline__ F3 bsdf_eval(const DevMaterial& m, const TexView& tv, const Shading& sd, F3 wi) {
    return bsdf_eval_i<-1>(m, tv, sd, wi);
}
template <int K>
__device__ __forceinline__ F3 bsdf_eval_k(const DevMaterial& m, const TexView& tv, const Shading& sd, F3 wi) {
    if constexpr (K < 0)
        return bsdf_eval(m, tv, sd, wi);
    else
        return bsdf_eval_i<K>(m, tv, sd, wi);
}

// BSDF::PDF for all kinds.
template <int K>
__device__ __forceinline__ float bsdf_pdf_i(const DevMaterial& m, const TexView& tv, const Shading& sd, F3 wi) {
    switch (K >= 0 ? K : m.kind) {
        case PGX_BSDF_DIFFUSE:
        case PGX_BSDF_ORENNAYAR:
            return cosine_pdf(to_local(sd.frame, wi));
        case PGX_BSDF_CONDUCTOR:
            return conductor_pdf(m, to_local(sd.frame, wi), to_local(sd.frame, sd.wo));
        case PGX_BSDF_DIELECTRIC: {
            float p;
            dielectric_eval_pdf_k<K>(m, zero3(), to_local(sd.frame, sd.wo), to_local(sd.frame, wi), nullptr, &p);
            return p;
        }
        case PGX_BSDF_PLASTIC: {
            F3 wil = to_local(sd.frame, wi), wol = to_local(sd.frame, sd.wo);
            if (wil.z <= 0.f || wol.z <= 0.f) return 0.f;
            F3 h = wil + wol;
            if (length_sq(h) < PGX_EPSILON) return 0.f;
            h = normalize(h);
            float e = plastic_exponent(m.alpha);
            float ks = fresnel_dielectric(dot(wol, h), m.int_ior, m.ext_ior);
            float kd = 1.f - ks;
            float ph = ((e + 1.f) * PGX_INV_2PI_F) * powf(s_max(h.z, 0.f), e);
            float gp = dot(wol, h) <= 0.f ? 0.f : (ph / (4.f * dot(wol, h)));
            float dp = cosine_pdf(wil);
            return (kd * dp) + (ks * gp);
        }
        default:
            return 0.f;
    }
    (void)tv;
}
static __device__ __noinline__ float bsdf_pdf(const DevMaterial& m, const TexView& tv, const Shading& sd, F3 wi) {
    return bsdf_pdf_i<-1>(m, tv, sd, wi);
}
template <int K>
__device__ __forceinline__ float bsdf_pdf_k(const DevMaterial& m, const TexView& tv, const Shading& sd, F3 wi) {
    if constexpr (K < 0)
        return bsdf_pdf(m, tv, sd, wi);
    else
        return bsdf_pdf_i<K>(m, tv, sd, wi);
}

// Samplers: the path's PCG32 stream, or the reference's TestSampler
// (Sampling.h:26-48: the first two draws are u and v, every later one 0.5).
struct PcgSampler {
    uint64_t& state;
    __device__ float next() { return pgx_rng_next(state); }
};
struct FixedSampler {
    float u, v;
    int called;
    __device__ float next() {
        float r = called == 0 ? u : (called == 1 ? v : 0.5f);
        called++;
        return r;
    }
};

// BSDF::sample for all kinds; draws from the sampler exactly like the reference.
template <int K, class Smp>
__device__ __forceinline__ F3 bsdf_sample_i(const DevMaterial& m, const TexView& tv, const Shading& sd, Smp& rng, F3& f,
                                            float& pdf) {
    switch (K >= 0 ? K : m.kind) {
        case PGX_BSDF_DIFFUSE:
        case PGX_BSDF_ORENNAYAR: {
            float r1 = rng.next();
            float r2 = rng.next();
            F3 wi = to_world(sd.frame, cosine_sample(r1, r2));
            f = bsdf_eval_k<K>(m, tv, sd, wi);
            pdf = bsdf_pdf_k<K>(m, tv, sd, wi);
            return wi;
        }
        case PGX_BSDF_MIRROR: {
            F3 wol = to_local(sd.frame, sd.wo);
            F3 wr = f3(-wol.x, -wol.y, wol.z);
            if (fabsf(wr.z) <= PGX_EPSILON) {
                pdf = 0.f;
                f = zero3();
                return f3(0.f, 0.f, 1.f);
            }
            f = divs(albedo_of(tv, m, sd), wr.z);
            pdf = 1.f;
            return to_world(sd.frame, wr);
        }
        case PGX_BSDF_CONDUCTOR: {
            F3 wol = to_local(sd.frame, sd.wo);
            if (wol.z <= 0.f) {
                pdf = 0.f;
                f = zero3();
                return f3(0.f, 0.f, 1.f);
            }
            if (m.alpha < PGX_EPSILON) {
                F3 wr = f3(-wol.x, -wol.y, wol.z);
                F3 F = fresnel_conductor_k<K>(wr.z, m.eta, m.k);
                f = divs(albedo_of(tv, m, sd), fabsf(wr.z)) * F;
                pdf = 1.f;
                return to_world(sd.frame, wr);
            }
            float r1 = rng.next();
            float r2 = rng.next();
            F3 h = ggx_sample_h(m.alpha, r1, r2);
            F3 wil = -wol + (h * 2.f) * dot(h, wol);
            F3 wi = to_world(sd.frame, wil);
            f = bsdf_eval_k<K>(m, tv, sd, wi);
            pdf = bsdf_pdf_k<K>(m, tv, sd, wi);
            return wi;
        }
        case PGX_BSDF_GLASS: {
            F3 wol = to_local(sd.frame, sd.wo);
            if (fabsf(wol.z) < PGX_EPSILON) {
                pdf = 0.f;
                f = zero3();
                return f3(0.f, 0.f, 1.f);
            }
            float F = fresnel_dielectric(wol.z, m.int_ior, m.ext_ior);
            float ci = wol.z;
            float eta = (ci < 0.f) ? (m.int_ior / m.ext_ior) : (m.ext_ior / m.int_ior);
            if (ci < 0.f) ci = fabsf(ci);
            F3 alb = albedo_of(tv, m, sd);
            if (rng.next() < F) {
                F3 wr = f3(-wol.x, -wol.y, wol.z);
                pdf = F;
                f = divs(alb, fabsf(wr.z)) * F;
                return to_world(sd.frame, wr);
            }
            float ci_sq = s_max(ci * ci, 0.f);
            float si_sq = s_max(1.f - ci_sq, 0.f);
            float eta_sq = eta * eta;
            float st_sq = eta_sq * si_sq;
            if (st_sq > 1.f) {
                F3 wr = f3(-wol.x, -wol.y, wol.z);
                pdf = F;
                f = divs(alb, fabsf(wr.z)) * F;
                return to_world(sd.frame, wr);
            }
            float ct = sqrtf(s_max(1.f - st_sq, 0.f));
            float wtz = (wol.z < 0.f) ? ct : -ct;
            F3 wt = f3(-eta * wol.x, -eta * wol.y, wtz);
            pdf = 1.f - F;
            f = (divs(alb, fabsf(wt.z)) * (1.f - F)) * eta_sq;
            return to_world(sd.frame, wt);
        }
        case PGX_BSDF_DIELECTRIC: {
            F3 wol = to_local(sd.frame, sd.wo);
            F3 alb = albedo_of(tv, m, sd);
            if (m.alpha < PGX_EPSILON) {
                float F = fresnel_dielectric(wol.z, m.int_ior, m.ext_ior);
                if (rng.next() < F) {
                    F3 w = f3(-wol.x, -wol.y, wol.z);
                    pdf = F;
                    f = divs(alb, fabsf(w.z)) * F;
                    return to_world(sd.frame, w);
                }
                float eta = wol.z > 0.f ? m.ext_ior / m.int_ior : m.int_ior / m.ext_ior;
                float eta_sq = eta * eta;
                float sgn = wol.z > 0.f ? -1.f : 1.f;
                float ci_sq = s_max(wol.z * wol.z, 0.f);
                float si_sq = s_max(1.f - ci_sq, 0.f);
                float st_sq = eta_sq * si_sq;
                if (st_sq > 1.f) {
                    F3 w = f3(-wol.x, -wol.y, wol.z);
                    pdf = F;
                    f = divs(alb, fabsf(w.z)) * F;
                    return to_world(sd.frame, w);
                }
                float ct = sqrtf(s_max(1.f - st_sq, 0.f));
                F3 w = f3(-eta * wol.x, -eta * wol.y, ct * sgn);
                pdf = 1.f - F;
                f = divs(alb, fabsf(w.z)) * (1.f - F);
                return to_world(sd.frame, w);
            }
            float r1 = rng.next(), r2 = rng.next();
            F3 h = ggx_sample_h(m.alpha, r1, r2);
            float F = fresnel_dielectric(dot(wol, h), m.int_ior, m.ext_ior);
            F3 wi;
            if (rng.next() < F) {
                wi = to_world(sd.frame, -wol + (h * 2.f) * dot(h, wol));
            } else {
                Frame hf = frame_from(h);
                F3 wo_h = to_local(hf, wol);
                float ci = wo_h.z;
                float eta = ci > 0.f ? m.ext_ior / m.int_ior : m.int_ior / m.ext_ior;
                float eta_sq = eta * eta;
                float sgn = ci > 0.f ? -1.f : 1.f;
                float ci_sq = s_max(ci * ci, 0.f);
                float si_sq = s_max(1.f - ci_sq, 0.f);
                float st_sq = eta_sq * si_sq;
                float ct = sqrtf(s_max(1.f - st_sq, 0.f));
                F3 w = f3(-eta * wo_h.x, -eta * wo_h.y, ct * sgn);
                wi = to_world(sd.frame, to_world(hf, w));
            }
            dielectric_eval_pdf_k<K>(m, alb, wol, to_local(sd.frame, wi), &f, &pdf);
            return wi;
        }
        case PGX_BSDF_PLASTIC: {
            F3 wol = to_local(sd.frame, sd.wo);
            float r1 = rng.next();
            float r2 = rng.next();
            float F = fresnel_dielectric(fabsf(wol.z), m.int_ior, m.ext_ior);
            F3 wil;
            if (rng.next() < F) {
                float e = plastic_exponent(m.alpha);
                float th = acosf(powf(1.f - r1, 1.f / (e + 1.f)));
                float ph = PGX_2PI_F * r2;
                F3 h = normalize(spherical_to_world(th, ph));
                wil = ((h * 2.f) * dot(wol, h)) - wol;
            } else {
                wil = cosine_sample(r1, r2);
            }
            F3 wi = to_world(sd.frame, wil);
            f = bsdf_eval_k<K>(m, tv, sd, wi);
            pdf = bsdf_pdf_k<K>(m, tv, sd, wi);
            return wi;
        }
        default:
            pdf = 0.f;
            f = zero3();
            return f3(0.f, 0.f, 1.f);
    }
}

template <class Smp>
static __device__ __noinline__ F3 bsdf_sample_s(const DevMaterial& m, const TexView& tv, const Shading& sd, Smp& rng,
                                                F3& f, float& pdf) {
    return bsdf_sample_i<-1>(m, tv, sd, rng, f, pdf);
}

__device__ __forceinline__ F3 bsdf_sample(const DevMaterial& m, const TexView& tv, const Shading& sd, uint64_t& rng,
                                          F3& f, float& pdf) {
    PcgSampler smp{rng};
    return bsdf_sample_s(m, tv, sd, smp, f, pdf);
}
template <int K>
__device__ __forceinline__ F3 bsdf_sample_k(const DevMaterial& m, const TexView& tv, const Shading& sd, uint64_t& rng,
                                            F3& f, float& pdf) {
    if constexpr (K < 0) {
        return bsdf_sample(m, tv, sd, rng, f, pdf);
    } else {
        PcgSampler smp{rng};
        return bsdf_sample_i<K>(m, tv, sd, smp, f, pdf);
    }
}

// BSDF::invert (Materials.h:163-171, 287-306, 673-681): the primary sample
// (u, v) that BSDF::sample would map to wi.  Delta lobes give (0, 0); the
// reference leaves the rough dielectric and plastic unimplemented
// (Materials.h:541-543, 782-784), so their (u, v) stay unchanged.
// The primary sample that the cosine-weighted hemisphere sampler of the
// diffuse BSDFs maps to wi in frame fr (BSDF::invert, Materials.h:163-171):
// u = cos^2 theta, v = phi / 2pi.
__device__ __forceinline__ void cosine_invert(const Frame& fr, F3 wi, float& u, float& v) {
    F3 wl = to_local(fr, wi);
    float theta = acosf(wl.z);
    float phi = spherical_phi(wl);
    float c = cosf(theta);
    u = c * c;
    v = phi * PGX_INV_2PI_F;
}

static __device__ __noinline__ void bsdf_invert(const DevMaterial& m, const Shading& sd, F3 wi, float& u, float& v) {
    switch (m.kind) {
        case PGX_BSDF_DIFFUSE:
        case PGX_BSDF_ORENNAYAR:
            cosine_invert(sd.frame, wi, u, v);
            break;
        case PGX_BSDF_CONDUCTOR: {
            if (m.alpha < PGX_EPSILON) {
                u = 0.f;
                v = 0.f;
                break;
            }
            F3 wil = to_local(sd.frame, wi), wol = to_local(sd.frame, sd.wo);
            F3 h = normalize(wil + wol);
            float theta = acosf(h.z);
            float phi = spherical_phi(h);
            float a2 = m.alpha * m.alpha;
            float a1 = a2 - 1.f;
            float c = cosf(theta);
            u = (a2 / ((c * c) * (a1 * a1) + a1)) - (1.f / a1);
            v = phi * PGX_INV_2PI_F;
            break;
        }
        case PGX_BSDF_MIRROR:
        case PGX_BSDF_GLASS:
            u = 0.f;
            v = 0.f;
            break;
        default:
            break;
    }
}

// ---- environment map (EnvironmentMap, Lights.h:128-228) ------------------------
// Distribution1D::binarySearch (Sampling.h:107-123) over cdf[0..size).
__device__ __forceinline__ int cdf_search(const float* cdf, int size, float u) {
    int first = 0, iter = size;
    while (iter > 0) {
        int half = iter / 2;
        int middle = first + half;
        if (cdf[middle] <= u) {
            first = middle + 1;
            iter -= (half + 1);
        } else {
            iter = half;
        }
    }
    int r = first - 1;
    r = (size - 2 < r) ? size - 2 : r;
    return r > 0 ? r : 0;
}
// cdf_search with a guide table (the cutpoint method, Chen and Asau 1974):
// guide[k] is the first index i with cdf_bucket(cdf[i]) >= k, guide[K] =
// size.  For a sorted CDF every entry before guide[k] is <= u and every
// entry from guide[k + 1] on is > u when u falls in bucket k, so the count
// of entries <= u -- what the binary search computes -- is found by the same
// search over [guide[k], guide[k + 1]), usually zero to two steps instead of
// log2(size).  The tables exist only for sorted CDFs.
__device__ __forceinline__ int cdf_search_guided(const float* cdf, int size, float u, const int* guide, int K) {
    const int k = cdf_bucket(u, K);
    int first = guide[k];
    int iter = guide[k + 1] - first;
    while (iter > 0) {
        int half = iter / 2;
        int middle = first + half;
        if (cdf[middle] <= u) {
            first = middle + 1;
            iter -= (half + 1);
        } else {
            iter = half;
        }
    }
    int r = first - 1;
    r = (size - 2 < r) ? size - 2 : r;
    return r > 0 ? r : 0;
}
// Distribution1D::sampleContinuous (Sampling.h:151-163); n = function size;
// guide: the CDF's guide table of n buckets, or nullptr.
__device__ __forceinline__ float sample_continuous(const float* func, const float* cdf, float integral, int n, float u,
                                                   float& pdf, int& off, const int* guide = nullptr) {
    off = guide ? cdf_search_guided(cdf, n + 1, u, guide, n) : cdf_search(cdf, n + 1, u);
    float du = u - cdf[off];
    if ((cdf[off + 1] - cdf[off]) > 0.f) du /= (cdf[off + 1] - cdf[off]);
    pdf = (integral > 0.f) ? (func[off] / integral) : 0.f;
    return ((float)off + du) / (float)n;
}

__device__ __forceinline__ F3 env_eval(const DevEnv& e, F3 wi) {
    if (!e.valid) return zero3();
    float u = atan2f(wi.z, wi.x);
    u = (u < 0.f) ? u + PGX_2PI_F : u;
    u = u * PGX_INV_2PI_F;
    float v = acosf(wi.y) * PGX_INV_PI_F;
    return tex_sample_raw(e.texels, 0, e.width, e.height, u, v);
}

// Distribution2D::PDF (Sampling.h:203-208) via EnvironmentMap::PDF.
__device__ __forceinline__ float env_pdf_i(const DevEnv& e, F3 wi) {
    float u = atan2f(wi.z, wi.x);
    u = (u < 0.f) ? u + PGX_2PI_F : u;
    u = u * PGX_INV_2PI_F;
    float v = acosf(wi.y) * PGX_INV_PI_F;
    float st = sinpif(v);  // sin(pi * v) of EnvironmentMap::PDF (Lights.h:188)
    if (st <= 0.f) return 0.f;
    float p;
    if (e.marg_int == 0.f) {
        p = 1.f;
    } else {
        int iu = min(max((int)(u * (float)e.width), 0), e.width - 1);
        int iv = min(max((int)(v * (float)e.height), 0), e.height - 1);
        p = e.cond_func[(size_t)iv * e.width + iu] / e.marg_int;
    }
    return p / (PGX_2PI2_F * st);
}
static __device__ __noinline__ float env_pdf(const DevEnv& e, F3 wi) { return env_pdf_i(e, wi); }

// EnvironmentMap::sample: direction (y-up), emitted colour and solid-angle pdf.
__device__ __forceinline__ F3 env_sample_i(const DevEnv& e, uint64_t& rng, F3& col, float& pdf) {
    float ru = pgx_rng_next(rng);
    float rv = pgx_rng_next(rng);
    float pv, pu;
    int dv, du;
    float v = sample_continuous(e.marg_func, e.marg_cdf, e.marg_int, e.height, rv, pv, dv, e.marg_guide);
    float u = sample_continuous(e.cond_func + (size_t)dv * e.width, e.cond_cdf + (size_t)dv * (e.width + 1),
                                e.cond_int[dv], e.width, ru, pu, du,
                                e.cond_guide ? e.cond_guide + (size_t)dv * (e.width + 1) : nullptr);
    float sp = pu * pv;
    float theta = PGX_PI_F * v;
    float phi = PGX_2PI_F * u;
    float ct = cosf(theta), cp = cosf(phi), st = sinf(theta), sp_ = sinf(phi);
    F3 wi = f3(cp * st, ct, sp_ * st);
    pdf = (st <= 0.f) ? 0.f : sp / (PGX_2PI2_F * st);
    col = (pdf <= 0.f) ? zero3() : env_eval(e, wi);
    return wi;
}
static __device__ __noinline__ F3 env_sample(const DevEnv& e, uint64_t& rng, F3& col, float& pdf) {
    return env_sample_i(e, rng, col, pdf);
}
