// The learned directional guide: a 6-layer MLP (78 encoded inputs -> 5
// hidden layers of 64 with ReLU -> 40 outputs) evaluated on the tensor
// cores with BF16 weights and activations and FP32 accumulation, whose
// outputs parameterise a mixture of 8 von Mises-Fisher lobes over the
// sphere of directions.
//
// Inputs of a query (position x, shading normal n, outgoing direction wo):
//   x' = (x - bmin) / (bmax - bmin), clamped to [0, 1]
//   feature c*24 + 2j     = sin(2^j * pi * x'_c)      j = 0..11, c = 0..2
//   feature c*24 + 2j + 1 = cos(2^j * pi * x'_c)
//   features 72..74 = n, 75..77 = wo, 78..79 = 0.
// Outputs: 8 lobe logits (softmax -> weights), 8 x 3 unnormalised mean
// directions, 8 concentrations kappa = softplus(r) + 0.01.
//
// Layer l's weights live on the device as a bf16 "image" in the tensor-core
// operand layout of pgx_tc.cuh (rows = 64 output features, padded with zero
// rows for the 40-output layer; K = input features), so a CTA copies them
// to shared memory with 16-byte loads.
#pragma once

#include <cstdint>

#include "pgx_shade.cuh"
#include "pgx_tc.cuh"

namespace mlp {

constexpr int kRows = 128;   // rows per tile = MMA M
constexpr int kIn = 80;      // input features of layer 0 (78 used)
constexpr int kHid = 64;
constexpr int kOut = 40;     // outputs used
constexpr int kLayers = 6;
constexpr int kLobes = 8;
constexpr int kFreq = 12;
constexpr float kKappaMin = 0.01f;

__host__ __device__ constexpr int layer_k(int l) { return l == 0 ? kIn : kHid; }
__host__ __device__ constexpr int layer_n(int l) { return l == kLayers - 1 ? kOut : kHid; }
// Bytes of layer l's weight image (64 rows x K bf16).
__host__ __device__ constexpr int image_bytes(int l) { return layer_k(l) * kHid * 2; }
__host__ __device__ constexpr int image_offset(int l) { return l == 0 ? 0 : image_bytes(0) + (l - 1) * image_bytes(1); }
constexpr int kImageBytes = image_bytes(0) + (kLayers - 1) * image_bytes(1);  // 51200
constexpr int kBiasFloats = kLayers * kHid;                                    // padded biases
// Parameters in API order: per layer W[n][k] row-major, then b[n].
__host__ __device__ constexpr int param_w(int l) {
    int off = 0;
    for (int i = 0; i < l; i++) off += layer_n(i) * layer_k(i) + layer_n(i);
    return off;
}
__host__ __device__ constexpr int param_b(int l) { return param_w(l) + layer_n(l) * layer_k(l); }
constexpr int kParams = param_w(kLayers);  // 24424
static_assert(kParams == 24424, "parameter count");

// Bytes of one row-major activation tile chunk column (128 rows x 8 bf16).
constexpr int kChunk = kRows * 16;

struct Bounds {
    float bmin[3];
    float inv_ext[3];
};

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t v) { return __uint_as_float(v & 0xFFFF0000u); }

// Writes 8 values as one 16-byte bf16 chunk of row r, column chunk c.
__device__ __forceinline__ void store_chunk(uint8_t* tile, int r, int c, const float* v) {
    uint4 q;
    q.x = pack_bf16x2(v[0], v[1]);
    q.y = pack_bf16x2(v[2], v[3]);
    q.z = pack_bf16x2(v[4], v[5]);
    q.w = pack_bf16x2(v[6], v[7]);
    *reinterpret_cast<uint4*>(tile + c * kChunk + r * 16) = q;
}
__device__ __forceinline__ void load_chunk(const uint8_t* tile, int r, int c, float* v) {
    uint4 q = *reinterpret_cast<const uint4*>(tile + c * kChunk + r * 16);
    v[0] = bf16_lo(q.x), v[1] = bf16_hi(q.x), v[2] = bf16_lo(q.y), v[3] = bf16_hi(q.y);
    v[4] = bf16_lo(q.z), v[5] = bf16_hi(q.z), v[6] = bf16_lo(q.w), v[7] = bf16_hi(q.w);
}

// The 80 input features of one query, written as bf16 into row r of the
// layer-0 tile.
__device__ __forceinline__ void encode_row(uint8_t* tile, int r, const Bounds& b, F3 x, F3 n, F3 wo) {
    float p[3] = {x.x, x.y, x.z};
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float t = (p[c] - b.bmin[c]) * b.inv_ext[c];
        t = fminf(fmaxf(t, 0.f), 1.f);
        float v[24];
        // sin/cos of 2^j pi t by the double-angle recurrence from j = 0
        // (absolute error below 2^j ulp, far under the bf16 step of 2^-8)
        float sn, cs;
        sincospif(t, &sn, &cs);
#pragma unroll
        for (int j = 0; j < kFreq; j++) {
            v[2 * j] = sn;
            v[2 * j + 1] = cs;
            float s2 = 2.f * sn * cs;
            cs = (cs - sn) * (cs + sn);
            sn = s2;
        }
        store_chunk(tile, r, 3 * c, v);
        store_chunk(tile, r, 3 * c + 1, v + 8);
        store_chunk(tile, r, 3 * c + 2, v + 16);
    }
    float tail[8] = {n.x, n.y, n.z, wo.x, wo.y, wo.z, 0.f, 0.f};
    store_chunk(tile, r, 9, tail);
}

// ---- the vMF mixture --------------------------------------------------------------
// Per query the renderer keeps 10 float4: lobe i = (mu.xyz, kappa) for
// i < 8, then the 8 lobe weights.
struct Mixture {
    float4 lobe[kLobes];
    float w[kLobes];
};

__device__ __forceinline__ float softplus(float x) { return x > 20.f ? x : log1pf(expf(x)); }

__device__ __forceinline__ void mixture_from_raw(const float* raw, Mixture& m) {
    float mx = raw[0];
#pragma unroll
    for (int i = 1; i < kLobes; i++) mx = fmaxf(mx, raw[i]);
    float sum = 0.f;
#pragma unroll
    for (int i = 0; i < kLobes; i++) {
        m.w[i] = expf(raw[i] - mx);
        sum += m.w[i];
    }
    float inv = 1.f / sum;
#pragma unroll
    for (int i = 0; i < kLobes; i++) {
        m.w[i] *= inv;
        float a = raw[8 + 3 * i], b = raw[9 + 3 * i], c = raw[10 + 3 * i];
        float len = sqrtf(a * a + b * b + c * c);
        float il = len > 1e-20f ? 1.f / len : 0.f;
        if (len <= 1e-20f) c = 1.f, il = 1.f;
        m.lobe[i] = make_float4(a * il, b * il, c * il, softplus(raw[32 + i]) + kKappaMin);
    }
}

// vMF density kappa / (2 pi (1 - e^{-2 kappa})) * exp(kappa (mu.w - 1)).
__device__ __forceinline__ float vmf_pdf(float4 l, F3 w) {
    float k = l.w;
    float cosv = l.x * w.x + l.y * w.y + l.z * w.z;
    float norm = k / (2.f * 3.14159265f * (-expm1f(-2.f * k)));
    return norm * expf(k * (cosv - 1.f));
}

__device__ __forceinline__ float mixture_pdf(const Mixture& m, F3 w) {
    float p = 0.f;
#pragma unroll
    for (int i = 0; i < kLobes; i++) p += m.w[i] * vmf_pdf(m.lobe[i], w);
    return p;
}

// Lobe chosen by u0, then w = 1 + log(u1 + (1 - u1) e^{-2 kappa}) / kappa
// about mu and a uniform azimuth 2 pi u2.
__device__ __forceinline__ F3 mixture_sample(const Mixture& m, float u0, float u1, float u2) {
    int pick = kLobes - 1;
    float acc = 0.f;
#pragma unroll
    for (int i = 0; i < kLobes; i++) {
        acc += m.w[i];
        if (u0 < acc && pick == kLobes - 1 && i < kLobes - 1) pick = i;
    }
    float4 l = m.lobe[0];
#pragma unroll
    for (int i = 1; i < kLobes; i++)
        if (i == pick) l = m.lobe[i];
    float k = l.w;
    float cw = 1.f + logf(u1 + (1.f - u1) * expf(-2.f * k)) / k;
    cw = fminf(fmaxf(cw, -1.f), 1.f);
    float sw = sqrtf(fmaxf(0.f, 1.f - cw * cw));
    float s, c;
    sincospif(2.f * u2, &s, &c);
    F3 mu = f3(l.x, l.y, l.z);
    // orthonormal basis about mu (Duff et al. 2017)
    float sign = copysignf(1.f, mu.z);
    float a = -1.f / (sign + mu.z);
    float bb = mu.x * mu.y * a;
    F3 t = f3(1.f + sign * mu.x * mu.x * a, sign * bb, -sign * mu.x);
    F3 bt = f3(bb, sign + mu.y * mu.y * a, -mu.y);
    return normalize(t * (sw * c) + bt * (sw * s) + mu * cw);
}

// ---- packed mixture, as the renderer keeps it per path ------------------------------
// 12 float4: lobe i = (mu.xyz, kappa) for i < 8; then c_0..c_7 with
// c_i = w_i kappa_i / (2 pi (1 - e^{-2 kappa_i})), so q(w) = sum_i c_i
// exp(kappa_i (mu_i.w - 1)); then the running sums of w_i for the lobe choice.
constexpr int kPacked = 12;

__device__ __forceinline__ void pack_mixture(const float* raw, float4* g) {
    Mixture m;
    mixture_from_raw(raw, m);
    float c[kLobes], cdf[kLobes];
    float acc = 0.f;
#pragma unroll
    for (int i = 0; i < kLobes; i++) {
        float k = m.lobe[i].w;
        c[i] = m.w[i] * k / (2.f * 3.14159265f * (-expm1f(-2.f * k)));
        acc += m.w[i];
        cdf[i] = acc;
        g[i] = m.lobe[i];
    }
    g[8] = make_float4(c[0], c[1], c[2], c[3]);
    g[9] = make_float4(c[4], c[5], c[6], c[7]);
    g[10] = make_float4(cdf[0], cdf[1], cdf[2], cdf[3]);
    g[11] = make_float4(cdf[4], cdf[5], cdf[6], cdf[7]);
}

__device__ __forceinline__ float packed_pdf(const float4* __restrict__ g, F3 w) {
    float4 c0 = g[8], c1 = g[9];
    float c[kLobes] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
    float p = 0.f;
#pragma unroll
    for (int i = 0; i < kLobes; i++) {
        float4 l = g[i];
        float cosv = l.x * w.x + l.y * w.y + l.z * w.z;
        p += c[i] * __expf(l.w * (cosv - 1.f));
    }
    return p;
}

__device__ __forceinline__ F3 packed_sample(const float4* __restrict__ g, float u0, float u1, float u2) {
    float4 a = g[10], b = g[11];
    float cdf[kLobes] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    int pick = kLobes - 1;
#pragma unroll
    for (int i = kLobes - 2; i >= 0; i--)
        if (u0 < cdf[i]) pick = i;
    float4 l = g[pick];
    float k = l.w;
    float cw = 1.f + __logf(u1 + (1.f - u1) * __expf(-2.f * k)) / k;
    cw = fminf(fmaxf(cw, -1.f), 1.f);
    float sw = sqrtf(fmaxf(0.f, 1.f - cw * cw));
    float s, c;
    sincospif(2.f * u2, &s, &c);
    F3 mu = f3(l.x, l.y, l.z);
    float sign = copysignf(1.f, mu.z);
    float aa = -1.f / (sign + mu.z);
    float bb = mu.x * mu.y * aa;
    F3 t = f3(1.f + sign * mu.x * mu.x * aa, sign * bb, -sign * mu.x);
    F3 bt = f3(bb, sign + mu.y * mu.y * aa, -mu.y);
    return normalize(t * (sw * c) + bt * (sw * s) + mu * cw);
}

// Loss of one training sample, -weight * log q(wi), and its gradient with
// respect to the 40 raw outputs (d[40]).
__device__ __forceinline__ float loss_grad(const float* raw, F3 wi, float weight, float* d) {
    Mixture m;
    mixture_from_raw(raw, m);
    float v[kLobes];
    float q = 0.f;
#pragma unroll
    for (int i = 0; i < kLobes; i++) {
        v[i] = vmf_pdf(m.lobe[i], wi);
        q += m.w[i] * v[i];
    }
    q = fmaxf(q, 1e-30f);
    float g = -weight / q;  // d loss / d q
#pragma unroll
    for (int i = 0; i < kLobes; i++) {
        // softmax logits
        d[i] = g * m.w[i] * (v[i] - q);
        // mean direction: d v / d m = v kappa (wi - (mu.wi) mu) / |m|
        float a = raw[8 + 3 * i], b = raw[9 + 3 * i], c = raw[10 + 3 * i];
        float len = sqrtf(a * a + b * b + c * c);
        float k = m.lobe[i].w;
        float cosv = m.lobe[i].x * wi.x + m.lobe[i].y * wi.y + m.lobe[i].z * wi.z;
        float s = len > 1e-20f ? g * m.w[i] * v[i] * k / len : 0.f;
        d[8 + 3 * i] = s * (wi.x - cosv * m.lobe[i].x);
        d[9 + 3 * i] = s * (wi.y - cosv * m.lobe[i].y);
        d[10 + 3 * i] = s * (wi.z - cosv * m.lobe[i].z);
        // concentration: d log v / d kappa = 1/kappa - 2/(e^{2 kappa} - 1) + cos - 1
        float dlk = 1.f / k - 2.f / expm1f(2.f * k) + (cosv - 1.f);
        float r = raw[32 + i];
        float sig = 1.f / (1.f + expf(-r));
        d[32 + i] = g * m.w[i] * v[i] * dlk * sig;
    }
    return -weight * logf(q);
}

// ---- one forward pass of a 128-row tile on the tensor cores ------------------------
// A tile is processed by a group of 128 threads (4 warps; thread t of the
// group owns row t, and its warp reads TMEM lanes 32 * (warp % 4) ..).  A CTA
// may run several groups on independent tiles; each group has its own
// activation tile, mbarrier, TMEM columns, wait flag and named barrier, and
// they share the weight images and biases.
struct FwdSmem {
    uint8_t* w;      // weight images (shared by the CTA's groups)
    float* bias;
    uint8_t* act;    // the group's activation tile, at least kIn/8 chunks
    uint64_t* mbar;  // the group's mbarrier
    int* flag;       // the group's wait result (shared memory)
    uint32_t tmem;   // the group's accumulator: 64 columns
    int bar;         // the group's named barrier (1..15)
    int tg;          // thread index within the group
};

__device__ __forceinline__ void group_sync(int bar) {
    asm volatile("bar.sync %0, 128;" ::"r"(bar) : "memory");
}

// Issue layer l: D(128 x 64) = act(128 x K) * W_l^T (one thread).
__device__ __forceinline__ void issue_layer(const FwdSmem& s, int l, const uint8_t* act) {
    const int K = layer_k(l);
    const uint32_t a0 = tc::smem_addr(act), b0 = tc::smem_addr(s.w + image_offset(l));
    const uint32_t idesc = tc::idesc_bf16(kRows, kHid);
    for (int k = 0; k < K / 16; k++) {
        uint64_t ad = tc::smem_desc(a0 + k * 2 * kChunk, kChunk, 128);
        uint64_t bd = tc::smem_desc(b0 + k * 2 * (kHid * 16), kHid * 16, 128);
        tc::mma_bf16(s.tmem, ad, bd, idesc, k > 0);
    }
    tc::mma_commit(s.mbar);
}

// Makes the group's shared-memory writes visible to the tensor core and
// orders them before the MMA issue.
__device__ __forceinline__ void publish_smem(int bar) {
    tc::fence_async_smem();
    tc::fence_before_sync();
    group_sync(bar);
    tc::fence_after_sync();
}

constexpr uint32_t kWaitPolls = 1u << 22;

// Thread 0 of the group waits (bounded) for the MMAs committed to s.mbar;
// the result reaches every thread of the group.  Returns false on timeout.
__device__ __forceinline__ bool group_wait(const FwdSmem& s, uint32_t& phase) {
    if (s.tg == 0) *s.flag = tc::mbar_wait(s.mbar, phase, kWaitPolls) ? 0 : 1;
    phase ^= 1u;
    group_sync(s.bar);
    bool ok = *s.flag == 0;
    tc::fence_after_sync();
    return ok;
}

// Runs the six layers on the tile already encoded in s.act; thread tg of
// the group receives row tg's 40 raw outputs.  `phase` is the mbarrier
// parity to wait for next (updated).  Returns false if an MMA did not
// complete in time (uniform across the group).  When keep_acts is given,
// layer l's input tile is s.act for l = 0 and keep_acts[l] for l > 0 (each
// kIn/8 or kHid/8 + 1 chunks), and is left in place for a backward pass.
__device__ __forceinline__ bool forward_tile(const FwdSmem& s, uint32_t& phase, float* out,
                                             uint8_t* const* keep_acts = nullptr) {
    const int t = s.tg;
    const int warp = t >> 5;
    for (int l = 0; l < kLayers; l++) {
        uint8_t* in = (l == 0 || !keep_acts) ? s.act : keep_acts[l];
        publish_smem(s.bar);
        if (t == 0) issue_layer(s, l, in);
        if (!group_wait(s, phase)) return false;
        const float* b = s.bias + l * kHid;
        // two halves of 32 accumulator columns, to keep registers low
#pragma unroll
        for (int half = 0; half < 2; half++) {
            float acc[32];
            tc::tmem_ld32(tc::tmem_at(s.tmem, warp * 32, 32 * half), acc);
            if (l < kLayers - 1) {
                uint8_t* dst = keep_acts ? keep_acts[l + 1] : s.act;
                // the MMA that read s.act has completed, so it may be overwritten
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    float v[8];
#pragma unroll
                    for (int j = 0; j < 8; j++) v[j] = fmaxf(acc[8 * c + j] + b[32 * half + 8 * c + j], 0.f);
                    store_chunk(dst, t, 4 * half + c, v);
                }
            } else {
#pragma unroll
                for (int j = 0; j < 32; j++)
                    if (32 * half + j < kOut) out[32 * half + j] = acc[j] + b[32 * half + j];
            }
        }
        tc::fence_before_sync();
    }
    return true;
}

}  // namespace mlp

// What the renderer needs of the network (mlp.cu).
struct MlpView {
    int valid;
    const uint8_t* image;   // weight images + biases
    mlp::Bounds bounds;
};
MlpView mlp_view(pgx_ctx* ctx);
int mlp_train_device(pgx_ctx* ctx, const float* samples, int64_t n, float lr, double* loss, bool update);
int mlp_query_device(pgx_ctx* ctx, const float* q, const float* aux, int64_t n, int mode, float* out, float* out2);
int mlp_online_step(pgx_ctx* ctx, const float* samples, int64_t n);
// QuadTree fallback of the learned guide: training samples counted per
// radiance-cache region; the counts of the current cache and the threshold
// below which a region counts as untrained (nullptr / 0 when off).
int mlp_count_regions(pgx_ctx* ctx, const float* samples, int64_t n);
int mlp_count_regions_reset(pgx_ctx* ctx);
const int* mlp_region_counts(pgx_ctx* ctx, int* min_samples);
int64_t mlp_train_batch(pgx_ctx* ctx);
int mlp_train_direct(pgx_ctx* ctx);
