// The learned guide's network: parameters, tensor-core forward queries,
// training (forward, loss, backward on tcgen05, Adam) and the C API
// (pgx_mlp_*).  The network and its mixture are defined in pgx_mlp.cuh.
//
// Training kernel, per 128-row tile of samples and per CTA:
//   forward: six MMAs chains as in inference, keeping every layer's input
//            tile X_l in shared memory (plus a constant-one feature column
//            after its last feature, so the weight-gradient MMA also yields
//            the bias gradient);
//   loss:    each thread turns its row's 40 outputs into dLoss/dOutput
//            (bf16, the tile dY);
//   backward, l = 5..0:
//            dW_l^T += X_l^T dY     (M = 128 input features incl. padding,
//                                    N = 64 outputs, K = 128 rows; both
//                                    operands read MN-major from the
//                                    row-major tiles; accumulated in tensor
//                                    memory across all tiles of the CTA)
//            dX = dY W_l            (l > 0; W_l's image read MN-major)
//            dY = dX * (X_l > 0)    (ReLU derivative, bf16)
// and finally each CTA adds its weight gradients to the global FP32
// gradient with one atomic per entry.
#include <cmath>
#include <cstring>
#include <vector>

#include "pgx_ctx.h"
#include "pgx_guide.cuh"
#include "pgx_mlp.cuh"

using namespace mlp;

namespace {

constexpr int kThreads = 128;

struct MlpState {
    DevBuf master, grad, m1, m2;   // kParams floats each
    DevBuf image;                  // kImageBytes weight images + kBiasFloats biases
    DevBuf scratch;                // queries / samples staged from the host
    DevBuf scratch2, scratch3;
    DevBuf loss;                   // double[2]: loss sum, weight sum
    DevBuf status;                 // int: MMA wait timeouts
    Bounds bounds{};
    float lr = 5e-3f, decay = 0.998f;
    int64_t batch = 262144;
    int steps = 4;
    int direct = 1;
    int64_t step = 0;
    bool valid = false;
    int sms = 0;
    // Training samples per radiance-cache region (the QuadTree guide's
    // regions), for the fallback: counts of cache build `count_gen`.
    DevBuf region_count;
    uint64_t count_gen = 0;
    int count_regions = 0;
    int fallback_min = 256;  // below this many samples a region uses the QuadTree guide (0: never)
};

MlpState* state(pgx_ctx* ctx) {
    if (!ctx->mlp_state) ctx->mlp_state = new MlpState();
    return static_cast<MlpState*>(ctx->mlp_state);
}

// PCG32 for the weight initialisation.
struct HostPcg {
    uint64_t s;
    explicit HostPcg(uint64_t seed) : s(pgx_rng_init(seed, 0x6d6c70ULL, 0)) {}
    float next() { return pgx_rng_next(s); }
};

// ---- weight images ------------------------------------------------------------------
__global__ void k_images(const float* __restrict__ master, uint8_t* __restrict__ image) {
    float* bias = reinterpret_cast<float*>(image + kImageBytes);
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    int stride = gridDim.x * blockDim.x;
    for (int l = 0; l < kLayers; l++) {
        const int K = layer_k(l), N = layer_n(l);
        __nv_bfloat16* img = reinterpret_cast<__nv_bfloat16*>(image + image_offset(l));
        for (int i = tid; i < kHid * K; i += stride) {
            int n = i / K, k = i % K;
            float v = n < N ? master[param_w(l) + n * K + k] : 0.f;
            img[tc::tile_offset(kHid, n, k) / 2] = __float2bfloat16_rn(v);
        }
        for (int j = tid; j < kHid; j += stride) bias[l * kHid + j] = j < N ? master[param_b(l) + j] : 0.f;
    }
}

// Loads the weight images and biases into shared memory (16-byte copies).
__device__ __forceinline__ void load_weights(const uint8_t* __restrict__ image, uint8_t* w, float* bias) {
    const uint4* src = reinterpret_cast<const uint4*>(image);
    uint4* dst = reinterpret_cast<uint4*>(w);
    for (int i = threadIdx.x; i < kImageBytes / 16; i += blockDim.x) dst[i] = src[i];
    const float* b = reinterpret_cast<const float*>(image + kImageBytes);
    for (int i = threadIdx.x; i < kBiasFloats; i += blockDim.x) bias[i] = b[i];
}

// ---- forward queries ------------------------------------------------------------------
enum QueryMode { Q_RAW = 0, Q_PDF = 1, Q_SAMPLE = 2 };

constexpr int kFwdSmem = kImageBytes + kBiasFloats * 4 + (kIn / 8) * kChunk;

__global__ void __launch_bounds__(kThreads) k_query(const uint8_t* __restrict__ image, Bounds bnd,
                                                    const float* __restrict__ q, const float* __restrict__ aux,
                                                    int64_t n, int mode, float* __restrict__ out,
                                                    float* __restrict__ out2, int* status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tslot;
    __shared__ int flag;
    FwdSmem s;
    s.w = smem;
    s.bias = reinterpret_cast<float*>(smem + kImageBytes);
    s.act = smem + kImageBytes + kBiasFloats * 4;
    s.mbar = &mbar;
    s.flag = &flag;
    s.bar = 1;
    s.tg = threadIdx.x;
    load_weights(image, s.w, s.bias);
    if (threadIdx.x == 0) tc::mbar_init(&mbar, 1);
    if (threadIdx.x < 32) {
        tc::tmem_alloc(&tslot, 64);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    s.tmem = tslot;
    uint32_t phase = 0;
    const int64_t ntiles = (n + kRows - 1) / kRows;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t r = tile * kRows + threadIdx.x;
        const bool live = r < n;
        F3 x = zero3(), nn = zero3(), wo = zero3();
        if (live) {
            const float* p = q + r * 9;
            x = f3(p[0], p[1], p[2]);
            nn = f3(p[3], p[4], p[5]);
            wo = f3(p[6], p[7], p[8]);
        }
        encode_row(s.act, threadIdx.x, bnd, x, nn, wo);
        float raw[kOut];
        if (!forward_tile(s, phase, raw)) {
            if (threadIdx.x == 0) atomicAdd(status, 1);
            break;
        }
        if (!live) continue;
        if (mode == Q_RAW) {
            for (int j = 0; j < kOut; j++) out[r * kOut + j] = raw[j];
        } else {
            // the renderer's packed form, so these queries see its numbers
            float4 g[kPacked];
            pack_mixture(raw, g);
            if (mode == Q_PDF) {
                const float* w = aux + r * 3;
                out[r] = packed_pdf(g, f3(w[0], w[1], w[2]));
            } else {
                const float* u = aux + r * 3;
                F3 w = packed_sample(g, u[0], u[1], u[2]);
                out[r * 3] = w.x;
                out[r * 3 + 1] = w.y;
                out[r * 3 + 2] = w.z;
                out2[r] = packed_pdf(g, w);
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_dealloc(s.tmem, 64);
}

// ---- training -----------------------------------------------------------------------------
// Shared memory: X_0 (11 chunks), X_1..X_5 (9 chunks each), dY (8 chunks),
// weight images, biases.  The weight-gradient MMA reads 16 chunks from each
// X_l; for X_5 the last 7 fall into dY, which is inside the allocation.
constexpr int kX0Chunks = kIn / 8 + 1;
constexpr int kXChunks = kHid / 8 + 1;
__host__ __device__ constexpr int x_offset(int l) { return l == 0 ? 0 : (kX0Chunks + (l - 1) * kXChunks) * kChunk; }
constexpr int kDyOffset = x_offset(kLayers);
constexpr int kTrainWOffset = kDyOffset + (kHid / 8) * kChunk;
constexpr int kTrainSmem = kTrainWOffset + kImageBytes + kBiasFloats * 4;
static_assert(x_offset(kLayers - 1) + 16 * kChunk <= kTrainWOffset, "weight-gradient reads stay in the tiles");
static_assert(kTrainSmem <= 227 * 1024, "training tile fits in shared memory");
constexpr uint32_t kTrainCols = 512;  // 64 (forward / dX) + 6 x 64 (dW^T)

// Sample record: position, normal, wo, wi, weight (13 floats).
constexpr int kSampleFloats = 13;

__global__ void __launch_bounds__(kThreads, 1) k_train(const uint8_t* __restrict__ image, Bounds bnd,
                                                       const float* __restrict__ samples, int64_t n,
                                                       const double* __restrict__ wsum, float* __restrict__ grad,
                                                       double* __restrict__ loss_out, int* status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tslot;
    __shared__ int flag;
    const int t = threadIdx.x, warp = t >> 5;
    FwdSmem s;
    s.w = smem + kTrainWOffset;
    s.bias = reinterpret_cast<float*>(smem + kTrainWOffset + kImageBytes);
    s.act = smem + x_offset(0);
    s.mbar = &mbar;
    s.flag = &flag;
    s.bar = 1;
    s.tg = t;
    uint8_t* xs[kLayers];
    for (int l = 0; l < kLayers; l++) xs[l] = smem + x_offset(l);
    uint8_t* dy = smem + kDyOffset;
    load_weights(image, s.w, s.bias);
    // constant-one feature after each tile's last feature (never read by the
    // forward MMAs, which stop at K)
    for (int l = 0; l < kLayers; l++) {
        float one[8] = {1.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        store_chunk(xs[l], t, layer_k(l) / 8, one);
    }
    if (t == 0) tc::mbar_init(&mbar, 1);
    if (t < 32) {
        tc::tmem_alloc(&tslot, kTrainCols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    s.tmem = tslot;
    const float scale = (float)(1.0 / fmax(*wsum, 1e-30));  // loss = sum(w l) / sum(w)
    uint32_t phase = 0;
    bool first = true, failed = false;
    double loss_acc = 0.0;
    const int64_t ntiles = (n + kRows - 1) / kRows;
    for (int64_t tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        const int64_t r = tile * kRows + t;
        const bool live = r < n;
        F3 x = zero3(), nn = zero3(), wo = zero3(), wi = f3(0.f, 0.f, 1.f);
        float wgt = 0.f;
        if (live) {
            const float* p = samples + r * kSampleFloats;
            x = f3(p[0], p[1], p[2]);
            nn = f3(p[3], p[4], p[5]);
            wo = f3(p[6], p[7], p[8]);
            wi = f3(p[9], p[10], p[11]);
            wgt = p[12];
        }
        encode_row(s.act, t, bnd, x, nn, wo);
        float raw[kOut];
        if (!forward_tile(s, phase, raw, xs)) {
            failed = true;
            break;
        }
        float d[kOut];
        float l = loss_grad(raw, wi, wgt * scale, d);
        if (live) loss_acc += (double)l;
        {
            float v[8];
#pragma unroll
            for (int c = 0; c < kHid / 8; c++) {
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    int f = 8 * c + j;
                    v[j] = (live && f < kOut) ? d[f] : 0.f;
                }
                store_chunk(dy, t, c, v);
            }
        }
        for (int lay = kLayers - 1; lay >= 0; lay--) {
            publish_smem(s.bar);
            if (t == 0) {
                // dW^T (+)= X^T dY
                const uint32_t xa = tc::smem_addr(xs[lay]), ya = tc::smem_addr(dy);
                const uint32_t id_w = tc::idesc_bf16(kRows, kHid, true, true);
                for (int k = 0; k < kRows / 16; k++) {
                    uint64_t ad = tc::smem_desc(xa + k * 256, 128, kChunk);
                    uint64_t bd = tc::smem_desc(ya + k * 256, 128, kChunk);
                    tc::mma_bf16(s.tmem + kHid + kHid * lay, ad, bd, id_w, !(first && k == 0));
                }
                if (lay > 0) {
                    // dX = dY W
                    const uint32_t wa = tc::smem_addr(s.w + image_offset(lay));
                    const uint32_t id_x = tc::idesc_bf16(kRows, kHid, false, true);
                    for (int k = 0; k < kHid / 16; k++) {
                        uint64_t ad = tc::smem_desc(ya + k * 2 * kChunk, kChunk, 128);
                        uint64_t bd = tc::smem_desc(wa + k * 256, 128, kHid * 16);
                        tc::mma_bf16(s.tmem, ad, bd, id_x, k > 0);
                    }
                }
                tc::mma_commit(&mbar);
            }
            if (!group_wait(s, phase)) {
                failed = true;
                break;
            }
            if (lay > 0) {
                float acc[64];
                tc::tmem_ld32(tc::tmem_at(s.tmem, warp * 32, 0), acc);
                tc::tmem_ld32(tc::tmem_at(s.tmem, warp * 32, 32), acc + 32);
#pragma unroll
                for (int c = 0; c < kHid / 8; c++) {
                    float xv[8], v[8];
                    load_chunk(xs[lay], t, c, xv);
#pragma unroll
                    for (int j = 0; j < 8; j++) v[j] = xv[j] > 0.f ? acc[8 * c + j] : 0.f;
                    store_chunk(dy, t, c, v);
                }
            }
            tc::fence_before_sync();
        }
        first = false;
    }
    if (failed) {
        if (t == 0) atomicAdd(status, 1);
    } else if (!first) {
        // this CTA's weight gradients: row t of dW_l^T is input feature t
        for (int lay = 0; lay < kLayers; lay++) {
            const int K = layer_k(lay), N = layer_n(lay);
            float acc[64];
            tc::tmem_ld32(tc::tmem_at(s.tmem + kHid + kHid * lay, warp * 32, 0), acc);
            tc::tmem_ld32(tc::tmem_at(s.tmem + kHid + kHid * lay, warp * 32, 32), acc + 32);
            if (t < K) {
                for (int j = 0; j < N; j++) atomicAdd(&grad[param_w(lay) + j * K + t], acc[j]);
            } else if (t == K) {
                for (int j = 0; j < N; j++) atomicAdd(&grad[param_b(lay) + j], acc[j]);
            }
        }
    }
    // loss: warp sums, one atomic per warp
    for (int o = 16; o > 0; o >>= 1) loss_acc += __shfl_xor_sync(0xffffffffu, loss_acc, o);
    if ((t & 31) == 0) atomicAdd(loss_out, loss_acc);
    tc::fence_before_sync();
    __syncthreads();
    if (t < 32) tc::tmem_dealloc(s.tmem, kTrainCols);
}

__global__ void k_weight_sum(const float* __restrict__ samples, int64_t n, double* out) {
    double acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc += (double)samples[i * kSampleFloats + 12];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    float gi = g[i];
    if (!isfinite(gi)) gi = 0.f;
    float a = b1 * m1[i] + (1.f - b1) * gi;
    float b = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    p[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
}

int ensure_ready(pgx_ctx* ctx, const char* who) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    PGX_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    MlpState* st = state(ctx);
    if (!st->valid) return pgx_fail(ctx, PGX_ERR_STATE, "%s: call pgx_mlp_init first", who);
    return PGX_OK;
}

int refresh_images(pgx_ctx* ctx) {
    MlpState* st = state(ctx);
    k_images<<<64, 256, 0, ctx->stream>>>(st->master.as<float>(), st->image.as<uint8_t>());
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    return PGX_OK;
}

int check_status(pgx_ctx* ctx, const char* who) {
    MlpState* st = state(ctx);
    int status = 0;
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&status, st->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (status != 0) return pgx_fail(ctx, PGX_ERR_TIMEOUT, "%s: tensor-core wait timed out in %d CTA(s)", who, status);
    return PGX_OK;
}

// Training samples (13 floats, position first) per radiance-cache region.
__global__ void k_count_regions(GuideView gv, const float* __restrict__ samples, int64_t n, int* __restrict__ counts) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float* sm = samples + i * kSampleFloats;
        const int r = guide_region_index(gv, f3(sm[0], sm[1], sm[2]));
        if (r >= 0) atomicAdd(counts + r, 1);
    }
}

}  // namespace

// ---- internal entry points for the renderer -------------------------------------------------
void mlp_state_free(pgx_ctx* ctx) {
    delete static_cast<MlpState*>(ctx->mlp_state);
    ctx->mlp_state = nullptr;
}

MlpView mlp_view(pgx_ctx* ctx) {
    MlpView v{};
    MlpState* st = ctx->mlp_state ? static_cast<MlpState*>(ctx->mlp_state) : nullptr;
    if (!st || !st->valid) return v;
    v.valid = 1;
    v.image = st->image.as<uint8_t>();
    v.bounds = st->bounds;
    return v;
}

int mlp_train_device(pgx_ctx* ctx, const float* samples, int64_t n, float lr, double* loss, bool update) {
    MlpState* st = state(ctx);
    if (n <= 0) return PGX_OK;
    cudaStream_t s = ctx->stream;
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(st->grad.p, 0, kParams * sizeof(float), s));
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(st->loss.p, 0, 2 * sizeof(double), s));
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(st->status.p, 0, sizeof(int), s));
    double* d_loss = st->loss.as<double>();
    k_weight_sum<<<std::min<int64_t>(1024, (n + 255) / 256), 256, 0, s>>>(samples, n, d_loss + 1);
    PGX_CUDA_TRY(ctx, cudaFuncSetAttribute(k_train, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrainSmem));
    const int64_t ntiles = (n + kRows - 1) / kRows;
    const int grid = (int)std::min<int64_t>(ntiles, st->sms);
    k_train<<<grid, kThreads, kTrainSmem, s>>>(st->image.as<uint8_t>(), st->bounds, samples, n, d_loss + 1,
                                               st->grad.as<float>(), d_loss, st->status.as<int>());
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    if (update) {
        st->step++;
        const float b1 = 0.9f, b2 = 0.99f;
        const float c1 = 1.f - powf(b1, (float)st->step), c2 = 1.f - powf(b2, (float)st->step);
        k_adam<<<(kParams + 255) / 256, 256, 0, s>>>(st->master.as<float>(), st->grad.as<float>(),
                                                      st->m1.as<float>(), st->m2.as<float>(), lr, b1, b2, 1e-8f,
                                                      c1, c2);
        PGX_CUDA_TRY(ctx, cudaGetLastError());
        PGX_TRY(refresh_images(ctx));
    }
    if (loss) {
        double h[2];
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(h, d_loss, sizeof(h), cudaMemcpyDeviceToHost, s));
        PGX_TRY(check_status(ctx, "pgx_mlp_train"));
        *loss = h[0];
    }
    return PGX_OK;
}

int mlp_query_device(pgx_ctx* ctx, const float* q, const float* aux, int64_t n, int mode, float* out, float* out2) {
    MlpState* st = state(ctx);
    PGX_CUDA_TRY(ctx, cudaFuncSetAttribute(k_query, cudaFuncAttributeMaxDynamicSharedMemorySize, kFwdSmem));
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(st->status.p, 0, sizeof(int), ctx->stream));
    const int64_t ntiles = (n + kRows - 1) / kRows;
    const int grid = (int)std::min<int64_t>(ntiles, (int64_t)st->sms * 3);
    if (grid > 0)
        k_query<<<grid, kThreads, kFwdSmem, ctx->stream>>>(st->image.as<uint8_t>(), st->bounds, q, aux, n, mode, out,
                                                            out2, st->status.as<int>());
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    return PGX_OK;
}

// ---- C API -------------------------------------------------------------------------------------
extern "C" int pgx_mlp_init(pgx_ctx* ctx, uint64_t seed, const float* bmin, const float* bmax) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    PGX_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    float lo[3], hi[3];
    if (bmin && bmax) {
        for (int i = 0; i < 3; i++) lo[i] = bmin[i], hi[i] = bmax[i];
    } else if (ctx->has_scene) {
        for (int i = 0; i < 3; i++) lo[i] = ctx->bounds.bmin[i], hi[i] = ctx->bounds.bmax[i];
    } else {
        return pgx_fail(ctx, PGX_ERR_STATE, "pgx_mlp_init: no bounds given and no scene uploaded");
    }
    MlpState* st = state(ctx);
    for (int i = 0; i < 3; i++) {
        float ext = hi[i] - lo[i];
        if (!(ext > 0.f) || !std::isfinite(ext)) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_mlp_init: empty bounds");
        st->bounds.bmin[i] = lo[i];
        st->bounds.inv_ext[i] = 1.f / ext;
    }
    int dev_sms = 0;
    PGX_CUDA_TRY(ctx, cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device));
    st->sms = dev_sms;
    // He-uniform weights for the ReLU layers, a 10x smaller last layer so
    // the initial mixture is broad; zero biases.
    std::vector<float> p(kParams, 0.f);
    HostPcg rng(seed);
    for (int l = 0; l < kLayers; l++) {
        const int K = layer_k(l), N = layer_n(l);
        float a = sqrtf(6.f / (float)(l == 0 ? 78 : K));
        if (l == kLayers - 1) a *= 0.1f;
        for (int i = 0; i < N * K; i++) p[param_w(l) + i] = (2.f * rng.next() - 1.f) * a;
    }
    size_t pb = kParams * sizeof(float);
    PGX_CUDA_TRY(ctx, st->master.reserve(pb));
    PGX_CUDA_TRY(ctx, st->grad.reserve(pb));
    PGX_CUDA_TRY(ctx, st->m1.reserve(pb));
    PGX_CUDA_TRY(ctx, st->m2.reserve(pb));
    PGX_CUDA_TRY(ctx, st->image.reserve(kImageBytes + kBiasFloats * 4));
    PGX_CUDA_TRY(ctx, st->loss.reserve(2 * sizeof(double)));
    PGX_CUDA_TRY(ctx, st->status.reserve(sizeof(int)));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(st->master.p, p.data(), pb, cudaMemcpyHostToDevice, ctx->stream));
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(st->m1.p, 0, pb, ctx->stream));
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(st->m2.p, 0, pb, ctx->stream));
    st->step = 0;
    st->valid = true;
    st->count_gen = 0;  // a new network has seen no samples anywhere
    PGX_TRY(refresh_images(ctx));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return PGX_OK;
}

extern "C" int pgx_mlp_get_params(pgx_ctx* ctx, float* params) {
    PGX_TRY(ensure_ready(ctx, "pgx_mlp_get_params"));
    if (!params) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_mlp_get_params: null output");
    MlpState* st = state(ctx);
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(params, st->master.p, kParams * sizeof(float), cudaMemcpyDeviceToHost,
                                      ctx->stream));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return PGX_OK;
}

extern "C" int pgx_mlp_set_params(pgx_ctx* ctx, const float* params) {
    PGX_TRY(ensure_ready(ctx, "pgx_mlp_set_params"));
    if (!params) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_mlp_set_params: null input");
    MlpState* st = state(ctx);
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(st->master.p, params, kParams * sizeof(float), cudaMemcpyHostToDevice,
                                      ctx->stream));
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(st->m1.p, 0, kParams * sizeof(float), ctx->stream));
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(st->m2.p, 0, kParams * sizeof(float), ctx->stream));
    st->step = 0;
    st->count_gen = 0;  // parameters from elsewhere: no samples counted against the cache
    PGX_TRY(refresh_images(ctx));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return PGX_OK;
}

static int query_host(pgx_ctx* ctx, const float* queries, const float* aux, int64_t n, int mode, float* out,
                      float* out2, const char* who) {
    PGX_TRY(ensure_ready(ctx, who));
    if (n < 0 || (n > 0 && (!queries || !out))) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "%s: bad arguments", who);
    if (n == 0) return PGX_OK;
    MlpState* st = state(ctx);
    const size_t qb = (size_t)n * 9 * sizeof(float);
    const size_t ab = (size_t)n * 3 * sizeof(float);
    const size_t ob = (size_t)n * (mode == Q_RAW ? kOut : (mode == Q_PDF ? 1 : 3)) * sizeof(float);
    PGX_CUDA_TRY(ctx, st->scratch.reserve(qb + ab));
    PGX_CUDA_TRY(ctx, st->scratch2.reserve(ob));
    PGX_CUDA_TRY(ctx, st->scratch3.reserve((size_t)n * sizeof(float)));
    float* dq = st->scratch.as<float>();
    float* da = reinterpret_cast<float*>(st->scratch.as<uint8_t>() + qb);
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(dq, queries, qb, cudaMemcpyHostToDevice, ctx->stream));
    if (aux) PGX_CUDA_TRY(ctx, cudaMemcpyAsync(da, aux, ab, cudaMemcpyHostToDevice, ctx->stream));
    PGX_TRY(mlp_query_device(ctx, dq, da, n, mode, st->scratch2.as<float>(), st->scratch3.as<float>()));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(out, st->scratch2.p, ob, cudaMemcpyDeviceToHost, ctx->stream));
    if (out2)
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(out2, st->scratch3.p, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost,
                                          ctx->stream));
    return check_status(ctx, who);
}

extern "C" int pgx_mlp_forward(pgx_ctx* ctx, const float* queries, int64_t n, float* raw) {
    return query_host(ctx, queries, nullptr, n, Q_RAW, raw, nullptr, "pgx_mlp_forward");
}

extern "C" int pgx_mlp_pdf(pgx_ctx* ctx, const float* queries, const float* dirs, int64_t n, float* pdf) {
    if (ctx && n > 0 && !dirs) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_mlp_pdf: null dirs");
    return query_host(ctx, queries, dirs, n, Q_PDF, pdf, nullptr, "pgx_mlp_pdf");
}

extern "C" int pgx_mlp_sample(pgx_ctx* ctx, const float* queries, const float* u3, int64_t n, float* dirs, float* pdf) {
    if (ctx && n > 0 && (!u3 || !pdf)) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_mlp_sample: null argument");
    return query_host(ctx, queries, u3, n, Q_SAMPLE, dirs, pdf, "pgx_mlp_sample");
}

static int train_host(pgx_ctx* ctx, const pgx_radiance_sample* samples, int64_t n, float lr, double* loss,
                      float* grad_out, bool update, const char* who) {
    PGX_TRY(ensure_ready(ctx, who));
    if (n <= 0 || !samples) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "%s: no samples", who);
    static_assert(sizeof(pgx_radiance_sample) == kSampleFloats * sizeof(float), "sample layout");
    MlpState* st = state(ctx);
    const size_t sb = (size_t)n * sizeof(pgx_radiance_sample);
    PGX_CUDA_TRY(ctx, st->scratch.reserve(sb));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(st->scratch.p, samples, sb, cudaMemcpyHostToDevice, ctx->stream));
    double l = 0.0;
    PGX_TRY(mlp_train_device(ctx, st->scratch.as<float>(), n, lr, &l, update));
    if (update) PGX_TRY(mlp_count_regions(ctx, st->scratch.as<float>(), n));
    if (loss) *loss = l;
    if (grad_out) {
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(grad_out, st->grad.p, kParams * sizeof(float), cudaMemcpyDeviceToHost,
                                          ctx->stream));
        PGX_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return PGX_OK;
}

extern "C" int pgx_mlp_gradient(pgx_ctx* ctx, const pgx_radiance_sample* samples, int64_t n, float* grad, double* loss) {
    if (ctx && !grad) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_mlp_gradient: null gradient");
    return train_host(ctx, samples, n, 0.f, loss, grad, false, "pgx_mlp_gradient");
}

extern "C" int pgx_mlp_train_step(pgx_ctx* ctx, const pgx_radiance_sample* samples, int64_t n, float lr, double* loss) {
    return train_host(ctx, samples, n, lr, loss, nullptr, true, "pgx_mlp_train_step");
}

extern "C" int pgx_mlp_configure(pgx_ctx* ctx, float lr, float decay, int64_t batch, int32_t steps,
                                 int32_t direct) {
    PGX_TRY(ensure_ready(ctx, "pgx_mlp_configure"));
    if (!(lr > 0.f) || !(decay > 0.f) || decay > 1.f || batch <= 0 || steps <= 0 || steps > 64 ||
        (direct != 0 && direct != 1))
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_mlp_configure: bad arguments");
    MlpState* st = state(ctx);
    st->lr = lr;
    st->decay = decay;
    st->batch = batch;
    st->steps = steps;
    st->direct = direct;
    return PGX_OK;
}

int mlp_train_direct(pgx_ctx* ctx) { return state(ctx)->direct; }

// Online training inside pgx_render: `steps` Adam steps on consecutive
// slices of the frame's samples (the last slice only if at least a quarter
// of a batch), learning rate lr * decay^step.
int mlp_online_step(pgx_ctx* ctx, const float* samples, int64_t n) {
    MlpState* st = state(ctx);
    if (!st->valid || n <= 0) return PGX_OK;
    int64_t used = 0;
    for (int k = 0; k < st->steps; k++) {
        int64_t off = (int64_t)k * st->batch;
        int64_t nk = std::min(st->batch, n - off);
        if (nk <= 0 || (k > 0 && nk < st->batch / 4)) break;
        float lr = st->lr * powf(st->decay, (float)st->step);
        PGX_TRY(mlp_train_device(ctx, samples + off * kSampleFloats, nk, lr, nullptr, true));
        used = off + nk;
    }
    return mlp_count_regions(ctx, samples, used);
}

// Adds the training samples' positions to the per-region counts of the
// current radiance cache (reset whenever the cache or the network is new).
int mlp_count_regions(pgx_ctx* ctx, const float* samples, int64_t n) {
    MlpState* st = state(ctx);
    if (!st->valid || n <= 0 || !guide_ready(ctx)) return PGX_OK;
    const GuideView gv = guide_view(ctx);
    if (gv.pss) return PGX_OK;  // primary-sample trees cannot stand in for directions
    const uint64_t gen = guide_generation(ctx);
    const int nreg = guide_regions(ctx);
    if (nreg <= 0) return PGX_OK;
    if (st->count_gen != gen || st->count_regions != nreg) {
        PGX_CUDA_TRY(ctx, st->region_count.reserve(sizeof(int) * (size_t)nreg));
        PGX_CUDA_TRY(ctx, cudaMemsetAsync(st->region_count.p, 0, sizeof(int) * (size_t)nreg, ctx->stream));
        st->count_gen = gen;
        st->count_regions = nreg;
    }
    k_count_regions<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, ctx->stream>>>(
        gv, samples, n, st->region_count.as<int>());
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    return PGX_OK;
}

const int* mlp_region_counts(pgx_ctx* ctx, int* min_samples) {
    MlpState* st = ctx->mlp_state ? static_cast<MlpState*>(ctx->mlp_state) : nullptr;
    *min_samples = 0;
    if (!st || !st->valid || st->fallback_min <= 0 || !guide_ready(ctx)) return nullptr;
    if (guide_view(ctx).pss || guide_regions(ctx) <= 0) return nullptr;
    if (st->count_gen != guide_generation(ctx) || st->count_regions != guide_regions(ctx)) {
        // nothing counted against this cache yet: every region is untrained
        if (mlp_count_regions_reset(ctx) != PGX_OK) return nullptr;
    }
    *min_samples = st->fallback_min;
    return st->region_count.as<int>();
}

int mlp_count_regions_reset(pgx_ctx* ctx) {
    MlpState* st = state(ctx);
    const int nreg = guide_regions(ctx);
    PGX_CUDA_TRY(ctx, st->region_count.reserve(sizeof(int) * (size_t)std::max(nreg, 1)));
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(st->region_count.p, 0, sizeof(int) * (size_t)std::max(nreg, 1), ctx->stream));
    st->count_gen = guide_generation(ctx);
    st->count_regions = nreg;
    return PGX_OK;
}

extern "C" int pgx_mlp_set_fallback(pgx_ctx* ctx, int32_t min_samples) {
    PGX_TRY(ensure_ready(ctx, "pgx_mlp_set_fallback"));
    if (min_samples < 0) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_mlp_set_fallback: negative count");
    state(ctx)->fallback_min = min_samples;
    return PGX_OK;
}

int64_t mlp_train_batch(pgx_ctx* ctx) { return state(ctx)->batch * state(ctx)->steps; }
