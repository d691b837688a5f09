// GPU binned-SAH BVH build (BVHNode::build, Geometry.h:419-446) and the
// conversion of any tree in the reference layout into the traversal layout.
//
// The build reproduces the reference's decisions exactly: centroids with
// the 0.3333f factor (Geometry.h:96-98), 16 bins over the centroid bounds
// of each axis, the left/right sweep and cost 1 + A_L/A_P*N_L*1.5 +
// A_R/A_P*N_R*1.5 against N*1.5 (Geometry.h:293-365), the partition test
// centroid[axis] < split position and the failed-split rule
// (Geometry.h:384-395), leaves at <= 4 triangles.  All of these are
// order-independent (counts, min/max, comparisons) and computed with
// unfused float ops, so every node owns the same triangle set as in the
// reference; only node numbering and the order of triangles inside a leaf
// differ (the reference partitions in place by swapping).
//
// Phase A (nodes with more than kSmall triangles) runs level by level:
// CTAs process 2048-triangle chunks of the active nodes — shared-memory
// binning, a per-node SAH sweep, then a block-scan partition into a second
// index buffer that also reduces the children's boxes.  Phase B hands each
// node of at most kSmall triangles to one thread, which finishes its
// subtree with the reference's sequential algorithm (in-place swap
// partition) and an explicit stack.
#include <algorithm>
#include <chrono>
#include <vector>

#include "pgx_ctx.h"
#include "pgx_trace.cuh"

namespace {

constexpr int kBins = 16;          // BUILD_BINS, Geometry.h:20
constexpr int kMaxLeaf = 4;        // MAXNODE_TRIANGLES, Geometry.h:17
constexpr int kSmall = 128;        // phase-B threshold
constexpr int kChunk = 2048;       // triangles per CTA chunk in phase A
constexpr int kThreads = 256;
constexpr int kPerThread = kChunk / kThreads;
constexpr int kSmallStack = 256;   // phase-B explicit stack depth
constexpr int kBinInts = 3 * kBins * 7;

struct BuildItem {
    int node;
    int start, count;
    int cmin[3], cmax[3];  // centroid bounds, ordered-int encoded
    int axis;
    float pos;
    int split;
    int lcur, rcur;
    int acc[2][12];  // per side: tbox min[3], tbox max[3], cent min[3], cent max[3] (ordered ints)
};

struct BuildMisc {
    int node_count;
    int rec_count;
    int nitems_next;
    int nsmall;
    int nchunks;
    int overflow;
    int root_acc[12];
};

__device__ __forceinline__ float area_x(float mnx, float mny, float mnz, float mxx, float mxy, float mxz) {
    // AABB::area, Geometry.h:212-215
    float sx = x_sub(mxx, mnx), sy = x_sub(mxy, mny), sz = x_sub(mxz, mnz);
    return x_mul(x_add(x_add(x_mul(sx, sy), x_mul(sy, sz)), x_mul(sx, sz)), 2.f);
}

// Triangle::centre and the triangle's vertex bounds.
__global__ void k_prep(const pgx_triangle* __restrict__ tris, int64_t n, float4* __restrict__ cent,
                       float4* __restrict__ tmin, float4* __restrict__ tmax) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const pgx_triangle& t = tris[i];
    xv3 p0 = mk(t.v[0].p[0], t.v[0].p[1], t.v[0].p[2]);
    xv3 p1 = mk(t.v[1].p[0], t.v[1].p[1], t.v[1].p[2]);
    xv3 p2 = mk(t.v[2].p[0], t.v[2].p[1], t.v[2].p[2]);
    xv3 c = x_scale(x_add(x_add(p0, p1), p2), 0.3333f);
    cent[i] = make_float4(c.x, c.y, c.z, 0.f);
    tmin[i] = make_float4(s_min(s_min(p0.x, p1.x), p2.x), s_min(s_min(p0.y, p1.y), p2.y),
                          s_min(s_min(p0.z, p1.z), p2.z), 0.f);
    tmax[i] = make_float4(s_max(s_max(p0.x, p1.x), p2.x), s_max(s_max(p0.y, p1.y), p2.y),
                          s_max(s_max(p0.z, p1.z), p2.z), 0.f);
}

__device__ __forceinline__ void warp_minmax(int& v, bool is_min) {
    for (int o = 16; o > 0; o >>= 1) {
        int w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
        v = is_min ? min(v, w) : max(v, w);
    }
}

// Root bounds: union of triangle boxes and of centroids.
__global__ void k_root_reduce(const float4* __restrict__ cent, const float4* __restrict__ tmin,
                              const float4* __restrict__ tmax, int64_t n, BuildMisc* misc) {
    int acc[12];
    for (int k = 0; k < 12; k++) acc[k] = ((k % 6) < 3) ? INT_MAX : INT_MIN;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float4 a = tmin[i], b = tmax[i], c = cent[i];
        acc[0] = min(acc[0], f2o(a.x));
        acc[1] = min(acc[1], f2o(a.y));
        acc[2] = min(acc[2], f2o(a.z));
        acc[3] = max(acc[3], f2o(b.x));
        acc[4] = max(acc[4], f2o(b.y));
        acc[5] = max(acc[5], f2o(b.z));
        acc[6] = min(acc[6], f2o(c.x));
        acc[7] = min(acc[7], f2o(c.y));
        acc[8] = min(acc[8], f2o(c.z));
        acc[9] = max(acc[9], f2o(c.x));
        acc[10] = max(acc[10], f2o(c.y));
        acc[11] = max(acc[11], f2o(c.z));
    }
    for (int k = 0; k < 12; k++) {
        bool is_min = (k % 6) < 3;
        warp_minmax(acc[k], is_min);
        if ((threadIdx.x & 31) == 0) {
            if (is_min)
                atomicMin(&misc->root_acc[k], acc[k]);
            else
                atomicMax(&misc->root_acc[k], acc[k]);
        }
    }
}

__global__ void k_root_init(pgx_bvh_node* nodes, BuildItem* items, BuildMisc* misc, int64_t n, int* small) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    pgx_bvh_node& r = nodes[0];
    for (int k = 0; k < 3; k++) {
        r.bmin[k] = o2f(misc->root_acc[k]);
        r.bmax[k] = o2f(misc->root_acc[3 + k]);
    }
    r.left_first = 0;
    r.used = (int)n;
    misc->node_count = 1;
    misc->rec_count = 0;
    misc->nitems_next = 0;
    misc->nsmall = 0;
    misc->overflow = 0;
    if (n <= kMaxLeaf) return;
    if (n <= kSmall) {
        small[0] = 0;
        misc->nsmall = 1;
        return;
    }
    BuildItem& it = items[0];
    it.node = 0;
    it.start = 0;
    it.count = (int)n;
    for (int k = 0; k < 3; k++) {
        it.cmin[k] = misc->root_acc[6 + k];
        it.cmax[k] = misc->root_acc[9 + k];
    }
    misc->nitems_next = 1;
}

// One chunk descriptor per kChunk triangles of each active node.
__global__ void k_chunks(BuildItem* items, int nitems, int2* chunks, BuildMisc* misc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nitems) return;
    BuildItem& it = items[i];
    it.split = 0;
    it.lcur = 0;
    it.rcur = 0;
    for (int s = 0; s < 2; s++)
        for (int k = 0; k < 12; k++) it.acc[s][k] = ((k % 6) < 3) ? INT_MAX : INT_MIN;
    int nch = (it.count + kChunk - 1) / kChunk;
    int base = atomicAdd(&misc->nchunks, nch);
    for (int c = 0; c < nch; c++) chunks[base + c] = make_int2(i, c * kChunk);
}

__global__ void k_bins_reset(int* bins, int nitems) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nitems * kBinInts) return;
    int k = (i % kBinInts) % 7;
    bins[i] = (k == 0) ? 0 : (k < 4 ? INT_MAX : INT_MIN);
}

// Bin the centroids of each chunk (findBestSplitPlane's binning loop,
// Geometry.h:313-323) into shared memory, then merge into the node's bins.
__global__ void __launch_bounds__(kThreads) k_bin(const BuildItem* __restrict__ items, const int2* __restrict__ chunks,
                                                  const BuildMisc* __restrict__ misc, const int* __restrict__ idx,
                                                  const float4* __restrict__ cent, const float4* __restrict__ tmin,
                                                  const float4* __restrict__ tmax, int* __restrict__ gbins) {
    __shared__ int sb[kBinInts];
    const int nchunks = misc->nchunks;
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        int2 ch = chunks[c];
        const BuildItem& it = items[ch.x];
        for (int k = threadIdx.x; k < kBinInts; k += blockDim.x) {
            int f = k % 7;
            sb[k] = (f == 0) ? 0 : (f < 4 ? INT_MAX : INT_MIN);
        }
        __syncthreads();
        float lo[3], scale[3];
        bool active[3];
        for (int ax = 0; ax < 3; ax++) {
            lo[ax] = o2f(it.cmin[ax]);
            float hi = o2f(it.cmax[ax]);
            active[ax] = !(lo[ax] == hi);
            scale[ax] = x_div((float)kBins, x_sub(hi, lo[ax]));
        }
        int end = min(it.count, ch.y + kChunk);
        for (int j = ch.y + threadIdx.x; j < end; j += blockDim.x) {
            int id = idx[it.start + j];
            float4 cc = cent[id];
            float4 a = tmin[id], b = tmax[id];
            float cv[3] = {cc.x, cc.y, cc.z};
            for (int ax = 0; ax < 3; ax++) {
                if (!active[ax]) continue;
                int bi = (int)x_mul(x_sub(cv[ax], lo[ax]), scale[ax]);
                bi = (bi < kBins - 1) ? bi : kBins - 1;
                int* b7 = sb + (ax * kBins + bi) * 7;
                atomicAdd(b7, 1);
                atomicMin(b7 + 1, f2o(a.x));
                atomicMin(b7 + 2, f2o(a.y));
                atomicMin(b7 + 3, f2o(a.z));
                atomicMax(b7 + 4, f2o(b.x));
                atomicMax(b7 + 5, f2o(b.y));
                atomicMax(b7 + 6, f2o(b.z));
            }
        }
        __syncthreads();
        int* g = gbins + (size_t)ch.x * kBinInts;
        for (int k = threadIdx.x; k < kBinInts; k += blockDim.x) {
            int bin_base = (k / 7) * 7;
            if (sb[bin_base] == 0) continue;
            int f = k % 7;
            if (f == 0)
                atomicAdd(g + k, sb[k]);
            else if (f < 4)
                atomicMin(g + k, sb[k]);
            else
                atomicMax(g + k, sb[k]);
        }
        __syncthreads();
    }
}

// Sweep of findBestSplitPlane (Geometry.h:325-362) for one axis given its
// bins; updates best/axis/pos exactly like the reference's loop.
__device__ void sweep_axis(const int* cnt, const float (*bmn)[3], const float (*bmx)[3], float lo, float hi,
                           float parent_area, int ax, float& best, int& axis, float& pos) {
    float left_area[kBins - 1], right_area[kBins - 1];
    int left_count[kBins - 1], right_count[kBins - 1];
    int lsum = 0, rsum = 0;
    float lmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lmx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    float rmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rmx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int i = 0; i < kBins - 1; i++) {
        lsum += cnt[i];
        left_count[i] = lsum;
        if (cnt[i] > 0) {
            for (int k = 0; k < 3; k++) {
                lmx[k] = s_max(lmx[k], bmn[i][k]);
                lmn[k] = s_min(lmn[k], bmn[i][k]);
            }
            for (int k = 0; k < 3; k++) {
                lmx[k] = s_max(lmx[k], bmx[i][k]);
                lmn[k] = s_min(lmn[k], bmx[i][k]);
            }
        }
        left_area[i] = (lsum > 0) ? area_x(lmn[0], lmn[1], lmn[2], lmx[0], lmx[1], lmx[2]) : 0.f;
        int r = kBins - 1 - i;
        rsum += cnt[r];
        right_count[kBins - 2 - i] = rsum;
        if (cnt[r] > 0) {
            for (int k = 0; k < 3; k++) {
                rmx[k] = s_max(rmx[k], bmn[r][k]);
                rmn[k] = s_min(rmn[k], bmn[r][k]);
            }
            for (int k = 0; k < 3; k++) {
                rmx[k] = s_max(rmx[k], bmx[r][k]);
                rmn[k] = s_min(rmn[k], bmx[r][k]);
            }
        }
        right_area[kBins - 2 - i] = (rsum > 0) ? area_x(rmn[0], rmn[1], rmn[2], rmx[0], rmx[1], rmx[2]) : 0.f;
    }
    float scale = x_div(x_sub(hi, lo), (float)kBins);
    for (int i = 0; i < kBins - 1; i++) {
        float la = x_div(left_area[i], parent_area);
        float ra = x_div(right_area[i], parent_area);
        float cost = x_add(x_add(1.f, x_mul(x_mul(la, (float)left_count[i]), 1.5f)),
                           x_mul(x_mul(ra, (float)right_count[i]), 1.5f));
        float cand = x_add(lo, x_mul(scale, (float)(i + 1)));
        if (cost < best) {
            pos = cand;
            axis = ax;
            best = cost;
        }
    }
}

// SAH decision per active node (subdivide, Geometry.h:367-381).
__global__ void k_split(BuildItem* items, int nitems, const int* __restrict__ gbins, pgx_bvh_node* nodes) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nitems) return;
    BuildItem& it = items[i];
    pgx_bvh_node& nd = nodes[it.node];
    float parent_area = area_x(nd.bmin[0], nd.bmin[1], nd.bmin[2], nd.bmax[0], nd.bmax[1], nd.bmax[2]);
    float best = FLT_MAX, pos = -FLT_MAX;
    int axis = -1;
    const int* g = gbins + (size_t)i * kBinInts;
    for (int ax = 0; ax < 3; ax++) {
        float lo = o2f(it.cmin[ax]), hi = o2f(it.cmax[ax]);
        if (lo == hi) continue;
        int cnt[kBins];
        float bmn[kBins][3], bmx[kBins][3];
        for (int b = 0; b < kBins; b++) {
            const int* b7 = g + (ax * kBins + b) * 7;
            cnt[b] = b7[0];
            for (int k = 0; k < 3; k++) {
                bmn[b][k] = o2f(b7[1 + k]);
                bmx[b][k] = o2f(b7[4 + k]);
            }
        }
        sweep_axis(cnt, bmn, bmx, lo, hi, parent_area, ax, best, axis, pos);
    }
    float no_split = x_mul((float)it.count, 1.5f);
    if (best >= no_split || axis == -1) {
        it.split = 0;
        nd.left_first = it.start;
        nd.used = it.count;
        return;
    }
    it.split = 1;
    it.axis = axis;
    it.pos = pos;
}

// Partition of each chunk by centroid[axis] < pos (Geometry.h:384-391) into
// the second index buffer, plus the children's box and centroid bounds.
__global__ void __launch_bounds__(kThreads) k_partition(BuildItem* __restrict__ items, const int2* __restrict__ chunks,
                                                        const BuildMisc* __restrict__ misc, const int* __restrict__ idx,
                                                        int* __restrict__ idx2, const float4* __restrict__ cent,
                                                        const float4* __restrict__ tmin,
                                                        const float4* __restrict__ tmax) {
    __shared__ int s_warp_l[kThreads / 32], s_warp_r[kThreads / 32];
    __shared__ int s_base_l, s_base_r;
    __shared__ int s_acc[24];
    const int nchunks = misc->nchunks;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        int2 ch = chunks[c];
        BuildItem& it = items[ch.x];
        if (!it.split) continue;  // uniform per block
        if (threadIdx.x < 24) s_acc[threadIdx.x] = ((threadIdx.x % 6) < 3) ? INT_MAX : INT_MIN;
        const int axis = it.axis;
        const float pos = it.pos;
        const int end = min(it.count, ch.y + kChunk);
        // Thread t owns positions ch.y + k*kThreads + t (coalesced reads).
        int ids[kPerThread];
        unsigned sides = 0;
        int nl = 0, nr = 0;
        int acc[24];
        for (int k = 0; k < 24; k++) acc[k] = ((k % 6) < 3) ? INT_MAX : INT_MIN;
        for (int k = 0; k < kPerThread; k++) {
            int j = ch.y + k * kThreads + threadIdx.x;
            ids[k] = -1;
            if (j >= end) continue;
            int id = idx[it.start + j];
            ids[k] = id;
            float4 cc = cent[id];
            float cv = axis == 0 ? cc.x : (axis == 1 ? cc.y : cc.z);
            int side = (cv < pos) ? 0 : 1;
            sides |= (unsigned)side << k;
            if (side == 0)
                nl++;
            else
                nr++;
            float4 a = tmin[id], b = tmax[id];
            int* s = acc + side * 12;
            s[0] = min(s[0], f2o(a.x));
            s[1] = min(s[1], f2o(a.y));
            s[2] = min(s[2], f2o(a.z));
            s[3] = max(s[3], f2o(b.x));
            s[4] = max(s[4], f2o(b.y));
            s[5] = max(s[5], f2o(b.z));
            s[6] = min(s[6], f2o(cc.x));
            s[7] = min(s[7], f2o(cc.y));
            s[8] = min(s[8], f2o(cc.z));
            s[9] = max(s[9], f2o(cc.x));
            s[10] = max(s[10], f2o(cc.y));
            s[11] = max(s[11], f2o(cc.z));
        }
        // Exclusive scan of nl / nr across the block.
        int il = nl, ir = nr;
        for (int o = 1; o < 32; o <<= 1) {
            int tl = __shfl_up_sync(0xFFFFFFFFu, il, o);
            int tr = __shfl_up_sync(0xFFFFFFFFu, ir, o);
            if (lane >= o) {
                il += tl;
                ir += tr;
            }
        }
        if (lane == 31) {
            s_warp_l[warp] = il;
            s_warp_r[warp] = ir;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int tl = 0, tr = 0;
            for (int w = 0; w < kThreads / 32; w++) {
                int a = s_warp_l[w], b = s_warp_r[w];
                s_warp_l[w] = tl;
                s_warp_r[w] = tr;
                tl += a;
                tr += b;
            }
            s_base_l = atomicAdd(&it.lcur, tl);
            s_base_r = atomicAdd(&it.rcur, tr);
        }
        __syncthreads();
        int offl = s_base_l + s_warp_l[warp] + il - nl;
        int offr = s_base_r + s_warp_r[warp] + ir - nr;
        for (int k = 0; k < kPerThread; k++) {
            if (ids[k] < 0) continue;
            if (((sides >> k) & 1u) == 0)
                idx2[it.start + (offl++)] = ids[k];
            else
                idx2[it.start + it.count - 1 - (offr++)] = ids[k];
        }
        for (int k = 0; k < 24; k++) {
            bool is_min = (k % 6) < 3;
            warp_minmax(acc[k], is_min);
            if (lane == 0) {
                if (is_min)
                    atomicMin(&s_acc[k], acc[k]);
                else
                    atomicMax(&s_acc[k], acc[k]);
            }
        }
        __syncthreads();
        if (threadIdx.x < 24) {
            int k = threadIdx.x;
            int* dst = &it.acc[k / 12][k % 12];
            if ((k % 6) < 3)
                atomicMin(dst, s_acc[k]);
            else
                atomicMax(dst, s_acc[k]);
        }
        __syncthreads();
    }
}

__global__ void k_copyback(const BuildItem* __restrict__ items, const int2* __restrict__ chunks,
                           const BuildMisc* __restrict__ misc, int* __restrict__ idx, const int* __restrict__ idx2) {
    const int nchunks = misc->nchunks;
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        int2 ch = chunks[c];
        const BuildItem& it = items[ch.x];
        if (!it.split) continue;
        int end = min(it.count, ch.y + kChunk);
        for (int j = ch.y + threadIdx.x; j < end; j += blockDim.x) idx[it.start + j] = idx2[it.start + j];
    }
}

// Child creation after the partition (Geometry.h:393-412).
__global__ void k_commit(BuildItem* items, int nitems, BuildItem* next, int next_cap, int* small, int small_cap,
                         pgx_bvh_node* nodes, int* node_rec, BuildMisc* misc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nitems) return;
    BuildItem& it = items[i];
    if (!it.split) return;
    pgx_bvh_node& nd = nodes[it.node];
    int L = it.lcur;
    if (L == 0 || L == it.count) {
        nd.left_first = it.start;
        nd.used = it.count;
        return;
    }
    int c = atomicAdd(&misc->node_count, 2);
    node_rec[it.node] = atomicAdd(&misc->rec_count, 1);
    nd.left_first = c;
    nd.used = 0;
    for (int side = 0; side < 2; side++) {
        int child = c + side;
        int cs = side ? it.start + L : it.start;
        int cn = side ? it.count - L : L;
        pgx_bvh_node& cnd = nodes[child];
        for (int k = 0; k < 3; k++) {
            cnd.bmin[k] = o2f(it.acc[side][k]);
            cnd.bmax[k] = o2f(it.acc[side][3 + k]);
        }
        cnd.left_first = cs;
        cnd.used = cn;
        if (cn <= kMaxLeaf) continue;
        if (cn <= kSmall) {
            int s = atomicAdd(&misc->nsmall, 1);
            if (s < small_cap)
                small[s] = child;
            else
                atomicExch(&misc->overflow, 1);
            continue;
        }
        int q = atomicAdd(&misc->nitems_next, 1);
        if (q >= next_cap) {
            atomicExch(&misc->overflow, 1);
            continue;
        }
        BuildItem& ni = next[q];
        ni.node = child;
        ni.start = cs;
        ni.count = cn;
        for (int k = 0; k < 3; k++) {
            ni.cmin[k] = it.acc[side][6 + k];
            ni.cmax[k] = it.acc[side][9 + k];
        }
    }
}

// Phase B: one thread finishes the subtree of a small node with the
// reference's sequential algorithm (Geometry.h:274-417).
__global__ void k_small(const int* __restrict__ small, const BuildMisc* __restrict__ misc_ro, int* __restrict__ idx,
                        const float4* __restrict__ cent, const float4* __restrict__ tmin,
                        const float4* __restrict__ tmax, pgx_bvh_node* nodes, int* node_rec, BuildMisc* misc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= misc_ro->nsmall) return;
    int stack[kSmallStack];
    int sp = 0;
    stack[sp++] = small[i];
    while (sp > 0) {
        int nid = stack[--sp];
        pgx_bvh_node nd = nodes[nid];
        int start = nd.left_first, cnt = nd.used;
        if (cnt <= kMaxLeaf) continue;
        float parent_area = area_x(nd.bmin[0], nd.bmin[1], nd.bmin[2], nd.bmax[0], nd.bmax[1], nd.bmax[2]);
        float best = FLT_MAX, pos = -FLT_MAX;
        int axis = -1;
        for (int ax = 0; ax < 3; ax++) {
            float lo = FLT_MAX, hi = -FLT_MAX;
            for (int k = 0; k < cnt; k++) {
                float4 c = cent[idx[start + k]];
                float cv = ax == 0 ? c.x : (ax == 1 ? c.y : c.z);
                lo = s_min(lo, cv);
                hi = s_max(hi, cv);
            }
            if (lo == hi) continue;
            int bc[kBins];
            float bmn[kBins][3], bmx[kBins][3];
            for (int b = 0; b < kBins; b++) {
                bc[b] = 0;
                for (int k = 0; k < 3; k++) {
                    bmn[b][k] = FLT_MAX;
                    bmx[b][k] = -FLT_MAX;
                }
            }
            float scale = x_div((float)kBins, x_sub(hi, lo));
            for (int k = 0; k < cnt; k++) {
                int id = idx[start + k];
                float4 c = cent[id];
                float cv = ax == 0 ? c.x : (ax == 1 ? c.y : c.z);
                int bi = (int)x_mul(x_sub(cv, lo), scale);
                bi = (bi < kBins - 1) ? bi : kBins - 1;
                float4 a = tmin[id], b = tmax[id];
                bc[bi]++;
                bmn[bi][0] = s_min(bmn[bi][0], a.x);
                bmn[bi][1] = s_min(bmn[bi][1], a.y);
                bmn[bi][2] = s_min(bmn[bi][2], a.z);
                bmx[bi][0] = s_max(bmx[bi][0], b.x);
                bmx[bi][1] = s_max(bmx[bi][1], b.y);
                bmx[bi][2] = s_max(bmx[bi][2], b.z);
            }
            sweep_axis(bc, bmn, bmx, lo, hi, parent_area, ax, best, axis, pos);
        }
        float no_split = x_mul((float)cnt, 1.5f);
        if (best >= no_split || axis == -1) continue;
        int a = start, b = start + cnt - 1;
        while (a <= b) {
            float4 c = cent[idx[a]];
            float cv = axis == 0 ? c.x : (axis == 1 ? c.y : c.z);
            if (cv < pos) {
                a++;
            } else {
                int t = idx[a];
                idx[a] = idx[b];
                idx[b] = t;
                b--;
            }
        }
        int L = a - start;
        if (L == 0 || L == cnt) continue;
        if (sp + 2 > kSmallStack) {
            atomicExch(&misc->overflow, 2);
            continue;
        }
        int c = atomicAdd(&misc->node_count, 2);
        node_rec[nid] = atomicAdd(&misc->rec_count, 1);
        nodes[nid].left_first = c;
        nodes[nid].used = 0;
        for (int side = 0; side < 2; side++) {
            int cs = side ? start + L : start;
            int cn = side ? cnt - L : L;
            float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            for (int k = 0; k < cn; k++) {
                int id = idx[cs + k];
                float4 ta = tmin[id], tb = tmax[id];
                mn[0] = s_min(mn[0], ta.x);
                mn[1] = s_min(mn[1], ta.y);
                mn[2] = s_min(mn[2], ta.z);
                mx[0] = s_max(mx[0], tb.x);
                mx[1] = s_max(mx[1], tb.y);
                mx[2] = s_max(mx[2], tb.z);
            }
            pgx_bvh_node& cnd = nodes[c + side];
            for (int k = 0; k < 3; k++) {
                cnd.bmin[k] = mn[k];
                cnd.bmax[k] = mx[k];
            }
            cnd.left_first = cs;
            cnd.used = cn;
        }
        stack[sp++] = c + 1;
        stack[sp++] = c;
    }
}

// Traversal records from the reference-layout tree.
__global__ void k_layout(const pgx_bvh_node* __restrict__ nodes, int64_t nnodes, const int* __restrict__ node_rec,
                         TravNode* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nnodes) return;
    const pgx_bvh_node& nd = nodes[i];
    if (nd.used > 0) return;
    int rec = node_rec[i];
    if (rec < 0) return;
    const pgx_bvh_node& L = nodes[nd.left_first];
    const pgx_bvh_node& R = nodes[nd.left_first + 1];
    int lref = L.used > 0 ? L.left_first : node_rec[nd.left_first];
    int rref = R.used > 0 ? R.left_first : node_rec[nd.left_first + 1];
    TravNode t;
    t.lmin = make_float4(L.bmin[0], L.bmin[1], L.bmin[2], __int_as_float(lref));
    t.lmax = make_float4(L.bmax[0], L.bmax[1], L.bmax[2], __int_as_float(L.used));
    t.rmin = make_float4(R.bmin[0], R.bmin[1], R.bmin[2], __int_as_float(rref));
    t.rmax = make_float4(R.bmax[0], R.bmax[1], R.bmax[2], __int_as_float(R.used));
    out[rec] = t;
}

// Leaf-ordered triangles: position p holds triangle idx[p] as v0, e0, e1.
__global__ void k_reorder(const pgx_triangle* __restrict__ tris, const int* __restrict__ idx, int64_t n,
                          TravTri* __restrict__ out) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int id = idx[p];
    const pgx_triangle& t = tris[id];
    xv3 v0 = mk(t.v[0].p[0], t.v[0].p[1], t.v[0].p[2]);
    xv3 e0 = x_sub(mk(t.v[1].p[0], t.v[1].p[1], t.v[1].p[2]), v0);
    xv3 e1 = x_sub(mk(t.v[2].p[0], t.v[2].p[1], t.v[2].p[2]), v0);
    TravTri o;
    o.v0 = make_float4(v0.x, v0.y, v0.z, __int_as_float(id));
    o.e0 = make_float4(e0.x, e0.y, e0.z, 0.f);
    o.e1 = make_float4(e1.x, e1.y, e1.z, 0.f);
    o.pad = make_float4(0.f, 0.f, 0.f, 0.f);
    out[p] = o;
}

__global__ void k_fill_int(int* p, int64_t n, int v) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}
__global__ void k_iota(int* p, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = (int)i;
}

inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

BvhView bvh_view(const pgx_ctx* ctx) {
    BvhView v;
    v.nodes = ctx->trav_nodes.as<TravNode>();
    v.tris = ctx->trav_tris.as<TravTri>();
    v.root = ctx->root;
    v.n_records = (int)ctx->n_records;
    v.n_tris = (int)ctx->ntris;
    if (!ctx->has_bvh) v.root.valid = 0;
    return v;
}

// Builds the traversal layout from ctx->bvh_nodes_ref / bvh_idx and a node ->
// record map (device buffer b_noderec, filled by the caller).
static int finish_layout(pgx_ctx* ctx) {
    cudaStream_t s = ctx->stream;
    int64_t n = ctx->ntris;
    PGX_CUDA_TRY(ctx, ctx->trav_nodes.reserve(sizeof(TravNode) * (size_t)std::max<int64_t>(ctx->n_records, 1)));
    PGX_CUDA_TRY(ctx, ctx->trav_tris.reserve(sizeof(TravTri) * (size_t)std::max<int64_t>(n, 1)));
    if (ctx->n_nodes > 0)
        k_layout<<<blocks_for(ctx->n_nodes, 256), 256, 0, s>>>(ctx->bvh_nodes_ref.as<pgx_bvh_node>(), ctx->n_nodes,
                                                               ctx->b_noderec.as<int>(), ctx->trav_nodes.as<TravNode>());
    if (n > 0)
        k_reorder<<<blocks_for(n, 256), 256, 0, s>>>(ctx->tris_in.as<pgx_triangle>(), ctx->bvh_idx.as<int>(), n,
                                                     ctx->trav_tris.as<TravTri>());
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    pgx_bvh_node root;
    int root_rec = -1;
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&root, ctx->bvh_nodes_ref.p, sizeof(root), cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&root_rec, ctx->b_noderec.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    TravRoot r{};
    for (int k = 0; k < 3; k++) {
        r.bmin[k] = root.bmin[k];
        r.bmax[k] = root.bmax[k];
    }
    if (root.used > 0) {
        r.ref = root.left_first;
        r.count = root.used;
    } else {
        r.ref = root_rec;
        r.count = 0;
    }
    r.valid = n > 0 ? 1 : 0;
    ctx->root = r;
    ctx->has_bvh = true;
    return PGX_OK;
}

int bvh_build_gpu(pgx_ctx* ctx) {
    if (!ctx->has_scene) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_bvh_build: no scene uploaded");
    auto t0 = std::chrono::steady_clock::now();
    cudaStream_t s = ctx->stream;
    const int64_t n = ctx->ntris;
    ctx->has_bvh = false;
    if (n == 0) {
        ctx->n_nodes = 0;
        ctx->n_records = 0;
        ctx->root = TravRoot{};
        ctx->has_bvh = true;
        return PGX_OK;
    }
    if (n > (int64_t)INT32_MAX / 2) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "too many triangles for a BVH");
    const int64_t max_nodes = 2 * n - 1;
    const int64_t item_cap = n / (kSmall / 2) + 64;
    const int64_t small_cap = n / (kMaxLeaf / 2) + 64;
    const int64_t chunk_cap = n / kChunk + item_cap + 64;
    PGX_CUDA_TRY(ctx, ctx->b_cent.reserve(sizeof(float4) * n));
    PGX_CUDA_TRY(ctx, ctx->b_tmin.reserve(sizeof(float4) * n));
    PGX_CUDA_TRY(ctx, ctx->b_tmax.reserve(sizeof(float4) * n));
    PGX_CUDA_TRY(ctx, ctx->b_idx2.reserve(sizeof(int) * n));
    PGX_CUDA_TRY(ctx, ctx->bvh_idx.reserve(sizeof(int) * n));
    PGX_CUDA_TRY(ctx, ctx->bvh_nodes_ref.reserve(sizeof(pgx_bvh_node) * max_nodes));
    PGX_CUDA_TRY(ctx, ctx->b_noderec.reserve(sizeof(int) * max_nodes));
    PGX_CUDA_TRY(ctx, ctx->b_items.reserve(sizeof(BuildItem) * item_cap));
    PGX_CUDA_TRY(ctx, ctx->b_items2.reserve(sizeof(BuildItem) * item_cap));
    PGX_CUDA_TRY(ctx, ctx->b_bins.reserve(sizeof(int) * kBinInts * item_cap));
    PGX_CUDA_TRY(ctx, ctx->b_chunks.reserve(sizeof(int2) * chunk_cap));
    PGX_CUDA_TRY(ctx, ctx->b_small.reserve(sizeof(int) * small_cap));
    PGX_CUDA_TRY(ctx, ctx->b_misc.reserve(sizeof(BuildMisc)));

    float4* cent = ctx->b_cent.as<float4>();
    float4* tmin = ctx->b_tmin.as<float4>();
    float4* tmax = ctx->b_tmax.as<float4>();
    int* idx = ctx->bvh_idx.as<int>();
    int* idx2 = ctx->b_idx2.as<int>();
    pgx_bvh_node* nodes = ctx->bvh_nodes_ref.as<pgx_bvh_node>();
    int* node_rec = ctx->b_noderec.as<int>();
    BuildItem* items = ctx->b_items.as<BuildItem>();
    BuildItem* items2 = ctx->b_items2.as<BuildItem>();
    int* bins = ctx->b_bins.as<int>();
    int2* chunks = ctx->b_chunks.as<int2>();
    int* small = ctx->b_small.as<int>();
    BuildMisc* misc = ctx->b_misc.as<BuildMisc>();

    k_prep<<<blocks_for(n, 256), 256, 0, s>>>(ctx->tris_in.as<pgx_triangle>(), n, cent, tmin, tmax);
    k_iota<<<blocks_for(n, 256), 256, 0, s>>>(idx, n);
    k_fill_int<<<blocks_for(max_nodes, 256), 256, 0, s>>>(node_rec, max_nodes, -1);
    BuildMisc hm{};
    for (int k = 0; k < 12; k++) hm.root_acc[k] = ((k % 6) < 3) ? INT_MAX : INT_MIN;
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(misc, &hm, sizeof(hm), cudaMemcpyHostToDevice, s));
    k_root_reduce<<<std::min<unsigned>(blocks_for(n, 256), 4 * pgx_num_sms()), 256, 0, s>>>(cent, tmin, tmax, n, misc);
    k_root_init<<<1, 32, 0, s>>>(nodes, items, misc, n, small);
    PGX_CUDA_TRY(ctx, cudaGetLastError());

    int nitems = 0;
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&nitems, &misc->nitems_next, sizeof(int), cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    int levels = 0;
    while (nitems > 0) {
        if (++levels > 200) return pgx_fail(ctx, PGX_ERR_OVERFLOW, "BVH build: too many levels");
        PGX_CUDA_TRY(ctx, cudaMemsetAsync(&misc->nchunks, 0, sizeof(int), s));
        PGX_CUDA_TRY(ctx, cudaMemsetAsync(&misc->nitems_next, 0, sizeof(int), s));
        k_chunks<<<blocks_for(nitems, 128), 128, 0, s>>>(items, nitems, chunks, misc);
        k_bins_reset<<<blocks_for((int64_t)nitems * kBinInts, 256), 256, 0, s>>>(bins, nitems);
        unsigned grid = (unsigned)std::min<int64_t>(n / kChunk + nitems, 8 * pgx_num_sms());
        k_bin<<<grid, kThreads, 0, s>>>(items, chunks, misc, idx, cent, tmin, tmax, bins);
        k_split<<<blocks_for(nitems, 64), 64, 0, s>>>(items, nitems, bins, nodes);
        k_partition<<<grid, kThreads, 0, s>>>(items, chunks, misc, idx, idx2, cent, tmin, tmax);
        k_copyback<<<grid, kThreads, 0, s>>>(items, chunks, misc, idx, idx2);
        k_commit<<<blocks_for(nitems, 128), 128, 0, s>>>(items, nitems, items2, (int)item_cap, small, (int)small_cap,
                                                          nodes, node_rec, misc);
        PGX_CUDA_TRY(ctx, cudaGetLastError());
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&nitems, &misc->nitems_next, sizeof(int), cudaMemcpyDeviceToHost, s));
        PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
        std::swap(items, items2);
    }
    int nsmall = 0;
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&nsmall, &misc->nsmall, sizeof(int), cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    if (nsmall > 0)
        k_small<<<blocks_for(nsmall, 64), 64, 0, s>>>(small, misc, idx, cent, tmin, tmax, nodes, node_rec, misc);
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    BuildMisc fin{};
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&fin, misc, sizeof(fin), cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    if (fin.overflow) return pgx_fail(ctx, PGX_ERR_OVERFLOW, "BVH build: work list overflow (%d)", fin.overflow);
    ctx->n_nodes = fin.node_count;
    ctx->n_records = fin.rec_count;
    PGX_TRY(finish_layout(ctx));
    auto t1 = std::chrono::steady_clock::now();
    ctx->bvh_build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    return PGX_OK;
}

int bvh_import_ref(pgx_ctx* ctx, const pgx_bvh_node* nodes, int64_t nnodes, const int32_t* idx) {
    if (!ctx->has_scene) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_bvh_import: no scene uploaded");
    const int64_t n = ctx->ntris;
    if (n == 0) {
        ctx->n_nodes = 0;
        ctx->n_records = 0;
        ctx->root = TravRoot{};
        ctx->has_bvh = true;
        return PGX_OK;
    }
    if (!nodes || !idx || nnodes <= 0) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_bvh_import: empty tree");
    // Validate the tree on the host and number interior nodes in array order.
    std::vector<int> rec((size_t)nnodes, -1);
    int next = 0;
    for (int64_t i = 0; i < nnodes; i++) {
        const pgx_bvh_node& nd = nodes[i];
        if (nd.used < 0) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_bvh_import: node %lld negative count", (long long)i);
        if (nd.used > 0) {
            if (nd.left_first < 0 || (int64_t)nd.left_first + nd.used > n)
                return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_bvh_import: leaf %lld out of range", (long long)i);
        } else {
            if (nd.left_first <= i || (int64_t)nd.left_first + 1 >= nnodes)
                return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_bvh_import: node %lld bad children", (long long)i);
            rec[(size_t)i] = next++;
        }
    }
    for (int64_t i = 0; i < n; i++)
        if (idx[i] < 0 || idx[i] >= n)
            return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_bvh_import: triangle index %lld out of range", (long long)i);
    cudaStream_t s = ctx->stream;
    PGX_CUDA_TRY(ctx, ctx->bvh_nodes_ref.reserve(sizeof(pgx_bvh_node) * nnodes));
    PGX_CUDA_TRY(ctx, ctx->bvh_idx.reserve(sizeof(int) * n));
    PGX_CUDA_TRY(ctx, ctx->b_noderec.reserve(sizeof(int) * nnodes));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->bvh_nodes_ref.p, nodes, sizeof(pgx_bvh_node) * nnodes,
                                      cudaMemcpyHostToDevice, s));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->bvh_idx.p, idx, sizeof(int) * n, cudaMemcpyHostToDevice, s));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->b_noderec.p, rec.data(), sizeof(int) * nnodes, cudaMemcpyHostToDevice, s));
    ctx->n_nodes = nnodes;
    ctx->n_records = next;
    ctx->has_bvh = false;
    return finish_layout(ctx);
}
