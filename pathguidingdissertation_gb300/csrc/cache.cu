// Radiance cache: the point BVH over path vertices
// (PointBVHNode::buildPointBVHNode, Renderer.h:85-142,189-211) built on the
// GPU, its k-nearest query, and the per-region QuadTree guide (pgx_guide.cuh).
//
// Build semantics follow the reference: a node holding more than 8 records
// splits on the longest axis of its bounds (ties to the lower axis) so that
// the left child receives the used/2 records with the smallest coordinate
// (std::nth_element at offset + used/2) and the right child the rest.  With
// distinct coordinates every node holds the same record set as the
// reference's.  Large nodes are split level by level with a 4-pass radix
// select on the ordered-int key (byte histograms per 2048-record chunk, then
// a block-scan partition that also reduces the children's bounds); nodes of
// at most 256 records are finished by one thread each with an in-place
// quickselect.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "pgx_ctx.h"
#include "pgx_guide.cuh"

namespace {

constexpr int kLeafMax = 8;      // MAX_CHILDNODE_RECORDS, Renderer.h:78
constexpr int kSmall = 256;      // one-thread subtrees at or below this size
constexpr int kChunk = 2048;
constexpr int kThreads = 256;
constexpr int kPer = kChunk / kThreads;
constexpr int kStack = 128;

struct PItem {
    int node;
    int offset, used;
    int axis;
    unsigned prefix;
    int k;
    int lcur, rcur, tie;
    int acc[2][6];      // child bounds: min xyz, max xyz (ordered ints)
};

struct PMisc {
    int node_count;
    int nitems_next;
    int nsmall;
    int nregions;
    int nchunks;
    int overflow;
};

struct CacheState {
    DevBuf recs_in, recs, pos, idx, idx2, nodes, trav, items, items2, hist, chunks, small, misc, regions, region_of;
    DevBuf wts_in, wts;  // flux weight per record (input order, then leaf order)
    DevBuf uvs;          // quadtree coordinates of each record's wi, leaf order (-1: outside the domain)
    DevBuf qroot, qnodes, knn_q, knn_i, knn_d, node_region;
    int64_t n_records = 0;
    int64_t n_nodes = 0;
    int n_regions = 0;
    uint64_t generation = 0;  // bumped by every build
    bool valid = false;
    bool pss = false;  // quadtrees over the diffuse BSDF's primary samples
    double build_ms = 0.0;
};

__device__ __forceinline__ unsigned key_of(float f) { return (unsigned)f2o(f) ^ 0x80000000u; }
__device__ __forceinline__ float axis_of(float4 p, int ax) { return ax == 0 ? p.x : (ax == 1 ? p.y : p.z); }

// Longest axis of a box (Renderer.h:90-95).
__device__ __forceinline__ int longest_axis(const pgx_cache_node& n) {
    float ex = n.bmax[0] - n.bmin[0], ey = n.bmax[1] - n.bmin[1], ez = n.bmax[2] - n.bmin[2];
    int ax = 0;
    if (ey > ex) ax = 1;
    float e = ax == 0 ? ex : ey;
    if (ez > e) ax = 2;
    return ax;
}

__global__ void k_pos(const pgx_path_vertex* __restrict__ r, int64_t n, float4* __restrict__ pos, int* idx) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pos[i] = make_float4(r[i].position[0], r[i].position[1], r[i].position[2], 0.f);
    idx[i] = (int)i;
}

__global__ void k_root(const float4* __restrict__ pos, int64_t n, PMisc* misc, pgx_cache_node* nodes, PItem* items,
                       int* small, int* acc, int region_max) {
    // acc: 6 ordered ints reduced by k_root_bounds
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    pgx_cache_node& r = nodes[0];
    for (int k = 0; k < 3; k++) {
        r.bmin[k] = o2f(acc[k]);
        r.bmax[k] = o2f(acc[3 + k]);
    }
    r.left = r.right = -1;
    r.offset = 0;
    r.used = (int)n;
    misc->node_count = 1;
    misc->nitems_next = 0;
    misc->nsmall = 0;
    misc->nregions = 0;
    misc->overflow = 0;
    if (n <= region_max) misc->nregions = 1;  // region 0 = the root, written by the host
    if (n <= kLeafMax) return;
    if (n <= kSmall) {
        small[0] = 0;
        misc->nsmall = 1;
        return;
    }
    PItem& it = items[0];
    it.node = 0;
    it.offset = 0;
    it.used = (int)n;
    misc->nitems_next = 1;
}

__global__ void k_root_bounds(const float4* __restrict__ pos, int64_t n, int* acc) {
    int a[6] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float4 p = pos[i];
        a[0] = min(a[0], f2o(p.x));
        a[1] = min(a[1], f2o(p.y));
        a[2] = min(a[2], f2o(p.z));
        a[3] = max(a[3], f2o(p.x));
        a[4] = max(a[4], f2o(p.y));
        a[5] = max(a[5], f2o(p.z));
    }
    for (int k = 0; k < 6; k++) {
        int v = a[k];
        for (int o = 16; o > 0; o >>= 1) {
            int w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
            v = k < 3 ? min(v, w) : max(v, w);
        }
        if ((threadIdx.x & 31) == 0) {
            if (k < 3)
                atomicMin(&acc[k], v);
            else
                atomicMax(&acc[k], v);
        }
    }
}

__global__ void k_pchunks(PItem* items, int nitems, const pgx_cache_node* nodes, int2* chunks, PMisc* misc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nitems) return;
    PItem& it = items[i];
    it.axis = longest_axis(nodes[it.node]);
    it.prefix = 0;
    it.k = it.used / 2;
    it.lcur = it.rcur = it.tie = 0;
    for (int s = 0; s < 2; s++)
        for (int k = 0; k < 6; k++) it.acc[s][k] = k < 3 ? INT_MAX : INT_MIN;
    int nch = (it.used + kChunk - 1) / kChunk;
    int base = atomicAdd(&misc->nchunks, nch);
    for (int c = 0; c < nch; c++) chunks[base + c] = make_int2(i, c * kChunk);
}

// Histogram of key byte `b` among records whose higher bytes equal the
// item's selected prefix.
__global__ void __launch_bounds__(kThreads) k_phist(const PItem* __restrict__ items, const int2* __restrict__ chunks,
                                                    const PMisc* __restrict__ misc, const int* __restrict__ idx,
                                                    const float4* __restrict__ pos, int* __restrict__ hist, int b) {
    __shared__ int sh[256];
    const int nchunks = misc->nchunks;
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        int2 ch = chunks[c];
        const PItem& it = items[ch.x];
        sh[threadIdx.x] = 0;
        __syncthreads();
        const int end = min(it.used, ch.y + kChunk);
        const unsigned hi_mask = (b == 3) ? 0u : (0xFFFFFFFFu << (8 * (b + 1)));
        for (int j = ch.y + threadIdx.x; j < end; j += blockDim.x) {
            unsigned key = key_of(axis_of(pos[idx[it.offset + j]], it.axis));
            if ((key & hi_mask) == (it.prefix & hi_mask)) atomicAdd(&sh[(key >> (8 * b)) & 255u], 1);
        }
        __syncthreads();
        int v = sh[threadIdx.x];
        if (v) atomicAdd(&hist[(size_t)ch.x * 256 + threadIdx.x], v);
        __syncthreads();
    }
}

__global__ void k_pselect(PItem* items, int nitems, int* hist, int b) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nitems) return;
    PItem& it = items[i];
    int* h = hist + (size_t)i * 256;
    int cum = 0;
    int bucket = 255;
    for (int v = 0; v < 256; v++) {
        if (cum + h[v] > it.k) {
            bucket = v;
            break;
        }
        cum += h[v];
    }
    it.prefix |= (unsigned)bucket << (8 * b);
    it.k -= cum;
    for (int v = 0; v < 256; v++) h[v] = 0;
}

// Partition around the selected key: < K left, > K right, == K left while
// the tie budget (it.k after the select) lasts.
__global__ void __launch_bounds__(kThreads) k_ppart(PItem* __restrict__ items, const int2* __restrict__ chunks,
                                                    const PMisc* __restrict__ misc, const int* __restrict__ idx,
                                                    int* __restrict__ idx2, const float4* __restrict__ pos) {
    __shared__ int s_wl[kThreads / 32], s_wr[kThreads / 32];
    __shared__ int s_bl, s_br;
    __shared__ int s_acc[12];
    const int nchunks = misc->nchunks;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        int2 ch = chunks[c];
        PItem& it = items[ch.x];
        if (threadIdx.x < 12) s_acc[threadIdx.x] = (threadIdx.x % 6) < 3 ? INT_MAX : INT_MIN;
        const int end = min(it.used, ch.y + kChunk);
        int ids[kPer];
        unsigned sides = 0;
        int nl = 0, nr = 0;
        int acc[12];
        for (int k = 0; k < 12; k++) acc[k] = (k % 6) < 3 ? INT_MAX : INT_MIN;
        for (int k = 0; k < kPer; k++) {
            int j = ch.y + k * kThreads + threadIdx.x;
            ids[k] = -1;
            if (j >= end) continue;
            int id = idx[it.offset + j];
            ids[k] = id;
            float4 p = pos[id];
            unsigned key = key_of(axis_of(p, it.axis));
            int side;
            if (key < it.prefix)
                side = 0;
            else if (key > it.prefix)
                side = 1;
            else
                side = (atomicAdd(&it.tie, 1) < it.k) ? 0 : 1;
            sides |= (unsigned)side << k;
            if (side == 0)
                nl++;
            else
                nr++;
            int* a = acc + 6 * side;
            a[0] = min(a[0], f2o(p.x));
            a[1] = min(a[1], f2o(p.y));
            a[2] = min(a[2], f2o(p.z));
            a[3] = max(a[3], f2o(p.x));
            a[4] = max(a[4], f2o(p.y));
            a[5] = max(a[5], f2o(p.z));
        }
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
            s_wl[warp] = il;
            s_wr[warp] = ir;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int tl = 0, tr = 0;
            for (int w = 0; w < kThreads / 32; w++) {
                int a = s_wl[w], bb = s_wr[w];
                s_wl[w] = tl;
                s_wr[w] = tr;
                tl += a;
                tr += bb;
            }
            s_bl = atomicAdd(&it.lcur, tl);
            s_br = atomicAdd(&it.rcur, tr);
        }
        __syncthreads();
        int offl = s_bl + s_wl[warp] + il - nl;
        int offr = s_br + s_wr[warp] + ir - nr;
        for (int k = 0; k < kPer; k++) {
            if (ids[k] < 0) continue;
            if (((sides >> k) & 1u) == 0)
                idx2[it.offset + (offl++)] = ids[k];
            else
                idx2[it.offset + it.used - 1 - (offr++)] = ids[k];
        }
        for (int k = 0; k < 12; k++) {
            int v = acc[k];
            bool mn = (k % 6) < 3;
            for (int o = 16; o > 0; o >>= 1) {
                int w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
                v = mn ? min(v, w) : max(v, w);
            }
            if (lane == 0) {
                if (mn)
                    atomicMin(&s_acc[k], v);
                else
                    atomicMax(&s_acc[k], v);
            }
        }
        __syncthreads();
        if (threadIdx.x < 12) {
            int k = threadIdx.x;
            int* dst = &it.acc[k / 6][k % 6];
            if ((k % 6) < 3)
                atomicMin(dst, s_acc[k]);
            else
                atomicMax(dst, s_acc[k]);
        }
        __syncthreads();
    }
}

__global__ void k_pcopy(const PItem* __restrict__ items, const int2* __restrict__ chunks,
                        const PMisc* __restrict__ misc, int* __restrict__ idx, const int* __restrict__ idx2) {
    const int nchunks = misc->nchunks;
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        int2 ch = chunks[c];
        const PItem& it = items[ch.x];
        int end = min(it.used, ch.y + kChunk);
        for (int j = ch.y + threadIdx.x; j < end; j += blockDim.x) idx[it.offset + j] = idx2[it.offset + j];
    }
}

__global__ void k_pcommit(PItem* items, int nitems, PItem* next, int next_cap, int* small, int small_cap,
                          pgx_cache_node* nodes, int2* regions, int* node_region, PMisc* misc, int region_max) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nitems) return;
    PItem& it = items[i];
    int half = it.used / 2;
    if (it.lcur != half) atomicExch(&misc->overflow, 3);
    int c = atomicAdd(&misc->node_count, 2);
    pgx_cache_node& nd = nodes[it.node];
    nd.left = c;
    nd.right = c + 1;
    nd.used = 0;
    for (int side = 0; side < 2; side++) {
        pgx_cache_node& ch = nodes[c + side];
        int cs = side ? it.offset + half : it.offset;
        int cn = side ? it.used - half : half;
        for (int k = 0; k < 3; k++) {
            ch.bmin[k] = o2f(it.acc[side][k]);
            ch.bmax[k] = o2f(it.acc[side][3 + k]);
        }
        ch.left = ch.right = -1;
        ch.offset = cs;
        ch.used = cn;
        if (cn <= region_max && it.used > region_max) {
            int r = atomicAdd(&misc->nregions, 1);
            regions[r] = make_int2(cs, cn);
            node_region[c + side] = r;
        }
        if (cn <= kLeafMax) continue;
        if (cn <= kSmall) {
            int s = atomicAdd(&misc->nsmall, 1);
            if (s < small_cap)
                small[s] = c + side;
            else
                atomicExch(&misc->overflow, 1);
            continue;
        }
        int q = atomicAdd(&misc->nitems_next, 1);
        if (q >= next_cap) {
            atomicExch(&misc->overflow, 2);
            continue;
        }
        next[q].node = c + side;
        next[q].offset = cs;
        next[q].used = cn;
    }
}

// In-place quickselect: afterwards idx[lo .. lo+nth) hold the nth smallest
// keys of idx[lo .. hi) (hi exclusive).
__device__ void quickselect(int* idx, int lo, int hi, int nth, const float4* pos, int ax) {
    int left = lo, right = hi - 1;
    int target = lo + nth;
    while (right > left) {
        int mid = left + (right - left) / 2;
        float a = axis_of(pos[idx[left]], ax), b = axis_of(pos[idx[mid]], ax), c = axis_of(pos[idx[right]], ax);
        float piv = (a < b) ? ((b < c) ? b : ((a < c) ? c : a)) : ((a < c) ? a : ((b < c) ? c : b));
        int i = left, j = right;
        while (i <= j) {
            while (i <= right && axis_of(pos[idx[i]], ax) < piv) i++;
            while (j >= left && piv < axis_of(pos[idx[j]], ax)) j--;
            if (i <= j) {
                int t = idx[i];
                idx[i] = idx[j];
                idx[j] = t;
                i++;
                j--;
            }
        }
        if (target <= j)
            right = j;
        else if (target >= i)
            left = i;
        else
            break;
    }
}

__global__ void k_psmall(const int* __restrict__ small, PMisc* misc, int* idx, const float4* __restrict__ pos,
                         pgx_cache_node* nodes) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= misc->nsmall) return;
    int stack[kStack];
    int sp = 0;
    stack[sp++] = small[i];
    while (sp > 0) {
        int nid = stack[--sp];
        pgx_cache_node nd = nodes[nid];
        if (nd.used <= kLeafMax) continue;
        int ax = longest_axis(nd);
        int half = nd.used / 2;
        quickselect(idx, nd.offset, nd.offset + nd.used, half, pos, ax);
        int c = atomicAdd(&misc->node_count, 2);
        nodes[nid].left = c;
        nodes[nid].right = c + 1;
        nodes[nid].used = 0;
        for (int side = 0; side < 2; side++) {
            int cs = side ? nd.offset + half : nd.offset;
            int cn = side ? nd.used - half : half;
            float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            for (int k = 0; k < cn; k++) {
                float4 p = pos[idx[cs + k]];
                mn[0] = s_min(mn[0], p.x);
                mn[1] = s_min(mn[1], p.y);
                mn[2] = s_min(mn[2], p.z);
                mx[0] = s_max(mx[0], p.x);
                mx[1] = s_max(mx[1], p.y);
                mx[2] = s_max(mx[2], p.z);
            }
            pgx_cache_node& ch = nodes[c + side];
            for (int k = 0; k < 3; k++) {
                ch.bmin[k] = mn[k];
                ch.bmax[k] = mx[k];
            }
            ch.left = ch.right = -1;
            ch.offset = cs;
            ch.used = cn;
        }
        if (sp + 2 > kStack) {
            atomicExch(&misc->overflow, 4);
            continue;
        }
        stack[sp++] = c + 1;
        stack[sp++] = c;
    }
}

// Default flux weight of a record: the luminance of its Li.  The quadtree
// build clamps weights at clamp_median x the region's median weight
// (pgx_guide_params; 0 = no clamp) so that a few very bright records (the
// sun seen through a specular chain) need not take the whole distribution.
__device__ __forceinline__ float record_lum(const pgx_path_vertex& v) {
    float w = ((0.2126f * v.Li[0]) + (0.7152f * v.Li[1])) + (0.0722f * v.Li[2]);
    return (isfinite(w) && w > 0.f) ? w : 0.f;
}

// Records into leaf order, with their flux weights (the given ones, the
// renderer's Lum(Li) |cos| / pdf, or Lum(Li); non-finite or negative -> 0)
// and the quadtree coordinates of their wi: the cylindrical map of the
// direction, or the diffuse sampler's primary sample (pss; (-1, -1) below
// the hemisphere, which no cell contains).
__global__ void k_gather(const pgx_path_vertex* __restrict__ in, const float* __restrict__ w_in,
                         const int* __restrict__ idx, int64_t n, pgx_path_vertex* __restrict__ out,
                         float* __restrict__ w_out, float2* __restrict__ uv_out, int pss) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int j = idx[i];
    const pgx_path_vertex v = in[j];
    out[i] = v;
    float w = w_in ? w_in[j] : record_lum(v);
    w_out[i] = (isfinite(w) && w > 0.f) ? w : 0.f;
    const F3 wi = f3(v.wi[0], v.wi[1], v.wi[2]);
    float u, vv;
    if (pss) {
        if (!pss_uv(f3(v.normal[0], v.normal[1], v.normal[2]), wi, u, vv)) u = vv = -1.f;
    } else {
        dir_to_uv(wi, u, vv);
    }
    uv_out[i] = make_float2(u, vv);
}

__global__ void k_trav(const pgx_cache_node* __restrict__ nodes, int64_t nn, CacheTravNode* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    const pgx_cache_node& n = nodes[i];
    CacheTravNode t;
    bool leaf = n.left < 0;
    t.bmin = make_float4(n.bmin[0], n.bmin[1], n.bmin[2], __int_as_float(leaf ? -(n.offset + 1) : n.left));
    t.bmax = make_float4(n.bmax[0], n.bmax[1], n.bmax[2], __int_as_float(leaf ? n.used : n.right));
    out[i] = t;
}

__global__ void k_regions(const int2* __restrict__ regions, int nreg, const pgx_path_vertex* __restrict__ recs,
                          float4* __restrict__ pos) {
    int r = blockIdx.x;
    if (r >= nreg) return;
    int2 g = regions[r];
    for (int i = threadIdx.x; i < g.y; i += blockDim.x) {
        const pgx_path_vertex& v = recs[g.x + i];
        pos[g.x + i] = make_float4(v.position[0], v.position[1], v.position[2], __int_as_float(r));
    }
}

__device__ __forceinline__ float warp_sum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}
__device__ __forceinline__ int warp_sum_i(int v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// One warp builds one region's quadtree (pgx_guide.cuh): the lanes stride
// over the region's records and reduce with shuffles; lane 0 keeps the BFS
// queue of cells in shared memory.
constexpr int kQtWarps = 4;

__global__ void __launch_bounds__(32 * kQtWarps) k_quadtree(const int2* __restrict__ regions, int nreg,
                                                            const float2* __restrict__ uvs,
                                                            const float* __restrict__ wts,
                                                            int* __restrict__ qroot, QuadNode* __restrict__ qnodes,
                                                            float clamp_median, float refine, float compensate) {
    __shared__ float s_u[kQtWarps][PGX_QT_MAX_NODES], s_v[kQtWarps][PGX_QT_MAX_NODES],
        s_s[kQtWarps][PGX_QT_MAX_NODES], s_c[kQtWarps][PGX_QT_MAX_NODES];
    __shared__ unsigned char s_d[kQtWarps][PGX_QT_MAX_NODES];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * kQtWarps + warp;
    if (r >= nreg) return;  // uniform per warp
    int2 g = regions[r];
    const float2* ruv = uvs + g.x;
    const float* rw = wts + g.x;
    // Median of the positive luminances by bisection on the value (only
    // needed for the clamp).
    float lo = FLT_MAX, hi = 0.f;
    int pos = 0;
    for (int i = lane; i < g.y; i += 32) {
        float w = rw[i];
        if (w > 0.f) {
            lo = fminf(lo, w);
            hi = fmaxf(hi, w);
            pos++;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xFFFFFFFFu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xFFFFFFFFu, hi, o));
    }
    pos = warp_sum_i(pos);
    if (pos == 0) {
        if (lane == 0) qroot[r] = -1;
        return;
    }
    const int half_count = (pos + 1) / 2;
    for (int it = 0; it < (clamp_median > 0.f ? 24 : 0); it++) {
        float mid = 0.5f * (lo + hi);
        int below = 0;
        for (int i = lane; i < g.y; i += 32) {
            float w = rw[i];
            if (w > 0.f && w <= mid) below++;
        }
        below = warp_sum_i(below);
        if (below >= half_count)
            hi = mid;
        else
            lo = mid;
    }
    const float clamp = clamp_median > 0.f ? clamp_median * hi : FLT_MAX;
    float total = 0.f;
    for (int i = lane; i < g.y; i += 32) total += fminf(rw[i], clamp);
    total = warp_sum(total);
    if (!(total > 0.f) || !isfinite(total)) {
        if (lane == 0) qroot[r] = -1;
        return;
    }
    QuadNode* out = qnodes + (size_t)r * PGX_QT_MAX_NODES;
    float* cu = s_u[warp];
    float* cv = s_v[warp];
    float* cs = s_s[warp];
    unsigned char* cd = s_d[warp];
    if (lane == 0) {
        cu[0] = 0.f;
        cv[0] = 0.f;
        cs[0] = 1.f;
        cd[0] = 0;
    }
    __syncwarp();
    int nn = 1, head = 0;
    const float thresh = refine * total;
    while (head < nn) {
        int node = head++;
        float u0 = cu[node], v0 = cv[node], sz = cs[node], half = sz * 0.5f;
        float flux[4] = {0.f, 0.f, 0.f, 0.f};
        int cnt[4] = {0, 0, 0, 0};
        for (int i = lane; i < g.y; i += 32) {
            float w = fminf(rw[i], clamp);
            if (!(w > 0.f)) continue;
            const float2 uv = ruv[i];
            const float u = uv.x, vv = uv.y;
            if (u < u0 || u >= u0 + sz || vv < v0 || vv >= v0 + sz) continue;
            int c = 2 * (vv >= v0 + half ? 1 : 0) + (u >= u0 + half ? 1 : 0);
            flux[c] += w;
            cnt[c]++;
        }
        QuadNode q;
        for (int c = 0; c < 4; c++) {
            q.flux[c] = warp_sum(flux[c]);
            int cc = warp_sum_i(cnt[c]);
            q.child[c] = -1;
            if (q.flux[c] > thresh && cc >= 2 && cd[node] + 1 < PGX_QT_MAX_DEPTH && nn < PGX_QT_MAX_NODES) {
                int k = nn++;
                if (lane == 0) {
                    cu[k] = u0 + half * (float)(c & 1);
                    cv[k] = v0 + half * (float)(c >> 1);
                    cs[k] = half;
                    cd[k] = (unsigned char)(cd[node] + 1);
                }
                q.child[c] = k;
            }
        }
        __syncwarp();
        if (lane == 0) out[node] = q;
    }
    if (compensate > 0.f && lane == 0) {
        // MIS compensation: leaves lose compensate x the mean flux over their
        // area (floored at 0); interior fluxes are the sums of their
        // children, computed leaves-up (reverse breadth-first order).
        const QuadNode root = out[0];
        const float tot = ((root.flux[0] + root.flux[1]) + root.flux[2]) + root.flux[3];
        float* comp = s_c[warp];
        for (int node = nn - 1; node >= 0; node--) {
            const QuadNode q = out[node];
            const float sub = compensate * tot * ldexpf(1.f, -2 * (cd[node] + 1));
            float sum = 0.f;
            for (int c = 0; c < 4; c++) sum += q.child[c] >= 0 ? comp[q.child[c]] : fmaxf(q.flux[c] - sub, 0.f);
            comp[node] = sum;
        }
        if (comp[0] >= 0.05f * tot) {
            for (int node = 0; node < nn; node++) {
                QuadNode q = out[node];
                const float sub = compensate * tot * ldexpf(1.f, -2 * (cd[node] + 1));
                for (int c = 0; c < 4; c++) q.flux[c] = q.child[c] >= 0 ? comp[q.child[c]] : fmaxf(q.flux[c] - sub, 0.f);
                out[node] = q;
            }
        }
    }
    if (lane == 0) qroot[r] = 0;  // region-relative; k_rebase makes it absolute
}

__global__ void k_rebase(int* qroot, int nreg) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nreg && qroot[r] >= 0) qroot[r] = r * PGX_QT_MAX_NODES;
}

// Child indices inside a region's quadtree are region-relative; make them
// absolute.
__global__ void k_rebase_children(QuadNode* q, const int* qroot, int nreg) {
    int r = blockIdx.x;
    if (r >= nreg || qroot[r] < 0) return;
    for (int i = threadIdx.x; i < PGX_QT_MAX_NODES; i += blockDim.x) {
        QuadNode& n = q[(size_t)r * PGX_QT_MAX_NODES + i];
        for (int c = 0; c < 4; c++)
            if (n.child[c] >= 0) n.child[c] += r * PGX_QT_MAX_NODES;
    }
}

// k nearest records per query (ascending distance, ties to lower index).
__global__ void k_knn(const CacheTravNode* __restrict__ nodes, const float4* __restrict__ pos, int nrec,
                      const float* __restrict__ q, int64_t nq, int k, int* __restrict__ out_i,
                      float* __restrict__ out_d) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nq) return;
    float x = q[3 * t], y = q[3 * t + 1], z = q[3 * t + 2];
    float bd[64];
    int bi[64];
    int cnt = 0;
    for (int j = 0; j < k; j++) {
        bd[j] = FLT_MAX;
        bi[j] = -1;
    }
    auto worse = [&](float d, int i, float d2, int i2) { return d > d2 || (d == d2 && i > i2); };
    auto box_d = [&](const CacheTravNode& c) {
        float dx = fmaxf(fmaxf(c.bmin.x - x, x - c.bmax.x), 0.f);
        float dy = fmaxf(fmaxf(c.bmin.y - y, y - c.bmax.y), 0.f);
        float dz = fmaxf(fmaxf(c.bmin.z - z, z - c.bmax.z), 0.f);
        return dx * dx + dy * dy + dz * dz;
    };
    if (nrec > 0) {
        int stack[64];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            int ni = stack[--sp];
            CacheTravNode n = nodes[ni];
            float lim = cnt < k ? FLT_MAX : bd[k - 1];
            if (box_d(n) > lim) continue;
            int l = __float_as_int(n.bmin.w), r = __float_as_int(n.bmax.w);
            if (l < 0) {
                int off = -l - 1;
                for (int j = 0; j < r; j++) {
                    float4 p = pos[off + j];
                    float dx = p.x - x, dy = p.y - y, dz = p.z - z;
                    float d = dx * dx + dy * dy + dz * dz;
                    int id = off + j;
                    if (cnt == k && !worse(bd[k - 1], bi[k - 1], d, id)) continue;
                    int m = cnt < k ? cnt++ : k - 1;
                    while (m > 0 && worse(bd[m - 1], bi[m - 1], d, id)) {
                        bd[m] = bd[m - 1];
                        bi[m] = bi[m - 1];
                        m--;
                    }
                    bd[m] = d;
                    bi[m] = id;
                }
            } else if (sp + 2 <= 64) {
                float da = box_d(nodes[l]), db = box_d(nodes[r]);
                if (da < db) {
                    stack[sp++] = r;
                    stack[sp++] = l;
                } else {
                    stack[sp++] = l;
                    stack[sp++] = r;
                }
            }
        }
    }
    for (int j = 0; j < k; j++) {
        out_i[t * k + j] = bi[j];
        out_d[t * k + j] = bd[j] == FLT_MAX ? INFINITY : bd[j];
    }
}

// Guide pdf / sample for explicit positions (pgx_guide_pdf / _sample).
__global__ void k_guide_query(GuideView g, const float* __restrict__ pos, const float* __restrict__ in, int64_t n,
                              int sample, float* __restrict__ dirs, float* __restrict__ pdf) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    F3 x = f3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    int root = guide_region_root(g, x);
    const float inv4pi = 1.f / (4.f * 3.14159265f);
    if (sample) {
        F3 w = f3(0.f, 0.f, 1.f);
        float p = 0.f;
        if (root >= 0) {
            float u, v;
            quad_sample(g.qnodes, root, in[2 * i], in[2 * i + 1], u, v);
            w = uv_to_dir(u, v);
            float pu, pv;
            dir_to_uv(w, pu, pv);
            p = quad_pdf(g.qnodes, root, pu, pv) * inv4pi;  // the quadtree alone
        }
        dirs[3 * i] = w.x;
        dirs[3 * i + 1] = w.y;
        dirs[3 * i + 2] = w.z;
        pdf[i] = p;
    } else {
        float p = 0.f;
        if (root >= 0) {
            float u, v;
            dir_to_uv(normalize(f3(in[3 * i], in[3 * i + 1], in[3 * i + 2])), u, v);
            p = quad_pdf(g.qnodes, root, u, v) * inv4pi;
        }
        pdf[i] = p;
    }
}

inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

CacheState* cstate(pgx_ctx* ctx) {
    if (!ctx->cache_state) ctx->cache_state = new CacheState();
    return static_cast<CacheState*>(ctx->cache_state);
}

}  // namespace

void cache_state_free(pgx_ctx* ctx) {
    delete static_cast<CacheState*>(ctx->cache_state);
    ctx->cache_state = nullptr;
}

GuideView guide_view(const pgx_ctx* ctx) {
    GuideView g{};
    const CacheState* cs = static_cast<const CacheState*>(ctx->cache_state);
    if (!cs || !cs->valid || cs->n_records == 0) return g;
    g.valid = 1;
    g.n_nodes = (int)cs->n_nodes;
    g.n_records = (int)cs->n_records;
    g.nodes = cs->trav.as<CacheTravNode>();
    g.rec_pos = cs->pos.as<float4>();
    g.region_qroot = cs->qroot.as<int>();
    g.qnodes = cs->qnodes.as<QuadNode>();
    g.node_region = cs->node_region.as<int>();
    g.pss = cs->pss ? 1 : 0;
    g.uniform = ctx->guide.uniform_share;
    g.min_alpha = ctx->guide.glossy_alpha;
    return g;
}

uint64_t guide_generation(const pgx_ctx* ctx) {
    const CacheState* cs = static_cast<const CacheState*>(ctx->cache_state);
    return cs ? cs->generation : 0;
}

int guide_regions(const pgx_ctx* ctx) {
    const CacheState* cs = static_cast<const CacheState*>(ctx->cache_state);
    return (cs && cs->valid && cs->n_records > 0) ? cs->n_regions : 0;
}

bool guide_ready(const pgx_ctx* ctx) {
    const CacheState* cs = static_cast<const CacheState*>(ctx->cache_state);
    return cs && cs->valid && cs->n_records > 0;
}

// Builds the cache from n records already on the device.
int cache_build_device(pgx_ctx* ctx, const pgx_path_vertex* d_records, int64_t n, bool pss,
                       const float* d_weights) {
    CacheState* cs = cstate(ctx);
    cs->valid = false;
    cs->generation++;
    cs->pss = pss;
    if (n < 0 || n > (int64_t)INT32_MAX / 2) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "cache: bad record count");
    auto t0 = std::chrono::steady_clock::now();
    cudaStream_t s = ctx->stream;
    cs->n_records = n;
    cs->n_nodes = 0;
    cs->n_regions = 0;
    if (n == 0) {
        cs->valid = true;
        return PGX_OK;
    }
    const int64_t max_nodes = 2 * n;
    const int64_t item_cap = n / (kSmall / 2) + 64;
    const int64_t chunk_cap = n / kChunk + item_cap + 64;
    const int64_t small_cap = n / (kLeafMax / 2) + 64;
    // Parameters of this build (later pgx_guide_configure calls shape the next one).
    const int region_max = ctx->guide.region_records;
    const float clamp_median = ctx->guide.clamp_median, refine = ctx->guide.refine_fraction;
    const float compensate = ctx->guide.compensate;
    const int64_t reg_cap = n / (region_max / 4) + 64;
    PGX_CUDA_TRY(ctx, cs->recs_in.reserve(sizeof(pgx_path_vertex) * n));
    PGX_CUDA_TRY(ctx, cs->recs.reserve(sizeof(pgx_path_vertex) * n));
    PGX_CUDA_TRY(ctx, cs->wts.reserve(sizeof(float) * n));
    PGX_CUDA_TRY(ctx, cs->uvs.reserve(sizeof(float2) * n));
    if (d_weights) {
        PGX_CUDA_TRY(ctx, cs->wts_in.reserve(sizeof(float) * n));
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(cs->wts_in.p, d_weights, sizeof(float) * n, cudaMemcpyDeviceToDevice,
                                          ctx->stream));
    }
    PGX_CUDA_TRY(ctx, cs->pos.reserve(sizeof(float4) * n));
    PGX_CUDA_TRY(ctx, cs->idx.reserve(sizeof(int) * n));
    PGX_CUDA_TRY(ctx, cs->idx2.reserve(sizeof(int) * n));
    PGX_CUDA_TRY(ctx, cs->nodes.reserve(sizeof(pgx_cache_node) * max_nodes));
    PGX_CUDA_TRY(ctx, cs->trav.reserve(sizeof(CacheTravNode) * max_nodes));
    PGX_CUDA_TRY(ctx, cs->items.reserve(sizeof(PItem) * item_cap));
    PGX_CUDA_TRY(ctx, cs->items2.reserve(sizeof(PItem) * item_cap));
    PGX_CUDA_TRY(ctx, cs->hist.reserve(sizeof(int) * 256 * item_cap));
    PGX_CUDA_TRY(ctx, cs->chunks.reserve(sizeof(int2) * chunk_cap));
    PGX_CUDA_TRY(ctx, cs->small.reserve(sizeof(int) * small_cap));
    PGX_CUDA_TRY(ctx, cs->misc.reserve(sizeof(PMisc) + sizeof(int) * 8));
    PGX_CUDA_TRY(ctx, cs->regions.reserve(sizeof(int2) * reg_cap));
    PGX_CUDA_TRY(ctx, cs->node_region.reserve(sizeof(int) * max_nodes));
    // -1 everywhere; region roots get their region index (the root: region 0
    // when the whole cache is one region).
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(cs->node_region.p, 0xFF, sizeof(int) * max_nodes, s));
    if (n <= region_max) PGX_CUDA_TRY(ctx, cudaMemsetAsync(cs->node_region.p, 0, sizeof(int), s));
    if (d_records != cs->recs_in.as<pgx_path_vertex>())
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(cs->recs_in.p, d_records, sizeof(pgx_path_vertex) * n,
                                          cudaMemcpyDeviceToDevice, s));
    float4* pos = cs->pos.as<float4>();
    int* idx = cs->idx.as<int>();
    int* idx2 = cs->idx2.as<int>();
    pgx_cache_node* nodes = cs->nodes.as<pgx_cache_node>();
    PItem* items = cs->items.as<PItem>();
    PItem* items2 = cs->items2.as<PItem>();
    int* hist = cs->hist.as<int>();
    int2* chunks = cs->chunks.as<int2>();
    int* small = cs->small.as<int>();
    PMisc* misc = cs->misc.as<PMisc>();
    int* acc = reinterpret_cast<int*>(misc + 1);
    int2* regions = cs->regions.as<int2>();

    k_pos<<<blocks_for(n, 256), 256, 0, s>>>(cs->recs_in.as<pgx_path_vertex>(), n, pos, idx);
    int hacc[8] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN, 0, 0};
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(acc, hacc, sizeof(hacc), cudaMemcpyHostToDevice, s));
    k_root_bounds<<<std::min<unsigned>(blocks_for(n, 256), 4 * pgx_num_sms()), 256, 0, s>>>(pos, n, acc);
    k_root<<<1, 32, 0, s>>>(pos, n, misc, nodes, items, small, acc, region_max);
    PGX_CUDA_TRY(ctx, cudaMemsetAsync(hist, 0, sizeof(int) * 256 * item_cap, s));
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    int nitems = 0;
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&nitems, &misc->nitems_next, sizeof(int), cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    int levels = 0;
    while (nitems > 0) {
        if (++levels > 64) return pgx_fail(ctx, PGX_ERR_OVERFLOW, "cache build: too many levels");
        PGX_CUDA_TRY(ctx, cudaMemsetAsync(&misc->nchunks, 0, sizeof(int), s));
        PGX_CUDA_TRY(ctx, cudaMemsetAsync(&misc->nitems_next, 0, sizeof(int), s));
        k_pchunks<<<blocks_for(nitems, 128), 128, 0, s>>>(items, nitems, nodes, chunks, misc);
        unsigned grid = (unsigned)std::min<int64_t>(n / kChunk + nitems, 8 * pgx_num_sms());
        for (int b = 3; b >= 0; b--) {
            k_phist<<<grid, kThreads, 0, s>>>(items, chunks, misc, idx, pos, hist, b);
            k_pselect<<<blocks_for(nitems, 64), 64, 0, s>>>(items, nitems, hist, b);
        }
        k_ppart<<<grid, kThreads, 0, s>>>(items, chunks, misc, idx, idx2, pos);
        k_pcopy<<<grid, kThreads, 0, s>>>(items, chunks, misc, idx, idx2);
        k_pcommit<<<blocks_for(nitems, 128), 128, 0, s>>>(items, nitems, items2, (int)item_cap, small,
                                                          (int)small_cap, nodes, regions, cs->node_region.as<int>(),
                                                          misc, region_max);
        PGX_CUDA_TRY(ctx, cudaGetLastError());
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&nitems, &misc->nitems_next, sizeof(int), cudaMemcpyDeviceToHost, s));
        PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
        std::swap(items, items2);
    }
    PMisc hm{};
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&hm, misc, sizeof(hm), cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    if (hm.nsmall > 0) k_psmall<<<blocks_for(hm.nsmall, 64), 64, 0, s>>>(small, misc, idx, pos, nodes);
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(&hm, misc, sizeof(hm), cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    if (hm.overflow) return pgx_fail(ctx, PGX_ERR_OVERFLOW, "cache build: internal overflow (%d)", hm.overflow);
    cs->n_nodes = hm.node_count;
    if (n <= region_max) {
        int2 r0 = make_int2(0, (int)n);
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(regions, &r0, sizeof(r0), cudaMemcpyHostToDevice, s));
        hm.nregions = 1;
    }
    cs->n_regions = hm.nregions;
    pgx_path_vertex* recs = cs->recs.as<pgx_path_vertex>();
    k_gather<<<blocks_for(n, 256), 256, 0, s>>>(cs->recs_in.as<pgx_path_vertex>(),
                                                d_weights ? cs->wts_in.as<float>() : nullptr, idx, n, recs,
                                                cs->wts.as<float>(), cs->uvs.as<float2>(), pss ? 1 : 0);
    k_trav<<<blocks_for(cs->n_nodes, 256), 256, 0, s>>>(nodes, cs->n_nodes, cs->trav.as<CacheTravNode>());
    // Records carry their region id; leaves below regions are inside them.
    k_regions<<<std::max(1, cs->n_regions), 128, 0, s>>>(regions, cs->n_regions, recs, pos);
    PGX_CUDA_TRY(ctx, cs->qroot.reserve(sizeof(int) * std::max(1, cs->n_regions)));
    PGX_CUDA_TRY(ctx, cs->qnodes.reserve(sizeof(QuadNode) * PGX_QT_MAX_NODES * (size_t)std::max(1, cs->n_regions)));
    k_quadtree<<<blocks_for(cs->n_regions, kQtWarps), 32 * kQtWarps, 0, s>>>(
        regions, cs->n_regions, cs->uvs.as<float2>(), cs->wts.as<float>(), cs->qroot.as<int>(),
        cs->qnodes.as<QuadNode>(), clamp_median, refine, compensate);
    k_rebase_children<<<std::max(1, cs->n_regions), 128, 0, s>>>(cs->qnodes.as<QuadNode>(), cs->qroot.as<int>(),
                                                                   cs->n_regions);
    k_rebase<<<blocks_for(cs->n_regions, 128), 128, 0, s>>>(cs->qroot.as<int>(), cs->n_regions);
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    cs->valid = true;
    cs->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return PGX_OK;
}

int64_t render_vertex_count(pgx_ctx* ctx);
const pgx_path_vertex* render_vertices(pgx_ctx* ctx);
const float* render_vertex_weights(pgx_ctx* ctx);

extern "C" int pgx_cache_build(pgx_ctx* ctx, const pgx_path_vertex* records, int64_t n) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (n < 0 || (n > 0 && !records)) return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_cache_build: bad arguments");
    PGX_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    CacheState* cs = cstate(ctx);
    PGX_CUDA_TRY(ctx, cs->recs_in.reserve(sizeof(pgx_path_vertex) * std::max<int64_t>(n, 1)));
    if (n > 0)
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(cs->recs_in.p, records, sizeof(pgx_path_vertex) * n, cudaMemcpyHostToDevice,
                                          ctx->stream));
    return cache_build_device(ctx, cs->recs_in.as<pgx_path_vertex>(), n);
}

extern "C" int pgx_cache_build_from_render(pgx_ctx* ctx) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    const pgx_path_vertex* v = render_vertices(ctx);
    int64_t n = render_vertex_count(ctx);
    if (!v) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_cache_build_from_render: no recorded path vertices");
    return cache_build_device(ctx, v, n, false, render_vertex_weights(ctx));
}

extern "C" int pgx_cache_get_stats(pgx_ctx* ctx, pgx_cache_stats* out) {
    if (!ctx || !out) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    CacheState* cs = static_cast<CacheState*>(ctx->cache_state);
    if (!cs || !cs->valid) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_cache_get_stats: no cache");
    *out = pgx_cache_stats{};
    out->records = cs->n_records;
    out->nodes = cs->n_nodes;
    out->build_ms = cs->build_ms;
    if (cs->n_nodes == 0) return PGX_OK;
    std::vector<pgx_cache_node> nodes((size_t)cs->n_nodes);
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(nodes.data(), cs->nodes.p, sizeof(pgx_cache_node) * nodes.size(),
                                      cudaMemcpyDeviceToHost, ctx->stream));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    // PointBVHNode::stats (Renderer.h:163-177,219-233).
    std::vector<std::pair<int, int>> st{{0, 0}};
    int mn = INT32_MAX, mx = -INT32_MAX;
    long long sum = 0;
    while (!st.empty()) {
        auto [i, d] = st.back();
        st.pop_back();
        const pgx_cache_node& nd = nodes[(size_t)i];
        if (nd.left < 0) {
            out->leaves++;
            mn = std::min(mn, d);
            mx = std::max(mx, d);
            sum += d;
        } else {
            st.push_back({nd.right, d + 1});
            st.push_back({nd.left, d + 1});
        }
    }
    out->min_leaf_depth = mn;
    out->max_leaf_depth = mx;
    out->mean_leaf_depth = out->leaves ? (double)sum / (double)out->leaves : 0.0;
    return PGX_OK;
}

extern "C" int pgx_cache_export(pgx_ctx* ctx, pgx_cache_node* nodes, int64_t* nnodes, pgx_path_vertex* records,
                                int64_t* nrecords) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    CacheState* cs = static_cast<CacheState*>(ctx->cache_state);
    if (!cs || !cs->valid) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_cache_export: no cache");
    if (nnodes) *nnodes = cs->n_nodes;
    if (nrecords) *nrecords = cs->n_records;
    if (nodes && cs->n_nodes > 0)
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(nodes, cs->nodes.p, sizeof(pgx_cache_node) * cs->n_nodes,
                                          cudaMemcpyDeviceToHost, ctx->stream));
    if (records && cs->n_records > 0)
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(records, cs->recs.p, sizeof(pgx_path_vertex) * cs->n_records,
                                          cudaMemcpyDeviceToHost, ctx->stream));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return PGX_OK;
}

extern "C" int pgx_cache_export_weights(pgx_ctx* ctx, float* weights, int64_t* nrecords) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    CacheState* cs = static_cast<CacheState*>(ctx->cache_state);
    if (!cs || !cs->valid) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_cache_export_weights: no cache");
    if (nrecords) *nrecords = cs->n_records;
    if (weights && cs->n_records > 0) {
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(weights, cs->wts.p, sizeof(float) * cs->n_records, cudaMemcpyDeviceToHost,
                                          ctx->stream));
        PGX_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return PGX_OK;
}

extern "C" int pgx_cache_knn(pgx_ctx* ctx, const float* queries, int64_t nq, int32_t k, int32_t* idx, float* d2) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (nq < 0 || k < 1 || k > 64 || (nq > 0 && (!queries || !idx || !d2)))
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_cache_knn: bad arguments (1 <= k <= 64)");
    CacheState* cs = static_cast<CacheState*>(ctx->cache_state);
    if (!cs || !cs->valid) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_cache_knn: no cache");
    if (nq == 0) return PGX_OK;
    cudaStream_t s = ctx->stream;
    PGX_CUDA_TRY(ctx, cs->knn_q.reserve(sizeof(float) * 3 * nq));
    PGX_CUDA_TRY(ctx, cs->knn_i.reserve(sizeof(int) * k * nq));
    PGX_CUDA_TRY(ctx, cs->knn_d.reserve(sizeof(float) * k * nq));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(cs->knn_q.p, queries, sizeof(float) * 3 * nq, cudaMemcpyHostToDevice, s));
    k_knn<<<blocks_for(nq, 128), 128, 0, s>>>(cs->trav.as<CacheTravNode>(), cs->pos.as<float4>(),
                                              (int)cs->n_records, cs->knn_q.as<float>(), nq, k, cs->knn_i.as<int>(),
                                              cs->knn_d.as<float>());
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(idx, cs->knn_i.p, sizeof(int) * k * nq, cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(d2, cs->knn_d.p, sizeof(float) * k * nq, cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return PGX_OK;
}

static int guide_query(pgx_ctx* ctx, const float* positions, const float* in, int64_t n, int sample, float* dirs,
                       float* pdf) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    if (n < 0 || (n > 0 && (!positions || !in || !pdf || (sample && !dirs))))
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_guide_*: bad arguments");
    if (!guide_ready(ctx)) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_guide_*: no radiance cache");
    if (cstate(ctx)->pss)
        return pgx_fail(ctx, PGX_ERR_STATE,
                        "pgx_guide_*: the cache was built by a PGX_MODE_GUIDED_PSS render (primary-sample trees)");
    if (n == 0) return PGX_OK;
    cudaStream_t s = ctx->stream;
    const size_t in_floats = sample ? 2 : 3;
    DevBuf dp, di, dd, dpdf;
    PGX_CUDA_TRY(ctx, dp.reserve(sizeof(float) * 3 * n));
    PGX_CUDA_TRY(ctx, di.reserve(sizeof(float) * in_floats * n));
    PGX_CUDA_TRY(ctx, dd.reserve(sizeof(float) * 3 * n));
    PGX_CUDA_TRY(ctx, dpdf.reserve(sizeof(float) * n));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(dp.p, positions, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(di.p, in, sizeof(float) * in_floats * n, cudaMemcpyHostToDevice, s));
    k_guide_query<<<blocks_for(n, 128), 128, 0, s>>>(guide_view(ctx), dp.as<float>(), di.as<float>(), n, sample,
                                                      dd.as<float>(), dpdf.as<float>());
    PGX_CUDA_TRY(ctx, cudaGetLastError());
    if (sample) PGX_CUDA_TRY(ctx, cudaMemcpyAsync(dirs, dd.p, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(pdf, dpdf.p, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return PGX_OK;
}

extern "C" int pgx_guide_pdf(pgx_ctx* ctx, const float* positions, const float* dirs, int64_t n, float* pdf) {
    return guide_query(ctx, positions, dirs, n, 0, nullptr, pdf);
}

extern "C" int pgx_guide_sample(pgx_ctx* ctx, const float* positions, const float* u2, int64_t n, float* dirs,
                                float* pdf) {
    return guide_query(ctx, positions, u2, n, 1, dirs, pdf);
}

extern "C" int pgx_guide_configure(pgx_ctx* ctx, const pgx_guide_params* params) {
    if (!ctx) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    const pgx_guide_params defaults{1024, 0.01f, 10.f, 0.2f, 0.f, 0.f};
    const pgx_guide_params p = params ? *params : defaults;
    if (p.region_records < 256 || p.region_records > (1 << 20))
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_guide_configure: region_records %d outside [256, 2^20]",
                        (int)p.region_records);
    if (!(p.refine_fraction > 0.f && p.refine_fraction <= 1.f))
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_guide_configure: refine_fraction must be in (0, 1]");
    if (!(p.clamp_median >= 0.f) || !std::isfinite(p.clamp_median))
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_guide_configure: clamp_median must be finite and >= 0");
    if (!(p.uniform_share >= 0.f && p.uniform_share < 1.f))
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_guide_configure: uniform_share must be in [0, 1)");
    if (!(p.compensate >= 0.f && p.compensate <= 4.f))
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_guide_configure: compensate must be in [0, 4]");
    if (!(p.glossy_alpha >= 0.f) || !std::isfinite(p.glossy_alpha))
        return pgx_fail(ctx, PGX_ERR_INVALID_ARG, "pgx_guide_configure: glossy_alpha must be finite and >= 0");
    ctx->guide = p;
    return PGX_OK;
}

extern "C" int pgx_guide_get_params(pgx_ctx* ctx, pgx_guide_params* out) {
    if (!ctx || !out) return PGX_ERR_INVALID_ARG;
    *out = ctx->guide;
    return PGX_OK;
}

extern "C" int pgx_guide_export(pgx_ctx* ctx, pgx_guide_region* regions, int32_t* nregions, pgx_quad_node* qnodes,
                                int32_t* pss) {
    if (!ctx || !nregions) return PGX_ERR_INVALID_ARG;
    ctx->err.clear();
    CacheState* cs = static_cast<CacheState*>(ctx->cache_state);
    if (!cs || !cs->valid) return pgx_fail(ctx, PGX_ERR_STATE, "pgx_guide_export: no cache");
    static_assert(sizeof(pgx_quad_node) == sizeof(QuadNode), "quad node layouts differ");
    static_assert(PGX_QT_MAX_NODES == PGX_GUIDE_MAX_QUAD_NODES, "quad node capacity differs");
    const int nreg = cs->n_records > 0 ? cs->n_regions : 0;
    *nregions = nreg;
    if (pss) *pss = cs->pss ? 1 : 0;
    if (!regions || nreg == 0) return PGX_OK;
    cudaStream_t s = ctx->stream;
    std::vector<int2> rg((size_t)nreg);
    std::vector<int> qr((size_t)nreg);
    std::vector<int> nr((size_t)cs->n_nodes);
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(rg.data(), cs->regions.p, sizeof(int2) * nreg, cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaMemcpyAsync(qr.data(), cs->qroot.p, sizeof(int) * nreg, cudaMemcpyDeviceToHost, s));
    if (cs->n_nodes > 0)
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(nr.data(), cs->node_region.p, sizeof(int) * nr.size(),
                                          cudaMemcpyDeviceToHost, s));
    if (qnodes)
        PGX_CUDA_TRY(ctx, cudaMemcpyAsync(qnodes, cs->qnodes.p, sizeof(QuadNode) * PGX_QT_MAX_NODES * (size_t)nreg,
                                          cudaMemcpyDeviceToHost, s));
    PGX_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    for (int r = 0; r < nreg; r++) regions[r] = pgx_guide_region{rg[(size_t)r].x, rg[(size_t)r].y, -1, qr[(size_t)r]};
    for (size_t i = 0; i < nr.size(); i++)
        if (nr[i] >= 0 && nr[i] < nreg) regions[nr[i]].node = (int32_t)i;
    return PGX_OK;
}
