// Stack traversal of the binary BVH: closest hit (BVHNode::traverse,
// Geometry.h:455-512) and any hit (BVHNode::traverseVisible,
// Geometry.h:514-567).
//
// The visit order is the reference's: at an interior node both child boxes
// are tested, a child whose entry distance is >= the current t (or maxT) is
// dropped, the nearer child is entered (the left one on ties), the farther
// one is pushed, and popped nodes are entered without re-testing their box.
// Triangles of a leaf are tested in index order and a hit replaces the best
// one only when 1e-4 < t < best, so ties keep the first triangle visited.
// Box and triangle arithmetic is exact (pgx_device.cuh), hence hits are
// bit-identical to the reference on the same tree.
//
// The stack holds (ref, count) child references in per-thread local memory
// (L1-cached).  Its depth is checked against PGX_STACK_SIZE: an overflow
// ends the ray with status 1 instead of writing out of bounds (the
// reference pushes unchecked, Geometry.h:509).
#pragma once

#include "pgx_device.cuh"

struct BvhView {
    const TravNode* __restrict__ nodes;
    const TravTri* __restrict__ tris;
    TravRoot root;
    int n_records;  // bound for interior references
    int n_tris;     // bound for leaf ranges
};

// 32 bytes through the read-only path in one 256-bit load (sm_100 and
// later); p must be 32-byte aligned.
__device__ __forceinline__ void ldg_256(const void* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

// A node record in two 256-bit loads: the traversal is bound by L1 request
// throughput (every lane of a warp reads its own node), and this halves the
// load instructions per node compared with four 128-bit loads.  Records are
// 64 bytes in a cudaMalloc'd (256-byte aligned) array, so each half is
// 32-byte aligned.
__device__ __forceinline__ TravNode load_node(const TravNode* __restrict__ nodes, int i) {
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    TravNode n;
    ldg_256(p + 0, n.lmin, n.lmax);
    ldg_256(p + 2, n.rmin, n.rmax);
    return n;
}

// Closest hit (ANY = false) or any hit (ANY = true).
// Returns: for ANY, 1 when an occluder was found (not visible); otherwise
// the hit fields are updated.  `status` gets 1 on stack overflow and 2 on
// a reference outside the tree (a corrupt imported BVH).
template <bool ANY, bool COUNT>
__device__ __forceinline__ bool bvh_trace(const BvhView& bvh, const xv3& o, const xv3& d, float tmax, int& hit_id,
                                          float& hit_t, float& hit_u, float& hit_v, int& status,
                                          unsigned long long& n_interior, unsigned long long& n_tris) {
    hit_id = -1;
    hit_t = tmax;
    status = 0;
    if (!bvh.root.valid) return false;
    xv3 inv = mk(x_div(1.f, d.x), x_div(1.f, d.y), x_div(1.f, d.z));
    float tb;
    if (!ray_box(bvh.root.bmin[0], bvh.root.bmin[1], bvh.root.bmin[2], bvh.root.bmax[0], bvh.root.bmax[1],
                 bvh.root.bmax[2], o, inv, tb))
        return false;
    if (tb > tmax) return false;

    int2 stack[PGX_STACK_SIZE];
    int sp = 0;
    int ref = bvh.root.ref;
    int cnt = bvh.root.count;
    for (;;) {
        if (cnt > 0) {
            // Leaf: test its triangles in order.
            if ((unsigned)ref > (unsigned)bvh.n_tris || cnt > bvh.n_tris - ref) {
                status = 2;  // corrupt tree: stop instead of reading out of bounds
                return false;
            }
            for (int k = 0; k < cnt; k++) {
                const float4* tp = reinterpret_cast<const float4*>(bvh.tris + ref + k);
                float4 a, b;
                ldg_256(tp, a, b);
                float4 c = __ldg(tp + 2);
                if (COUNT) n_tris++;
                float t, u, v;
                if (ray_tri(mk(a), mk(b), mk(c), o, d, t, u, v)) {
                    if (ANY) {
                        if (t > PGX_EPSILON && t < tmax) return true;
                    } else if (t > PGX_EPSILON && t < hit_t) {
                        hit_t = t;
                        hit_id = __float_as_int(a.w);
                        hit_u = u;
                        hit_v = v;
                    }
                }
            }
            if (sp == 0) break;
            --sp;
            ref = stack[sp].x;
            cnt = stack[sp].y;
            continue;
        }
        if (COUNT) n_interior++;
        if ((unsigned)ref >= (unsigned)bvh.n_records) {
            status = 2;
            return false;
        }
        TravNode n = load_node(bvh.nodes, ref);
        const float lim = ANY ? tmax : hit_t;
        float dl = 0.f, dr = 0.f;
        if (!ray_box(n.lmin.x, n.lmin.y, n.lmin.z, n.lmax.x, n.lmax.y, n.lmax.z, o, inv, dl) || dl >= lim)
            dl = FLT_MAX;
        if (!ray_box(n.rmin.x, n.rmin.y, n.rmin.z, n.rmax.x, n.rmax.y, n.rmax.z, o, inv, dr) || dr >= lim)
            dr = FLT_MAX;
        int nref = __float_as_int(n.lmin.w), ncnt = __float_as_int(n.lmax.w);
        int fref = __float_as_int(n.rmin.w), fcnt = __float_as_int(n.rmax.w);
        if (dl > dr) {
            float tf = dl;
            dl = dr;
            dr = tf;
            int t0 = nref;
            nref = fref;
            fref = t0;
            t0 = ncnt;
            ncnt = fcnt;
            fcnt = t0;
        }
        if (dl == FLT_MAX) {
            if (sp == 0) break;
            --sp;
            ref = stack[sp].x;
            cnt = stack[sp].y;
        } else {
            ref = nref;
            cnt = ncnt;
            if (dr != FLT_MAX) {
                if (sp >= PGX_STACK_SIZE) {
                    status = 1;
                    return false;
                }
                stack[sp] = make_int2(fref, fcnt);
                sp++;
            }
        }
    }
    return false;
}

// ---- persistent traversal with lane refill ----------------------------------
// Stack of one lane of the persistent traversal (PGX_STACK_SIZE entries, the
// reference's depth): the top SHORT entries live in shared memory (one column
// per thread of the block, so a warp's accesses fall in distinct banks),
// deeper ones spill to local memory.  SHORT trades shared memory (8 bytes x
// 128 threads per entry, so resident blocks) against local-memory traffic;
// the batch autotuner picks it from kShortStackChoices.
constexpr int kShortStack = 8;
constexpr int kShortStackChoices[] = {4, 8, 16};
constexpr int kTraceMaxBlock = 128;  // block size of every kernel using trace_persistent
template <int SHORT = kShortStack>
struct TraceStack {
    int2* sh;  // this thread's column: entry i at sh[i * kTraceMaxBlock]
    int2 loc[PGX_STACK_SIZE - SHORT];
    __device__ __forceinline__ void put(int i, int2 v) {
        if (i < SHORT)
            sh[i * kTraceMaxBlock] = v;
        else
            loc[i - SHORT] = v;
    }
    __device__ __forceinline__ int2 get(int i) const { return i < SHORT ? sh[i * kTraceMaxBlock] : loc[i - SHORT]; }
};

// The same per-ray algorithm as bvh_trace, cut into steps (one interior node
// or one triangle) so that a warp can keep stepping while its lanes finish at
// different times: every few steps, lanes whose ray is done fetch the next
// ray index from a global counter (warp-aggregated atomicAdd).  Each ray still
// visits its nodes and triangles in exactly bvh_trace's order, so results are
// identical; only which rays share a warp instruction changes.
struct TraceLane {
    xv3 o, d, inv;
    float tmax;   // ANY: the visibility limit; closest: the current best t
    float hu, hv;
    int hit_id;
    int ref, cnt, k;  // current node reference; for leaves, next triangle k
    int sp;
    int status;
    bool finite;  // every component of inv is finite (see ray_box_finite)
};

// Starts a ray at `root`; returns false when the root box is missed (finished).
__device__ __forceinline__ bool lane_start(const TravRoot& root, TraceLane& L, xv3 o, xv3 d, float tmax) {
    L.o = o;
    L.d = d;
    L.tmax = tmax;
    L.hit_id = -1;
    L.hu = 0.f;
    L.hv = 0.f;
    L.sp = 0;
    L.k = 0;
    L.status = 0;
    if (!root.valid) return false;
    L.inv = mk(x_div(1.f, d.x), x_div(1.f, d.y), x_div(1.f, d.z));
    L.finite = isfinite(L.inv.x) && isfinite(L.inv.y) && isfinite(L.inv.z);
    float tb;
    if (!ray_box(root.bmin[0], root.bmin[1], root.bmin[2], root.bmax[0], root.bmax[1], root.bmax[2], o, L.inv, tb))
        return false;
    if (tb > tmax) return false;
    L.ref = root.ref;
    L.cnt = root.count;
    return true;
}

// The tree's own root for every ray (one scene).
struct SceneRoot {
    __device__ __forceinline__ const TravRoot& operator()(unsigned, const BvhView& bvh) const { return bvh.root; }
};

// One step; returns true when the ray is finished (for ANY, hit_id >= 0
// marks an occluder).
template <bool ANY, bool COUNT, class Stack>
__device__ __forceinline__ bool lane_step(const BvhView& bvh, TraceLane& L, Stack& stack, unsigned long long& n_interior,
                                          unsigned long long& n_tris) {
    if (L.cnt > 0) {
        if ((unsigned)L.ref > (unsigned)bvh.n_tris || L.cnt > bvh.n_tris - L.ref) {
            L.status = 2;
            return true;
        }
        const float4* tp = reinterpret_cast<const float4*>(bvh.tris + L.ref + L.k);
        float4 a, b;
        ldg_256(tp, a, b);
        float4 c = __ldg(tp + 2);
        if (COUNT) n_tris++;
        float t, u, v;
        if (ray_tri(mk(a), mk(b), mk(c), L.o, L.d, t, u, v)) {
            if (ANY) {
                if (t > PGX_EPSILON && t < L.tmax) {
                    L.hit_id = __float_as_int(a.w);
                    return true;
                }
            } else if (t > PGX_EPSILON && t < L.tmax) {
                L.tmax = t;
                L.hit_id = __float_as_int(a.w);
                L.hu = u;
                L.hv = v;
            }
        }
        if (++L.k < L.cnt) return false;
        L.k = 0;
        if (L.sp == 0) return true;
        --L.sp;
        {
            int2 e = stack.get(L.sp);
            L.ref = e.x;
            L.cnt = e.y;
        }
        return false;
    }
    if (COUNT) n_interior++;
    if ((unsigned)L.ref >= (unsigned)bvh.n_records) {
        L.status = 2;
        return true;
    }
    TravNode n = load_node(bvh.nodes, L.ref);
    const float lim = L.tmax;
    float dl = 0.f, dr = 0.f;
    bool hl, hr;
    if (L.finite) {
        hl = ray_box_finite(n.lmin.x, n.lmin.y, n.lmin.z, n.lmax.x, n.lmax.y, n.lmax.z, L.o, L.inv, dl);
        hr = ray_box_finite(n.rmin.x, n.rmin.y, n.rmin.z, n.rmax.x, n.rmax.y, n.rmax.z, L.o, L.inv, dr);
    } else {
        hl = ray_box(n.lmin.x, n.lmin.y, n.lmin.z, n.lmax.x, n.lmax.y, n.lmax.z, L.o, L.inv, dl);
        hr = ray_box(n.rmin.x, n.rmin.y, n.rmin.z, n.rmax.x, n.rmax.y, n.rmax.z, L.o, L.inv, dr);
    }
    if (!hl || dl >= lim) dl = FLT_MAX;
    if (!hr || dr >= lim) dr = FLT_MAX;
    int nref = __float_as_int(n.lmin.w), ncnt = __float_as_int(n.lmax.w);
    int fref = __float_as_int(n.rmin.w), fcnt = __float_as_int(n.rmax.w);
    if (dl > dr) {
        float tf = dl;
        dl = dr;
        dr = tf;
        int t0 = nref;
        nref = fref;
        fref = t0;
        t0 = ncnt;
        ncnt = fcnt;
        fcnt = t0;
    }
    if (dl == FLT_MAX) {
        if (L.sp == 0) return true;
        --L.sp;
        {
            int2 e = stack.get(L.sp);
            L.ref = e.x;
            L.cnt = e.y;
        }
        return false;
    }
    L.ref = nref;
    L.cnt = ncnt;
    if (dr != FLT_MAX) {
        if (L.sp >= PGX_STACK_SIZE) {
            L.status = 1;
            return true;
        }
        stack.put(L.sp, make_int2(fref, fcnt));
        L.sp++;
    }
    return false;
}

// Persistent warp loop over rays [0, n): `load(i, o, d, tmax)` fetches ray i,
// `store(i, lane)` consumes a finished ray, `root_of(i, bvh)` gives the tree
// root ray i starts from (several trees can share the node and triangle
// arrays).  `next` is a zeroed counter.  Must be called by whole warps.
template <bool ANY, bool COUNT, class Load, class Store, class RootOf = SceneRoot, int SHORT = kShortStack>
__device__ __forceinline__ void trace_persistent(const BvhView& bvh, unsigned n, unsigned* next, Load load,
                                                 Store store, unsigned long long& n_interior,
                                                 unsigned long long& n_tris, unsigned& status_or,
                                                 RootOf root_of = RootOf()) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    constexpr int kRefillBelow = 24;  // refill when fewer lanes than this are busy
    constexpr int kMaxSteps = 64;
    constexpr int kCheckEvery = 8;    // steps between occupancy votes
    const int lane = threadIdx.x & 31;
    __shared__ int2 s_stack[SHORT * kTraceMaxBlock];
    TraceStack<SHORT> stack;
    stack.sh = s_stack + threadIdx.x;
    TraceLane L;
    int ray = -1;
    bool exhausted = false;
    for (;;) {
        // Refill idle lanes (possibly several rounds when roots are missed).
        for (;;) {
            bool need = ray < 0 && !exhausted;
            unsigned m = __ballot_sync(kFull, need);
            if (!m) break;
            int leader = __ffs(m) - 1;
            unsigned base = 0;
            if (lane == leader) base = atomicAdd(next, (unsigned)__popc(m));
            base = __shfl_sync(kFull, base, leader);
            if (need) {
                unsigned idx = base + __popc(m & ((1u << lane) - 1u));
                if (idx < n) {
                    xv3 o, d;
                    float tmax;
                    load(idx, o, d, tmax);
                    if (lane_start(root_of(idx, bvh), L, o, d, tmax)) {
                        ray = (int)idx;
                    } else {
                        store(idx, L);  // missed the root: finished
                    }
                } else {
                    exhausted = true;
                }
            }
        }
        if (__all_sync(kFull, ray < 0)) break;  // every lane idle and the queue is drained
        for (int s = 0; s < kMaxSteps; s++) {
            // Branch vote: lanes at a leaf (triangle tests) and lanes at an
            // interior node (two slab tests) take different code; when a warp
            // holds both, only the larger group steps this time and the other
            // waits one step.  A ray's own sequence of nodes and triangles is
            // unchanged (it only pauses), so results stay bit-identical.
            const unsigned act = __ballot_sync(kFull, ray >= 0);
            const unsigned leaf = __ballot_sync(kFull, ray >= 0 && L.cnt > 0);
            const bool leaf_turn = 2 * __popc(leaf) >= __popc(act);
            if (ray >= 0 && (L.cnt > 0) == leaf_turn) {
                if (lane_step<ANY, COUNT>(bvh, L, stack, n_interior, n_tris)) {
                    status_or |= (unsigned)L.status;
                    store((unsigned)ray, L);
                    ray = -1;
                }
            }
            if (kCheckEvery > 1 && (s % kCheckEvery) != kCheckEvery - 1) continue;
            unsigned busy = __ballot_sync(kFull, ray >= 0);
            if (__popc(busy) < kRefillBelow && !__all_sync(kFull, exhausted || ray >= 0)) break;
            if (busy == 0) break;
        }
    }
}
