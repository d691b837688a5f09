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

__device__ __forceinline__ TravNode load_node(const TravNode* __restrict__ nodes, int i) {
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    TravNode n;
    n.lmin = __ldg(p + 0);
    n.lmax = __ldg(p + 1);
    n.rmin = __ldg(p + 2);
    n.rmax = __ldg(p + 3);
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
                float4 a = __ldg(tp + 0);
                float4 b = __ldg(tp + 1);
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
