/* CPU restatement of the reference's hot path — the ORACLE (test
 * infrastructure only; see pgx_oracle.h).
 *
 * Arithmetic follows the reference expression by expression:
 *  - Vec4 dot is (x*x' + y*y') + z*z' (MyMath.h:118), cross as MyMath.h:134-140;
 *  - std::min(a, b) is (b < a) ? b : a and std::max(a, b) is (a < b) ? b : a,
 *    which fixes what happens to NaNs in the slab test;
 *  - division by a scalar multiplies by its reciprocal (MyMath.h:95-98).
 * Build with -ffp-contract=off -fno-fast-math. */
#include "pgx_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "pgx_oracle_rng.h"

#define ORC_EPSILON 1e-4f             /* Geometry.h:13 */
#define ORC_MT_EPSILON 1e-8f          /* Geometry.h:14 */
#define ORC_MAXNODE_TRIANGLES 4       /* Geometry.h:17 */
#define ORC_BOUNDS_COST 1.f           /* Geometry.h:18 */
#define ORC_INTERSECT_COST 1.5f       /* Geometry.h:19 */
#define ORC_BUILD_BINS 16             /* Geometry.h:20 */
#define ORC_STACK 64                  /* Geometry.h:461 */

typedef struct {
    float x, y, z;
} ov3;

static inline ov3 v3(float x, float y, float z) {
    ov3 r = {x, y, z};
    return r;
}
static inline ov3 v3_from(const float* p) { return v3(p[0], p[1], p[2]); }
static inline ov3 v3_sub(ov3 a, ov3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline ov3 v3_add(ov3 a, ov3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline ov3 v3_mul(ov3 a, ov3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline ov3 v3_scale(ov3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline float v3_dot(ov3 a, ov3 b) { return ((a.x * b.x) + (a.y * b.y)) + (a.z * b.z); }
static inline ov3 v3_cross(ov3 a, ov3 b) {
    return v3((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x));
}
static inline float v3_comp(ov3 a, int ax) { return ax == 0 ? a.x : (ax == 1 ? a.y : a.z); }
/* std::min / std::max argument order semantics. */
static inline float smin(float a, float b) { return (b < a) ? b : a; }
static inline float smax(float a, float b) { return (a < b) ? b : a; }
static inline ov3 v3_min(ov3 a, ov3 b) { return v3(smin(a.x, b.x), smin(a.y, b.y), smin(a.z, b.z)); }
static inline ov3 v3_max(ov3 a, ov3 b) { return v3(smax(a.x, b.x), smax(a.y, b.y), smax(a.z, b.z)); }

/* ------------------------------------------------------------------------ */
/* AABB (Geometry.h:156-229)                                                */
/* ------------------------------------------------------------------------ */
typedef struct {
    ov3 mx, mn;
} obox;

static inline void box_reset(obox* b) {
    b->mx = v3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
    b->mn = v3(FLT_MAX, FLT_MAX, FLT_MAX);
}
/* AABB::extend, Geometry.h:170-173 */
static inline void box_extend(obox* b, ov3 p) {
    b->mx = v3_max(b->mx, p);
    b->mn = v3_min(b->mn, p);
}
/* AABB::area, Geometry.h:212-215 */
static inline float box_area(const obox* b) {
    ov3 s = v3_sub(b->mx, b->mn);
    return (((s.x * s.y) + (s.y * s.z)) + (s.x * s.z)) * 2.f;
}

/* AABB::rayAABB, Geometry.h:175-192. */
static inline int ray_box(ov3 bmin, ov3 bmax, ov3 o, ov3 inv, float* t) {
    ov3 tmin = v3_mul(v3_sub(bmin, o), inv);
    ov3 tmax = v3_mul(v3_sub(bmax, o), inv);
    ov3 ten = v3_min(tmin, tmax);
    ov3 tex = v3_max(tmin, tmax);
    float fen = smax(ten.x, smax(ten.y, ten.z));
    float fex = smin(tex.x, smin(tex.y, tex.z));
    if (fen > fex || fex < 0.f) return 0;
    *t = smax(0.f, fen);
    return 1;
}

/* Triangle::rayIntersect (Möller–Trumbore), Geometry.h:101-130. */
static inline int ray_tri(const pgx_triangle* tri, ov3 o, ov3 d, float* t, float* u, float* v) {
    ov3 p0 = v3_from(tri->v[0].p);
    ov3 e0 = v3_sub(v3_from(tri->v[1].p), p0);
    ov3 e1 = v3_sub(v3_from(tri->v[2].p), p0);
    ov3 p = v3_cross(d, e1);
    float det = v3_dot(e0, p);
    if (fabsf(det) < ORC_MT_EPSILON) return 0;
    float inv_det = 1.f / det;
    ov3 T = v3_sub(o, p0);
    *u = v3_dot(T, p) * inv_det;
    if (*u < 0.f || *u > 1.f) return 0;
    ov3 q = v3_cross(T, e0);
    *v = v3_dot(d, q) * inv_det;
    if (*v < 0.f || *v > 1.f || (*u + *v > 1.f)) return 0;
    *t = v3_dot(e1, q) * inv_det;
    return *t >= 0.f;
}

/* Triangle::centre, Geometry.h:96-98 (note the 0.3333f). */
static inline ov3 tri_centre(const pgx_triangle* tri) {
    ov3 s = v3_add(v3_add(v3_from(tri->v[0].p), v3_from(tri->v[1].p)), v3_from(tri->v[2].p));
    return v3_scale(s, 0.3333f);
}

/* ------------------------------------------------------------------------ */
/* Binned-SAH build (Geometry.h:268-446)                                     */
/* ------------------------------------------------------------------------ */
typedef struct {
    obox b;
    int left_first, used;
} onode;

typedef struct {
    const pgx_triangle* tris;
    onode* nodes;
    int32_t* idx;
    int64_t nodes_used;
} obuild;

/* BVHNode::updateBounds, Geometry.h:274-287 */
static void build_update_bounds(obuild* B, int64_t i) {
    onode* nd = &B->nodes[i];
    box_reset(&nd->b);
    for (int k = 0; k < nd->used; k++) {
        const pgx_triangle* t = &B->tris[B->idx[nd->left_first + k]];
        box_extend(&nd->b, v3_from(t->v[0].p));
        box_extend(&nd->b, v3_from(t->v[1].p));
        box_extend(&nd->b, v3_from(t->v[2].p));
    }
}

/* BVHNode::findBestSplitPlane, Geometry.h:293-365 */
static float build_best_split(obuild* B, const onode* nd, int* axis, float* split_pos) {
    float parent_area = box_area(&nd->b);
    float best = FLT_MAX;
    for (int ax = 0; ax < 3; ax++) {
        float lo = FLT_MAX, hi = -FLT_MAX;
        for (int k = 0; k < nd->used; k++) {
            float c = v3_comp(tri_centre(&B->tris[B->idx[nd->left_first + k]]), ax);
            lo = smin(lo, c);
            hi = smax(hi, c);
        }
        if (lo == hi) continue;
        obox bin_box[ORC_BUILD_BINS];
        int bin_count[ORC_BUILD_BINS];
        for (int b = 0; b < ORC_BUILD_BINS; b++) {
            box_reset(&bin_box[b]);
            bin_count[b] = 0;
        }
        float scale = (float)ORC_BUILD_BINS / (hi - lo);
        for (int k = 0; k < nd->used; k++) {
            const pgx_triangle* t = &B->tris[B->idx[nd->left_first + k]];
            int bi = (int)((v3_comp(tri_centre(t), ax) - lo) * scale);
            bi = (bi < ORC_BUILD_BINS - 1) ? bi : ORC_BUILD_BINS - 1;
            bin_count[bi]++;
            box_extend(&bin_box[bi], v3_from(t->v[0].p));
            box_extend(&bin_box[bi], v3_from(t->v[1].p));
            box_extend(&bin_box[bi], v3_from(t->v[2].p));
        }
        float left_area[ORC_BUILD_BINS - 1], right_area[ORC_BUILD_BINS - 1];
        int left_count[ORC_BUILD_BINS - 1], right_count[ORC_BUILD_BINS - 1];
        int lsum = 0, rsum = 0;
        obox lb, rb;
        box_reset(&lb);
        box_reset(&rb);
        for (int i = 0; i < ORC_BUILD_BINS - 1; i++) {
            lsum += bin_count[i];
            left_count[i] = lsum;
            if (bin_count[i] > 0) {
                box_extend(&lb, bin_box[i].mn);
                box_extend(&lb, bin_box[i].mx);
            }
            left_area[i] = (lsum > 0) ? box_area(&lb) : 0.f;
            int r = ORC_BUILD_BINS - 1 - i;
            rsum += bin_count[r];
            right_count[ORC_BUILD_BINS - 2 - i] = rsum;
            if (bin_count[r] > 0) {
                box_extend(&rb, bin_box[r].mn);
                box_extend(&rb, bin_box[r].mx);
            }
            right_area[ORC_BUILD_BINS - 2 - i] = (rsum > 0) ? box_area(&rb) : 0.f;
        }
        scale = (hi - lo) / (float)ORC_BUILD_BINS;
        for (int i = 0; i < ORC_BUILD_BINS - 1; i++) {
            float la = left_area[i] / parent_area;
            float ra = right_area[i] / parent_area;
            float cost = ORC_BOUNDS_COST + ((la * (float)left_count[i]) * ORC_INTERSECT_COST) +
                         ((ra * (float)right_count[i]) * ORC_INTERSECT_COST);
            float cand = lo + scale * (float)(i + 1);
            if (cost < best) {
                *split_pos = cand;
                *axis = ax;
                best = cost;
            }
        }
    }
    return best;
}

/* BVHNode::subdivide, Geometry.h:367-417 (recursion depth is the tree
 * depth, bounded by the float resolution of the centroids). */
static void build_subdivide(obuild* B, int64_t i) {
    onode* nd = &B->nodes[i];
    if (nd->used <= ORC_MAXNODE_TRIANGLES) return;
    int axis = -1;
    float split_pos = -FLT_MAX;
    float split_cost = build_best_split(B, nd, &axis, &split_pos);
    float no_split = (float)nd->used * ORC_INTERSECT_COST;
    if (split_cost >= no_split || axis == -1) return;
    int a = nd->left_first;
    int b = a + nd->used - 1;
    while (a <= b) {
        float c = v3_comp(tri_centre(&B->tris[B->idx[a]]), axis);
        if (c < split_pos) {
            a++;
        } else {
            int32_t tmp = B->idx[a];
            B->idx[a] = B->idx[b];
            B->idx[b] = tmp;
            b--;
        }
    }
    int left_count = a - nd->left_first;
    if (left_count == 0 || left_count == nd->used) return;
    int64_t l = B->nodes_used++;
    int64_t r = B->nodes_used++;
    B->nodes[l].left_first = nd->left_first;
    B->nodes[l].used = left_count;
    B->nodes[r].left_first = a;
    B->nodes[r].used = nd->used - left_count;
    nd->left_first = (int)l;
    nd->used = 0;
    build_update_bounds(B, l);
    build_update_bounds(B, r);
    build_subdivide(B, l);
    build_subdivide(B, r);
}

/* BVHNode::build, Geometry.h:419-446 */
int64_t orc_bvh_build(const pgx_triangle* tris, int64_t n, pgx_bvh_node* out, int32_t* idx) {
    if (n <= 0) return 0;
    obuild B;
    B.tris = tris;
    B.idx = idx;
    B.nodes = (onode*)calloc((size_t)(2 * n - 1), sizeof(onode));
    B.nodes_used = 1;
    for (int64_t i = 0; i < n; i++) idx[i] = (int32_t)i;
    B.nodes[0].left_first = 0;
    B.nodes[0].used = (int)n;
    build_update_bounds(&B, 0);
    build_subdivide(&B, 0);
    for (int64_t i = 0; i < B.nodes_used; i++) {
        out[i].bmin[0] = B.nodes[i].b.mn.x;
        out[i].bmin[1] = B.nodes[i].b.mn.y;
        out[i].bmin[2] = B.nodes[i].b.mn.z;
        out[i].bmax[0] = B.nodes[i].b.mx.x;
        out[i].bmax[1] = B.nodes[i].b.mx.y;
        out[i].bmax[2] = B.nodes[i].b.mx.z;
        out[i].left_first = B.nodes[i].left_first;
        out[i].used = B.nodes[i].used;
    }
    int64_t cnt = B.nodes_used;
    free(B.nodes);
    return cnt;
}

static double node_area_d(const pgx_bvh_node* n) {
    double sx = (double)n->bmax[0] - n->bmin[0];
    double sy = (double)n->bmax[1] - n->bmin[1];
    double sz = (double)n->bmax[2] - n->bmin[2];
    return 2.0 * (sx * sy + sy * sz + sx * sz);
}

double orc_sah_cost(const pgx_bvh_node* nodes, int64_t nnodes) {
    if (nnodes <= 0) return 0.0;
    double root = node_area_d(&nodes[0]);
    if (!(root > 0.0)) return 0.0;
    double cost = 0.0;
    for (int64_t i = 0; i < nnodes; i++) {
        double a = node_area_d(&nodes[i]) / root;
        if (nodes[i].used > 0)
            cost += a * nodes[i].used * (double)ORC_INTERSECT_COST;
        else
            cost += a * (double)ORC_BOUNDS_COST;
    }
    return cost;
}

/* ------------------------------------------------------------------------ */
/* Traversal (Geometry.h:448-567)                                            */
/* ------------------------------------------------------------------------ */
static inline ov3 node_min(const pgx_bvh_node* n) { return v3(n->bmin[0], n->bmin[1], n->bmin[2]); }
static inline ov3 node_max(const pgx_bvh_node* n) { return v3(n->bmax[0], n->bmax[1], n->bmax[2]); }

/* BVHNode::traverse, Geometry.h:455-512.  `best_t` enters as the initial
 * intersection.t (FLT_MAX in the reference).  Returns 0 on stack overflow
 * (the reference would write past its 64-entry stack). */
static int trace_one_closest(const pgx_triangle* tris, const pgx_bvh_node* nodes, const int32_t* idx,
                             ov3 o, ov3 d, float t0, pgx_hit* hit, int64_t* iv, int64_t* tt) {
    ov3 inv = v3(1.f / d.x, 1.f / d.y, 1.f / d.z); /* Ray::init, Geometry.h:35 */
    hit->id = -1;
    hit->t = t0;
    hit->u = 0.f;
    hit->v = 0.f;
    int stack[ORC_STACK];
    int sp = 0;
    const pgx_bvh_node* node = &nodes[0];
    float tb;
    if (!ray_box(node_min(node), node_max(node), o, inv, &tb)) return 1;
    if (tb > hit->t) return 1;
    for (;;) {
        if (node->used > 0) {
            for (int k = 0; k < node->used; k++) {
                int ti = idx[node->left_first + k];
                float t, u, v;
                (*tt)++;
                if (ray_tri(&tris[ti], o, d, &t, &u, &v)) {
                    if (t > ORC_EPSILON && t < hit->t) {
                        hit->t = t;
                        hit->id = ti;
                        hit->u = u;
                        hit->v = v;
                    }
                }
            }
            if (sp == 0) break;
            node = &nodes[stack[--sp]];
            continue;
        }
        (*iv)++;
        int li = node->left_first, ri = node->left_first + 1;
        const pgx_bvh_node* L = &nodes[li];
        const pgx_bvh_node* R = &nodes[ri];
        float dl = 0.f, dr = 0.f;
        if (!ray_box(node_min(L), node_max(L), o, inv, &dl) || dl >= hit->t) dl = FLT_MAX;
        if (!ray_box(node_min(R), node_max(R), o, inv, &dr) || dr >= hit->t) dr = FLT_MAX;
        if (dl > dr) {
            float tf = dl;
            dl = dr;
            dr = tf;
            const pgx_bvh_node* tn = L;
            L = R;
            R = tn;
            int ti = li;
            li = ri;
            ri = ti;
        }
        if (dl == FLT_MAX) {
            if (sp == 0) break;
            node = &nodes[stack[--sp]];
        } else {
            node = L;
            if (dr != FLT_MAX) {
                if (sp >= ORC_STACK) return 0;
                stack[sp++] = ri;
            }
        }
    }
    return 1;
}

/* BVHNode::traverseVisible, Geometry.h:514-567 */
static int trace_one_any(const pgx_triangle* tris, const pgx_bvh_node* nodes, const int32_t* idx, ov3 o,
                         ov3 d, float max_t, int64_t* iv, int64_t* tt) {
    ov3 inv = v3(1.f / d.x, 1.f / d.y, 1.f / d.z);
    int stack[ORC_STACK];
    int sp = 0;
    const pgx_bvh_node* node = &nodes[0];
    float tb;
    if (!ray_box(node_min(node), node_max(node), o, inv, &tb)) return 1;
    if (tb > max_t) return 1;
    for (;;) {
        if (node->used > 0) {
            for (int k = 0; k < node->used; k++) {
                int ti = idx[node->left_first + k];
                float t, u, v;
                (*tt)++;
                if (ray_tri(&tris[ti], o, d, &t, &u, &v)) {
                    if (t > ORC_EPSILON && t < max_t) return 0;
                }
            }
            if (sp == 0) break;
            node = &nodes[stack[--sp]];
            continue;
        }
        (*iv)++;
        int li = node->left_first, ri = node->left_first + 1;
        const pgx_bvh_node* L = &nodes[li];
        const pgx_bvh_node* R = &nodes[ri];
        float dl = 0.f, dr = 0.f;
        if (!ray_box(node_min(L), node_max(L), o, inv, &dl) || dl >= max_t) dl = FLT_MAX;
        if (!ray_box(node_min(R), node_max(R), o, inv, &dr) || dr >= max_t) dr = FLT_MAX;
        if (dl > dr) {
            float tf = dl;
            dl = dr;
            dr = tf;
            const pgx_bvh_node* tn = L;
            L = R;
            R = tn;
            int ti = li;
            li = ri;
            ri = ti;
        }
        if (dl == FLT_MAX) {
            if (sp == 0) break;
            node = &nodes[stack[--sp]];
        } else {
            node = L;
            if (dr != FLT_MAX) {
                if (sp >= ORC_STACK) return 1;
                stack[sp++] = ri;
            }
        }
    }
    return 1;
}

void orc_trace_closest(const pgx_triangle* tris, const pgx_bvh_node* nodes, const int32_t* idx,
                       const pgx_ray* rays, int64_t n, pgx_hit* hits, int64_t* interior_visits,
                       int64_t* tri_tests) {
    int64_t iv = 0, tt = 0;
    for (int64_t i = 0; i < n; i++) {
        trace_one_closest(tris, nodes, idx, v3_from(rays[i].o), v3_from(rays[i].d), rays[i].tmax, &hits[i],
                          &iv, &tt);
    }
    if (interior_visits) *interior_visits += iv;
    if (tri_tests) *tri_tests += tt;
}

void orc_trace_any(const pgx_triangle* tris, const pgx_bvh_node* nodes, const int32_t* idx,
                   const pgx_ray* rays, int64_t n, uint8_t* visible, int64_t* interior_visits,
                   int64_t* tri_tests) {
    int64_t iv = 0, tt = 0;
    for (int64_t i = 0; i < n; i++) {
        visible[i] = (uint8_t)trace_one_any(tris, nodes, idx, v3_from(rays[i].o), v3_from(rays[i].d),
                                            rays[i].tmax, &iv, &tt);
    }
    if (interior_visits) *interior_visits += iv;
    if (tri_tests) *tri_tests += tt;
}

typedef struct {
    const pgx_triangle* tris;
    const pgx_bvh_node* nodes;
    const int32_t* idx;
    const pgx_ray* rays;
    pgx_hit* hits;
    int64_t begin, end;
} otrace_job;

static void* trace_worker(void* arg) {
    otrace_job* j = (otrace_job*)arg;
    orc_trace_closest(j->tris, j->nodes, j->idx, j->rays + j->begin, j->end - j->begin, j->hits + j->begin,
                      NULL, NULL);
    return NULL;
}

void orc_trace_closest_mt(const pgx_triangle* tris, const pgx_bvh_node* nodes, const int32_t* idx,
                          const pgx_ray* rays, int64_t n, pgx_hit* hits, int32_t threads) {
    if (threads < 1) threads = 1;
    pthread_t* th = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    otrace_job* jobs = (otrace_job*)calloc((size_t)threads, sizeof(otrace_job));
    for (int i = 0; i < threads; i++) {
        jobs[i].tris = tris;
        jobs[i].nodes = nodes;
        jobs[i].idx = idx;
        jobs[i].rays = rays;
        jobs[i].hits = hits;
        jobs[i].begin = n * i / threads;
        jobs[i].end = n * (i + 1) / threads;
        pthread_create(&th[i], NULL, trace_worker, &jobs[i]);
    }
    for (int i = 0; i < threads; i++) pthread_join(th[i], NULL);
    free(th);
    free(jobs);
}

void orc_rng_floats(uint64_t seed, uint64_t pixel, uint64_t sample, int32_t count, float* out) {
    uint64_t s = orc_pcg_init(seed, pixel, sample);
    for (int32_t i = 0; i < count; i++) out[i] = orc_pcg_next_float(&s);
}
