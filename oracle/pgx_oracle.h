/* CPU restatement of the reference's hot path — the ORACLE.
 *
 * TEST INFRASTRUCTURE ONLY.  Tests, `__graft_entry__.smoke()` and the CPU
 * baseline leg of bench.py may load this library as the checker; the
 * product (libpgx) never links or calls it.
 *
 * Every function restates a reference function, cited by file:line in
 * pgx_oracle.c, with the reference's float operation order (the library is
 * built with -ffp-contract=off so no FMA is formed).  Its outputs are pinned
 * against the reference compiled headless (oracle/ref_harness.cpp) by
 * tests/test_oracle_pin.py and by the fixtures in tests/golden/. */
#ifndef PGX_ORACLE_H_
#define PGX_ORACLE_H_

#include <stdint.h>

#include "../include/pgx.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Binned-SAH BVH (BVHNode::build).  nodes needs room for 2n-1 entries, idx
 * for n.  Returns the node count. */
int64_t orc_bvh_build(const pgx_triangle* tris, int64_t n, pgx_bvh_node* nodes, int32_t* idx);

/* SAH cost of a tree: sum over interior nodes of A/A_root * 1 plus sum over
 * leaves of A/A_root * used * 1.5 (constants of Geometry.h:17-20). */
double orc_sah_cost(const pgx_bvh_node* nodes, int64_t nnodes);

/* Closest hit (BVHNode::traverse) and any hit (BVHNode::traverseVisible)
 * over a tree in the reference layout.  Counters (may be NULL) add the
 * number of interior nodes whose two child boxes were tested and the
 * number of ray/triangle tests. */
void orc_trace_closest(const pgx_triangle* tris, const pgx_bvh_node* nodes, const int32_t* idx,
                       const pgx_ray* rays, int64_t n, pgx_hit* hits, int64_t* interior_visits,
                       int64_t* tri_tests);
void orc_trace_any(const pgx_triangle* tris, const pgx_bvh_node* nodes, const int32_t* idx,
                   const pgx_ray* rays, int64_t n, uint8_t* visible, int64_t* interior_visits,
                   int64_t* tri_tests);

/* Multi-threaded closest hit for CPU timing (same arithmetic). */
void orc_trace_closest_mt(const pgx_triangle* tris, const pgx_bvh_node* nodes, const int32_t* idx,
                          const pgx_ray* rays, int64_t n, pgx_hit* hits, int32_t threads);

/* PCG32 stream (pgx_oracle_rng.h) exposed for the GPU stream test. */
void orc_rng_floats(uint64_t seed, uint64_t pixel, uint64_t sample, int32_t count, float* out);

#ifdef __cplusplus
}
#endif

#endif
