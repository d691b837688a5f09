/*
 * pgx.h — C ABI of the GB300-native wavefront path tracer.
 *
 * The reference (IsaGeriler/PathGuidingDissertation) is a header-only C++
 * class API with no FFI: `Scene` (Scene.h:76-176), `RayTracer`
 * (Renderer.h:236-752), the `BSDF` (Materials.h:121-134) and `Light`
 * (Lights.h:16-26) virtual interfaces, the triangle BVH (Geometry.h:268-567)
 * and the path-vertex cache `PointBVHNode` (Renderer.h:71-234).  Each entry
 * point below names the reference member it stands in for.  The C++ façade
 * in pgx.hpp rebuilds the reference's class names on top of these calls.
 *
 * Conventions
 *  - Every function returns an int status (PGX_OK == 0).  On failure
 *    pgx_last_error(ctx) gives a message.  Nothing exits or asserts.
 *  - Inputs are copied at the call; the caller keeps ownership of its
 *    buffers.  Outputs go to caller-allocated host buffers unless the name
 *    ends in `_device`, where device pointers are borrowed for the call.
 *  - One context owns one CUDA stream and all device memory it allocates.
 *    Calls on one context must not overlap; separate contexts may be used
 *    from separate threads.
 *  - Floating point is IEEE binary32 throughout; triangle/box intersection
 *    reproduces the reference's arithmetic exactly (no FMA contraction).
 */
#ifndef PGX_H_
#define PGX_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define PGX_OK 0
#define PGX_ERR_INVALID_ARG 1 /* null pointer, negative size, bad enum      */
#define PGX_ERR_OOM 2         /* device or host allocation failed           */
#define PGX_ERR_CUDA 3        /* a CUDA runtime call failed                 */
#define PGX_ERR_OVERFLOW 4    /* traversal stack / queue capacity exceeded  */
#define PGX_ERR_TIMEOUT 5     /* a bounded device wait gave up              */
#define PGX_ERR_STATE 6       /* call out of order (e.g. render w/o scene)  */

/* ---- scene description --------------------------------------------------- */

/* Reference `Vertex` (MyMath.h:146-149) without the Vec4 w lanes. */
typedef struct pgx_vertex {
    float p[3];
    float n[3];
    float u, v;
} pgx_vertex;

/* Reference `Triangle` inputs (Geometry.h:76-94): three vertices and the
 * index of its material.  Edges, normal and area are derived on upload
 * exactly as `Triangle::init` derives them. */
typedef struct pgx_triangle {
    pgx_vertex v[3];
    uint32_t material;
} pgx_triangle;

/* BSDF kinds, one per reference class in Materials.h. */
enum pgx_bsdf_kind {
    PGX_BSDF_DIFFUSE = 0,    /* DiffuseBSDF     Materials.h:136-189 */
    PGX_BSDF_MIRROR = 1,     /* MirrorBSDF      Materials.h:191-234 */
    PGX_BSDF_CONDUCTOR = 2,  /* ConductorBSDF   Materials.h:236-358 */
    PGX_BSDF_GLASS = 3,      /* GlassBSDF       Materials.h:360-440 */
    PGX_BSDF_DIELECTRIC = 4, /* DielectricBSDF  Materials.h:442-639 */
    PGX_BSDF_ORENNAYAR = 5,  /* OrenNayarBSDF   Materials.h:641-721 */
    PGX_BSDF_PLASTIC = 6     /* PlasticBSDF     Materials.h:724-853 */
};

/* One material: the constructor arguments of the reference BSDF classes.
 * `roughness` is converted to alpha = 1.62142*sqrt(roughness) as the
 * reference constructors do (Materials.h:249,455,737).  `albedo_texture`
 * indexes the texture table given to pgx_scene_upload (the reference's
 * `Texture*` albedo); -1 means a 1x1 texture holding `albedo`.
 * `emission` with positive luminance turns the material into an area light
 * (`BSDF::addLight`, `Scene::build` Scene.h:92-100).  `layered` != 0 wraps
 * it in the pass-through LayeredBSDF (Materials.h:855-897). */
typedef struct pgx_material {
    int32_t kind;
    int32_t albedo_texture;
    float albedo[3];
    float eta[3];
    float k[3];
    float int_ior;
    float ext_ior;
    float roughness;
    float sigma;
    float emission[3];
    int32_t layered;
} pgx_material;

/* RGB float texture (reference `Texture`, Imaging.h:23-138). */
typedef struct pgx_texture {
    int32_t width;
    int32_t height;
    const float* rgb; /* width*height*3, row-major, row 0 first */
} pgx_texture;

/* Pinhole camera as `loadScene` sets it up (SceneLoader.h:226-243):
 * Matrix::perspective(0.001, 10000, width/height, fov) and the inverse of
 * Matrix::lookAt(from, to, up). */
typedef struct pgx_camera {
    float from[3];
    float to[3];
    float up[3];
    float fov_degrees;
    int32_t width;
    int32_t height;
    int32_t flip_x;
} pgx_camera;

/* ---- rays and hits -------------------------------------------------------- */

/* A ray.  Closest hit starts its search at t = tmax (FLT_MAX gives the
 * reference's `IntersectionData` default, Geometry.h:247-253); any hit
 * reports an occluder only for t in (1e-4, tmax) (Geometry.h:514-567). */
typedef struct pgx_ray {
    float o[3];
    float tmax;
    float d[3];
    float pad;
} pgx_ray;

/* Closest hit: triangle index (-1 on a miss), distance, and the barycentric
 * beta (u) and gamma (v); alpha = 1 - (u + v) as in Geometry.h:478-480. */
typedef struct pgx_hit {
    int32_t id;
    float t;
    float u;
    float v;
} pgx_hit;

/* One node of a binary BVH in the reference's layout (BVHBuildNode,
 * Geometry.h:255-261): children of an interior node are left_first and
 * left_first + 1; a leaf (used > 0) owns tri_index[left_first ..
 * left_first + used). */
typedef struct pgx_bvh_node {
    float bmin[3];
    float bmax[3];
    int32_t left_first;
    int32_t used;
} pgx_bvh_node;

typedef struct pgx_bvh_stats {
    int64_t nodes;
    int64_t leaves;
    int32_t max_depth;
    int32_t max_leaf_size;
    double sah_cost; /* sum_int A/A_root*1 + sum_leaf A/A_root*N*1.5 */
    double build_ms;
} pgx_bvh_stats;

/* ---- rendering ---------------------------------------------------------- */

enum pgx_render_mode {
    /* `RayTracer::pathTrace` (Renderer.h:531-618): NEE + MIS, RR from
     * depth > 3 on throughput, stop at depth 8. */
    PGX_MODE_PLAIN = 0,
    /* `RayTracer::guidedPath` with GUIDED_PATH (Renderer.h:368-528): image =
     * BSDF-sampled incoming radiance, fixed RR 0.7, path vertices recorded
     * and back-propagated; the cache is rebuilt after frames while the
     * frame count is below 16 (Renderer.h:720-746). */
    PGX_MODE_GUIDED_LI = 1,
    /* Extension: plain estimator whose continuation directions are drawn
     * by one-sample MIS between the BSDF and the radiance-cache QuadTree
     * guide (the design sketched in Renderer.h:398-414). */
    PGX_MODE_GUIDED_QUADTREE = 2,
    /* Extension: the same estimator with the learned guide (pgx_mlp_*): at
     * every non-specular vertex the network's vMF mixture for (position,
     * shading normal, wo) is evaluated on the tensor cores and mixed with
     * the BSDF by one-sample MIS; needs pgx_mlp_init. */
    PGX_MODE_GUIDED_MLP = 3,
    /* Extension: guiding in the BSDF's primary sample space, the design of
     * Renderer.h:398-414 (record (position, wi, Li), invert the BSDF's
     * sampling, sample the primary sample space): the radiance cache's
     * regions hold quadtrees over the primary samples that the diffuse
     * BSDFs' cosine sampler maps to the records' wi (BSDF::invert,
     * Materials.h:163-171); at a diffuse or Oren-Nayar vertex a primary
     * sample drawn from the region's quadtree (probability guide_fraction,
     * else uniform) goes through BSDF::sample, and the pdf is the quadtree
     * mixture's density at the sample times the BSDF pdf.  A render in this
     * mode with record_paths builds the cache in this form. */
    PGX_MODE_GUIDED_PSS = 4
};

typedef struct pgx_render_config {
    int32_t mode;          /* pgx_render_mode                              */
    int32_t max_depth;     /* reference: 8                                 */
    uint64_t seed;         /* PCG32 streams are hash(seed, pixel, sample)  */
    float guide_fraction;  /* probability of sampling the guide (0.5)      */
    int32_t record_paths;  /* cache training: guided Li — non-zero keeps the
                            * vertices of the last frame with SPP < 16, as the
                            * reference does; plain / QuadTree — N > 0 records
                            * the last N frames of the call with the full
                            * NEE+MIS incident radiance.  The cache is rebuilt
                            * from the records when the call ends. */
    int32_t flags;         /* PGX_RENDER_* below                            */
    int32_t guide_depth;   /* guided modes: guide the first guide_depth
                            * bounces only (0: every bounce)               */
} pgx_render_config;

/* pgx_render_config.flags */
/* Per-stage CUDA-event times and device counters of the node and triangle
 * fetches (the traversal kernels then run a counting variant). */
#define PGX_RENDER_PROFILE 1
/* Splat with the Mitchell-Netravali filter, B = C = 1/3, radius 2
 * (MitchellNetravaliFilter, Imaging.h:153-176) instead of the box filter
 * RayTracer::init installs (Renderer.h:255). */
#define PGX_RENDER_FILTER_MITCHELL 2
/* PGX_MODE_GUIDED_MLP: after every frame, the configured Adam steps of the
 * learned guide on the radiance samples that frame's paths produced
 * (pgx_mlp_configure). */
#define PGX_RENDER_TRAIN_GUIDE 4
/* Per-stage CUDA-event times only: the kernels are the ones a render without
 * flags runs. */
#define PGX_RENDER_TIMING 8

/* Statistics of the last pgx_render call.  The per-stage times are filled
 * with PGX_RENDER_PROFILE or PGX_RENDER_TIMING, the node/triangle fetch counts
 * only with PGX_RENDER_PROFILE. */
typedef struct pgx_render_stats {
    int64_t paths;
    int64_t extension_rays;
    int64_t shadow_rays;
    int64_t path_vertices;
    int64_t kernel_launches;
    int64_t extend_launches;
    int64_t extend_interior_visits; /* 64-byte node records fetched        */
    int64_t extend_tri_tests;       /* 48-byte triangles fetched           */
    int64_t shadow_interior_visits;
    int64_t shadow_tri_tests;
    double ms_total;
    double ms_extend;
    double ms_shadow;
    double ms_shade;
    int64_t guide_fallbacks;  /* learned-guide vertices guided by the QuadTree
                                 instead (pgx_mlp_set_fallback)              */
} pgx_render_stats;

/* Reference `PathVertex` (Renderer.h:42-47) without the Vec4 w lanes. */
typedef struct pgx_path_vertex {
    float position[3];
    float normal[3];
    float wi[3];
    float Li[3];
} pgx_path_vertex;

/* Point-BVH node (PointBVHNode, Renderer.h:71-81) flattened: interior
 * nodes have left/right child indices; leaves (left == -1) own
 * records [offset, offset + used). */
typedef struct pgx_cache_node {
    float bmin[3];
    float bmax[3];
    int32_t left;
    int32_t right;
    int32_t offset;
    int32_t used;
} pgx_cache_node;

typedef struct pgx_cache_stats {
    int64_t records;
    int64_t nodes;
    int64_t leaves;
    int32_t min_leaf_depth;
    int32_t max_leaf_depth;
    double mean_leaf_depth;
    double build_ms;
} pgx_cache_stats;

/* ---- context -------------------------------------------------------------- */

typedef struct pgx_ctx pgx_ctx;

/* Creates a context on CUDA device `device`. */
int pgx_create(int32_t device, pgx_ctx** out);
int pgx_destroy(pgx_ctx* ctx);
/* Message of the last failed call on ctx ("" if none).  ctx may be NULL for
 * failures of pgx_create. */
const char* pgx_last_error(const pgx_ctx* ctx);
/* Library version string. */
const char* pgx_version(void);

/* `Scene::init` (Scene.h:121-137): copies triangles, materials, textures,
 * the optional environment map (`EnvironmentMap`, Lights.h:128-228; NULL
 * gives the reference's black `BackgroundColour`) and the camera to the
 * device, builds the emitter list (Scene.h:92-100), the scene bounds
 * (SceneLoader.h:267-268) and the environment sampling tables
 * (`Distribution2D`, Sampling.h:171-189).  Does not build the BVH. */
int pgx_scene_upload(pgx_ctx* ctx, const pgx_triangle* tris, int64_t ntris,
                     const pgx_material* mats, int32_t nmats,
                     const pgx_texture* textures, int32_t ntextures,
                     const pgx_texture* envmap, const pgx_camera* camera);

/* `BVHNode::build` (Geometry.h:419-446) on the GPU: binned SAH, 16 bins per
 * axis, leaves of at most 4 triangles unless splitting costs more. */
int pgx_bvh_build(pgx_ctx* ctx);
/* Installs a BVH built elsewhere (e.g. exported from the reference) in the
 * reference layout; the traversal then visits nodes in the reference's
 * order. */
int pgx_bvh_import(pgx_ctx* ctx, const pgx_bvh_node* nodes, int64_t nnodes,
                   const int32_t* tri_index);
/* Copies the current BVH out in the reference layout.  Pass NULL buffers to
 * query the sizes. */
int pgx_bvh_export(pgx_ctx* ctx, pgx_bvh_node* nodes, int64_t* nnodes,
                   int32_t* tri_index, int64_t* ntri_index);
int pgx_bvh_get_stats(pgx_ctx* ctx, pgx_bvh_stats* out);

/* `BVHNode::traverse` (Geometry.h:448-512) for a batch of host rays. */
int pgx_trace_closest(pgx_ctx* ctx, const pgx_ray* rays, int64_t n, pgx_hit* hits);
/* `BVHNode::traverseVisible` (Geometry.h:514-567): visible[i] = 1 when no
 * triangle is hit in (1e-4, tmax). */
int pgx_trace_any(pgx_ctx* ctx, const pgx_ray* rays, int64_t n, uint8_t* visible);
/* Allocation-free variant of pgx_trace_closest.  No counterpart in the
 * reference (whose BVH queries are plain CPU calls).  It is meant for
 * callers that cannot have the library allocate device memory while they
 * run: for example an application whose device memory is handed out by its
 * own pool allocator (or by another framework that reserved the GPU's memory
 * up front), where a cudaMalloc inside the library would fail or break the
 * memory budget, or a frame loop that must not wait on the allocator.
 * The call allocates and frees nothing: rays and hits are staged in a fixed
 * device array of PGX_NOALLOC_MAX_RAYS rays that libpgx declares at file
 * scope, so the memory is reserved on every GPU that loads the library for
 * the life of the process.  Larger batches are rejected with
 * PGX_ERR_INVALID_ARG (split them).  Hits are identical to pgx_trace_closest.
 * The first call on a device looks up the array's device address (set-up);
 * make that first call before any stream capture starts.  The address is kept
 * for the life of the process and belongs to the device's primary context:
 * a process that resets the device (cudaDeviceReset) must not call this
 * entry point afterwards.  All
 * calls, from every context on a device, share the one array: calls that
 * overlap on the GPU (another thread, another context) race on it and must
 * be serialised by the caller. */
#define PGX_NOALLOC_MAX_RAYS 65536
int pgx_trace_closest_noalloc(pgx_ctx* ctx, const pgx_ray* rays, int64_t n, pgx_hit* hits);
/* Device-pointer variants on a caller stream (cudaStream_t or NULL). */
int pgx_trace_closest_device(pgx_ctx* ctx, const pgx_ray* d_rays, int64_t n,
                             pgx_hit* d_hits, void* stream);
int pgx_trace_any_device(pgx_ctx* ctx, const pgx_ray* d_rays, int64_t n,
                         uint8_t* d_visible, void* stream);
/* Node/triangle fetch counters of the last trace call (algorithmic bytes). */
int pgx_trace_counters(pgx_ctx* ctx, int64_t* nodes_visited, int64_t* tris_tested);

/* Camera rays (`Camera::generateRay`, Scene.h:253-265) for pixel sample
 * positions px, py (n of each). */
int pgx_camera_rays(pgx_ctx* ctx, const float* px, const float* py, int64_t n, pgx_ray* rays);

/* Moves the camera (RTCamera::updateCamera -> Camera::updateView,
 * SceneLoader.h:85-89, Scene.h:32-43).  The image size must stay the same;
 * the film is not cleared (call pgx_clear as the reference's viewer does). */
int pgx_set_camera(pgx_ctx* ctx, const pgx_camera* camera);

/* `RayTracer::render` (Renderer.h:648-747) called `frames` times: each frame
 * is one sample per pixel accumulated into the film. */
int pgx_render(pgx_ctx* ctx, const pgx_render_config* cfg, int32_t frames);
/* `RayTracer::clear` (Renderer.h:265-267). */
int pgx_clear(pgx_ctx* ctx);
/* `RayTracer::getSPP` (Renderer.h:749). */
int pgx_get_spp(pgx_ctx* ctx, int32_t* spp);
/* Film sums (`Film::film`, Imaging.h:186-217) to host: rgb = sum of samples
 * per pixel (divide by spp for `Film::save`), rgb2 = sum of squares (may be
 * NULL).  Both width*height*3 floats. */
int pgx_film_read(pgx_ctx* ctx, float* rgb, float* rgb2, int32_t* spp);
int pgx_render_get_stats(pgx_ctx* ctx, pgx_render_stats* out);
/* Film::tonemap for every pixel (Imaging.h:220-244): film / SPP * exposure,
 * extended Reinhard with white point lmax_white, gamma 1/2.2, clamped to
 * 8 bits.  rgb8: width*height*3 bytes (the reference's window back buffer). */
int pgx_film_tonemap(pgx_ctx* ctx, float exposure, float lmax_white, uint8_t* rgb8);

/* ---- BSDF queries -------------------------------------------------------- */

/* `BSDF::sample` (Materials.h:124) for `count` shading points with normal
 * normals[i] (shading = geometric normal, frame from Frame::fromVector) and
 * outgoing direction wo[i], driven by the reference's TestSampler
 * (Sampling.h:26-48): the first two draws are uv[2i], uv[2i+1], later draws
 * 0.5.  Writes the sampled direction, the BSDF value (may be NULL) and the
 * pdf (may be NULL).  The material must have a constant albedo. */
int pgx_bsdf_sample_batch(pgx_ctx* ctx, const pgx_material* mat, const float* normals, const float* wo,
                          const float* uv, int64_t count, float* wi, float* f, float* pdf);
/* `BSDF::invert` (Materials.h:125,163-171,287-306,673-681): the primary
 * sample (u, v) that maps to wi[i]. */
int pgx_bsdf_invert_batch(pgx_ctx* ctx, const pgx_material* mat, const float* normals, const float* wo,
                          const float* wi, int64_t count, float* uv);

/* ---- radiance cache ------------------------------------------------------ */

/* `PointBVHNode::buildPointBVHNode` (Renderer.h:189-211) over host records. */
int pgx_cache_build(pgx_ctx* ctx, const pgx_path_vertex* records, int64_t n);
/* Builds the cache from the path vertices the last guided render kept. */
int pgx_cache_build_from_render(pgx_ctx* ctx);
int pgx_cache_get_stats(pgx_ctx* ctx, pgx_cache_stats* out);
/* Copies the cache out: nodes (root first) and the records in leaf order. */
int pgx_cache_export(pgx_ctx* ctx, pgx_cache_node* nodes, int64_t* nnodes,
                     pgx_path_vertex* records, int64_t* nrecords);
/* Flux weight of each exported record, in the same order (extension; the
 * QuadTree guide's deposits): Lum(Li) |cos(normal, wi)| / pdf(wi) for the
 * records of plain, QuadTree, PSS and learned-guide renders (pdf: the density
 * wi was sampled with, so the weights estimate Li |cos| whatever sampled
 * them, Mueller et al. 2017), Lum(Li) for host records and guided-Li
 * records; non-finite or negative weights are 0.  weights == NULL: count
 * only. */
int pgx_cache_export_weights(pgx_ctx* ctx, float* weights, int64_t* nrecords);
/* k nearest cached records to each query point (extension; the reference
 * has no cache query).  idx is nq*k record indices into the exported record
 * order (-1 when fewer than k exist), d2 the squared distances, ascending,
 * ties broken by the lower index. */
int pgx_cache_knn(pgx_ctx* ctx, const float* queries, int64_t nq, int32_t k,
                  int32_t* idx, float* d2);

/* Guide queries (extension; the reference has no guiding distribution).
 * For each position, the QuadTree of its cache region (found by descending
 * the point BVH towards the position): pgx_guide_pdf gives the solid-angle
 * pdf of direction dirs[i] under the QuadTree alone (0 where the region has
 * no recorded flux); pgx_guide_sample maps two uniforms u2[2i], u2[2i+1] to a
 * QuadTree direction and its pdf (pdf 0 and direction (0,0,1) when the
 * region has no flux).  The renderer mixes this distribution with a
 * uniform share (pgx_guide_params).  positions, dirs: n*3 floats. */
int pgx_guide_pdf(pgx_ctx* ctx, const float* positions, const float* dirs, int64_t n, float* pdf);
int pgx_guide_sample(pgx_ctx* ctx, const float* positions, const float* u2, int64_t n, float* dirs, float* pdf);

/* Parameters of the QuadTree guide (extension; Mueller et al. 2017 fix rho =
 * 1 % and leave the rest to the implementation).  Defaults in brackets.
 *   region_records  regions are the point-BVH subtrees whose record count
 *                   first drops to this (256 .. 2^20) [1024]
 *   refine_fraction a quadtree cell is split while one of its children holds
 *                   more than this share of the region's flux (0, 1] [0.01]
 *   clamp_median    a record's flux (luminance of Li) is clamped at this
 *                   multiple of the region's median flux; 0: no clamp [10]
 *   uniform_share   share of the guide's samples drawn uniformly over the
 *                   sphere (or the primary-sample square) [0, 1) [0.2]
 *   compensate      MIS compensation (Karlik et al. 2019): every leaf's flux
 *                   less compensate x the region's mean flux over the leaf's
 *                   area, floored at 0, so the guide concentrates on what
 *                   the BSDF samples poorly; regions left with under 5 % of
 *                   their flux keep the plain tree; 0: off [0, 4] [0]
 *   glossy_alpha    conductor vertices whose GGX alpha is below this sample
 *                   their BSDF alone in PGX_MODE_GUIDED_QUADTREE (the tree
 *                   holds Li |cos|, not the product with a narrow lobe);
 *                   0: every non-specular surface is guided [>= 0] [0]
 * region_records, refine_fraction, clamp_median and compensate shape the next
 * cache build; uniform_share and glossy_alpha apply to every later render
 * (uniform_share also to guide queries). */
typedef struct pgx_guide_params {
    int32_t region_records;
    float refine_fraction;
    float clamp_median;
    float uniform_share;
    float compensate;
    float glossy_alpha;
} pgx_guide_params;
/* params == NULL restores the defaults; out-of-range values are rejected
 * with PGX_ERR_INVALID_ARG and change nothing. */
int pgx_guide_configure(pgx_ctx* ctx, const pgx_guide_params* params);
int pgx_guide_get_params(pgx_ctx* ctx, pgx_guide_params* out);

/* One region of the QuadTree guide: the point-BVH subtree (root node `node`)
 * whose record count first drops to pgx_guide_params.region_records (the
 * whole cache when it holds at most that many records), owning records
 * [first, first + count) of the exported record order; its quadtree starts
 * at quad node `qroot` (-1: no flux). */
typedef struct pgx_guide_region {
    int32_t first;
    int32_t count;
    int32_t node;
    int32_t qroot;
} pgx_guide_region;

/* QuadTree cell (extension; the reference's QuadTree.h:24-174 holds points,
 * not flux): the flux of its four children (index 2*y + x over the cell's
 * halves in (u, v)) and their quad node indices (-1: leaf). */
typedef struct pgx_quad_node {
    float flux[4];
    int32_t child[4];
} pgx_quad_node;

#define PGX_GUIDE_MAX_QUAD_NODES 256 /* per region */
/* Copies the guide out for inspection: nregions regions and, when qnodes is
 * not NULL, nregions * PGX_GUIDE_MAX_QUAD_NODES quad nodes (region r's block
 * starts at r * PGX_GUIDE_MAX_QUAD_NODES; child indices and qroot are
 * absolute; cells not reachable from a region's root are undefined).  Call
 * with regions == NULL to get the count.  `pss` gets 1 when the trees are
 * over the diffuse sampler's primary samples (a PGX_MODE_GUIDED_PSS cache),
 * 0 for directions. */
int pgx_guide_export(pgx_ctx* ctx, pgx_guide_region* regions, int32_t* nregions, pgx_quad_node* qnodes,
                     int32_t* pss);

/* ---- learned guide (extension; the reference has no learned component) ----
 * A 6-layer MLP (inputs: position encoded with 12 sin/cos frequencies per
 * axis after normalising to the scene bounds, shading normal, wo — 78
 * values padded to 80; 5 hidden layers of 64 with ReLU; 40 outputs) with
 * BF16 weights and activations and FP32 accumulation on the tensor cores.
 * Outputs: 8 lobe logits (softmax weights), 8 unnormalised mean directions
 * (3 each), 8 concentrations kappa = softplus(r) + 0.01; the guide is the
 * mixture of the 8 von Mises-Fisher lobes.
 *
 * Parameters (FP32 master copy, PGX_MLP_PARAMS floats) are, per layer l,
 * W_l[n][k] row-major followed by b_l[n], with (k, n) = (80, 64), (64, 64)
 * x 4, (64, 40).  Queries are 9 floats each: position, normal, wo. */
#define PGX_MLP_PARAMS 24424
#define PGX_MLP_OUTPUTS 40

/* One training sample: the direction wi continued from (position, normal,
 * wo) and its weight, e.g. Lum(incident radiance along wi) / pdf(wi). */
typedef struct pgx_radiance_sample {
    float position[3];
    float normal[3];
    float wo[3];
    float wi[3];
    float weight;
} pgx_radiance_sample;

/* Creates (or re-initialises) the network with He-uniform weights from
 * `seed`; positions are normalised to [bmin, bmax] (both NULL: the uploaded
 * scene's bounds).  Resets the optimiser. */
int pgx_mlp_init(pgx_ctx* ctx, uint64_t seed, const float* bmin, const float* bmax);
int pgx_mlp_get_params(pgx_ctx* ctx, float* params);
/* Replaces the parameters and resets the optimiser moments. */
int pgx_mlp_set_params(pgx_ctx* ctx, const float* params);
/* Raw outputs (n x 40) of n queries. */
int pgx_mlp_forward(pgx_ctx* ctx, const float* queries, int64_t n, float* raw);
/* Mixture pdf (solid angle) of dirs[i] for query i. */
int pgx_mlp_pdf(pgx_ctx* ctx, const float* queries, const float* dirs, int64_t n, float* pdf);
/* Samples the mixture with three uniforms per query (lobe, cos, azimuth);
 * dirs: n x 3, pdf: n. */
int pgx_mlp_sample(pgx_ctx* ctx, const float* queries, const float* u3, int64_t n, float* dirs, float* pdf);
/* Gradient of the loss sum_i w_i (-log q(wi_i | query_i)) / sum_i w_i with
 * respect to the parameters (PGX_MLP_PARAMS floats), without an update. */
int pgx_mlp_gradient(pgx_ctx* ctx, const pgx_radiance_sample* samples, int64_t n, float* grad, double* loss);
/* One Adam step (beta1 0.9, beta2 0.99, eps 1e-8) with learning rate lr on
 * the same loss; loss (may be NULL) gets its value before the step. */
int pgx_mlp_train_step(pgx_ctx* ctx, const pgx_radiance_sample* samples, int64_t n, float lr, double* loss);
/* Online training inside pgx_render (PGX_RENDER_TRAIN_GUIDE): after every
 * frame, `steps` Adam steps on disjoint batches of at most `batch` of that
 * frame's radiance samples, learning rate lr * decay^step (defaults 5e-3,
 * 0.998, 262144, 4).  direct = 1 trains on the full incident radiance of a
 * continuation (the default); 0 leaves out the emission reached directly
 * from the vertex, which next-event estimation also samples. */
int pgx_mlp_configure(pgx_ctx* ctx, float lr, float decay, int64_t batch, int32_t steps, int32_t direct);
/* The QuadTree guide as the learned guide's fallback.  While a radiance
 * cache with direction quadtrees exists (pgx_cache_build, or a render with
 * record_paths), the radiance samples the network is trained on (online or
 * pgx_mlp_train_step) are counted per cache region; in PGX_MODE_GUIDED_MLP a
 * vertex whose region has fewer than min_samples of them is guided by the
 * region's quadtree instead of the network (the same one-sample MIS with the
 * BSDF).  A new network, new parameters or a rebuilt cache start every
 * region at zero.  Default 256; 0 turns the fallback off. */
int pgx_mlp_set_fallback(pgx_ctx* ctx, int32_t min_samples);

/* ---- differentiable rendering (extension; the reference renders forward only) ----
 * Plain path tracing with NEE + MIS (PGX_MODE_PLAIN's estimator, box
 * filter, one thread per pixel) whose sampling decisions -- directions,
 * pdfs, MIS weights, Russian roulette and the environment's sampling
 * tables -- use the uploaded scene, while radiance is evaluated with the
 * "evaluation parameters": environment texels, a per-material albedo
 * offset (added to the sampled albedo texture; for constant albedos this is
 * the albedo itself) and per-material GGX roughness.  The estimator stays
 * unbiased for every evaluation-parameter value, and its derivative with
 * the sampling held fixed is an unbiased estimate of the image's gradient. */

/* Sets the evaluation parameters; NULL keeps the uploaded value (env W*H*3,
 * albedo_offset nmats*3 -- zero is the uploaded albedo -- roughness nmats). */
int pgx_diff_set_params(pgx_ctx* ctx, const float* env_rgb, const float* albedo_offset, const float* roughness);
/* Mean of spp samples per pixel (seeds hash(seed, pixel, sample)) in double,
 * summed in a fixed order, so two calls differ only through the samples a
 * parameter change touches.  image: W*H*3. */
int pgx_diff_render(pgx_ctx* ctx, int32_t spp, uint64_t seed, int32_t max_depth, double* image);
/* Gradient of sum_p dloss_dimage[p] . image[p] (the image of
 * pgx_diff_render with the same spp, seed and max_depth) with respect to the
 * environment texels (W*H*3), the albedo offsets (nmats*3) and the
 * roughness values (nmats), by replaying every sample from its seed (path
 * replay back-propagation; no path state is stored).  Albedo gradients are
 * computed for diffuse, Oren-Nayar, mirror and conductor materials, roughness
 * gradients for rough conductors; outputs may be NULL. */
int pgx_diff_adjoint(pgx_ctx* ctx, int32_t spp, uint64_t seed, int32_t max_depth, const float* dloss_dimage,
                     float* grad_env, float* grad_albedo, float* grad_roughness);

/* ---- batched rendering (extension) ----------------------------------------
 * Renders many independent scenes -- each uploaded into its own context on
 * the same device, with its BVH built -- as one wavefront: their traversal
 * nodes, triangles, shading data, materials, textures and area lights are
 * merged into one set of arrays at pgx_batch_create, and a render runs the
 * extend / shade / shadow pipeline over waves of (scene, pixel, sample)
 * items whose paths share the queues and every launch; each path starts
 * traversal at its scene's root and samples its scene's lights.  Paths use
 * PGX_MODE_PLAIN's estimator (NEE + MIS, box filter) and the PCG32 key
 * (seed, pixel, sample) of pgx_render, so a scene's image equals
 * pgx_render's for the same seed.  The waves of one call are captured in
 * one CUDA graph, replayed while spp, max_depth and the tuning stay the
 * same.  Environment maps are read from the scenes' own contexts. */
typedef struct pgx_batch pgx_batch;

typedef struct pgx_batch_tuning {
    int64_t wave_paths;           /* queue capacity: paths per wave            */
    int32_t trace_blocks_per_sm;  /* persistent traversal blocks per SM (1-8)  */
    int32_t shade_blocks_per_sm;  /* camera / shade / splat blocks per SM      */
    int32_t stack_shared;         /* traversal stack entries kept in shared
                                     memory (4, 8 or 16 of the 64; the rest
                                     spill to local memory)                     */
} pgx_batch_tuning;

typedef struct pgx_batch_stats {
    int64_t paths;          /* items of the last pgx_batch_render           */
    double ms;              /* its device time                              */
    int32_t graph_replayed; /* 1 when the captured graph was replayed       */
} pgx_batch_stats;

/* The contexts must outlive the batch; their films accumulate.  Geometry
 * changed after creation is not seen (the arrays are copied). */
int pgx_batch_create(pgx_ctx* const* scenes, int32_t n, pgx_batch** out);
int pgx_batch_destroy(pgx_batch* batch);
/* Adds spp samples per pixel to every scene's film. */
int pgx_batch_render(pgx_batch* batch, int32_t spp, uint64_t seed, int32_t max_depth);
/* Times candidate tunings on `spp` samples of the batch into a scratch film
 * (the scenes' films are not touched), keeps the fastest and returns it:
 * every wave capacity (1M-32M paths) x traversal and shading grid size with
 * the default stack split, then the shared-memory part of the traversal
 * stack (4, 8 or 16 of its 64 entries, the reference's depth) at the best
 * of those. */
int pgx_batch_autotune(pgx_batch* batch, int32_t spp, int32_t max_depth, pgx_batch_tuning* best);
int pgx_batch_set_tuning(pgx_batch* batch, const pgx_batch_tuning* tuning);
int pgx_batch_get_stats(pgx_batch* batch, pgx_batch_stats* stats);
const char* pgx_batch_last_error(pgx_batch* batch);

/* ---- image decoding (scene ingestion) --------------------------------------
 * Texture::load (Imaging.h:44-79) reads albedo maps with stb_image; the
 * loader decodes PNG, HDR, BMP and TGA itself and JPEG here, on the host (no
 * context or GPU needed).  Baseline, extended (8-bit) and progressive
 * Huffman-coded JPEG with 1 or 3 components: 8-bit samples, rows top-down,
 * interleaved.  With out == NULL only width, height and channels are filled.
 * Returns PGX_ERR_INVALID_ARG for malformed or unsupported data (msg, when
 * not NULL, gets a description of at most msg_size bytes). */
int pgx_image_decode_jpeg(const uint8_t* data, int64_t size, int32_t* width, int32_t* height, int32_t* channels,
                          uint8_t* out, int64_t out_size, char* msg, int32_t msg_size);

/* ---- scene files (the reference's format) ------------------------------------
 * `loadScene(dir)` (SceneLoader.h:222-269) on the host: `dir`/scene.json
 * (GEMScene::load, GEMLoader.h:853-882), the .gem meshes it names
 * (GEMModelLoader::load, GEMLoader.h:430-457) and their textures
 * (Texture::load, Imaging.h:44-79: PNG, JPEG, BMP, TGA; Radiance HDR for the
 * environment map), assembled with loadInstance's rules
 * (SceneLoader.h:104-220): one material per instance, float32 world
 * transforms, zero-area triangles dropped, distinct texture files shared.  A
 * texture that cannot be read becomes 1x1 white, as in the reference.
 * pgx_scene_read returns the upload arrays (owned by the result; release
 * with pgx_scene_data_free); on failure (missing scene.json or mesh, a
 * malformed file) it returns PGX_ERR_INVALID_ARG and a message in msg.  The
 * reference prints and continues or exits instead. */
typedef struct pgx_scene_data {
    pgx_triangle* triangles;
    int64_t ntris;
    pgx_material* materials;
    int32_t nmats;
    pgx_texture* textures; /* albedo textures, first use first */
    int32_t ntextures;
    int32_t has_env;
    pgx_texture env;       /* the environment map when has_env */
    pgx_camera camera;
    void* internal;        /* owner of the arrays */
} pgx_scene_data;
int pgx_scene_read(const char* dir, pgx_scene_data** out, char* msg, int32_t msg_size);
void pgx_scene_data_free(pgx_scene_data* data);
/* pgx_scene_read followed by pgx_scene_upload: the whole of `loadScene`
 * (without the BVH build, which is pgx_bvh_build, `Scene::build`). */
int pgx_scene_load(pgx_ctx* ctx, const char* dir);

#ifdef __cplusplus
}
#endif

#endif /* PGX_H_ */
