/*
 * rt_oracle.h -- CPU restatement of the reference's LBVH build, traversal,
 * shading rays and path tracer.  TEST INFRASTRUCTURE ONLY: the parity tests,
 * the smoke check and the CPU-baseline leg of bench.py call it as the
 * checker.  The GPU product path never links or calls it.
 *
 * Every function cites the reference file:line it restates (paths are
 * relative to the elfrank/raytracer-gpupro4 checkout).  Floating point is
 * evaluated in IEEE binary32 with the reference's operation order; the
 * library is compiled with -ffp-contract=off so no multiply-add is fused.
 * Parity of build and traversal is pinned against the reference's own
 * LBVH::Build / LBVH::IntersectP (compiled by oracle/ref/build_ref.sh) and
 * the committed golden fixtures under tests/golden/.
 */
#ifndef RT_ORACLE_H
#define RT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* LBVHNode, LBVH.h:25-28 / Structures.hlsl:18-26 (32 bytes). */
typedef struct or_node {
    float mn[3];
    float mx[3];
    int32_t prim_count; /* (count << 3) | leaf*4 | axis */
    int32_t prim_pos;
} or_node;

/* Sentinel written to heap slots no path reaches (LBVH.hlsl:151-154). */
#define OR_SENTINEL (-2147483647)

/* Pinhole camera (restates CSPrimaryRays.hlsl:36-56 with an explicit basis). */
typedef struct or_camera {
    float eye[3];
    float right[3];
    float up[3];
    float fwd[3];
    float tan_half_fovy;
    uint32_t width, height;
} or_camera;

/* Closest-hit record {id, u, v, t} (Intersection, Structures.hlsl:44-50). */
typedef struct or_hit {
    int32_t id;
    float u, v, t;
} or_hit;

/* --- build (LBVH.cpp:488-632) ------------------------------------------ */
void or_scene_bounds(const float* tris, uint32_t n, float out6[6]);
void or_morton(const float* tris, uint32_t n, const float bounds6[6], uint32_t* keys);
void or_sort_pairs(uint32_t* keys, uint32_t* ids, uint32_t n);
void or_lbvh_emit(const float* tris, const uint32_t* keys, const uint32_t* ids,
                  uint32_t n, uint32_t depth, or_node* nodes, uint8_t* reached);
/* All of the above in order; nodes has 1<<depth slots. */
void or_lbvh_build(const float* tris, uint32_t n, uint32_t depth,
                   or_node* nodes, uint32_t* ids, uint32_t* keys, uint8_t* reached);

/* --- traversal (LBVH.hlsl:363-440, Intersection.hlsl:18-78) ------------- */
/* rays: n x 8 floats {ox,oy,oz, dx,dy,dz, tmax, exclude_id}.
 * stats (nullable): 2 x uint32 per ray {box tests, triangle tests}.
 * any_hit != 0 stops at the first accepted hit (shadow rays). */
void or_trace(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
              const float* rays, uint32_t nrays, or_hit* hits, uint32_t* stats, int any_hit,
              int nthreads);

/* The same with the walk started at heap node starts[i] (NULL or values
 * <= 1: the root), the iRoot restart of LBVH_IntersectP (LBVH.hlsl:363-376);
 * leaves (nullable) receives the node whose triangles gave each closest hit
 * (1 for a miss).  A start must be a node the build reached. */
void or_trace_from(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
                   const float* rays, uint32_t nrays, const uint32_t* starts, or_hit* hits, uint32_t* leaves,
                   uint32_t* stats, int any_hit, int nthreads);

/* The reference's own walk order, LBVH_IntersectP (LBVH.hlsl:363-440): the
 * stackless trail walk started at heap node starts[i] (NULL: the root), a
 * closest-hit walk whose exact ties keep the first triangle it tests;
 * stats = {visited nodes, triangle tests} (its iVisitedNodes counter). */
void or_trace_hlsl(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
                   const float* rays, uint32_t nrays, const uint32_t* starts, or_hit* hits, uint32_t* leaves,
                   uint32_t* stats, int nthreads);

void or_shadow_mirror_hlsl(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
                           const or_camera* cam, const float light[3], const or_hit* prim, const uint32_t* prim_leaves,
                           uint8_t* vis, or_hit* mirror, uint32_t* shadow_stats, uint32_t* mirror_stats,
                           int nthreads);

/* --- ray generation and shading rays (CSPrimaryRays.hlsl, CSComputeColorRT.hlsl) */
void or_primary_rays(const or_camera* cam, float* rays /* w*h x 8 */);
/* From primary hits: shadow-ray visibility code per pixel
 *   0 primary miss, 1 light on the other side of the surface,
 *   2 occluded, 3 lit
 * and the mirror-reflection closest hit (id -2 where the primary missed). */
void or_shadow_mirror(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
                      const or_camera* cam, const float light[3], const or_hit* prim,
                      uint8_t* vis, or_hit* mirror, uint32_t* shadow_stats, uint32_t* mirror_stats,
                      int nthreads);

/* The same with each pixel's shading rays started at its primary hit's leaf
 * (prim_leaves from or_trace_from; NULL: the root); mirror_leaves
 * (nullable) receives the mirror hit's leaf.  Hits equal or_shadow_mirror's. */
void or_shadow_mirror_from(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
                           const or_camera* cam, const float light[3], const or_hit* prim,
                           const uint32_t* prim_leaves, uint8_t* vis, or_hit* mirror, uint32_t* mirror_leaves,
                           uint32_t* shadow_stats, uint32_t* mirror_stats, int nthreads);

/* --- path tracer (CSComputeColorGI.hlsl:19-238, ConstantBuffers.h:85-110) */
typedef struct or_pt_params {
    uint32_t spp;
    uint32_t bounces;   /* segments traced = bounces + 1 */
    uint64_t seed;
    float sky[3];       /* radiance added on a miss (reference: white, i.e. 1) */
    uint32_t first_sample;  /* n0: samples 0 .. n0-1 are already in image (ConstantBuffers.h:102-109) */
    /* pixel window [x0, x0 + win_w) x [y0, y0 + win_h) of the cam->width x
     * cam->height image (win_w = 0: the whole image); image / d_image hold
     * the window's pixels only, row-major */
    uint32_t x0, y0, win_w, win_h;
} or_pt_params;
void or_pathtrace(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
                  const float* albedo /* n x 3 */, const float* emission /* n x 3 */,
                  const or_camera* cam, const or_pt_params* p, float* image /* w*h x 4 */,
                  int nthreads);
/* FP64 adjoint of an L2 image loss: d_image = dL/dI (w*h x 4, float).
 * Paths are replayed with the same fp32 traversal; gradient arithmetic is
 * double.  d_albedo: n x 3, d_emission_scale: scalar multiplier of every
 * emitting triangle's radiance. */
void or_pathtrace_adjoint(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
                          const float* albedo, const float* emission, const or_camera* cam,
                          const or_pt_params* p, const float* d_image,
                          double* d_albedo, double* d_emission_scale, int nthreads);

/* --- colour stage with its bounce loop (CSComputeColorRT.hlsl:18-262,
 * RayTracerCS.cpp:284-295), no textures ------------------------------- */
typedef struct or_material {  /* Material, Structures.hlsl:69-78 */
    float ambient[4];
    float diffuse[4];
    float specular[4];
    float shininess;
    float alpha;
} or_material;
typedef struct or_shade_params {
    uint32_t bounces;        /* colour stages run = bounces + 1 */
    int32_t shadows;         /* g_bIsShadowOn */
    int32_t phong;           /* g_bIsPhongShadingOn (needs per-corner normals) */
    int32_t gloss_mapping;   /* g_bIsGlossMappingOn */
    int32_t env_mapping;     /* g_iEnvMappingFlag: -1 on, 0 off */
    float env_color[3];      /* the environment map's colour */
    uint32_t seed;           /* reflection / refraction choice */
} or_shade_params;
/* normals (nullable): n x 9 per-corner normals; mat_ids (nullable): n;
 * accum / result: w*h x 4 (g_uAccumulation, g_uResultTexture). */
void or_render_whitted(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
                       const float* normals, const int32_t* mat_ids, const or_material* mats, uint32_t nmat,
                       const or_camera* cam, const float light[3], const or_shade_params* sp, float* accum,
                       float* result, int nthreads);
/* The uniform number of the reflection / refraction choice. */
float or_whitted_rand(uint32_t seed, uint32_t pixel, uint32_t bounce);

/* --- the reference's SAH BVH (LinearBVHNode, bvh.cpp:272-293), traced as
 * BVH_IntersectP (BVH.hlsl:124-217) ----------------------------------- */
void or_bvh_trace(const or_node* nodes, uint32_t num_nodes, const uint32_t* ids, uint32_t n, const float* tris,
                  const float* rays, uint32_t nrays, or_hit* hits, uint32_t* stats, int any_hit, int nthreads);
void or_bvh_shadow_mirror(const or_node* nodes, uint32_t num_nodes, const uint32_t* ids, uint32_t n,
                          const float* tris, const or_camera* cam, const float light[3], const or_hit* prim,
                          uint8_t* vis, or_hit* mirror, uint32_t* shadow_stats, uint32_t* mirror_stats,
                          int nthreads);

/* PCG32 helpers shared with the tests (O'Neill, pcg-random.org, pcg32_srandom_r). */
uint32_t or_pcg32_first(uint64_t initstate, uint64_t initseq, uint32_t count, uint32_t* out);

#ifdef __cplusplus
}
#endif
#endif
