/*
 * rt_api.h -- C ABI of the GB300 (sm_103a) LBVH ray-tracing core.
 *
 * The entry points replace the per-frame GPU path of the reference demo
 * (elfrank/raytracer-gpupro4): the acceleration-structure interface
 * (AccelerationStructures/AccelerationStructure.h:40-67 and
 * AccelerationStructures/LBVH/LBVH.h:70-118), the GPU build stage
 * (RayTracerCS/StructureConstruction.h:67-91) and the per-frame render
 * stages (RayTracerCS/RayTracerCS.h:64-144, RayTracerCS.cpp:241-311).
 * Direct3D devices and contexts become an opaque rt_ctx bound to one CUDA
 * device and stream; every call is asynchronous on that stream unless it
 * says otherwise, returns an rt_status and never throws.
 *
 * Plain C types only: pointers marked "device" are CUDA device addresses,
 * "host" pointers are ordinary host memory (pinned memory makes the copies
 * asynchronous).  A stream is passed as void* (a cudaStream_t).
 */
#ifndef RT_API_H
#define RT_API_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RT_API_VERSION 1

/* Errors.  The reference returned void / HRESULT and called exit()
 * (Common/Scenes/Model.cpp:220-222, DeviceCore/D3DComputeShader.cpp:84-92). */
typedef enum rt_status {
    RT_OK = 0,
    RT_ERR_INVALID = 1,   /* bad argument (null pointer, n == 0, depth out of range, ...) */
    RT_ERR_CAPACITY = 2,  /* more triangles / pixels than the object was created for */
    RT_ERR_CUDA = 3,      /* a CUDA runtime call failed; see rt_last_error() */
    RT_ERR_TIMEOUT = 4,   /* a bounded device-side wait gave up (see rt_ctx_check) */
    RT_ERR_NONFINITE = 5  /* the triangle soup holds NaN or infinite coordinates */
} rt_status;

/* LBVHNode (LBVH.h:25-28) / Node (Shaders/Structures.hlsl:18-26), 32 bytes.
 * prim_count = (count << 3) | leaf * 4 | axis;  heap layout: root at 1,
 * children of i at 2i and 2i+1, slot 0 unused, 1 << depth slots. */
typedef struct rt_node {
    float min[3];
    float max[3];
    int32_t prim_count;
    int32_t prim_pos;
} rt_node;

/* Value written to prim_count and prim_pos of heap slots that no path
 * reaches when RT_BUILD_CLEAR_UNREACHED is set (LBVH.hlsl:151-154). */
#define RT_NODE_SENTINEL (-2147483647)

/* Closest hit: {iTriangleId, fU, fV, fT} of Intersection
 * (Shaders/Structures.hlsl:44-50), 16 bytes.  id = -1: no hit. */
typedef struct rt_hit {
    int32_t id;
    float u, v, t;
} rt_hit;

/* A ray for rt_trace_rays (Ray, Shaders/Structures.hlsl:28-35, without the
 * shading factor), 32 bytes.  exclude_id: triangle the ray must ignore
 * (the triangle it leaves from), -1 for none. */
typedef struct rt_ray {
    float o[3];
    int32_t exclude_id;
    float d[3];
    float tmax;
} rt_ray;

/* Pinhole camera (CSPrimaryRays.hlsl:36-56 with an explicit basis instead
 * of the inverse world matrix): pixel (i, j) looks along
 * normalize(right*x*tan + up*y*tan + fwd), x = (2i+1-W)/H, y = -(2j+1-H)/H. */
typedef struct rt_camera {
    float eye[3];
    float right[3];
    float up[3];
    float fwd[3];
    float tan_half_fovy;
    uint32_t width, height;
} rt_camera;

typedef struct rt_ctx rt_ctx;
typedef struct rt_lbvh rt_lbvh;

/* ---- context ------------------------------------------------------- */
/* Replaces the D3D device + immediate context (RayTracerCS.cpp:67-83). */
rt_status rt_ctx_create(int device, void* stream, rt_ctx** out);
rt_status rt_ctx_destroy(rt_ctx* ctx);
rt_status rt_ctx_set_stream(rt_ctx* ctx, void* stream);
/* Work budget of the camera, shading and generic ray traces: a ray that has
 * spent more than `budget` box + triangle tests in the per-lane traversal is
 * handed to a second kernel that traces it with a whole warp (same hit).
 * 0 turns the hand-over off.  rt_ctx_set_trace_budget sets every kind;
 * rt_ctx_set_trace_budget_kind one (0 primary rays, 1 shadow / mirror rays,
 * 2 rt_trace_rays).  Defaults: 384, 768, 384 (the fastest on a 2.1 M-triangle
 * frame).  Path tracing never hands over. */
rt_status rt_ctx_set_trace_budget(rt_ctx* ctx, uint32_t budget);
rt_status rt_ctx_set_trace_budget_kind(rt_ctx* ctx, uint32_t kind, uint32_t budget);
/* How the handed-over rays are traced, per trace kind in `kinds` (bit 0
 * primary rays, bit 1 shadow / mirror rays, bit 2 rt_trace_rays): a set bit
 * traces each with a whole block of 128 threads (suits a few hundred very
 * long rays), a clear bit with a warp (suits thousands).  Same hits either
 * way.  Default 2 (the shading rays a block per ray: the fastest on a
 * 2.1 M-triangle frame). */
rt_status rt_ctx_set_heavy_block(rt_ctx* ctx, uint32_t kinds);
/* Heavy-first tile order: for each trace kind in `kinds` (bit 0 primary
 * rays, bit 1 shadow / mirror rays, bit 2 rt_trace_rays) a call first
 * traces the tiles that were the most expensive in the previous call of the
 * same kind on this context, then the rest in image order.  Results do not
 * depend on the order.  Default: primary rays only (1). */
rt_status rt_ctx_set_tile_order(rt_ctx* ctx, uint32_t kinds);
rt_status rt_ctx_sync(rt_ctx* ctx);
/* Synchronises, then reports a device-side error flag raised since the
 * last check (RT_ERR_TIMEOUT, RT_ERR_NONFINITE) and clears it. */
rt_status rt_ctx_check(rt_ctx* ctx);
const char* rt_last_error(const rt_ctx* ctx);
const char* rt_status_string(rt_status s);
int rt_api_version(void);

/* ---- LBVH ---------------------------------------------------------- */
/* Creates an LBVH with room for max_tris triangles and 1 << depth heap
 * slots (LBVH(Primitive**, N, n = 1 << depth), LBVH.h:104; lbvh_depth of
 * conf.ini:61).  All device memory is allocated here; rebuilds reuse it. */
rt_status rt_lbvh_create(rt_ctx* ctx, uint32_t max_tris, uint32_t depth, rt_lbvh** out);
rt_status rt_lbvh_destroy(rt_lbvh* lbvh);

#define RT_BUILD_CLEAR_UNREACHED 1u  /* write RT_NODE_SENTINEL to unreached slots */
#define RT_BUILD_COMPACT 2u          /* also build the compact layout (rt_lbvh_compact_get) and trace it */

/* Full rebuild from a device triangle soup (n x 9 floats: A, B, C):
 * scene bounds, 30-bit Morton codes, stable LSD radix sort, node emission,
 * bottom-up refit.  Replaces LBVH::Build (LBVH.cpp:488-632) and
 * StructureConstruction::GPUBuildStructure (StructureConstruction.cpp:86-131). */
rt_status rt_lbvh_build(rt_ctx* ctx, rt_lbvh* lbvh, const float* d_tris, uint32_t n, uint32_t flags);
/* Same from a host soup; the host-to-device copy is part of the call. */
rt_status rt_lbvh_build_host(rt_ctx* ctx, rt_lbvh* lbvh, const float* h_tris, uint32_t n, uint32_t flags);
/* Uses a tree built elsewhere (e.g. the reference's CPU LBVH::Build):
 * host nodes (1 << depth), ordered ids (n) and the soup are uploaded
 * (RayTracerCS::SelectAccelerationStructure, RayTracerCS.cpp:590-624). */
rt_status rt_lbvh_import_host(rt_ctx* ctx, rt_lbvh* lbvh, const rt_node* h_nodes, const uint32_t* h_ids,
                              const float* h_tris, uint32_t n);

/* Allocation-free rebuild.  No counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc when they rebuild -- an engine whose
 * own allocator owns all device memory (a caching pool that has reserved
 * the free memory, or a budgeted heap that must account for every byte),
 * or a real-time loop that cannot absorb the implicit device-wide
 * synchronisation of cudaMalloc / cudaFree.  The caller passes the device
 * soup (n x 9 floats) and every output: d_nodes (1 << depth rt_node), d_ids
 * and d_keys (n each), d_sorted_tris (n x 12 floats, the layout of
 * rt_lbvh_view).  The results equal rt_lbvh_build's.  All scratch lives in
 * one fixed device array of 5,577,088 bytes that every GPU loading this
 * library holds until the process exits; n above RT_NOALLOC_MAX_TRIS or
 * depth above RT_NOALLOC_MAX_DEPTH returns RT_ERR_CAPACITY.  flags may hold
 * RT_BUILD_CLEAR_UNREACHED only (the compact layout needs allocated
 * buffers: RT_ERR_INVALID).  The first call on a device looks up that
 * array's device address (cudaGetSymbolAddress, once per device, with the
 * device current), so make it before any stream capture.  `stream` must
 * belong to the current device.  Every call reuses the same array and
 * clears what must start at zero; calls that overlap on the GPU race on it
 * and must be serialised by the caller.  ctx may be NULL.  If given, it
 * must be bound to the current device; it receives the error message
 * (rt_last_error) and the kernels' device-side errors (a non-finite soup,
 * a look-back wait that gave up), which rt_ctx_check reports.  With
 * ctx == NULL device-side errors are not reported.  Asynchronous on
 * `stream`; calls no allocating routine. */
#define RT_NOALLOC_MAX_TRIS 262144u
#define RT_NOALLOC_MAX_DEPTH 20u
rt_status rt_lbvh_build_noalloc(rt_ctx* ctx, void* stream, const float* d_tris, uint32_t n, uint32_t depth,
                                uint32_t flags, rt_node* d_nodes, uint32_t* d_ids, uint32_t* d_keys,
                                float* d_sorted_tris);

/* ---- sort stage ------------------------------------------------------ */
/* Stable LSD radix sort of n (key, value) pairs by the full 32-bit key, in
 * place: four 8-bit passes (one digit histogram kernel, then per pass
 * warp-ballot ranks, a bounded decoupled look-back over 4,096-key tiles
 * taken in groups of 32 tiles, as the build's sort does, and a
 * shared-memory-staged scatter).  Equal keys keep their input order.
 * Replaces the sort stage of the GPU build, BitonicSort::GPUSort
 * (RayTracerCS/BitonicSort.cpp:56-117, 45 dispatches over a fixed 512 x 512
 * array) and RadixSort::Sort (RayTracerCS/RadixSort.cpp:46-74), without
 * their fixed size.  d_scratch: device memory of at least
 * rt_radix_sort_scratch_bytes(n) bytes, 16-byte aligned (the caller owns
 * it; the call allocates nothing).  Asynchronous on the context stream;
 * a look-back wait that gives up is reported by rt_ctx_check
 * (RT_ERR_TIMEOUT). */
size_t rt_radix_sort_scratch_bytes(uint32_t n);
rt_status rt_radix_sort(rt_ctx* ctx, uint32_t* d_keys, uint32_t* d_values, uint32_t n, void* d_scratch,
                        size_t scratch_bytes);
/* Test hook of the bounded look-back wait (no counterpart in the
 * reference): runs the first radix pass of rt_radix_sort with its first
 * tile never started, so the waits of the other tiles of its group for its
 * digit counts can never complete; each gives up after spin_limit polls,
 * records RT_ERR_TIMEOUT for rt_ctx_check and goes on, and the pass returns.  Every access stays inside the buffers; d_keys
 * and d_values are left untouched (the pass writes into the scratch).
 * n must exceed 4,096 (two tiles). */
rt_status rt_radix_sort_stall_test(rt_ctx* ctx, const uint32_t* d_keys, const uint32_t* d_values, uint32_t n,
                                   void* d_scratch, size_t scratch_bytes, uint32_t spin_limit);

/* Device views (GetPtrToElements / GetOrderedElementsIds, LBVH.h:109-113). */
typedef struct rt_lbvh_view {
    const rt_node* nodes;      /* device, num_nodes entries */
    const uint32_t* ids;       /* device, n: triangle id at sorted position */
    const uint32_t* keys;      /* device, n: sorted Morton codes (valid after rt_lbvh_build) */
    const float* sorted_tris;  /* device, n x 12 floats: A.xyz,id  B.xyz,0  C.xyz,0 in sorted order */
    uint32_t n;
    uint32_t depth;
    uint32_t num_nodes;        /* 1 << depth (GetNumberOfElements) */
    uint32_t node_size;        /* 32 (GetSizeOfElement) */
} rt_lbvh_view;
rt_status rt_lbvh_view_get(const rt_lbvh* lbvh, rt_lbvh_view* out);
/* The compact node layout that rt_lbvh_build with RT_BUILD_COMPACT adds and
 * the traversal then uses (the heap above stays the reference layout): slot 1 = root, the reachable nodes in
 * sibling pairs at even slots, and in an internal node PrimPos holds the slot
 * of its children pair instead of its first primitive.  *slots = the
 * capacity of the array (2 + 2 x internal nodes are used).  RT_ERR_INVALID
 * when the last build did not make it (imported trees are traced in the heap). */
rt_status rt_lbvh_compact_get(const rt_lbvh* lbvh, const rt_node** d_nodes, uint32_t* slots);
/* WorldBound() = root box (LBVH.h:115).  Synchronous. */
rt_status rt_lbvh_world_bound(rt_ctx* ctx, const rt_lbvh* lbvh, float out_min_max[6]);
/* Synchronous copies to host; any pointer may be NULL. */
rt_status rt_lbvh_download(rt_ctx* ctx, const rt_lbvh* lbvh, rt_node* h_nodes, uint32_t* h_ids, uint32_t* h_keys);

/* ---- tracing ------------------------------------------------------- */
/* Optional per-ray statistics: 2 x uint32 {box tests, triangle tests},
 * the iVisitedNodes counter of LBVH.hlsl:389,404 split in two. */

/* Primary rays + closest hit (CSGeneratePrimaryRays + CSComputeIntersections
 * -> LBVH_IntersectP, CSPrimaryRays.hlsl:22-69, LBVH.hlsl:363-440).
 * d_hits: width*height, row-major. */
rt_status rt_trace_primary(rt_ctx* ctx, const rt_lbvh* lbvh, const rt_camera* cam, rt_hit* d_hits,
                           uint32_t* d_stats);
/* Shadow + mirror rays from primary hits (CSComputeColorRT.hlsl:57-177,
 * 203-210, flat normals).  d_vis per pixel: 0 primary miss, 1 light on the
 * far side of the surface, 2 occluded, 3 lit.  d_mirror: closest hit of the
 * mirror ray (id -2 where the primary ray missed).  Either output may be
 * NULL to skip that ray type. */
rt_status rt_trace_shadow_mirror(rt_ctx* ctx, const rt_lbvh* lbvh, const rt_camera* cam, const float light[3],
                                 const rt_hit* d_primary, uint8_t* d_vis, rt_hit* d_mirror,
                                 uint32_t* d_shadow_stats, uint32_t* d_mirror_stats);
/* Arbitrary rays, closest hit (any_hit = 0) or first hit (any_hit = 1). */
rt_status rt_trace_rays(rt_ctx* ctx, const rt_lbvh* lbvh, const rt_ray* d_rays, uint32_t n, int any_hit,
                        rt_hit* d_hits, uint32_t* d_stats);

/* Traversal restart: the iRoot of LBVH_IntersectP(ray, nodeNum)
 * (LBVH.hlsl:363-376), which the reference feeds with the leaf where the
 * previous intersection was found (CSIntersections.hlsl:32,
 * CSComputeColorRT.hlsl:160).  A walk started at heap node k visits k's
 * subtree and the siblings of k's ancestors, which together hold every
 * triangle, so the hits equal a walk from the root (up to the order
 * dependence every walk has between two triangles hit within an ulp of each
 * other); a ray leaving a surface near its last hit reaches fewer boxes.  A start of 0 or 1 is the root; any
 * other start must be a node the current build reached, such as a leaf one
 * of these calls reported (1 is reported for a miss, for a ray handed to the
 * warp-per-ray pass, and for every ray when the compact layout is built).
 * d_leaves / d_mirror_leaves (nullable): the heap node whose triangles gave
 * each closest hit. */
rt_status rt_trace_primary_leaves(rt_ctx* ctx, const rt_lbvh* lbvh, const rt_camera* cam, rt_hit* d_hits,
                                  uint32_t* d_leaves, uint32_t* d_stats);
rt_status rt_trace_shadow_mirror_from(rt_ctx* ctx, const rt_lbvh* lbvh, const rt_camera* cam,
                                      const float light[3], const rt_hit* d_primary,
                                      const uint32_t* d_primary_leaves, uint8_t* d_vis, rt_hit* d_mirror,
                                      uint32_t* d_mirror_leaves, uint32_t* d_shadow_stats, uint32_t* d_mirror_stats);
rt_status rt_trace_rays_from(rt_ctx* ctx, const rt_lbvh* lbvh, const rt_ray* d_rays, uint32_t n, int any_hit,
                             const uint32_t* d_starts, rt_hit* d_hits, uint32_t* d_leaves, uint32_t* d_stats);

/* ---- the reference's SAH BVH: a second structure ---------------------- */
/* BVH (AccelerationStructures/BVH/bvh.h, PBRT's SAH build) keeps its tree as
 * a depth-first LinearBVHNode array (FlattenBVHTree, bvh.cpp:272-293), the
 * same 32-byte record as rt_node: prim_count = nPrimitives (> 0: a leaf of
 * that many entries of the ordered primitive ids from prim_pos; <= 0: an
 * interior node split on axis -prim_count whose first child is the next
 * record and whose second child is at prim_pos).  An rt_bvh holds such a
 * tree on the device, and BVH_IntersectP (BVH.hlsl:124-217) traces it:
 * visited node boxes tested with IntersectBox, the child on the ray's
 * negative side of the split axis first.  All leaf triangles are tested
 * (the shader tests a leaf's first one only, which is the same for the
 * one-primitive leaves it supports); ties at equal t keep the smaller id. */
typedef struct rt_bvh rt_bvh;
rt_status rt_bvh_create(rt_ctx* ctx, uint32_t max_nodes, uint32_t max_tris, rt_bvh** out);
rt_status rt_bvh_destroy(rt_bvh* bvh);
/* Uploads a tree the reference built (BVH::GetPtrToElements,
 * GetOrderedElementsIds) and the soup it was built over (host pointers,
 * n x 9 floats).  The tree is checked first: every child inside the array
 * and after its parent, every leaf range inside the ids, every id below n,
 * split axes 0..2 (RT_ERR_INVALID otherwise). */
rt_status rt_bvh_import_host(rt_ctx* ctx, rt_bvh* bvh, const rt_node* h_nodes, uint32_t num_nodes,
                             const uint32_t* h_ids, const float* h_tris, uint32_t n);
/* The tracing calls of the LBVH, over the BVH. */
rt_status rt_bvh_trace_primary(rt_ctx* ctx, const rt_bvh* bvh, const rt_camera* cam, rt_hit* d_hits,
                               uint32_t* d_stats);
rt_status rt_bvh_trace_shadow_mirror(rt_ctx* ctx, const rt_bvh* bvh, const rt_camera* cam, const float light[3],
                                     const rt_hit* d_primary, uint8_t* d_vis, rt_hit* d_mirror,
                                     uint32_t* d_shadow_stats, uint32_t* d_mirror_stats);
rt_status rt_bvh_trace_rays(rt_ctx* ctx, const rt_bvh* bvh, const rt_ray* d_rays, uint32_t n, int any_hit,
                            rt_hit* d_hits, uint32_t* d_stats);

/* ---- colour stage ---------------------------------------------------- */
/* Material (Structures.hlsl:69-78; the MTL colours of Model::LoadFile):
 * shininess = Ns / 1000, alpha = d or 1 - Tr (the probability of the mirror
 * bounce), ambient[3] = the refraction index of the refracted bounce. */
typedef struct rt_material {
    float ambient[4];
    float diffuse[4];
    float specular[4];
    float shininess;
    float alpha;
} rt_material;

/* Switches of the colour stage (cbInputOutput, ConstantBuffers.h:35-70). */
typedef struct rt_shade_params {
    uint32_t bounces;       /* num_reflex: colour stages run = bounces + 1 */
    int32_t shadows;        /* bIsShadowOn */
    int32_t phong;          /* bIsPhongShadingOn: interpolate d_normals (flat when NULL) */
    int32_t gloss_mapping;  /* bIsGlossMappingOn: keep specular.w */
    int32_t env_mapping;    /* iEnvMapping: -1 a miss takes env_color and ends the ray; 0 it shows 1 */
    float env_color[3];     /* stands in for the environment cube map */
    uint32_t seed;          /* the mirror / refraction choice (stands in for the random texture) */
} rt_shade_params;

/* RayTracerCS::Render without global illumination (RayTracerCS.cpp:284-295):
 * primary rays, then bounces + 1 times the intersection stage
 * (CSIntersections.hlsl:18-39, each walk restarted at the pixel's previous
 * leaf) and the colour stage (CSComputeColorRT.hlsl:18-262 without textures
 * or normal maps: flat or Phong normal, shadow ray, specular^49 and diffuse
 * terms, mirror or refracted next ray, environment colour on a miss).
 * d_material_ids (nullable: all 0): n; d_materials: num_materials (>= 1);
 * d_normals (nullable): n x 9 per-corner normals.  d_accum / d_result
 * (w*h x 4 floats, row-major; d_result nullable): g_uAccumulation and
 * g_uResultTexture after the last bounce.  The triangles are the soup of
 * the last build (indexed by triangle id); the walks use the heap layout. */
rt_status rt_render_whitted(rt_ctx* ctx, const rt_lbvh* lbvh, const rt_camera* cam, const float light[3],
                            const rt_shade_params* params, const int32_t* d_material_ids,
                            const rt_material* d_materials, uint32_t num_materials, const float* d_normals,
                            float* d_accum, float* d_result);

/* A frame (primary, shadow, mirror rays) traced in the reference's own walk
 * order: LBVH_IntersectP (LBVH.hlsl:363-440) as the shader runs it, a
 * stackless trail walk with one box test per visited node, the child picked
 * by the stored axis field first, closest hit for every ray (the shadow ray
 * too, as CSComputeColorRT.hlsl:160 issues it) and exact ties resolved as
 * the shader resolves them (the first triangle tested stays); the shading
 * rays restart at the primary hit's leaf.  One lane per ray: slower than
 * rt_trace_primary + rt_trace_shadow_mirror, which keep the smaller id on
 * an exact tie.  The optional stats are the shader's iVisitedNodes per ray
 * {visited nodes, triangle tests}; the trace's algorithmic bytes are
 * defined on them.  vis / mirror may be NULL. */
rt_status rt_trace_frame_shader_order(rt_ctx* ctx, const rt_lbvh* lbvh, const rt_camera* cam, const float light[3],
                                      rt_hit* d_primary, uint8_t* d_vis, rt_hit* d_mirror, uint32_t* d_primary_stats,
                                      uint32_t* d_shadow_stats, uint32_t* d_mirror_stats);

/* One frame of the dynamic path (RayTracerCS::Render with dynamic=1,
 * RayTracerCS.cpp:258-295): rebuild from a host soup, primary, shadow and
 * mirror rays (started at the primary hits' leaves), results copied back to
 * host buffers (any may be NULL). */
rt_status rt_render_frame_host(rt_ctx* ctx, rt_lbvh* lbvh, const float* h_tris, uint32_t n,
                               const rt_camera* cam, const float light[3], rt_hit* h_primary,
                               uint8_t* h_vis, rt_hit* h_mirror);
/* The same frame, queued on the context stream without waiting: the host
 * buffers must stay untouched until rt_ctx_sync (pinned memory makes the
 * copies asynchronous).  Two contexts on two streams, used for alternate
 * frames, overlap one frame's copies with the other frame's kernels. */
rt_status rt_render_frame_host_async(rt_ctx* ctx, rt_lbvh* lbvh, const float* h_tris, uint32_t n,
                                     const rt_camera* cam, const float light[3], rt_hit* h_primary,
                                     uint8_t* h_vis, rt_hit* h_mirror);

/* ---- one frame as a CUDA graph ------------------------------------- */
/* The dynamic per-frame path (RayTracerCS::Render with dynamic=1,
 * RayTracerCS.cpp:258-295: rebuild, primary rays, shadow + mirror rays)
 * captured once and replayed with one launch.  All pointers, the camera and
 * the light are fixed at capture; write new vertex data into d_tris (or
 * capture one rt_frame per soup buffer).  d_vis / d_mirror may be NULL.
 * Capturing synchronises the context stream; rt_frame_launch is
 * asynchronous on it.  rt_frame_node_count: nodes in the captured graph. */
typedef struct rt_frame rt_frame;
rt_status rt_frame_capture(rt_ctx* ctx, rt_lbvh* lbvh, const float* d_tris, uint32_t n, uint32_t flags,
                           const rt_camera* cam, const float light[3], rt_hit* d_primary, uint8_t* d_vis,
                           rt_hit* d_mirror, rt_frame** out);
rt_status rt_frame_launch(rt_ctx* ctx, rt_frame* frame);
uint32_t rt_frame_node_count(const rt_frame* frame);
/* A captured frame holds a reference on its rt_lbvh (rt_batch): while it
 * exists the structure's grow-on-demand buffers keep their size (a call that
 * would grow them fails with RT_ERR_CAPACITY), and rt_lbvh_destroy /
 * rt_batch_destroy only marks the structure; the last rt_frame_destroy frees
 * it. */
rt_status rt_frame_destroy(rt_frame* frame);
/* rt_frame_capture with host buffers: the upload of the pinned host soup,
 * the rebuild, the trace and the read-back of the results into pinned host
 * buffers (any output may be NULL), captured as one graph; every launch of
 * it is one frame of rt_render_frame_host.  All host buffers must be
 * page-locked (RT_ERR_INVALID otherwise); the caller writes the next frame's
 * vertices into h_tris between launches. */
rt_status rt_frame_capture_host(rt_ctx* ctx, rt_lbvh* lbvh, const float* h_tris, uint32_t n, uint32_t flags,
                                const rt_camera* cam, const float light[3], rt_hit* h_primary, uint8_t* h_vis,
                                rt_hit* h_mirror, rt_frame** out);

/* ---- double-buffered host frames ------------------------------------- */
/* The dynamic per-frame path with host buffers, pipelined (replaces the
 * vertex-buffer update + RayTracerCS::Render loop of a dynamic model,
 * RayTracerCS.cpp:241-311, which the D3D immediate context serialises).
 * rt_pipe_create captures two frames (rt_frame_capture) over two device soup
 * slots and two sets of device result buffers.  rt_pipe_submit queues frame
 * k in slot k mod 2: the upload of the pinned host soup on a private copy
 * stream, the captured rebuild + trace on the context stream (frames run
 * their kernels one after another), the read-back into the pinned host
 * buffers on a second private copy stream.  So frame k's upload and frame
 * k-1's read-back run while frame k-1's or k's kernels do, and no two
 * frames' kernels share the GPU.  The host soup of frame k may be rewritten
 * once rt_pipe_wait(k) has returned; its host results are complete then.
 * Waiting on a ticket whose slot a later frame has reused waits for that
 * later frame.  want_vis / want_mirror select the shading outputs (0: the
 * frame traces primary rays only and h_vis / h_mirror must be NULL).  Host
 * buffers must be page-locked (RT_ERR_INVALID otherwise).  Device-side
 * errors are reported by rt_ctx_check (it waits for the context stream).
 * The pipe holds a reference on lbvh, as a captured frame does. */
typedef struct rt_pipe rt_pipe;
rt_status rt_pipe_create(rt_ctx* ctx, rt_lbvh* lbvh, uint32_t n, uint32_t flags, const rt_camera* cam,
                         const float light[3], int want_vis, int want_mirror, rt_pipe** out);
rt_status rt_pipe_submit(rt_pipe* pipe, const float* h_tris, rt_hit* h_primary, uint8_t* h_vis, rt_hit* h_mirror,
                         uint64_t* ticket);
rt_status rt_pipe_wait(rt_pipe* pipe, uint64_t ticket);
rt_status rt_pipe_destroy(rt_pipe* pipe);

/* ---- batched scenes ------------------------------------------------- */
/* Up to 256 independent scenes rebuilt and traced together: one pass of the
 * build kernels over the concatenated soups and one persistent trace kernel
 * over (scene, 8x4 pixel tile) work items, in place of n_scenes rounds of
 * Model::RebuildStructure (Model.cpp:163-205) + RayTracerCS::Render
 * (RayTracerCS.cpp:241-311).  Scene s is triangles [off_s, off_s + count_s)
 * of the soup passed to rt_batch_build, off_s = count_0 + ... + count_{s-1};
 * its tree equals rt_lbvh_build of those triangles alone (same nodes,
 * scene-local PrimPos and ids), stored in its own 1 << depth heap.
 * rt_batch_create allocates everything once for the given scene sizes
 * (every scene non-empty, depth <= RT_BATCH_MAX_DEPTH); rt_batch_build and
 * rt_batch_trace allocate nothing, so both can be captured in a graph
 * (rt_batch_frame_capture). */
#define RT_BATCH_MAX_SCENES 256u
#define RT_BATCH_MAX_DEPTH 23u
typedef struct rt_batch rt_batch;
rt_status rt_batch_create(rt_ctx* ctx, uint32_t n_scenes, const uint32_t* h_tri_counts, uint32_t depth,
                          rt_batch** out);
rt_status rt_batch_destroy(rt_batch* batch);
uint32_t rt_batch_scene_count(const rt_batch* batch);
/* d_tris: device, (sum of counts) x 9 floats.  The soup stays borrowed
 * until the next build (the shadow rays read it). */
rt_status rt_batch_build(rt_ctx* ctx, rt_batch* batch, const float* d_tris, uint32_t flags);
/* Scene `scene`'s tree, in the layout of a single-scene view (device
 * pointers into the batch's arrays). */
rt_status rt_batch_view_get(const rt_batch* batch, uint32_t scene, rt_lbvh_view* out);
/* Synchronous copies of scene `scene`'s nodes (1 << depth), scene-local
 * ids and sorted codes (its triangle count each); any pointer may be NULL. */
rt_status rt_batch_download(rt_ctx* ctx, const rt_batch* batch, uint32_t scene, rt_node* h_nodes, uint32_t* h_ids,
                            uint32_t* h_keys);
/* Per-scene cameras (host, n_scenes, one common width x height) and point
 * lights (host, n_scenes x 3 floats), copied to the device on the context
 * stream; the host arrays may be reused when the call returns. */
rt_status rt_batch_set_views(rt_ctx* ctx, rt_batch* batch, const rt_camera* h_cams, const float* h_lights);
/* Primary rays (rt_trace_primary) and, when d_vis is not NULL, shadow rays
 * (rt_trace_shadow_mirror's vis codes) of every pixel of every scene.
 * d_hits: device, n_scenes x width x height rt_hit (scene-major, each
 * scene row-major, hit ids scene-local); d_vis: the same shape in bytes. */
rt_status rt_batch_trace(rt_ctx* ctx, const rt_batch* batch, rt_hit* d_hits, uint8_t* d_vis);
/* Launch shape of rt_batch_trace.  threads: 64, 128 or 256 per block;
 * blocks_per_sm: 0 = as many as fit; grab: tiles a warp takes per
 * work-counter increment (1 to 16); order: 0 = scene-major work items
 * (the tiles of one scene are consecutive), 1 = interleaved (tile-major). */
typedef struct rt_batch_tuning {
    uint32_t threads;
    uint32_t blocks_per_sm;
    uint32_t grab;
    uint32_t order;
} rt_batch_tuning;
rt_status rt_batch_set_tuning(rt_ctx* ctx, rt_batch* batch, const rt_batch_tuning* t);
rt_status rt_batch_get_tuning(const rt_batch* batch, rt_batch_tuning* t);
/* One batched frame (rt_batch_build + rt_batch_trace with the current
 * views and tuning) captured as a CUDA graph; launch / destroy it with
 * rt_frame_launch / rt_frame_destroy. */
rt_status rt_batch_frame_capture(rt_ctx* ctx, rt_batch* batch, const float* d_tris, uint32_t flags, rt_hit* d_hits,
                                 uint8_t* d_vis, rt_frame** out);

/* ---- path tracing (CSComputeColorGI.hlsl, ConstantBuffers.h:85-110) --- */
typedef struct rt_pt_params {
    uint32_t spp;
    uint32_t bounces;   /* segments traced per path = bounces + 1 (RayTracerCS.cpp:289) */
    uint64_t seed;
    float sky[3];       /* radiance of a miss; the reference adds white (1,1,1) */
    uint32_t first_sample;  /* n0: samples already averaged into d_image (0 = start afresh) */
} rt_pt_params;
/* Every bounce's walk starts at the leaf that held the previous hit (the
 * iRoot of CSIntersections.hlsl:32); the camera segment at the root.
 * d_albedo, d_emission: n x 3 floats indexed by triangle id.
 * d_image: width*height float4 (rgb, 1), the progressive mean over samples
 * n0 .. n0 + spp - 1 blended into the mean of samples 0 .. n0 - 1 that
 * d_image holds on entry: per sample n the image is scaled by n / (n + 1)
 * and the sample added with weight 1 / (n + 1), the factors of
 * cbGlobalIllumination::Update (ConstantBuffers.h:102-109) applied in
 * CSPrimaryRays.hlsl:62-63.  n0 plays the reference's frame counter
 * (RayTracerCS.cpp:306), and n0 = 0 its reset on camera motion
 * (RayTracerCS.cpp:246-250); d_image is not read when n0 = 0.  Sample n of
 * a pixel has its own PCG32 stream, so two calls of k samples with n0 = 0
 * and n0 = k give the image of one call of 2k samples, bit for bit. */
rt_status rt_pathtrace(rt_ctx* ctx, const rt_lbvh* lbvh, const float* d_albedo, const float* d_emission,
                       const rt_camera* cam, const rt_pt_params* p, float* d_image);
/* rt_pathtrace that also adds its walk counts to d_counts (device, 4 x
 * uint64, not cleared by the call): segments traced, box tests, triangle
 * tests, segments that hit a triangle.  Same image; the counting makes it
 * slower, so it serves measurement (the path tracer's algorithmic bytes are
 * defined on these counts), not rendering. */
rt_status rt_pathtrace_counted(rt_ctx* ctx, const rt_lbvh* lbvh, const float* d_albedo, const float* d_emission,
                               const rt_camera* cam, const rt_pt_params* p, float* d_image,
                               unsigned long long* d_counts);
/* Adjoint of rt_pathtrace by path replay: given dL/dImage (width*height
 * float4), accumulates dL/dalbedo (n x 3) and dL/dLe (3 floats: the shared
 * radiance of every emitting triangle) into the output buffers (not
 * cleared by the call).  With n0 = first_sample > 0 it differentiates the
 * samples n0 .. n0 + spp - 1 of that call (each with its weight in the
 * final mean); the n0 samples already in the image are constants. */
rt_status rt_pathtrace_adjoint(rt_ctx* ctx, const rt_lbvh* lbvh, const float* d_albedo, const float* d_emission,
                               const rt_camera* cam, const rt_pt_params* p, const float* d_dimage,
                               float* d_dalbedo, float* d_demission);

#ifdef __cplusplus
}
#endif
#endif /* RT_API_H */
