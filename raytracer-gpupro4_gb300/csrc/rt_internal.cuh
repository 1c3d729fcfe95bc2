// rt_internal.cuh -- shared definitions of the sm_103a LBVH core.
//
// Arithmetic on the parity-critical paths (Morton quantisation, ray
// generation, ray/box and ray/triangle tests, shading rays) goes through
// the __f*_rn intrinsics below: IEEE binary32, round to nearest, never
// contracted into a fused multiply-add, so each result equals the
// reference's CPU evaluation (LBVH.cpp, AccelerationStructure.h:70-97,
// Geometry.h Cross/Dot) bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/rt_api.h"

// ---------------------------------------------------------------------------
// exact fp32 helpers
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return mk3(fsub(a.x, b.x), fsub(a.y, b.y), fsub(a.z, b.z)); }
// Dot (Geometry.h): (x*x' + y*y') + z*z'
__device__ __forceinline__ float dot3(f3 a, f3 b) {
    return fadd(fadd(fmul(a.x, b.x), fmul(a.y, b.y)), fmul(a.z, b.z));
}
// Cross (Geometry.h)
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
    return mk3(fsub(fmul(a.y, b.z), fmul(a.z, b.y)), fsub(fmul(a.z, b.x), fmul(a.x, b.z)),
               fsub(fmul(a.x, b.y), fmul(a.y, b.x)));
}
// Normalize (Geometry.h): divide each component by the length
__device__ __forceinline__ f3 normalize3(f3 v) {
    float l = fsqrt(dot3(v, v));
    return mk3(fdiv(v.x, l), fdiv(v.y, l), fdiv(v.z, l));
}

// std::min / std::max as the reference's CPU code evaluates them:
// min(a,b) = (b < a) ? b : a, max(a,b) = (a < b) ? b : a (NaN-sensitive).
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }

// ---------------------------------------------------------------------------
// Device error word (bit set by kernels, read by rt_ctx_check).
enum : uint32_t {
    RT_DEVERR_TIMEOUT = 1u,
    RT_DEVERR_NONFINITE = 2u,
    RT_DEVERR_BOUNDS = 4u,  // a bounds guard rejected an index (corrupt tree or scratch)
};

// Scene bounds and Morton parameters produced on the device by the bounds
// kernel (cbScene of ConstantBuffers.h:112-142 computed instead of uploaded).
struct SceneInfo {
    float bmin[3], bmax[3];  // VertMin / VertMax (LBVH.cpp:513-514)
    float lo3[3];            // 3 * VertMin (LBVH.cpp:522)
    float f[3];              // 1024 / (3*VertMax - 3*VertMin) (LBVH.cpp:523-526)
    uint32_t nonfinite;
    uint32_t pad[3];
};

// Tiling constants
constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096 keys per onesweep tile
constexpr int kSortPasses = 4;                        // 8-bit digits over 30-bit codes
constexpr int kEmitThreads = 256;
constexpr int kEmitItems = 8;
constexpr int kEmitTile = kEmitThreads * kEmitItems;  // 2048 elements per emission tile
constexpr int kMaxDepth = 26;
constexpr uint32_t kMaxTris = (1u << 29);

// ---------------------------------------------------------------------------
// Heavy-ray hand-over (see Spill in rt_traverse.cuh): list capacity and the
// default budget of box + triangle tests a lane spends on one ray before it
// hands the ray to the warp-per-ray kernel.
constexpr uint32_t kSpillCap = 1u << 20;
constexpr uint32_t kDefaultHeavyTeam = 2u;
constexpr uint32_t kDefaultTraceBudget = 384;
constexpr uint32_t kDefaultShadeBudget = 768;
// Heavy-first tile order (TileOrder in rt_traverse.cuh): per trace kind two
// lists of kOrderCap tiles and two bitmaps, in one allocation.
constexpr uint32_t kOrderCap = 1u << 20;
constexpr size_t kOrderWords = 2 * (size_t)kOrderCap + 2 * (size_t)(kOrderCap / 32);
constexpr int kOrderKinds = 3;

struct rt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    uint32_t* d_err = nullptr;   // device error word (d_words[0])
    uint32_t* d_work = nullptr;  // work counters of the persistent kernels (d_words[16..])
    uint32_t* d_spill_count = nullptr;  // heavy-ray list length (d_words[32]; shading rays: [33], claims [34])
    uint32_t* d_words = nullptr; // 64 device words
    uint32_t* d_spill = nullptr; // heavy-ray list, kSpillCap entries
    uint32_t* d_order = nullptr; // heavy-first tile order, kOrderKinds x kOrderWords (parity / counts: d_words[40..])
    // hand-over budget per trace kind (0 primary, 1 shading, 2 generic rays); 0: no hand-over
    uint32_t trace_budget[3] = {kDefaultTraceBudget, kDefaultShadeBudget, kDefaultTraceBudget};
    // per trace kind (bit 0 primary, 1 shading, 2 generic rays): the handed-over
    // rays are traced a block per ray (k_trace_heavy_team) instead of a warp
    uint32_t heavy_team = kDefaultHeavyTeam;
    uint32_t tile_order = 1u;  // heavy-first tile order per kind: bit 0 primary, 1 shading, 2 generic rays
    int num_sms = 0;
};

struct rt_lbvh {
    uint32_t cap = 0, depth = 0, num_nodes = 0, n = 0;
    bool built_keys = false;
    rt_node* nodes = nullptr;
    uint32_t* keys = nullptr;
    uint32_t* ids = nullptr;
    uint32_t* keys_alt = nullptr;
    uint32_t* ids_alt = nullptr;
    float4* sorted_tris = nullptr;  // 3 x float4 per triangle
    // compact layout used by the traversal: slot 1 = root, the children of
    // internal node x at slots 2 r + 2, 2 r + 3 with r = the rank of x among
    // the reachable internal nodes in heap order (its PrimPos holds 2 r + 2)
    rt_node* cnodes = nullptr;
    uint32_t ccap = 0;              // slots of cnodes
    uint32_t* inner = nullptr;      // bitmap of reachable internal heap slots (num_nodes / 32 words, >= 1)
    uint32_t* inner_rank = nullptr; // exclusive popcount prefix of inner
    bool compact_valid = false;     // cnodes describe the current tree
    float* tris = nullptr;          // device copy of the soup (host builds / imports)
    const float* src_tris = nullptr; // soup of the last build / import, indexed by triangle id (borrowed)
    // build scratch
    SceneInfo* scene = nullptr;
    float* partials = nullptr;       // bounds partial reductions, 8 floats per block
    uint32_t* counters = nullptr;    // [0] bounds ticket, [1..4] sort tile tickets, [5] leaf count, [6] refit epoch
    uint32_t* hist = nullptr;        // 4 x 256 digit histograms
    uint32_t* lookback = nullptr;    // 4 passes x sort tiles x 256 status words
    uint32_t* scan = nullptr;        // emission tiles x 4 (fwd agg, bwd agg, fwd prefix, bwd suffix)
    uint32_t* leaf_list = nullptr;   // cap
    uint32_t* arrive = nullptr;      // 1 << (depth-1) refit arrival words (epoch-tagged)
    uint2* items = nullptr;          // emission items (heap index, mask) of every merge level: 6 x emit tiles x 64
    uint32_t* item_counts = nullptr; // 8 x emit tiles: item counts of every level (6x), tile unit counts, merge tickets
    uint32_t sort_tiles_cap = 0, emit_tiles_cap = 0, bounds_blocks = 0;
    // frame buffers for rt_render_frame_host (grown on demand)
    rt_hit* f_primary = nullptr;
    rt_hit* f_mirror = nullptr;
    uint8_t* f_vis = nullptr;
    size_t f_pixels = 0;
    // compacted shading-ray lists (shadow pixels, mirror pixels, primary leaves, then the start
    // nodes of the listed rays, 2 x), 5 x s_pixels
    uint32_t* s_lists = nullptr;
    float4* s_rays = nullptr;  // the listed rays, 2 x 2 x s_pixels float4 (ensure_shade_lists)
    size_t s_pixels = 0;
    // per-pixel state of the colour stage's bounce loop (rt_render_whitted)
    void* w_buf = nullptr;
    size_t w_pixels = 0;
    // captured frames that point into this structure's buffers: while any
    // exists the grow-on-demand buffers keep their size, and a destroy
    // waits for the last one
    uint32_t graph_refs = 0;
    bool destroy_pending = false;
};

// Frees an rt_lbvh / rt_batch and its device buffers.
void free_lbvh(rt_lbvh* l);
void free_batch(rt_batch* b);

// Many independent scenes built in one pass of the build kernels and traced
// by one persistent kernel.  Scene s owns triangles [tri_off[s], tri_off[s+1])
// of the concatenated soup and heap slots [node_off[s], node_off[s+1]).
struct rt_batch {
    uint32_t S = 0, depth = 0, total = 0;
    uint32_t graph_refs = 0;       // captured frames pointing into the batch (see rt_lbvh)
    bool destroy_pending = false;
    std::vector<uint32_t> h_tri_off;
    uint32_t* tri_off = nullptr;   // S + 1
    uint32_t* node_off = nullptr;  // S + 1
    uint32_t* chunks = nullptr;    // (scene, begin, end) triples, one scene each
    uint32_t nchunks = 0;
    rt_node* nodes = nullptr;      // S << depth
    uint32_t *keys = nullptr, *ids = nullptr, *keys_alt = nullptr, *ids_alt = nullptr;
    uint32_t *res_keys = nullptr, *res_ids = nullptr;  // buffers holding the sorted pairs
    uint32_t* ids_local = nullptr;  // scene-local triangle id at each sorted position
    float4* sorted_tris = nullptr;  // 3 x float4 per triangle, w of the first = scene-local id
    float* sbounds = nullptr;       // 8 floats per scene (min xyz, max xyz)
    uint32_t* counters = nullptr;   // [0..4] sort tickets, [5] leaf count, [6] refit epoch
    uint32_t* hist = nullptr;       // 5 x 256
    uint32_t* lookback = nullptr;   // 5 x 256 x sort tiles
    uint32_t* scan = nullptr;       // 4 per emission tile
    uint32_t* leaf_list = nullptr;  // total
    uint32_t* arrive = nullptr;     // S << (depth - 1)
    const float* src_tris = nullptr;
    bool built = false;
    // views of the batched trace (rt_batch_set_views)
    rt_camera* cams = nullptr;      // S, device
    float* lights = nullptr;        // 3 S, device
    uint32_t width = 0, height = 0;
    // the shadow rays of a batched trace, listed by the primary pass (batch
    // pixel s * width * height + p, ray, start node) for the lane-refill
    // pass; s_cap = 0: no list (the primary pass traces them itself)
    uint32_t* s_lists = nullptr;    // s_cap pixels, then s_cap start nodes
    float4* s_rays = nullptr;       // 2 s_cap
    uint32_t s_cap = 0;
    rt_batch_tuning tuning = {128u, 0u, 1u, 0u};
};

// ---------------------------------------------------------------------------
// error plumbing (host)
rt_status rt_fail(rt_ctx* ctx, rt_status s, const char* fmt, ...);

// Programmatic dependent launch.  A kernel launched with launch_pdl may be
// scheduled while the kernel before it on the stream drains (in a captured
// graph the edge between the two becomes a programmatic one), which hides
// the launch and block-scheduling gap between dependent kernels.  Every
// kernel launched this way begins with grid_dep_wait(): it returns once the
// previous kernel has completed and its writes are visible (at once for an
// ordinary launch), so the stream order of memory effects is unchanged.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... P, typename... A>
inline void launch_pdl(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, A... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, args...);  // an error is left for RT_CHECK_LAUNCH
}

#define RT_CHECK_CUDA(ctx, call)                                                               \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return rt_fail((ctx), RT_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

#define RT_CHECK_LAUNCH(ctx, what)                                                              \
    do {                                                                                        \
        cudaError_t e_ = cudaGetLastError();                                                    \
        if (e_ != cudaSuccess)                                                                  \
            return rt_fail((ctx), RT_ERR_CUDA, "launch of %s failed: %s", what, cudaGetErrorString(e_)); \
    } while (0)

// Bounded spin used by every device-side wait (look-back): after this many
// polls the waiter records RT_DEVERR_TIMEOUT and stops waiting.  A poll that
// finds nothing new sleeps ~100 ns first, so a wait gives up within about a
// second (2^20 polls x (sleep + an L2 round trip)).
constexpr uint32_t kSpinLimit = 1u << 20;

// Grid of a persistent kernel: as many blocks as fit on every SM at once,
// capped by the number of 32-item tiles.
template <typename K>
inline uint32_t persistent_blocks(const rt_ctx* ctx, K kernel, int threads, uint32_t tiles) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const uint64_t full = (uint64_t)per_sm * (uint64_t)ctx->num_sms;
    const uint64_t need = ((uint64_t)tiles * 32 + threads - 1) / threads;
    return (uint32_t)std::max<uint64_t>(1, std::min(full, need));
}

// Work-counter slots (ctx->d_work) of the persistent kernels.
enum : int {
    kWorkPrimary = 0,
    kWorkSecondary = 1,
    kWorkRays = 2,
    kWorkPath = 3,
    kWorkAdjoint = 4,
    kWorkBatch = 5,
    kWorkHeavy = 6,
    kWorkShade = 7,
    kShadeCounts = 8  // two words: shadow-list and mirror-list lengths
};

// Grows the compacted shading-ray lists of l to px pixels (synchronises the
// context stream when it allocates; call before a stream capture).
rt_status ensure_shade_lists(rt_ctx* ctx, rt_lbvh* l, size_t px);
// Grows the per-frame result buffers of l (f_primary, f_vis, f_mirror) to px
// pixels (synchronises the context stream when it allocates).
rt_status ensure_frame_buffers(rt_ctx* ctx, rt_lbvh* l, size_t px);
// Primary rays, then (d_vis or d_mirror set) the shading rays started at the
// primary leaves; the shading lists must hold the image (ensure_shade_lists).
rt_status trace_frame(rt_ctx* ctx, rt_lbvh* l, const rt_camera* cam, const float light[3], rt_hit* d_primary,
                      uint8_t* d_vis, rt_hit* d_mirror, const char* who);

inline rt_status reset_work(rt_ctx* ctx, int slot) {
    RT_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->d_work + slot, 0, sizeof(uint32_t), ctx->stream));
    return RT_OK;
}

