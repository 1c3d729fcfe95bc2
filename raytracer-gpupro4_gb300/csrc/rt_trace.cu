// rt_trace.cu -- primary, shadow and mirror rays over the LBVH on sm_103a.
//
// Replaces the per-bounce dispatches of RayTracerCS::Render
// (RayTracerCS/RayTracerCS.cpp:284-295): CSGeneratePrimaryRays
// (Shaders/CS/CSPrimaryRays.hlsl:22-69) and CSComputeIntersections
// (CSIntersections.hlsl:18-39) are fused into k_trace_primary (rays are made
// in registers, no 48-byte ray buffer round trip); the shadow ray and the
// mirror bounce of CSComputeColor (CSComputeColorRT.hlsl:57-177, 203-210,
// flat normals, no textures) are k_trace_secondary.
//
// All three kernels are persistent: a grid sized to fill every SM once, each
// warp pulling 32-ray tiles (8 x 4 pixels) from a work counter until the
// image is done.  Ray cost varies by three orders of magnitude across the
// image, so a static grid leaves SMs idle behind the last heavy tiles.
#include <algorithm>
#include <cstring>

#include "rt_traverse.cuh"

using namespace rt;

namespace {

constexpr int kTraceThreads = 128;

__device__ __forceinline__ void store_hit(rt_hit* out, const Hit& h) {
    *reinterpret_cast<int4*>(out) = make_int4(h.id, __float_as_int(h.u), __float_as_int(h.v), __float_as_int(h.t));
}

// Heavy-ray list entries: kind in the top two bits, pixel or ray index below.
enum : uint32_t { kHeavyPrimary = 0, kHeavyShadow = 1, kHeavyMirror = 2, kHeavyRay = 3 };
constexpr uint32_t kHeavyIndexMask = (1u << 30) - 1u;

__device__ __forceinline__ void spill_record(uint32_t* list, int slot, uint32_t kind, size_t index) {
    list[slot] = (kind << 30) | (uint32_t)index;
}

constexpr uint32_t kNoSlot = 0xffffffffu;

// Warp-aggregated append of the lanes' pixels to a list (a warp's pixels in
// lane order, so neighbouring rays stay neighbours).  Returns the lane's
// slot, or kNoSlot.
__device__ __forceinline__ uint32_t append_pixel(bool take, uint32_t p, uint32_t* list, uint32_t cap,
                                                 uint32_t* count) {
    const uint32_t m = __ballot_sync(0xffffffffu, take);
    if (!m) return kNoSlot;
    uint32_t base = 0;
    if ((threadIdx.x & 31) == 0) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    const uint32_t k = base + __popc(m & ((1u << (threadIdx.x & 31)) - 1u));
    if (!take || k >= cap) return kNoSlot;
    list[k] = p;
    return k;
}

// The shading-ray lists of a frame (shadow pixels, then mirror pixels) and
// the results that need no ray.  A frame's primary pass fills them as it
// goes (lists != nullptr), so no separate pass re-reads the primary hits.
// Beside each listed pixel its ray (two float4: origin and tmax, direction
// and the excluded triangle) and the node its walk starts at, so the
// tracing kernel neither re-reads the primary hit and the triangle nor
// rebuilds the ray.
struct ShadeLists {
    const float* soup;
    float lx, ly, lz;
    uint8_t* vis;
    rt_hit* mirror;
    uint32_t* lists;
    uint32_t cap;
    uint32_t* counts;  // 2 words
    float4* rays;      // 2 x cap rays (2 float4 each), by list slot
    uint32_t* starts;  // 2 x cap start nodes, by list slot
};

__device__ __forceinline__ void put_ray(float4* q, const RayState& r) {
    q[0] = make_float4(r.o.x, r.o.y, r.o.z, r.tmax);
    q[1] = make_float4(r.d.x, r.d.y, r.d.z, __int_as_float(r.exclude));
}

// One pixel's shading-ray setup from its primary hit ph (all lanes call):
// visibility 0 (no hit) or 1 (light behind the surface) and the mirror
// miss record are written, the pixels that cast a shadow ray and those that
// cast a mirror ray are appended to the two lists with their rays and
// `start`, the restart node of the walks (the primary hit's leaf, or 1).
__device__ __forceinline__ void shade_setup_pixel(const ShadeLists& sl, const rt_camera& cam, int4 ph, bool valid,
                                                  uint32_t i, uint32_t j, size_t p, uint32_t start) {
    const ShadeRays s = shade_rays(sl.soup, cam, sl.lx, sl.ly, sl.lz, ph, valid, i, j, sl.mirror != nullptr);
    if (valid) {
        if (sl.vis && !(s.has && s.cast)) sl.vis[p] = vis_code(s.has, s.cast, false);
        if (sl.mirror && !s.has) {
            Hit mh;
            mh.id = -2; mh.u = -1.0f; mh.v = -1.0f; mh.t = 0.0f;
            store_hit(sl.mirror + p, mh);
        }
    }
    const uint32_t ks = append_pixel(sl.vis && valid && s.has && s.cast, (uint32_t)p, sl.lists, sl.cap, sl.counts);
    const uint32_t km = append_pixel(sl.mirror && valid && s.has, (uint32_t)p, sl.lists + sl.cap, sl.cap, sl.counts + 1);
    if (ks != kNoSlot) {
        put_ray(sl.rays + 2 * (size_t)ks, s.shadow);
        sl.starts[ks] = start;
    }
    if (km != kNoSlot) {
        put_ray(sl.rays + 2 * ((size_t)sl.cap + km), s.mirror);
        sl.starts[sl.cap + km] = start;
    }
}

// At most 72 registers (seven blocks per SM, no spills): a little faster
// than the 80 the compiler picks unbounded; 64 spills and is slower.
template <bool STATS>
__global__ void __launch_bounds__(kTraceThreads, 7) k_trace_primary(TreeRef tr, rt_camera cam,
                                                                 rt_hit* __restrict__ hits,
                                                                 uint32_t* __restrict__ leaves,
                                                                 uint32_t* __restrict__ stats, uint32_t* work,
                                                                 uint32_t num_tiles, Spill spill,
                                                                 uint32_t* __restrict__ list, TileOrder ord,
                                                                 ShadeLists sl) {
    grid_dep_wait();
    const uint32_t wbuf = *ord.parity, rbuf = wbuf ^ 1u, heavy = min(ord.counts[rbuf], ord.cap);
    for (uint32_t tile = next_ordered_tile(work, ord, rbuf, heavy, num_tiles); tile < num_tiles;
         tile = next_ordered_tile(work, ord, rbuf, heavy, num_tiles)) {
        uint32_t i, j;
        const bool valid = tile_pixel(tile, threadIdx.x & 31, cam.width, cam.height, &i, &j);
        if (!valid) i = j = 0;  // lanes past the image edge only help the warp
        const f3 d = primary_dir(cam, i, j);
        const RayState r = make_ray(mk3(cam.eye[0], cam.eye[1], cam.eye[2]), d, 1e16f, -1);
        uint32_t nb = 0, nt = 0, leaf = 1;
        int slot = -1;
        const Hit h = trace_ray<STATS>(r, valid, tr, false, &nb, &nt, &spill, &slot, 1u, &leaf);
        const size_t p = (size_t)j * cam.width + i;
        if (valid) {
            if (slot >= 0) {
                spill_record(list, slot, kHeavyPrimary, p);
            } else {
                store_hit(hits + p, h);
                if (leaves) leaves[p] = leaf;
            }
            if (STATS) {
                stats[2 * p] = nb;
                stats[2 * p + 1] = nt;
            }
        }
        if (sl.lists) {  // uniform; a handed-over pixel is set up by the warp-per-ray pass
            const int4 ph = make_int4(h.id, __float_as_int(h.u), __float_as_int(h.v), __float_as_int(h.t));
            shade_setup_pixel(sl, cam, ph, valid && slot < 0, i, j, p, leaf);
        }
        record_tile_cost(ord, wbuf, tile, nb + nt);
    }
}


// Shadow (any hit) and mirror (closest hit) rays of one pixel whose primary
// hit is ph.  Called by all lanes of the warp together (valid == false for
// lanes past the image edge); rays of pixels whose primary ray missed, or
// whose light is behind the surface, are traced with active == false.
template <bool STATS>
__device__ __forceinline__ void secondary_pixel(const TreeRef& tr, const float* __restrict__ soup,
                                                const rt_camera& cam, float lx, float ly, float lz, int4 ph,
                                                uint8_t* __restrict__ vis, rt_hit* __restrict__ mirror,
                                                uint32_t* __restrict__ sstats, uint32_t* __restrict__ mstats,
                                                bool valid, uint32_t i, uint32_t j, const Spill* spill,
                                                uint32_t* __restrict__ list, uint32_t* tests, uint32_t start,
                                                uint32_t* __restrict__ mirror_leaves) {
    const size_t p = (size_t)j * cam.width + i;
    const ShadeRays s = shade_rays(soup, cam, lx, ly, lz, ph, valid, i, j, mirror != nullptr);
    uint32_t snb = 0, snt = 0, mnb = 0, mnt = 0;
    if (vis) {  // uniform across the warp
        int slot = -1;
        const Hit sh = trace_ray<STATS>(s.shadow, s.cast, tr, true, &snb, &snt, spill, &slot, start);
        if (valid) {
            if (slot >= 0) spill_record(list, slot, kHeavyShadow, p);
            else vis[p] = vis_code(s.has, s.cast, sh.id >= 0);
        }
    }
    if (mirror) {
        int slot = -1;
        uint32_t leaf = 1;
        Hit mh = trace_ray<STATS>(s.mirror, s.has, tr, false, &mnb, &mnt, spill, &slot, start, &leaf);
        if (!s.has) {
            mh.id = -2; mh.u = -1.0f; mh.v = -1.0f; mh.t = 0.0f;
        }
        if (valid) {
            if (slot >= 0) {
                spill_record(list, slot, kHeavyMirror, p);
            } else {
                store_hit(mirror + p, mh);
                if (mirror_leaves) mirror_leaves[p] = leaf;
            }
        }
    }
    if (STATS && valid) {
        if (sstats) { sstats[2 * p] = snb; sstats[2 * p + 1] = snt; }
        if (mstats) { mstats[2 * p] = mnb; mstats[2 * p + 1] = mnt; }
    }
    if (tests) *tests = snb + snt + mnb + mnt;
}

// Restart node of a pixel's shading rays: its primary hit's leaf, or the root.
__device__ __forceinline__ uint32_t shade_start(const uint32_t* __restrict__ prim_leaves, int4 ph, bool valid,
                                                size_t p) {
    return (prim_leaves && valid && ph.x >= 0) ? __ldg(prim_leaves + p) : 1u;
}

template <bool STATS>
__global__ void __launch_bounds__(kTraceThreads) k_trace_secondary(
    TreeRef tr, const float* __restrict__ soup, rt_camera cam, float lx, float ly, float lz,
    const rt_hit* __restrict__ prim, const uint32_t* __restrict__ prim_leaves, uint8_t* __restrict__ vis,
    rt_hit* __restrict__ mirror, uint32_t* __restrict__ mirror_leaves, uint32_t* __restrict__ sstats,
    uint32_t* __restrict__ mstats, uint32_t* work, uint32_t num_tiles, Spill spill, uint32_t* __restrict__ list,
    TileOrder ord) {
    const uint32_t wbuf = *ord.parity, rbuf = wbuf ^ 1u, heavy = min(ord.counts[rbuf], ord.cap);
    for (uint32_t tile = next_ordered_tile(work, ord, rbuf, heavy, num_tiles); tile < num_tiles;
         tile = next_ordered_tile(work, ord, rbuf, heavy, num_tiles)) {
        uint32_t i, j;
        const bool valid = tile_pixel(tile, threadIdx.x & 31, cam.width, cam.height, &i, &j);
        if (!valid) i = j = 0;
        int4 ph = make_int4(-1, 0, 0, 0);
        if (valid) ph = __ldg(reinterpret_cast<const int4*>(prim + (size_t)j * cam.width + i));
        uint32_t tests = 0;
        secondary_pixel<STATS>(tr, soup, cam, lx, ly, lz, ph, vis, mirror, sstats, mstats, valid, i, j, &spill,
                               list, &tests, shade_start(prim_leaves, ph, valid, (size_t)j * cam.width + i),
                               mirror_leaves);
        record_tile_cost(ord, wbuf, tile, tests);
    }
}

// Production path of the shading rays, in two passes.  k_shade_setup runs
// over the pixels in 8x4-tile order, writes the results that need no ray (no
// primary hit: visibility 0 and the mirror miss record; light behind the
// surface: visibility 1) and appends the pixels that cast a shadow ray and
// those that cast a mirror ray to two lists, a warp's pixels in order, so
// neighbouring rays stay neighbours, each with the ray the tile pass would
// cast and its start node.  k_trace_shade then traces the lists 32 rays per
// warp with every lane busy (the tile pass leaves the lanes of sky pixels and
// of pixels without a cast ray idle).
__global__ void __launch_bounds__(256) k_shade_setup(const float* __restrict__ soup, rt_camera cam, float lx, float ly,
                                                     float lz, const rt_hit* __restrict__ prim, uint8_t* __restrict__ vis,
                                                     rt_hit* __restrict__ mirror, uint32_t* __restrict__ mirror_leaves,
                                                     const uint32_t* __restrict__ prim_leaves,
                                                     uint32_t* __restrict__ lists, uint32_t cap, uint32_t* counts,
                                                     float4* __restrict__ rays, uint32_t* __restrict__ starts,
                                                     uint32_t num_tiles) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t t = warp; t < num_tiles; t += nwarps) {
        uint32_t i, j;
        const bool valid = tile_pixel(t, lane, cam.width, cam.height, &i, &j);
        if (!valid) i = j = 0;
        const size_t p = (size_t)j * cam.width + i;
        int4 ph = make_int4(-1, 0, 0, 0);
        if (valid) ph = __ldg(reinterpret_cast<const int4*>(prim + p));
        const ShadeLists sl{soup, lx, ly, lz, vis, mirror, lists, cap, counts, rays, starts};
        shade_setup_pixel(sl, cam, ph, valid, i, j, p, shade_start(prim_leaves, ph, valid, p));
        if (valid && mirror_leaves && ph.x < 0) mirror_leaves[p] = 1u;
    }
}

// k_trace_shade keeps every lane busy: a lane whose ray has finished takes
// the next list entry as soon as kRefillLanes lanes of its warp are idle
// (the newcomers take consecutive entries, so they stay neighbours), instead
// of idling until the warp's slowest ray is done (dynamic ray fetch, Aila
// and Laine 2009).  Each ray's walk and result are those of a whole-warp
// trace_ray: the same start, the same descent, the same leaf phase.
//
// A lane expands at most kShadeSteps internal nodes per round before the
// warp's leaf phase, so that lanes holding a leaf do not wait out one lane's
// long descent (shading rays start on the surface, where descents vary
// most).  At 2.1 M triangles / 1080p, with at most 72 registers (7 blocks per
// SM), 4 steps and a refill at 24 idle lanes were the fastest pair of those
// tried (steps 1-16, refill at 8-32 idle lanes): 9 % faster than an unbounded
// descent with a refill at 16.  The primary walk is fastest unbounded.
constexpr int kRefillLanes = 24;
constexpr int kShadeSteps = 4;

// The scenes of a batch as seen by k_trace_shade (nodes == nullptr: one tree):
// a listed pixel g belongs to scene g / px, whose heap is at nodes + (s <<
// depth) and whose triangles are [tri_off[s], tri_off[s + 1]) of the batch's
// sorted-triangle array.
struct BatchTrees {
    const rt_node* nodes;
    const uint32_t* tri_off;
    uint32_t depth, px;
};

template <bool BATCH>
__global__ void __launch_bounds__(kTraceThreads, 7) k_trace_shade(
    TreeRef tr0, const float* __restrict__ soup, rt_camera cam, float lx, float ly, float lz,
    const rt_hit* __restrict__ prim, const uint32_t* __restrict__ prim_leaves, uint8_t* __restrict__ vis,
    rt_hit* __restrict__ mirror, uint32_t* __restrict__ mirror_leaves, const uint32_t* __restrict__ lists,
    uint32_t cap, const uint32_t* counts, const float4* __restrict__ rays, const uint32_t* __restrict__ starts,
    uint32_t* work, Spill spill, uint32_t* __restrict__ list, BatchTrees bt) {
    grid_dep_wait();
    TreeRef tr = tr0;  // per lane: a batch's lanes may walk different scenes
    constexpr uint32_t kFull = 0xffffffffu;
    const uint32_t ns = min(counts[0], cap), nm = min(counts[1], cap), total = ns + nm;
    const int lane = threadIdx.x & 31;
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t stack_node[kStackSize];
    float stack_t0[kStackSize];
    RayState r = make_ray(mk3(0.f, 0.f, 0.f), mk3(0.f, 0.f, 1.f), 1.0f, -1);
    Best b;
    b.key = 0;
    b.t = 0.f;
    b.u = b.v = -1.f;
    b.id = -1;
    b.leaf = 1u;
    uint64_t bound = 0;
    NodeBox cur;
    cur.a = make_float4(0.f, 0.f, 0.f, 0.f);
    cur.b = cur.a;
    uint32_t sp = 0, node = 1, nbox = 0, ntri = 0, p = 0;
    int slot = -1;
    bool live = false, have = false, shadow = false, budgeted = false, drained = false;
    for (;;) {
        const uint32_t idle = __ballot_sync(kFull, !live);
        if (!drained && (idle == kFull || __popc(idle) >= kRefillLanes)) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(work, (uint32_t)__popc(idle));
            base = __shfl_sync(kFull, base, 0);
            if (base + (uint32_t)__popc(idle) >= total) drained = true;
            const uint32_t k = base + __popc(idle & lt);
            const bool take = !live && k < total;
            uint32_t start = 1u;
            if (take) {
                shadow = k < ns;
                const uint32_t q = shadow ? k : cap + (k - ns);  // list slot: pixel, ray, start node
                p = __ldg(lists + q);
                if (BATCH) {
                    const uint32_t sc = p / bt.px;
                    tr.nodes = bt.nodes + ((size_t)sc << bt.depth);
                    tr.tri_base = __ldg(bt.tri_off + sc);
                    tr.n = __ldg(bt.tri_off + sc + 1);
                }
                const float4 ra = __ldg(rays + 2 * (size_t)q), rb = __ldg(rays + 2 * (size_t)q + 1);
                r = make_ray(mk3(ra.x, ra.y, ra.z), mk3(rb.x, rb.y, rb.z), ra.w, __float_as_int(rb.w));
                start = __ldg(starts + q);
                b.key = hit_key(r.tmax, 0);
                b.id = -1;
                b.u = b.v = -1.0f;
                b.t = r.tmax;
                b.leaf = 1u;
                bound = b.key;
                sp = 0;
                nbox = ntri = 0;
                slot = -1;
                budgeted = spill.count != nullptr;
                live = true;
            }
            const bool ex = __any_sync(kFull, take && r.exact);  // warp-uniform choice of the box test
            if (take) {
                have = ex ? start_walk<true>(r, tr, start, b.t, stack_node, stack_t0, sp, node, cur, nbox)
                          : start_walk<false>(r, tr, start, b.t, stack_node, stack_t0, sp, node, cur, nbox);
            }
        }
        if (!__any_sync(kFull, live)) {
            if (drained) break;
            continue;
        }
        // one round of the walk: descend (at most kShadeSteps nodes) towards a
        // leaf, test the held leaves together, pop
        const bool ex = __any_sync(kFull, have && r.exact);
        bool leaf = false;
        if (have) {
            have = ex ? descend<true, false, true>(tr, r, b.t, node, cur, stack_node, stack_t0, sp, 0u, nbox,
                                                   kShadeSteps, &leaf)
                      : descend<false, false, true>(tr, r, b.t, node, cur, stack_node, stack_t0, sp, 0u, nbox,
                                                    kShadeSteps, &leaf);
        }
        __syncwarp();
        if (__any_sync(kFull, have && leaf)) leaf_phase<false>(tr, r, have && leaf, cur, node, bound, b, ntri);
        if (have && leaf) {
            if (shadow && b.id >= 0) {
                have = false;  // any hit
            } else {
                have = pop_node(tr, b.t, node, cur, stack_node, stack_t0, sp, 0u);
                if (budgeted && have && nbox + ntri > spill.budget) {
                    const uint32_t s = atomicAdd(spill.count, 1u);
                    if (s < spill.cap) {
                        slot = (int)s;
                        have = false;
                    } else {
                        budgeted = false;  // list full: finish here
                    }
                }
            }
        }
        if (live && !have) {  // the walk is over: the ray's result
            if (slot >= 0) {
                spill_record(list, slot, shadow ? kHeavyShadow : kHeavyMirror, p);
            } else if (shadow) {
                vis[p] = vis_code(true, true, b.id >= 0);
            } else {
                Hit h;
                h.id = b.id;
                h.u = b.u;
                h.v = b.v;
                h.t = b.t;
                store_hit(mirror + p, h);
                if (mirror_leaves) mirror_leaves[p] = tr.compact ? 1u : b.leaf;
            }
            live = false;
        }
    }
}

__device__ __forceinline__ RayState load_ray(const rt_ray* __restrict__ rays, uint32_t k, bool valid) {
    float4 a = make_float4(0.f, 0.f, 0.f, __int_as_float(-1)), b = make_float4(0.f, 0.f, 1.f, 1.f);
    if (valid) {
        a = __ldg(reinterpret_cast<const float4*>(rays + k));
        b = __ldg(reinterpret_cast<const float4*>(rays + k) + 1);
    }
    return make_ray(mk3(a.x, a.y, a.z), mk3(b.x, b.y, b.z), b.w, __float_as_int(a.w));
}

template <bool STATS>
__global__ void __launch_bounds__(kTraceThreads) k_trace_rays(TreeRef tr, const rt_ray* __restrict__ rays, uint32_t n,
                                                              int any_hit, const uint32_t* __restrict__ starts,
                                                              rt_hit* __restrict__ hits, uint32_t* __restrict__ leaves,
                                                              uint32_t* __restrict__ stats, uint32_t* work,
                                                              Spill spill, uint32_t* __restrict__ list,
                                                              TileOrder ord) {
    const uint32_t num_tiles = (n + 31) / 32;
    const uint32_t wbuf = *ord.parity, rbuf = wbuf ^ 1u, heavy = min(ord.counts[rbuf], ord.cap);
    for (uint32_t tile = next_ordered_tile(work, ord, rbuf, heavy, num_tiles); tile < num_tiles;
         tile = next_ordered_tile(work, ord, rbuf, heavy, num_tiles)) {
        const uint32_t k = tile * 32 + (threadIdx.x & 31);
        const bool valid = k < n;
        const RayState r = load_ray(rays, k, valid);
        const uint32_t start = (starts && valid) ? __ldg(starts + k) : 1u;
        uint32_t nb = 0, nt = 0, leaf = 1;
        int slot = -1;
        const Hit h = trace_ray<STATS>(r, valid, tr, any_hit != 0, &nb, &nt, &spill, &slot, start, &leaf);
        if (valid) {
            if (slot >= 0) {
                spill_record(list, slot, kHeavyRay, k);
            } else {
                store_hit(hits + k, h);
                if (leaves) leaves[k] = leaf;
            }
            if (STATS) {
                stats[2 * k] = nb;
                stats[2 * k + 1] = nt;
            }
        }
        record_tile_cost(ord, wbuf, tile, nb + nt);
    }
}

// Second pass over the rays the first pass handed over: one ray per warp
// (trace_wide), rebuilt from its list entry exactly as the first pass made
// it, and its result written where the first pass would have written it.
struct HeavyArgs {
    TreeRef tr;
    const float* soup;
    rt_camera cam;
    float lx, ly, lz;
    const rt_hit* prim;   // primary hits (shadow / mirror entries)
    rt_hit* hits;         // primary or generic-ray output
    uint8_t* vis;
    rt_hit* mirror;
    const rt_ray* rays;
    int any_hit;          // generic rays
    uint32_t* leaves;     // primary / generic-ray leaf output (nullable)
    uint32_t* mirror_leaves;
    uint32_t wide_cap;    // frontier-stack entries per warp (wide_stack_entries of the tree depth)
    uint32_t team_cap;    // frontier-stack entries per block (team_stack_entries of the tree depth)
    ShadeLists sl;        // primary entries: set up their pixel's shading rays too (sl.lists != nullptr)
    const uint32_t* list;
    const uint32_t* count;
    uint32_t cap;
    uint32_t* work;
};

__global__ void __launch_bounds__(kTraceThreads) k_trace_heavy(HeavyArgs a) {
    grid_dep_wait();
    const uint32_t n = min(*a.count, a.cap);
    const int lane = threadIdx.x & 31;
    for (uint32_t e = next_tile(a.work); e < n; e = next_tile(a.work)) {
        const uint32_t entry = __ldg(a.list + e);
        const uint32_t kind = entry >> 30, idx = entry & kHeavyIndexMask;
        if (kind == kHeavyPrimary) {
            const uint32_t i = idx % a.cam.width, j = idx / a.cam.width;
            const RayState r = make_ray(mk3(a.cam.eye[0], a.cam.eye[1], a.cam.eye[2]), primary_dir(a.cam, i, j),
                                        1e16f, -1);
            const Hit h = trace_wide(r, a.tr, false, a.wide_cap);
            if (lane == 0) {
                store_hit(a.hits + idx, h);
                if (a.leaves) a.leaves[idx] = 1u;  // the root: a valid restart node
            }
            if (a.sl.lists) {
                const int4 ph = make_int4(h.id, __float_as_int(h.u), __float_as_int(h.v), __float_as_int(h.t));
                shade_setup_pixel(a.sl, a.cam, ph, lane == 0, i, j, idx, 1u);
            }
        } else if (kind == kHeavyRay) {
            const RayState r = load_ray(a.rays, idx, true);
            const Hit h = trace_wide(r, a.tr, a.any_hit != 0, a.wide_cap);
            if (lane == 0) {
                store_hit(a.hits + idx, h);
                if (a.leaves) a.leaves[idx] = 1u;
            }
        } else {
            const uint32_t i = idx % a.cam.width, j = idx / a.cam.width;
            const int4 ph = __ldg(reinterpret_cast<const int4*>(a.prim + idx));
            const ShadeRays s = shade_rays(a.soup, a.cam, a.lx, a.ly, a.lz, ph, true, i, j, kind == kHeavyMirror);
            if (kind == kHeavyShadow) {
                const Hit h = trace_wide(s.shadow, a.tr, true, a.wide_cap);
                if (lane == 0) a.vis[idx] = vis_code(s.has, s.cast, h.id >= 0);
            } else {
                const Hit h = trace_wide(s.mirror, a.tr, false, a.wide_cap);
                if (lane == 0) {
                    store_hit(a.mirror + idx, h);
                    if (a.mirror_leaves) a.mirror_leaves[idx] = 1u;
                }
            }
        }
    }
}

// k_trace_heavy with a block per ray (traverse_team): for the handed-over
// shading rays, a few hundred grazing rays whose walks run for thousands of
// tests, where a warp per ray leaves the GPU waiting on the longest few.
__global__ void __launch_bounds__(kTeamThreads) k_trace_heavy_team(HeavyArgs a) {
    grid_dep_wait();
    __shared__ TeamShared ts;
    __shared__ uint32_t s_e;
    const uint32_t n = min(*a.count, a.cap);
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) s_e = atomicAdd(a.work, 1u);
        __syncthreads();
        const uint32_t e = s_e;
        __syncthreads();
        if (e >= n) break;
        const uint32_t entry = __ldg(a.list + e);
        const uint32_t kind = entry >> 30, idx = entry & kHeavyIndexMask;
        if (kind == kHeavyPrimary) {
            const uint32_t i = idx % a.cam.width, j = idx / a.cam.width;
            const RayState r = make_ray(mk3(a.cam.eye[0], a.cam.eye[1], a.cam.eye[2]), primary_dir(a.cam, i, j),
                                        1e16f, -1);
            const Hit h = trace_team(r, a.tr, false, a.team_cap, ts);
            if (tid == 0) {
                store_hit(a.hits + idx, h);
                if (a.leaves) a.leaves[idx] = 1u;  // the root: a valid restart node
            }
            if (a.sl.lists && tid < 32) {
                const int4 ph = make_int4(h.id, __float_as_int(h.u), __float_as_int(h.v), __float_as_int(h.t));
                shade_setup_pixel(a.sl, a.cam, ph, tid == 0, i, j, idx, 1u);
            }
        } else if (kind == kHeavyRay) {
            const RayState r = load_ray(a.rays, idx, true);
            const Hit h = trace_team(r, a.tr, a.any_hit != 0, a.team_cap, ts);
            if (tid == 0) {
                store_hit(a.hits + idx, h);
                if (a.leaves) a.leaves[idx] = 1u;
            }
        } else {
            const uint32_t i = idx % a.cam.width, j = idx / a.cam.width;
            const int4 ph = __ldg(reinterpret_cast<const int4*>(a.prim + idx));
            const ShadeRays sr = shade_rays(a.soup, a.cam, a.lx, a.ly, a.lz, ph, true, i, j, kind == kHeavyMirror);
            if (kind == kHeavyShadow) {
                const Hit h = trace_team(sr.shadow, a.tr, true, a.team_cap, ts);
                if (tid == 0) a.vis[idx] = vis_code(sr.has, sr.cast, h.id >= 0);
            } else {
                const Hit h = trace_team(sr.mirror, a.tr, false, a.team_cap, ts);
                if (tid == 0) {
                    store_hit(a.mirror + idx, h);
                    if (a.mirror_leaves) a.mirror_leaves[idx] = 1u;
                }
            }
        }
    }
}


uint32_t pixel_tiles(const rt_camera* cam) {
    return (uint32_t)(((cam->width + 7) / 8) * ((cam->height + 3) / 4));
}

rt_status check_trace_args(rt_ctx* ctx, const rt_lbvh* l, const rt_camera* cam, const char* who) {
    if (!ctx) return RT_ERR_INVALID;
    if (!l || !cam) return rt_fail(ctx, RT_ERR_INVALID, "%s: null argument", who);
    if (l->n == 0) return rt_fail(ctx, RT_ERR_INVALID, "%s: the LBVH has not been built", who);
    if (cam->width == 0 || cam->height == 0 || (uint64_t)cam->width * cam->height > (1ull << 31))
        return rt_fail(ctx, RT_ERR_INVALID, "%s: bad image size %ux%u", who, cam->width, cam->height);
    return RT_OK;
}

}  // namespace

rt_status ensure_shade_lists(rt_ctx* ctx, rt_lbvh* l, size_t px) {
    if (px <= l->s_pixels) return RT_OK;
    if (l->graph_refs > 0)
        return rt_fail(ctx, RT_ERR_CAPACITY,
                       "shading lists of %zu pixels cannot grow to %zu while a captured frame uses them",
                       l->s_pixels, px);
    RT_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (l->s_lists) cudaFree(l->s_lists);
    if (l->s_rays) cudaFree(l->s_rays);
    l->s_lists = nullptr;
    l->s_rays = nullptr;
    l->s_pixels = 0;
    // shadow-ray pixels, mirror-ray pixels, primary leaves of a frame, start
    // nodes of the listed rays (2 x px); the listed rays (2 x px x 32 bytes)
    RT_CHECK_CUDA(ctx, cudaMalloc((void**)&l->s_lists, 5 * sizeof(uint32_t) * px));
    RT_CHECK_CUDA(ctx, cudaMalloc((void**)&l->s_rays, 4 * sizeof(float4) * px));
    l->s_pixels = px;
    return RT_OK;
}

TreeRef tree_ref(const rt_ctx* ctx, const rt_lbvh* l) {
    TreeRef t;
    t.compact = l->compact_valid;
    t.tri_base = 0;
    t.nodes = t.compact ? l->cnodes : l->nodes;
    t.num_nodes = t.compact ? l->ccap : l->num_nodes;
    t.tris = l->sorted_tris;
    t.n = l->n;
    t.err = ctx->d_err;
    return t;
}

namespace {

// Heavy-ray hand-over of one trace call: the list is emptied before the
// first pass (budget 0 or a counting pass: no hand-over), and the second pass
// drains it.
// The shading rays keep their own list length and claim counter, so a frame
// zeroes both passes' counters in one launch before its primary pass.
Spill spill_of(rt_ctx* ctx, bool enabled, int kind) {
    Spill sp;
    sp.budget = ctx->trace_budget[kind];
    const bool shade = kind == 1;
    sp.count = (enabled && sp.budget) ? ctx->d_spill_count + (shade ? 1 : 0) : nullptr;
    sp.work = shade ? ctx->d_spill_count + 2 : ctx->d_work + kWorkHeavy;
    sp.cap = kSpillCap;
    return sp;
}

// A trace call zeroes its counters (words of ctx->d_words) in one small
// kernel launched before its first pass, k_order_begin where the call has a
// tile order to advance, k_reset_words otherwise: one graph node instead of a
// memset per counter, and a programmatic edge to the pass.
uint64_t word_bit(const rt_ctx* ctx, const uint32_t* p) { return 1ull << (uint32_t)(p - ctx->d_words); }

// The list length and the warp-per-ray pass's claim counter.
uint64_t spill_reset_bits(const rt_ctx* ctx, const Spill& sp) {
    return sp.count ? word_bit(ctx, sp.count) | word_bit(ctx, sp.work) : 0ull;
}

// The counters of the compacted shading-ray pass.
uint64_t shade_reset_bits(const rt_ctx* ctx, const Spill& sp) {
    return word_bit(ctx, ctx->d_work + kWorkSecondary) | word_bit(ctx, ctx->d_work + kWorkShade) |
           spill_reset_bits(ctx, sp);
}

__device__ __forceinline__ void zero_words(uint32_t* words, unsigned long long mask) {
    if (threadIdx.x < 64 && ((mask >> threadIdx.x) & 1ull)) words[threadIdx.x] = 0u;
}

__global__ void k_reset_words(uint32_t* words, unsigned long long mask) {
    grid_dep_wait();
    zero_words(words, mask);
}

rt_status reset_words(rt_ctx* ctx, uint64_t mask) {
    if (!mask) return RT_OK;
    launch_pdl(k_reset_words, 1, 64, 0, ctx->stream, ctx->d_words, (unsigned long long)mask);
    RT_CHECK_LAUNCH(ctx, "k_reset_words");
    return RT_OK;
}

rt_status launch_heavy(rt_ctx* ctx, const Spill& sp, HeavyArgs a, int kind) {
    if (!sp.count) return RT_OK;
    a.list = ctx->d_spill;
    a.count = sp.count;
    a.cap = kSpillCap;
    a.work = sp.work;
    if ((ctx->heavy_team >> kind) & 1u) {
        const size_t smem = team_smem_bytes(a.team_cap);
        if (smem > 48u * 1024u)
            RT_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_trace_heavy_team, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)smem));
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_heavy_team, kTeamThreads, smem) !=
                cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        launch_pdl(k_trace_heavy_team, (uint32_t)per_sm * ctx->num_sms, kTeamThreads, smem, ctx->stream, a);
        RT_CHECK_LAUNCH(ctx, "k_trace_heavy_team");
        return RT_OK;
    }
    const size_t smem = wide_smem_bytes(a.wide_cap);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_heavy, kTraceThreads, smem) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    launch_pdl(k_trace_heavy, (uint32_t)per_sm * ctx->num_sms, kTraceThreads, smem, ctx->stream, a);
    RT_CHECK_LAUNCH(ctx, "k_trace_heavy");
    return RT_OK;
}

__global__ void k_order_begin(TileOrder o, uint32_t* words, unsigned long long reset) {
    grid_dep_wait();
    zero_words(words, reset);
    __shared__ uint32_t s_w;
    if (threadIdx.x == 0) {
        const uint32_t w = *o.parity ^ 1u;
        *o.parity = w;
        s_w = w;
    }
    __syncthreads();
    const uint32_t w = s_w;
    const uint32_t n = min(o.counts[w], o.cap);
    __syncthreads();
    // the buffer this call writes was read two calls ago: clear its bits
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t t = o.lists[(size_t)w * o.cap + i];
        if (t < o.cap) o.bits[(size_t)w * (o.cap / 32) + t / 32] = 0u;
    }
    __syncthreads();
    if (threadIdx.x == 0) o.counts[w] = 0u;
}

// Tile order of one trace kind (0 primary, 1 shading, 2 generic rays),
// advanced to this call; enabled == false gives image order (cap 0: no list
// is read or written).  reset: the call's counters to zero (word_bit mask).
rt_status order_begin(rt_ctx* ctx, int kind, bool enabled, TileOrder* out, uint64_t reset = 0) {
    TileOrder o;
    o.cap = enabled ? kOrderCap : 0u;
    o.parity = ctx->d_words + 40 + 4 * kind;
    o.counts = o.parity + 1;
    o.lists = ctx->d_order + (size_t)kind * kOrderWords;
    o.bits = o.lists + 2 * (size_t)kOrderCap;
    if (enabled) {
        launch_pdl(k_order_begin, 1, 256, 0, ctx->stream, o, ctx->d_words, (unsigned long long)reset);
        RT_CHECK_LAUNCH(ctx, "k_order_begin");
    } else {
        rt_status s = reset_words(ctx, reset);
        if (s != RT_OK) return s;
    }
    *out = o;
    return RT_OK;
}

HeavyArgs heavy_args(rt_ctx* ctx, const rt_lbvh* l) {
    HeavyArgs a;
    memset(&a, 0, sizeof(a));
    a.tr = tree_ref(ctx, l);
    a.wide_cap = wide_stack_entries(l->depth);
    a.team_cap = team_stack_entries(l->depth);
    return a;
}

}  // namespace

namespace {

// sl (nullable): a frame's shading lists, filled by this pass as it goes
// (their counts are zeroed with this call's counters); the statistics
// variant never fills them.
rt_status trace_primary(rt_ctx* ctx, const rt_lbvh* l, const rt_camera* cam, rt_hit* d_hits, uint32_t* d_leaves,
                        uint32_t* d_stats, const char* who, const ShadeLists* sl = nullptr,
                        uint64_t extra_reset = 0) {
    rt_status s = check_trace_args(ctx, l, cam, who);
    if (s != RT_OK) return s;
    if (!d_hits) return rt_fail(ctx, RT_ERR_INVALID, "%s: null output", who);
    const Spill sp = spill_of(ctx, !d_stats && (uint64_t)cam->width * cam->height <= kHeavyIndexMask, 0);
    uint64_t reset = word_bit(ctx, ctx->d_work + kWorkPrimary) | spill_reset_bits(ctx, sp) | extra_reset;
    if (sl && !d_stats) reset |= word_bit(ctx, sl->counts) | word_bit(ctx, sl->counts + 1);
    TileOrder ord;
    if ((s = order_begin(ctx, 0, ctx->tile_order & 1u, &ord, reset)) != RT_OK) return s;
    const uint32_t tiles = pixel_tiles(cam);
    uint32_t* work = ctx->d_work + kWorkPrimary;
    ShadeLists none;
    memset(&none, 0, sizeof(none));
    const ShadeLists lists = (sl && !d_stats) ? *sl : none;
    if (d_stats) {
        auto k = k_trace_primary<true>;
        k<<<persistent_blocks(ctx, k, kTraceThreads, tiles), kTraceThreads, 0, ctx->stream>>>(
            tree_ref(ctx, l), *cam, d_hits, d_leaves, d_stats, work, tiles, sp, ctx->d_spill, ord, none);
    } else {
        auto k = k_trace_primary<false>;
        launch_pdl(k, persistent_blocks(ctx, k, kTraceThreads, tiles), kTraceThreads, 0, ctx->stream,
                   tree_ref(ctx, l), *cam, d_hits, d_leaves, (uint32_t*)nullptr, work, tiles, sp, ctx->d_spill, ord,
                   lists);
    }
    RT_CHECK_LAUNCH(ctx, "k_trace_primary");
    HeavyArgs a = heavy_args(ctx, l);
    a.cam = *cam;
    a.hits = d_hits;
    a.leaves = d_leaves;
    a.sl = lists;
    return launch_heavy(ctx, sp, a, 0);
}

// prebuilt: the frame's primary pass has filled the shading lists (and the
// results that need no ray), so the setup pass is skipped, and the counters
// of this pass were zeroed with the primary pass's (shade_reset_bits).
rt_status trace_shadow_mirror(rt_ctx* ctx, const rt_lbvh* l, const rt_camera* cam, const float light[3],
                              const rt_hit* d_primary, const uint32_t* d_prim_leaves, uint8_t* d_vis,
                              rt_hit* d_mirror, uint32_t* d_mirror_leaves, uint32_t* d_shadow_stats,
                              uint32_t* d_mirror_stats, const char* who, bool prebuilt = false) {
    rt_status s = check_trace_args(ctx, l, cam, who);
    if (s != RT_OK) return s;
    if (!light || !d_primary) return rt_fail(ctx, RT_ERR_INVALID, "%s: null argument", who);
    if (!l->src_tris) return rt_fail(ctx, RT_ERR_INVALID, "%s: no triangle soup bound", who);
    const bool stats = d_shadow_stats || d_mirror_stats;
    const Spill sp = spill_of(ctx, !stats && (uint64_t)cam->width * cam->height <= kHeavyIndexMask, 1);
    uint64_t reset = word_bit(ctx, ctx->d_work + kWorkSecondary) | spill_reset_bits(ctx, sp);
    const uint32_t tiles = pixel_tiles(cam);
    if (stats) {  // per-pixel counts in the oracle's order: the tile pass
        TileOrder ord;
        if ((s = order_begin(ctx, 1, ctx->tile_order & 2u, &ord, reset)) != RT_OK) return s;
        uint32_t* work = ctx->d_work + kWorkSecondary;
        auto k = k_trace_secondary<true>;
        k<<<persistent_blocks(ctx, k, kTraceThreads, tiles), kTraceThreads, 0, ctx->stream>>>(
            tree_ref(ctx, l), l->src_tris, *cam, light[0], light[1], light[2], d_primary, d_prim_leaves, d_vis,
            d_mirror, d_mirror_leaves, d_shadow_stats, d_mirror_stats, work, tiles, sp, ctx->d_spill, ord);
        RT_CHECK_LAUNCH(ctx, "k_trace_secondary");
    } else {  // compacted shading-ray lists
        const size_t px = (size_t)cam->width * cam->height;
        if ((s = ensure_shade_lists(ctx, const_cast<rt_lbvh*>(l), px)) != RT_OK) return s;
        uint32_t* counts = ctx->d_work + kShadeCounts;
        if (!prebuilt) {
            reset = shade_reset_bits(ctx, sp) | word_bit(ctx, counts) | word_bit(ctx, counts + 1);
            if ((s = reset_words(ctx, reset)) != RT_OK) return s;
        }
        const uint32_t cap = (uint32_t)l->s_pixels;
        if (!prebuilt) {
            const uint32_t sblocks = std::max(1u, std::min((tiles + 7) / 8, (uint32_t)ctx->num_sms * 8));
            k_shade_setup<<<sblocks, 256, 0, ctx->stream>>>(l->src_tris, *cam, light[0], light[1], light[2], d_primary,
                                                             d_vis, d_mirror, d_mirror_leaves, d_prim_leaves,
                                                             l->s_lists, cap, counts, l->s_rays,
                                                             l->s_lists + 3 * l->s_pixels,
                                                             tiles);
            RT_CHECK_LAUNCH(ctx, "k_shade_setup");
        }
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_shade<false>, kTraceThreads, 0) !=
                cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        launch_pdl(k_trace_shade<false>, (uint32_t)per_sm * ctx->num_sms, kTraceThreads, 0, ctx->stream, tree_ref(ctx, l),
                   l->src_tris, *cam, light[0], light[1], light[2], d_primary, d_prim_leaves, d_vis, d_mirror,
                   d_mirror_leaves, (const uint32_t*)l->s_lists, cap, (const uint32_t*)counts,
                   (const float4*)l->s_rays, (const uint32_t*)(l->s_lists + 3 * l->s_pixels), ctx->d_work + kWorkShade,
                   sp, ctx->d_spill, BatchTrees{nullptr, nullptr, 0u, 0u});
        RT_CHECK_LAUNCH(ctx, "k_trace_shade");
    }
    HeavyArgs a = heavy_args(ctx, l);
    a.soup = l->src_tris;
    a.cam = *cam;
    a.lx = light[0];
    a.ly = light[1];
    a.lz = light[2];
    a.prim = d_primary;
    a.vis = d_vis;
    a.mirror = d_mirror;
    a.mirror_leaves = d_mirror_leaves;
    return launch_heavy(ctx, sp, a, 1);
}

rt_status trace_rays(rt_ctx* ctx, const rt_lbvh* l, const rt_ray* d_rays, uint32_t n, int any_hit,
                     const uint32_t* d_starts, rt_hit* d_hits, uint32_t* d_leaves, uint32_t* d_stats,
                     const char* who) {
    if (!ctx) return RT_ERR_INVALID;
    if (!l || !d_rays || !d_hits) return rt_fail(ctx, RT_ERR_INVALID, "%s: null argument", who);
    if (l->n == 0) return rt_fail(ctx, RT_ERR_INVALID, "%s: the LBVH has not been built", who);
    if (n == 0) return RT_OK;
    const Spill sp = spill_of(ctx, !d_stats && n <= kHeavyIndexMask, 2);
    const uint64_t reset = word_bit(ctx, ctx->d_work + kWorkRays) | spill_reset_bits(ctx, sp);
    TileOrder ord;
    rt_status s = order_begin(ctx, 2, ctx->tile_order & 4u, &ord, reset);
    if (s != RT_OK) return s;
    const uint32_t tiles = (n + 31) / 32;
    uint32_t* work = ctx->d_work + kWorkRays;
    if (d_stats) {
        auto k = k_trace_rays<true>;
        k<<<persistent_blocks(ctx, k, kTraceThreads, tiles), kTraceThreads, 0, ctx->stream>>>(
            tree_ref(ctx, l), d_rays, n, any_hit, d_starts, d_hits, d_leaves, d_stats, work, sp, ctx->d_spill, ord);
    } else {
        auto k = k_trace_rays<false>;
        k<<<persistent_blocks(ctx, k, kTraceThreads, tiles), kTraceThreads, 0, ctx->stream>>>(
            tree_ref(ctx, l), d_rays, n, any_hit, d_starts, d_hits, d_leaves, nullptr, work, sp, ctx->d_spill, ord);
    }
    RT_CHECK_LAUNCH(ctx, "k_trace_rays");
    HeavyArgs a = heavy_args(ctx, l);
    a.rays = d_rays;
    a.any_hit = any_hit;
    a.hits = d_hits;
    a.leaves = d_leaves;
    return launch_heavy(ctx, sp, a, 2);
}

}  // namespace

extern "C" rt_status rt_trace_primary(rt_ctx* ctx, const rt_lbvh* l, const rt_camera* cam, rt_hit* d_hits,
                                      uint32_t* d_stats) {
    return trace_primary(ctx, l, cam, d_hits, nullptr, d_stats, "rt_trace_primary");
}

extern "C" rt_status rt_trace_primary_leaves(rt_ctx* ctx, const rt_lbvh* l, const rt_camera* cam, rt_hit* d_hits,
                                             uint32_t* d_leaves, uint32_t* d_stats) {
    return trace_primary(ctx, l, cam, d_hits, d_leaves, d_stats, "rt_trace_primary_leaves");
}

extern "C" rt_status rt_trace_shadow_mirror(rt_ctx* ctx, const rt_lbvh* l, const rt_camera* cam, const float light[3],
                                            const rt_hit* d_primary, uint8_t* d_vis, rt_hit* d_mirror,
                                            uint32_t* d_shadow_stats, uint32_t* d_mirror_stats) {
    return trace_shadow_mirror(ctx, l, cam, light, d_primary, nullptr, d_vis, d_mirror, nullptr, d_shadow_stats,
                               d_mirror_stats, "rt_trace_shadow_mirror");
}

extern "C" rt_status rt_trace_shadow_mirror_from(rt_ctx* ctx, const rt_lbvh* l, const rt_camera* cam,
                                                 const float light[3], const rt_hit* d_primary,
                                                 const uint32_t* d_primary_leaves, uint8_t* d_vis, rt_hit* d_mirror,
                                                 uint32_t* d_mirror_leaves, uint32_t* d_shadow_stats,
                                                 uint32_t* d_mirror_stats) {
    return trace_shadow_mirror(ctx, l, cam, light, d_primary, d_primary_leaves, d_vis, d_mirror, d_mirror_leaves,
                               d_shadow_stats, d_mirror_stats, "rt_trace_shadow_mirror_from");
}

extern "C" rt_status rt_trace_rays(rt_ctx* ctx, const rt_lbvh* l, const rt_ray* d_rays, uint32_t n, int any_hit,
                                   rt_hit* d_hits, uint32_t* d_stats) {
    return trace_rays(ctx, l, d_rays, n, any_hit, nullptr, d_hits, nullptr, d_stats, "rt_trace_rays");
}

extern "C" rt_status rt_trace_rays_from(rt_ctx* ctx, const rt_lbvh* l, const rt_ray* d_rays, uint32_t n, int any_hit,
                                        const uint32_t* d_starts, rt_hit* d_hits, uint32_t* d_leaves,
                                        uint32_t* d_stats) {
    return trace_rays(ctx, l, d_rays, n, any_hit, d_starts, d_hits, d_leaves, d_stats, "rt_trace_rays_from");
}

// The trace stages of one frame: primary rays, then the shading rays started
// at each primary hit's leaf (the iRoot restart; the leaves live in the third
// segment of the shading lists, which the caller has sized).
rt_status trace_frame(rt_ctx* ctx, rt_lbvh* l, const rt_camera* cam, const float light[3], rt_hit* d_primary,
                      uint8_t* d_vis, rt_hit* d_mirror, const char* who) {
    const size_t px = (size_t)cam->width * cam->height;
    uint32_t* leaves = (d_vis || d_mirror) && l->s_pixels >= px ? l->s_lists + 2 * l->s_pixels : nullptr;
    if (!leaves) return trace_primary(ctx, l, cam, d_primary, nullptr, nullptr, who);
    if (!l->src_tris) return rt_fail(ctx, RT_ERR_INVALID, "%s: no triangle soup bound", who);
    // the primary pass (and its warp-per-ray pass) fills the shading lists
    ShadeLists sl{l->src_tris, light[0], light[1], light[2], d_vis,     d_mirror,
                  l->s_lists, (uint32_t)l->s_pixels, ctx->d_work + kShadeCounts, l->s_rays,
                  l->s_lists + 3 * l->s_pixels};
    // the shading pass's counters are zeroed with the primary pass's
    const Spill ssp = spill_of(ctx, px <= kHeavyIndexMask, 1);
    rt_status s = trace_primary(ctx, l, cam, d_primary, leaves, nullptr, who, &sl, shade_reset_bits(ctx, ssp));
    if (s == RT_OK)
        s = trace_shadow_mirror(ctx, l, cam, light, d_primary, leaves, d_vis, d_mirror, nullptr, nullptr, nullptr, who,
                                true);
    return s;
}

rt_status ensure_frame_buffers(rt_ctx* ctx, rt_lbvh* l, size_t px) {
    if (px <= l->f_pixels) return RT_OK;  // frame buffers grow on the first call at a new size
    if (l->graph_refs > 0)
        return rt_fail(ctx, RT_ERR_CAPACITY,
                       "frame buffers of %zu pixels cannot grow to %zu while a captured frame uses them",
                       l->f_pixels, px);
    RT_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (l->f_primary) cudaFree(l->f_primary);
    if (l->f_mirror) cudaFree(l->f_mirror);
    if (l->f_vis) cudaFree(l->f_vis);
    l->f_primary = nullptr; l->f_mirror = nullptr; l->f_vis = nullptr; l->f_pixels = 0;
    RT_CHECK_CUDA(ctx, cudaMalloc((void**)&l->f_primary, sizeof(rt_hit) * px));
    RT_CHECK_CUDA(ctx, cudaMalloc((void**)&l->f_mirror, sizeof(rt_hit) * px));
    RT_CHECK_CUDA(ctx, cudaMalloc((void**)&l->f_vis, px));
    l->f_pixels = px;
    return RT_OK;
}

static rt_status render_frame_host(rt_ctx* ctx, rt_lbvh* l, const float* h_tris, uint32_t n, const rt_camera* cam,
                                   const float light[3], rt_hit* h_primary, uint8_t* h_vis, rt_hit* h_mirror,
                                   bool sync, const char* who) {
    if (!ctx) return RT_ERR_INVALID;
    if (!l || !h_tris || !cam || !light) return rt_fail(ctx, RT_ERR_INVALID, "%s: null argument", who);
    const size_t px = (size_t)cam->width * cam->height;
    if (px == 0 || px > (1ull << 31)) return rt_fail(ctx, RT_ERR_INVALID, "%s: bad image size", who);
    rt_status s = ensure_frame_buffers(ctx, l, px);
    if (s != RT_OK) return s;
    if (h_vis || h_mirror) {
        if ((s = ensure_shade_lists(ctx, l, px)) != RT_OK) return s;
    }
    if ((s = rt_lbvh_build_host(ctx, l, h_tris, n, 0)) != RT_OK) return s;
    if ((s = trace_frame(ctx, l, cam, light, l->f_primary, h_vis ? l->f_vis : nullptr, h_mirror ? l->f_mirror : nullptr,
                         who)) != RT_OK)
        return s;
    cudaStream_t st = ctx->stream;
    if (h_primary) RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_primary, l->f_primary, sizeof(rt_hit) * px, cudaMemcpyDeviceToHost, st));
    if (h_vis) RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_vis, l->f_vis, px, cudaMemcpyDeviceToHost, st));
    if (h_mirror) RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_mirror, l->f_mirror, sizeof(rt_hit) * px, cudaMemcpyDeviceToHost, st));
    if (sync) RT_CHECK_CUDA(ctx, cudaStreamSynchronize(st));
    return RT_OK;
}

extern "C" rt_status rt_render_frame_host(rt_ctx* ctx, rt_lbvh* l, const float* h_tris, uint32_t n,
                                          const rt_camera* cam, const float light[3], rt_hit* h_primary,
                                          uint8_t* h_vis, rt_hit* h_mirror) {
    return render_frame_host(ctx, l, h_tris, n, cam, light, h_primary, h_vis, h_mirror, true, "rt_render_frame_host");
}

extern "C" rt_status rt_render_frame_host_async(rt_ctx* ctx, rt_lbvh* l, const float* h_tris, uint32_t n,
                                                const rt_camera* cam, const float light[3], rt_hit* h_primary,
                                                uint8_t* h_vis, rt_hit* h_mirror) {
    return render_frame_host(ctx, l, h_tris, n, cam, light, h_primary, h_vis, h_mirror, false,
                             "rt_render_frame_host_async");
}

// ---------------------------------------------------------------------------
// The frame in the reference's own walk order: LBVH_IntersectP
// (LBVH.hlsl:363-440) as the shader runs it, a stackless walk over the heap
// driven by a trail word, one box test per visited node, the child picked by
// dirIsNeg[axis field] first, leaf triangles tested in order and a
// candidate kept only when strictly nearer (an exact tie keeps the first
// one tested, as the shader does).  Primary rays start at the root; the
// shadow ray (a closest-hit walk, as CSComputeColorRT.hlsl:160 issues it)
// and the mirror ray restart at the primary hit's leaf (iRoot).  One lane
// per ray.  Its per-ray counts are the shader's iVisitedNodes (visited nodes,
// triangle tests), the figures the trace's algorithmic bytes are defined by.
namespace {

template <bool EXACT>
__device__ __forceinline__ Hit shader_walk(const RayState& r, bool active, const TreeRef& tr, uint32_t node,
                                           uint32_t* visits_out, uint32_t* ntri_out, uint32_t* leaf_out) {
    Hit best;
    best.id = -1;
    best.u = -1.0f;
    best.v = -1.0f;
    best.t = r.tmax;
    uint32_t root = 1, visits = 0, ntri = 0;
    if (node < 1u) node = 1u;
    uint32_t trail = 1u << (31 - __clz(node));
    const uint32_t limit = 2u * tr.num_nodes + 64u;  // a tree walk visits each node once at most
    while (active) {
        if (node >= tr.num_nodes || visits >= limit) {
            atomicOr(tr.err, RT_DEVERR_BOUNDS);
            break;
        }
        const NodeBox nb = load_node(tr.nodes, node);
        const int p = __ffs(trail + 1u) - 1;
        ++visits;
        float t0;
        // IntersectBox, entered unless T0 > closest t or T1 < 0
        if (!box_enter<EXACT>(r, nb.a.x, nb.a.y, nb.a.z, nb.a.w, nb.b.x, nb.b.y, best.t, &t0)) {
            trail = (trail >> p) + 1u;
            node = (node >> p) ^ 1u;
        } else if (__float_as_int(nb.b.z) & 4) {
            const int cnt = __float_as_int(nb.b.z) >> 3, pos = __float_as_int(nb.b.w);
            if (pos < 0 || cnt < 0 || (uint32_t)pos + (uint32_t)cnt > tr.n) {
                atomicOr(tr.err, RT_DEVERR_BOUNDS);
                break;
            }
            for (int i = 0; i < cnt; ++i) {
                const float4* tp = tr.tris + 3 * (size_t)(pos + i);
                const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                ++ntri;
                const int id = __float_as_int(a.w);
                float u, v, t;
                if (id != r.exclude && tri_test(r, a, b, c, &u, &v, &t) && t < best.t) {
                    best.id = id;
                    best.u = u;
                    best.v = v;
                    best.t = t;
                    root = node;
                }
            }
            trail = (trail >> p) + 1u;
            node = (node >> p) ^ 1u;
        } else {
            const int field = __float_as_int(nb.b.z) & 3;
            const float ia = field == 0 ? r.inv.x : (field == 1 ? r.inv.y : r.inv.z);
            trail <<= 1;
            node = (node << 1) | (ia < 0.0f ? 1u : 0u);
        }
        if (trail <= 1u) break;
    }
    if (visits_out) *visits_out = visits;
    if (ntri_out) *ntri_out = ntri;
    if (leaf_out) *leaf_out = root;
    return best;
}

__device__ __forceinline__ Hit shader_trace(const RayState& r, bool active, const TreeRef& tr, uint32_t node,
                                            uint32_t* visits, uint32_t* ntri, uint32_t* leaf) {
    if (__any_sync(0xffffffffu, active && r.exact)) return shader_walk<true>(r, active, tr, node, visits, ntri, leaf);
    return shader_walk<false>(r, active, tr, node, visits, ntri, leaf);
}

__global__ void __launch_bounds__(kTraceThreads) k_shader_primary(TreeRef tr, rt_camera cam, rt_hit* __restrict__ hits,
                                                                  uint32_t* __restrict__ leaves,
                                                                  uint32_t* __restrict__ stats, uint32_t* work,
                                                                  uint32_t num_tiles) {
    for (uint32_t tile = next_tile(work); tile < num_tiles; tile = next_tile(work)) {
        uint32_t i, j;
        const bool valid = tile_pixel(tile, threadIdx.x & 31, cam.width, cam.height, &i, &j);
        if (!valid) i = j = 0;
        const RayState r = make_ray(mk3(cam.eye[0], cam.eye[1], cam.eye[2]), primary_dir(cam, i, j), 1e16f, -1);
        uint32_t nv = 0, nt = 0, leaf = 1;
        const Hit h = shader_trace(r, valid, tr, 1u, &nv, &nt, &leaf);
        if (valid) {
            const size_t p = (size_t)j * cam.width + i;
            store_hit(hits + p, h);
            leaves[p] = leaf;
            if (stats) {
                stats[2 * p] = nv;
                stats[2 * p + 1] = nt;
            }
        }
    }
}

__global__ void __launch_bounds__(kTraceThreads) k_shader_shade(TreeRef tr, const float* __restrict__ soup,
                                                                rt_camera cam, float lx, float ly, float lz,
                                                                const rt_hit* __restrict__ prim,
                                                                const uint32_t* __restrict__ leaves,
                                                                uint8_t* __restrict__ vis, rt_hit* __restrict__ mirror,
                                                                uint32_t* __restrict__ sstats,
                                                                uint32_t* __restrict__ mstats, uint32_t* work,
                                                                uint32_t num_tiles) {
    for (uint32_t tile = next_tile(work); tile < num_tiles; tile = next_tile(work)) {
        uint32_t i, j;
        const bool valid = tile_pixel(tile, threadIdx.x & 31, cam.width, cam.height, &i, &j);
        if (!valid) i = j = 0;
        const size_t p = (size_t)j * cam.width + i;
        int4 ph = make_int4(-1, 0, 0, 0);
        if (valid) ph = __ldg(reinterpret_cast<const int4*>(prim + p));
        const ShadeRays s = shade_rays(soup, cam, lx, ly, lz, ph, valid, i, j, mirror != nullptr);
        const uint32_t start = (valid && s.has) ? __ldg(leaves + p) : 1u;
        uint32_t snv = 0, snt = 0, mnv = 0, mnt = 0;
        if (vis) {  // uniform across the grid
            const Hit sh = shader_trace(s.shadow, valid && s.cast, tr, start, &snv, &snt, nullptr);
            if (valid) vis[p] = vis_code(s.has, s.cast, sh.id >= 0);
        }
        if (mirror) {
            Hit mh = shader_trace(s.mirror, valid && s.has, tr, start, &mnv, &mnt, nullptr);
            if (!s.has) {
                mh.id = -2; mh.u = -1.0f; mh.v = -1.0f; mh.t = 0.0f;
            }
            if (valid) store_hit(mirror + p, mh);
        }
        if (valid) {
            if (sstats) { sstats[2 * p] = snv; sstats[2 * p + 1] = snt; }
            if (mstats) { mstats[2 * p] = mnv; mstats[2 * p + 1] = mnt; }
        }
    }
}

}  // namespace

extern "C" rt_status rt_trace_frame_shader_order(rt_ctx* ctx, const rt_lbvh* l, const rt_camera* cam,
                                                 const float light[3], rt_hit* d_primary, uint8_t* d_vis,
                                                 rt_hit* d_mirror, uint32_t* d_primary_stats,
                                                 uint32_t* d_shadow_stats, uint32_t* d_mirror_stats) {
    rt_status s = check_trace_args(ctx, l, cam, "rt_trace_frame_shader_order");
    if (s != RT_OK) return s;
    if (!light || !d_primary) return rt_fail(ctx, RT_ERR_INVALID, "rt_trace_frame_shader_order: null argument");
    if ((d_vis || d_mirror) && !l->src_tris)
        return rt_fail(ctx, RT_ERR_INVALID, "rt_trace_frame_shader_order: no triangle soup bound");
    const size_t px = (size_t)cam->width * cam->height;
    // the primary leaves live in the third segment of the shading lists
    if ((s = ensure_shade_lists(ctx, const_cast<rt_lbvh*>(l), px)) != RT_OK) return s;
    uint32_t* leaves = l->s_lists + 2 * l->s_pixels;
    TreeRef tr;  // the reference's walk runs over the heap
    tr.compact = false;
    tr.tri_base = 0;
    tr.nodes = l->nodes;
    tr.num_nodes = l->num_nodes;
    tr.tris = l->sorted_tris;
    tr.n = l->n;
    tr.err = ctx->d_err;
    const uint32_t tiles = pixel_tiles(cam);
    if ((s = reset_work(ctx, kWorkPrimary)) != RT_OK) return s;
    k_shader_primary<<<persistent_blocks(ctx, k_shader_primary, kTraceThreads, tiles), kTraceThreads, 0, ctx->stream>>>(
        tr, *cam, d_primary, leaves, d_primary_stats, ctx->d_work + kWorkPrimary, tiles);
    RT_CHECK_LAUNCH(ctx, "k_shader_primary");
    if (d_vis || d_mirror) {
        if ((s = reset_work(ctx, kWorkSecondary)) != RT_OK) return s;
        k_shader_shade<<<persistent_blocks(ctx, k_shader_shade, kTraceThreads, tiles), kTraceThreads, 0,
                         ctx->stream>>>(tr, l->src_tris, *cam, light[0], light[1], light[2], d_primary, leaves, d_vis,
                                        d_mirror, d_shadow_stats, d_mirror_stats, ctx->d_work + kWorkSecondary, tiles);
        RT_CHECK_LAUNCH(ctx, "k_shader_shade");
    }
    return RT_OK;
}

// ---------------------------------------------------------------------------
// Batched trace: primary + shadow rays of every pixel of every scene of an
// rt_batch.  A work item is one 8 x 4 tile of one scene; warps take `grab`
// consecutive items per increment of one work counter, so the scenes with
// the costliest rays never hold the grid back.  The primary pass lists the
// pixels that cast a shadow ray (with the ray and its start node, the
// primary leaf) and the lane-refill kernel traces them, lanes of one warp
// walking different scenes: in the tile pass only one lane in seven had a
// shadow ray to trace.  Without a list the tile pass traces them itself.
namespace {

struct BatchTraceArgs {
    const rt_node* nodes;
    const float4* sorted_tris;
    const float* soup;
    const uint32_t* tri_off;
    const rt_camera* cams;
    const float* lights;
    rt_hit* hits;
    uint8_t* vis;
    uint32_t* err;
    uint32_t S, depth, width, height, tiles_per_scene, grab, order;
};

// The shadow-ray list of a batched trace.  (A separate kernel argument:
// with these fields inside BatchTraceArgs the compiler gives k_batch_trace
// 78 registers instead of 64, and its primary rays run 20 % slower.)
struct BatchListArgs {
    uint32_t* lists;
    uint32_t cap;
    uint32_t* counts;
    float4* rays;
    uint32_t* starts;
};

// LIST: the shadow rays are listed (a.lists set), else traced here (a.vis
// set) or not cast (a.vis null).
template <bool LIST>
__device__ __forceinline__ void batch_trace_body(const BatchTraceArgs& a, const BatchListArgs& la, uint32_t* work) {
    const uint32_t total = a.S * a.tiles_per_scene;
    const uint32_t lane = threadIdx.x & 31;
    const size_t px = (size_t)a.width * a.height;
    for (;;) {
        uint32_t g0 = 0;
        if (lane == 0) g0 = atomicAdd(work, a.grab);
        g0 = __shfl_sync(0xffffffffu, g0, 0);
        if (g0 >= total) break;
        const uint32_t g1 = min(total, g0 + a.grab);
        for (uint32_t g = g0; g < g1; ++g) {
            const uint32_t s = a.order ? g % a.S : g / a.tiles_per_scene;
            const uint32_t tile = a.order ? g / a.S : g % a.tiles_per_scene;
            const uint32_t toff = __ldg(a.tri_off + s);
            TreeRef tr;
            tr.compact = false;
            tr.tri_base = 0;
            tr.nodes = a.nodes + ((size_t)s << a.depth);
            tr.tris = a.sorted_tris + 3 * (size_t)toff;
            tr.num_nodes = 1u << a.depth;
            tr.n = __ldg(a.tri_off + s + 1) - toff;
            tr.err = a.err;
            const rt_camera cam = a.cams[s];
            uint32_t i, j;
            const bool valid = tile_pixel(tile, lane, a.width, a.height, &i, &j);
            if (!valid) i = j = 0;
            const f3 d = primary_dir(cam, i, j);
            const RayState r = make_ray(mk3(cam.eye[0], cam.eye[1], cam.eye[2]), d, 1e16f, -1);
            uint32_t nb = 0, nt = 0, leaf = 1;
            const Hit h = trace_ray<false>(r, valid, tr, false, &nb, &nt, nullptr, nullptr, 1u, &leaf);
            const size_t p = (size_t)j * a.width + i;
            if (valid) store_hit(a.hits + s * px + p, h);
            if (LIST) {  // the shadow ray (restarting at the primary leaf) goes to the list
                const int4 ph = make_int4(h.id, __float_as_int(h.u), __float_as_int(h.v), __float_as_int(h.t));
                const ShadeLists sl{a.soup + 9 * (size_t)toff, __ldg(a.lights + 3 * s), __ldg(a.lights + 3 * s + 1),
                                    __ldg(a.lights + 3 * s + 2), a.vis, nullptr, la.lists, la.cap, la.counts,
                                    la.rays, la.starts};
                shade_setup_pixel(sl, cam, ph, valid, i, j, s * px + p, h.id >= 0 ? leaf : 1u);
            } else if (a.vis) {  // uniform across the grid; the shadow ray restarts at the primary leaf
                const int4 ph = make_int4(h.id, __float_as_int(h.u), __float_as_int(h.v), __float_as_int(h.t));
                secondary_pixel<false>(tr, a.soup + 9 * (size_t)toff, cam, __ldg(a.lights + 3 * s),
                                       __ldg(a.lights + 3 * s + 1), __ldg(a.lights + 3 * s + 2), ph,
                                       a.vis + s * px, nullptr, nullptr, nullptr, valid, i, j, nullptr, nullptr,
                                       nullptr, h.id >= 0 ? leaf : 1u, nullptr);
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_batch_trace(BatchTraceArgs a, uint32_t* work) {
    grid_dep_wait();
    const BatchListArgs none = {nullptr, 0u, nullptr, nullptr, nullptr};
    batch_trace_body<false>(a, none, work);
}

__global__ void __launch_bounds__(256) k_batch_list(BatchTraceArgs a, BatchListArgs la, uint32_t* work) {
    grid_dep_wait();
    batch_trace_body<true>(a, la, work);
}

}  // namespace

extern "C" rt_status rt_batch_set_views(rt_ctx* ctx, rt_batch* b, const rt_camera* h_cams, const float* h_lights) {
    if (!ctx) return RT_ERR_INVALID;
    if (!b || !h_cams || !h_lights) return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_set_views: null argument");
    const uint32_t w = h_cams[0].width, h = h_cams[0].height;
    if (w == 0 || h == 0 || (uint64_t)w * h * b->S > (1ull << 34))
        return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_set_views: bad image size %ux%u", w, h);
    for (uint32_t s = 1; s < b->S; ++s)
        if (h_cams[s].width != w || h_cams[s].height != h)
            return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_set_views: scene %u is %ux%u, scene 0 is %ux%u", s,
                           h_cams[s].width, h_cams[s].height, w, h);
    RT_CHECK_CUDA(ctx, cudaMemcpyAsync(b->cams, h_cams, sizeof(rt_camera) * b->S, cudaMemcpyHostToDevice, ctx->stream));
    RT_CHECK_CUDA(ctx, cudaMemcpyAsync(b->lights, h_lights, sizeof(float) * 3 * b->S, cudaMemcpyHostToDevice,
                                       ctx->stream));
    // the shadow-ray list: one entry per pixel of the batch at most
    const uint64_t cap = (uint64_t)w * h * b->S;
    if (cap > b->s_cap && cap <= (1ull << 31)) {
        if (b->graph_refs > 0)
            return rt_fail(ctx, RT_ERR_CAPACITY,
                           "rt_batch_set_views: the shadow-ray list cannot grow while a captured frame uses it");
        RT_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (b->s_lists) cudaFree(b->s_lists);
        if (b->s_rays) cudaFree(b->s_rays);
        b->s_lists = nullptr;
        b->s_rays = nullptr;
        b->s_cap = 0;
        RT_CHECK_CUDA(ctx, cudaMalloc((void**)&b->s_lists, 2 * sizeof(uint32_t) * cap));
        RT_CHECK_CUDA(ctx, cudaMalloc((void**)&b->s_rays, 2 * sizeof(float4) * cap));
        b->s_cap = (uint32_t)cap;
    }
    b->width = w;
    b->height = h;
    return RT_OK;
}

extern "C" rt_status rt_batch_set_tuning(rt_ctx* ctx, rt_batch* b, const rt_batch_tuning* t) {
    if (!ctx) return RT_ERR_INVALID;
    if (!b || !t) return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_set_tuning: null argument");
    if (t->threads != 64 && t->threads != 128 && t->threads != 256)
        return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_set_tuning: threads must be 64, 128 or 256");
    if (t->grab < 1 || t->grab > 16) return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_set_tuning: grab must be in [1, 16]");
    if (t->order > 1) return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_set_tuning: order must be 0 or 1");
    if (t->blocks_per_sm > 64) return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_set_tuning: blocks_per_sm above 64");
    b->tuning = *t;
    return RT_OK;
}

extern "C" rt_status rt_batch_get_tuning(const rt_batch* b, rt_batch_tuning* t) {
    if (!b || !t) return RT_ERR_INVALID;
    *t = b->tuning;
    return RT_OK;
}

extern "C" rt_status rt_batch_trace(rt_ctx* ctx, const rt_batch* b, rt_hit* d_hits, uint8_t* d_vis) {
    if (!ctx) return RT_ERR_INVALID;
    if (!b || !d_hits) return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_trace: null argument");
    if (!b->built) return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_trace: the batch has not been built");
    if (b->width == 0) return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_trace: no views set (rt_batch_set_views)");
    const uint64_t cap = (uint64_t)b->width * b->height * b->S;
    const bool listed = d_vis && b->s_cap >= cap && cap > 0;
    uint32_t* counts = ctx->d_work + kShadeCounts;
    uint64_t reset = word_bit(ctx, ctx->d_work + kWorkBatch);
    if (listed)
        reset |= word_bit(ctx, ctx->d_work + kWorkShade) | word_bit(ctx, counts) | word_bit(ctx, counts + 1);
    rt_status s = reset_words(ctx, reset);
    if (s != RT_OK) return s;
    BatchTraceArgs a;
    a.nodes = b->nodes;
    a.sorted_tris = b->sorted_tris;
    a.soup = b->src_tris;
    a.tri_off = b->tri_off;
    a.cams = b->cams;
    a.lights = b->lights;
    a.hits = d_hits;
    a.vis = d_vis;
    a.err = ctx->d_err;
    a.S = b->S;
    a.depth = b->depth;
    a.width = b->width;
    a.height = b->height;
    a.tiles_per_scene = ((b->width + 7) / 8) * ((b->height + 3) / 4);
    a.grab = b->tuning.grab;
    a.order = b->tuning.order;
    const BatchListArgs la = {b->s_lists, (uint32_t)cap, counts, b->s_rays, b->s_lists + cap};
    const int threads = (int)b->tuning.threads;
    int per_sm = 0;
    const cudaError_t oe = listed ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_list, threads, 0)
                                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_trace, threads, 0);
    if (oe != cudaSuccess || per_sm < 1) per_sm = 1;
    if (b->tuning.blocks_per_sm) per_sm = std::min(per_sm, (int)b->tuning.blocks_per_sm);
    const uint64_t items = (uint64_t)a.S * a.tiles_per_scene;
    const uint64_t need = (items * 32 + threads - 1) / threads;
    const uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)per_sm * ctx->num_sms, need));
    if (listed)
        launch_pdl(k_batch_list, blocks, threads, 0, ctx->stream, a, la, ctx->d_work + kWorkBatch);
    else
        launch_pdl(k_batch_trace, blocks, threads, 0, ctx->stream, a, ctx->d_work + kWorkBatch);
    RT_CHECK_LAUNCH(ctx, "k_batch_trace");
    if (!listed) return RT_OK;
    TreeRef tr;  // the batch's whole sorted-triangle array; nodes, tri_base and n set per lane
    tr.compact = false;
    tr.tri_base = 0;
    tr.nodes = b->nodes;
    tr.tris = b->sorted_tris;
    tr.num_nodes = 1u << b->depth;
    tr.n = 0;
    tr.err = ctx->d_err;
    Spill none;
    memset(&none, 0, sizeof(none));
    int shade_per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&shade_per_sm, k_trace_shade<true>, kTraceThreads, 0) !=
            cudaSuccess ||
        shade_per_sm < 1)
        shade_per_sm = 1;
    rt_camera cam0;
    memset(&cam0, 0, sizeof(cam0));
    launch_pdl(k_trace_shade<true>, (uint32_t)shade_per_sm * ctx->num_sms, kTraceThreads, 0, ctx->stream, tr,
               (const float*)nullptr, cam0, 0.0f, 0.0f, 0.0f, (const rt_hit*)nullptr, (const uint32_t*)nullptr, d_vis,
               (rt_hit*)nullptr, (uint32_t*)nullptr, (const uint32_t*)b->s_lists, (uint32_t)cap,
               (const uint32_t*)counts, (const float4*)b->s_rays, (const uint32_t*)(b->s_lists + cap),
               ctx->d_work + kWorkShade, none, (uint32_t*)nullptr,
               BatchTrees{b->nodes, b->tri_off, b->depth, b->width * b->height});
    RT_CHECK_LAUNCH(ctx, "k_trace_shade");
    return RT_OK;
}
