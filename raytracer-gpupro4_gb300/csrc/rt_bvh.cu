// rt_bvh.cu -- the reference's SAH BVH as a second structure on the GPU.
//
// The reference builds a PBRT-style SAH BVH on the CPU
// (AccelerationStructures/BVH/bvh.cpp) and uploads its depth-first
// LinearBVHNode array and ordered primitive ids for the shader BVH_IntersectP
// (RayTracerCS/Shaders/AccelerationStructures/BVH.hlsl:124-217,
// RayTracerCS.cpp:590-624).  rt_bvh_import_host uploads such a tree after a
// host-side structural check, gathers the triangles into leaf order (3 x
// float4, the id in the first w), and the kernels walk it as the shader does:
// the box of each visited node is tested (IntersectBox, pruned when T1 < 0 or
// T0 > closest t), a leaf's triangles are tested, an interior node enters the
// child on the ray's negative side of its split axis and stacks the other.
// One lane per ray, persistent warps over 32-ray tiles; the SAH tree's
// one-primitive leaves leave no long leaf loops to share across the warp.
#include <algorithm>
#include <cstring>
#include <vector>

#include "rt_traverse.cuh"

using namespace rt;

struct rt_bvh {
    uint32_t max_nodes = 0, max_tris = 0;
    uint32_t num_nodes = 0, n = 0;
    rt_node* nodes = nullptr;
    uint32_t* ids = nullptr;
    float4* sorted_tris = nullptr;  // leaf order, 3 x float4 per entry
    float* tris = nullptr;          // the soup by triangle id
};

namespace {

constexpr int kBvhThreads = 128;
constexpr int kBvhStack = 64;  // the reference's CPU walk uses 64 (bvh.cpp:303)

// Work-counter slots (ctx->d_work) of the BVH kernels.
enum : int { kWorkBvhPrimary = 15, kWorkBvhRays = 15, kWorkBvhShade = 15 };

struct BvhRef {
    const rt_node* __restrict__ nodes;
    const float4* __restrict__ tris;
    uint32_t num_nodes, n;
    uint32_t* err;
};

template <bool EXACT>
__device__ __forceinline__ Hit bvh_walk(const RayState& r, bool active, const BvhRef& b, bool any_hit,
                                        uint32_t* nbox_out, uint32_t* ntri_out) {
    uint64_t best = hit_key(r.tmax, 0);
    float bt = r.tmax, bu = -1.0f, bv = -1.0f;
    int bid = -1;
    uint32_t nbox = 0, ntri = 0;
    uint32_t stack[kBvhStack];
    int sp = 0;
    uint32_t node = 0;
    bool live = active && r.tmax > 0.0f && b.num_nodes > 0;  // no t satisfies 0 <= t < tmax otherwise
    while (live) {
        if (nbox >= b.num_nodes) {  // a tree walk visits each node once at most
            atomicOr(b.err, RT_DEVERR_BOUNDS);
            break;
        }
        const NodeBox nb = load_node(b.nodes, node);
        ++nbox;
        float t0;
        bool next = false;
        if (box_enter<EXACT>(r, nb.a.x, nb.a.y, nb.a.z, nb.a.w, nb.b.x, nb.b.y, bt, &t0)) {
            const int pc = __float_as_int(nb.b.z);
            const uint32_t pos = (uint32_t)__float_as_int(nb.b.w);
            if (pc > 0) {
                if ((uint64_t)pos + (uint64_t)pc > b.n) {
                    atomicOr(b.err, RT_DEVERR_BOUNDS);
                    break;
                }
                for (int i = 0; i < pc; ++i) {
                    const float4* tp = b.tris + 3 * (size_t)(pos + (uint32_t)i);
                    const float4 ta = __ldg(tp), tb = __ldg(tp + 1), tc = __ldg(tp + 2);
                    ++ntri;
                    const int id = __float_as_int(ta.w);
                    float u, v, t;
                    if (id != r.exclude && tri_test(r, ta, tb, tc, &u, &v, &t)) {
                        const uint64_t k = hit_key(t, id);
                        if (k < best) {
                            best = k;
                            bt = t;
                            bu = u;
                            bv = v;
                            bid = id;
                        }
                    }
                }
                if (any_hit && bid >= 0) break;
            } else {
                const int axis = -pc;
                const float ia = axis == 0 ? r.inv.x : (axis == 1 ? r.inv.y : r.inv.z);
                const bool neg = ia < 0.0f;  // dirIsNeg of BVH.hlsl:199-201
                const uint32_t first = node + 1, second = pos;
                if (axis > 2 || first >= b.num_nodes || second >= b.num_nodes || sp >= kBvhStack) {
                    atomicOr(b.err, RT_DEVERR_BOUNDS);
                    break;
                }
                stack[sp++] = neg ? first : second;
                node = neg ? second : first;
                next = true;
            }
        }
        if (!next) {
            if (sp == 0) break;
            node = stack[--sp];
        }
    }
    if (nbox_out) *nbox_out = nbox;
    if (ntri_out) *ntri_out = ntri;
    Hit h;
    h.id = bid;
    h.u = bu;
    h.v = bv;
    h.t = bt;
    return h;
}

__device__ __forceinline__ Hit bvh_trace(const RayState& r, bool active, const BvhRef& b, bool any_hit,
                                         uint32_t* nbox, uint32_t* ntri) {
    if (__any_sync(0xffffffffu, active && r.exact)) return bvh_walk<true>(r, active, b, any_hit, nbox, ntri);
    return bvh_walk<false>(r, active, b, any_hit, nbox, ntri);
}

__device__ __forceinline__ void put_hit(rt_hit* out, const Hit& h) {
    *reinterpret_cast<int4*>(out) = make_int4(h.id, __float_as_int(h.u), __float_as_int(h.v), __float_as_int(h.t));
}

template <bool STATS>
__global__ void __launch_bounds__(kBvhThreads) k_bvh_primary(BvhRef b, rt_camera cam, rt_hit* __restrict__ hits,
                                                             uint32_t* __restrict__ stats, uint32_t* work,
                                                             uint32_t num_tiles) {
    for (uint32_t tile = next_tile(work); tile < num_tiles; tile = next_tile(work)) {
        uint32_t i, j;
        const bool valid = tile_pixel(tile, threadIdx.x & 31, cam.width, cam.height, &i, &j);
        if (!valid) i = j = 0;
        const RayState r = make_ray(mk3(cam.eye[0], cam.eye[1], cam.eye[2]), primary_dir(cam, i, j), 1e16f, -1);
        uint32_t nb = 0, nt = 0;
        const Hit h = bvh_trace(r, valid, b, false, &nb, &nt);
        if (valid) {
            const size_t p = (size_t)j * cam.width + i;
            put_hit(hits + p, h);
            if (STATS) {
                stats[2 * p] = nb;
                stats[2 * p + 1] = nt;
            }
        }
    }
}

template <bool STATS>
__global__ void __launch_bounds__(kBvhThreads) k_bvh_shade(BvhRef b, const float* __restrict__ soup, rt_camera cam,
                                                           float lx, float ly, float lz,
                                                           const rt_hit* __restrict__ prim, uint8_t* __restrict__ vis,
                                                           rt_hit* __restrict__ mirror, uint32_t* __restrict__ sstats,
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
        uint32_t snb = 0, snt = 0, mnb = 0, mnt = 0;
        if (vis) {  // uniform across the grid
            const Hit sh = bvh_trace(s.shadow, valid && s.cast, b, true, &snb, &snt);
            if (valid) vis[p] = vis_code(s.has, s.cast, sh.id >= 0);
        }
        if (mirror) {
            Hit mh = bvh_trace(s.mirror, valid && s.has, b, false, &mnb, &mnt);
            if (!s.has) {
                mh.id = -2; mh.u = -1.0f; mh.v = -1.0f; mh.t = 0.0f;
            }
            if (valid) put_hit(mirror + p, mh);
        }
        if (STATS && valid) {
            if (sstats) { sstats[2 * p] = snb; sstats[2 * p + 1] = snt; }
            if (mstats) { mstats[2 * p] = mnb; mstats[2 * p + 1] = mnt; }
        }
    }
}

template <bool STATS>
__global__ void __launch_bounds__(kBvhThreads) k_bvh_rays(BvhRef b, const rt_ray* __restrict__ rays, uint32_t n,
                                                          int any_hit, rt_hit* __restrict__ hits,
                                                          uint32_t* __restrict__ stats, uint32_t* work) {
    const uint32_t num_tiles = (n + 31) / 32;
    for (uint32_t tile = next_tile(work); tile < num_tiles; tile = next_tile(work)) {
        const uint32_t k = tile * 32 + (threadIdx.x & 31);
        const bool valid = k < n;
        float4 a = make_float4(0.f, 0.f, 0.f, __int_as_float(-1)), c = make_float4(0.f, 0.f, 1.f, 1.f);
        if (valid) {
            a = __ldg(reinterpret_cast<const float4*>(rays + k));
            c = __ldg(reinterpret_cast<const float4*>(rays + k) + 1);
        }
        const RayState r = make_ray(mk3(a.x, a.y, a.z), mk3(c.x, c.y, c.z), c.w, __float_as_int(a.w));
        uint32_t nb = 0, nt = 0;
        const Hit h = bvh_trace(r, valid, b, any_hit != 0, &nb, &nt);
        if (valid) {
            put_hit(hits + k, h);
            if (STATS) {
                stats[2 * k] = nb;
                stats[2 * k + 1] = nt;
            }
        }
    }
}

// Leaf-order triangles: entry k = the triangle ids[k], its id in the first w.
__global__ void k_bvh_gather(const float* __restrict__ soup, const uint32_t* __restrict__ ids, uint32_t n,
                             float4* __restrict__ out) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t id = __ldg(ids + k);
        const float* t = soup + 9 * (size_t)id;
        out[3 * (size_t)k] = make_float4(t[0], t[1], t[2], __int_as_float((int)id));
        out[3 * (size_t)k + 1] = make_float4(t[3], t[4], t[5], 0.f);
        out[3 * (size_t)k + 2] = make_float4(t[6], t[7], t[8], 0.f);
    }
}

BvhRef bvh_ref(const rt_ctx* ctx, const rt_bvh* b) {
    BvhRef r;
    r.nodes = b->nodes;
    r.tris = b->sorted_tris;
    r.num_nodes = b->num_nodes;
    r.n = b->n;
    r.err = ctx->d_err;
    return r;
}

uint32_t bvh_tiles(const rt_camera* cam) {
    return (uint32_t)(((cam->width + 7) / 8) * ((cam->height + 3) / 4));
}

rt_status check_bvh(rt_ctx* ctx, const rt_bvh* b, const char* who) {
    if (!ctx) return RT_ERR_INVALID;
    if (!b) return rt_fail(ctx, RT_ERR_INVALID, "%s: null BVH", who);
    if (b->num_nodes == 0) return rt_fail(ctx, RT_ERR_INVALID, "%s: no tree imported", who);
    return RT_OK;
}

rt_status check_cam(rt_ctx* ctx, const rt_camera* cam, const char* who) {
    if (!cam) return rt_fail(ctx, RT_ERR_INVALID, "%s: null camera", who);
    if (cam->width == 0 || cam->height == 0 || (uint64_t)cam->width * cam->height > (1ull << 31))
        return rt_fail(ctx, RT_ERR_INVALID, "%s: bad image size", who);
    return RT_OK;
}

}  // namespace

extern "C" rt_status rt_bvh_create(rt_ctx* ctx, uint32_t max_nodes, uint32_t max_tris, rt_bvh** out) {
    if (!ctx) return RT_ERR_INVALID;
    if (!out || max_nodes == 0 || max_tris == 0) return rt_fail(ctx, RT_ERR_INVALID, "rt_bvh_create: bad argument");
    if (max_tris > kMaxTris || max_nodes > 2 * kMaxTris)
        return rt_fail(ctx, RT_ERR_CAPACITY, "rt_bvh_create: too large");
    rt_bvh* b = new rt_bvh();
    b->max_nodes = max_nodes;
    b->max_tris = max_tris;
    cudaError_t e = cudaMalloc((void**)&b->nodes, sizeof(rt_node) * max_nodes);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->ids, sizeof(uint32_t) * max_tris);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->sorted_tris, 3 * sizeof(float4) * max_tris);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->tris, 9 * sizeof(float) * max_tris);
    if (e != cudaSuccess) {
        rt_bvh_destroy(b);
        return rt_fail(ctx, RT_ERR_CUDA, "rt_bvh_create: allocation failed: %s", cudaGetErrorString(e));
    }
    *out = b;
    return RT_OK;
}

extern "C" rt_status rt_bvh_destroy(rt_bvh* b) {
    if (!b) return RT_OK;
    void* ptrs[] = {b->nodes, b->ids, b->sorted_tris, b->tris};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete b;
    return RT_OK;
}

extern "C" rt_status rt_bvh_import_host(rt_ctx* ctx, rt_bvh* b, const rt_node* h_nodes, uint32_t num_nodes,
                                        const uint32_t* h_ids, const float* h_tris, uint32_t n) {
    if (!ctx) return RT_ERR_INVALID;
    if (!b || !h_nodes || !h_ids || !h_tris || num_nodes == 0 || n == 0)
        return rt_fail(ctx, RT_ERR_INVALID, "rt_bvh_import_host: bad argument");
    if (num_nodes > b->max_nodes || n > b->max_tris)
        return rt_fail(ctx, RT_ERR_CAPACITY, "rt_bvh_import_host: %u nodes / %u triangles exceed the capacity",
                       num_nodes, n);
    // structural check: indices inside the arrays, children after their
    // parent, and every node but the root the child of exactly one node, so
    // a walk visits each node at most once
    for (uint32_t i = 0; i < n; ++i)
        if (h_ids[i] >= n) return rt_fail(ctx, RT_ERR_INVALID, "rt_bvh_import_host: id %u out of range", h_ids[i]);
    std::vector<uint8_t> parents(num_nodes, 0);
    for (uint32_t i = 0; i < num_nodes; ++i) {
        const int pc = h_nodes[i].prim_count;
        const uint32_t pos = (uint32_t)h_nodes[i].prim_pos;
        if (pc > 0) {
            if ((uint64_t)pos + (uint64_t)pc > n)
                return rt_fail(ctx, RT_ERR_INVALID, "rt_bvh_import_host: leaf %u range out of bounds", i);
        } else {
            if (pc < -2 || i + 1 >= num_nodes || pos <= i + 1 || pos >= num_nodes || parents[i + 1] || parents[pos])
                return rt_fail(ctx, RT_ERR_INVALID, "rt_bvh_import_host: interior node %u is malformed", i);
            parents[i + 1] = parents[pos] = 1;
        }
    }
    for (uint32_t i = 1; i < num_nodes; ++i)
        if (!parents[i]) return rt_fail(ctx, RT_ERR_INVALID, "rt_bvh_import_host: node %u has no parent", i);
    cudaStream_t st = ctx->stream;
    RT_CHECK_CUDA(ctx, cudaMemcpyAsync(b->nodes, h_nodes, sizeof(rt_node) * num_nodes, cudaMemcpyHostToDevice, st));
    RT_CHECK_CUDA(ctx, cudaMemcpyAsync(b->ids, h_ids, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st));
    RT_CHECK_CUDA(ctx, cudaMemcpyAsync(b->tris, h_tris, 9 * sizeof(float) * n, cudaMemcpyHostToDevice, st));
    k_bvh_gather<<<std::max(1u, std::min((n + 255) / 256, (uint32_t)ctx->num_sms * 8)), 256, 0, st>>>(
        b->tris, b->ids, n, b->sorted_tris);
    RT_CHECK_LAUNCH(ctx, "k_bvh_gather");
    // the host buffers may be reused as soon as the call returns
    RT_CHECK_CUDA(ctx, cudaStreamSynchronize(st));
    b->num_nodes = num_nodes;
    b->n = n;
    return RT_OK;
}

extern "C" rt_status rt_bvh_trace_primary(rt_ctx* ctx, const rt_bvh* b, const rt_camera* cam, rt_hit* d_hits,
                                          uint32_t* d_stats) {
    rt_status s = check_bvh(ctx, b, "rt_bvh_trace_primary");
    if (s != RT_OK || (s = check_cam(ctx, cam, "rt_bvh_trace_primary")) != RT_OK) return s;
    if (!d_hits) return rt_fail(ctx, RT_ERR_INVALID, "rt_bvh_trace_primary: null output");
    if ((s = reset_work(ctx, kWorkBvhPrimary)) != RT_OK) return s;
    const uint32_t tiles = bvh_tiles(cam);
    uint32_t* work = ctx->d_work + kWorkBvhPrimary;
    if (d_stats) {
        auto k = k_bvh_primary<true>;
        k<<<persistent_blocks(ctx, k, kBvhThreads, tiles), kBvhThreads, 0, ctx->stream>>>(bvh_ref(ctx, b), *cam, d_hits,
                                                                                           d_stats, work, tiles);
    } else {
        auto k = k_bvh_primary<false>;
        k<<<persistent_blocks(ctx, k, kBvhThreads, tiles), kBvhThreads, 0, ctx->stream>>>(bvh_ref(ctx, b), *cam, d_hits,
                                                                                           nullptr, work, tiles);
    }
    RT_CHECK_LAUNCH(ctx, "k_bvh_primary");
    return RT_OK;
}

extern "C" rt_status rt_bvh_trace_shadow_mirror(rt_ctx* ctx, const rt_bvh* b, const rt_camera* cam,
                                                const float light[3], const rt_hit* d_primary, uint8_t* d_vis,
                                                rt_hit* d_mirror, uint32_t* d_shadow_stats, uint32_t* d_mirror_stats) {
    rt_status s = check_bvh(ctx, b, "rt_bvh_trace_shadow_mirror");
    if (s != RT_OK || (s = check_cam(ctx, cam, "rt_bvh_trace_shadow_mirror")) != RT_OK) return s;
    if (!light || !d_primary) return rt_fail(ctx, RT_ERR_INVALID, "rt_bvh_trace_shadow_mirror: null argument");
    if ((s = reset_work(ctx, kWorkBvhShade)) != RT_OK) return s;
    const uint32_t tiles = bvh_tiles(cam);
    uint32_t* work = ctx->d_work + kWorkBvhShade;
    if (d_shadow_stats || d_mirror_stats) {
        auto k = k_bvh_shade<true>;
        k<<<persistent_blocks(ctx, k, kBvhThreads, tiles), kBvhThreads, 0, ctx->stream>>>(
            bvh_ref(ctx, b), b->tris, *cam, light[0], light[1], light[2], d_primary, d_vis, d_mirror, d_shadow_stats,
            d_mirror_stats, work, tiles);
    } else {
        auto k = k_bvh_shade<false>;
        k<<<persistent_blocks(ctx, k, kBvhThreads, tiles), kBvhThreads, 0, ctx->stream>>>(
            bvh_ref(ctx, b), b->tris, *cam, light[0], light[1], light[2], d_primary, d_vis, d_mirror, nullptr,
            nullptr, work, tiles);
    }
    RT_CHECK_LAUNCH(ctx, "k_bvh_shade");
    return RT_OK;
}

extern "C" rt_status rt_bvh_trace_rays(rt_ctx* ctx, const rt_bvh* b, const rt_ray* d_rays, uint32_t n, int any_hit,
                                       rt_hit* d_hits, uint32_t* d_stats) {
    rt_status s = check_bvh(ctx, b, "rt_bvh_trace_rays");
    if (s != RT_OK) return s;
    if (!d_rays || !d_hits) return rt_fail(ctx, RT_ERR_INVALID, "rt_bvh_trace_rays: null argument");
    if (n == 0) return RT_OK;
    if ((s = reset_work(ctx, kWorkBvhRays)) != RT_OK) return s;
    const uint32_t tiles = (n + 31) / 32;
    uint32_t* work = ctx->d_work + kWorkBvhRays;
    if (d_stats) {
        auto k = k_bvh_rays<true>;
        k<<<persistent_blocks(ctx, k, kBvhThreads, tiles), kBvhThreads, 0, ctx->stream>>>(bvh_ref(ctx, b), d_rays, n,
                                                                                           any_hit, d_hits, d_stats,
                                                                                           work);
    } else {
        auto k = k_bvh_rays<false>;
        k<<<persistent_blocks(ctx, k, kBvhThreads, tiles), kBvhThreads, 0, ctx->stream>>>(bvh_ref(ctx, b), d_rays, n,
                                                                                           any_hit, d_hits, nullptr,
                                                                                           work);
    }
    RT_CHECK_LAUNCH(ctx, "k_bvh_rays");
    return RT_OK;
}
