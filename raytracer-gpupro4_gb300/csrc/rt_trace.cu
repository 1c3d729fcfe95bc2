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

#include "rt_traverse.cuh"

using namespace rt;

namespace {

constexpr int kTraceThreads = 128;

__device__ __forceinline__ void store_hit(rt_hit* out, const Hit& h) {
    *reinterpret_cast<int4*>(out) = make_int4(h.id, __float_as_int(h.u), __float_as_int(h.v), __float_as_int(h.t));
}

template <bool STATS>
__global__ void __launch_bounds__(kTraceThreads) k_trace_primary(TreeRef tr, rt_camera cam,
                                                                 rt_hit* __restrict__ hits,
                                                                 uint32_t* __restrict__ stats, uint32_t* work,
                                                                 uint32_t num_tiles) {
    for (uint32_t tile = next_tile(work); tile < num_tiles; tile = next_tile(work)) {
        uint32_t i, j;
        const bool valid = tile_pixel(tile, threadIdx.x & 31, cam.width, cam.height, &i, &j);
        if (!valid) i = j = 0;  // lanes past the image edge only help the warp
        const f3 d = primary_dir(cam, i, j);
        const RayState r = make_ray(mk3(cam.eye[0], cam.eye[1], cam.eye[2]), d, 1e16f, -1);
        uint32_t nb = 0, nt = 0;
        const Hit h = trace_ray<STATS>(r, valid, tr, false, &nb, &nt);
        if (valid) {
            const size_t p = (size_t)j * cam.width + i;
            store_hit(hits + p, h);
            if (STATS) {
                stats[2 * p] = nb;
                stats[2 * p + 1] = nt;
            }
        }
    }
}

// Shadow (any hit) and mirror (closest hit) rays of one pixel.  Called by
// all lanes of the warp together (valid == false for lanes past the image
// edge); rays of pixels whose primary ray missed, or whose light is behind
// the surface, are traced with active == false.
template <bool STATS>
__device__ __forceinline__ void secondary_pixel(const TreeRef& tr, const float* __restrict__ soup,
                                                const rt_camera& cam, float lx, float ly, float lz,
                                                const rt_hit* __restrict__ prim, uint8_t* __restrict__ vis,
                                                rt_hit* __restrict__ mirror, uint32_t* __restrict__ sstats,
                                                uint32_t* __restrict__ mstats, bool valid, uint32_t i, uint32_t j) {
    const size_t p = (size_t)j * cam.width + i;
    int4 ph = make_int4(-1, 0, 0, 0);
    if (valid) ph = __ldg(reinterpret_cast<const int4*>(prim + p));
    const int id = ph.x;
    const bool has = valid && id >= 0;
    uint32_t snb = 0, snt = 0, mnb = 0, mnt = 0;
    f3 N = mk3(0.f, 0.f, 1.f), Nf = N, P = mk3(0.f, 0.f, 0.f), L = mk3(0.f, 0.f, 1.f), d = mk3(0.f, 0.f, 1.f);
    float dist = 1.0f;
    bool cast = false;
    if (has) {
        const float t = __int_as_float(ph.w);
        d = primary_dir(cam, i, j);
        const f3 o = mk3(cam.eye[0], cam.eye[1], cam.eye[2]);
        const float* tp = soup + 9 * (size_t)id;
        const f3 A = mk3(__ldg(tp), __ldg(tp + 1), __ldg(tp + 2));
        const f3 B = mk3(__ldg(tp + 3), __ldg(tp + 4), __ldg(tp + 5));
        const f3 C = mk3(__ldg(tp + 6), __ldg(tp + 7), __ldg(tp + 8));
        N = normalize3(cross3(sub3(B, A), sub3(C, A)));            // CSComputeColorRT.hlsl:61-63,75
        Nf = N;
        if (dot3(Nf, d) > 0.0f) Nf = mk3(-N.x, -N.y, -N.z);        // :126-131
        P = mk3(fadd(o.x, fmul(t, d.x)), fadd(o.y, fmul(t, d.y)), fadd(o.z, fmul(t, d.z)));  // :134-135
        L = mk3(fsub(P.x, lx), fsub(P.y, ly), fsub(P.z, lz));      // :136
        dist = fsqrt(dot3(L, L));                                  // :137
        L = mk3(fdiv(L.x, dist), fdiv(L.y, dist), fdiv(L.z, dist)); // :138
        const float ls = dot3(N, L), rs = dot3(N, d);              // :145-146
        cast = fmul(ls, rs) > 0.0f;                                // :147
    }
    if (vis) {  // uniform across the warp
        const RayState sr = make_ray(P, mk3(-L.x, -L.y, -L.z), dist, id);  // :149-153
        const Hit sh = trace_ray<STATS>(sr, cast, tr, true, &snb, &snt);
        if (valid) vis[p] = !has ? 0 : (!cast ? 1 : (sh.id >= 0 ? 2 : 3));
    }
    if (mirror) {
        f3 R = mk3(0.f, 0.f, 1.f);
        if (has) {
            const float k = fmul(2.0f, dot3(d, Nf));               // reflect(d, N) = d - 2*dot(d,N)*N
            R = normalize3(mk3(fsub(d.x, fmul(k, Nf.x)), fsub(d.y, fmul(k, Nf.y)), fsub(d.z, fmul(k, Nf.z))));
        }
        const RayState mr = make_ray(P, R, 1e16f, id);
        Hit mh = trace_ray<STATS>(mr, has, tr, false, &mnb, &mnt);
        if (!has) {
            mh.id = -2; mh.u = -1.0f; mh.v = -1.0f; mh.t = 0.0f;
        }
        if (valid) store_hit(mirror + p, mh);
    }
    if (STATS && valid) {
        if (sstats) { sstats[2 * p] = snb; sstats[2 * p + 1] = snt; }
        if (mstats) { mstats[2 * p] = mnb; mstats[2 * p + 1] = mnt; }
    }
}

template <bool STATS>
__global__ void __launch_bounds__(kTraceThreads) k_trace_secondary(
    TreeRef tr, const float* __restrict__ soup, rt_camera cam, float lx, float ly, float lz,
    const rt_hit* __restrict__ prim, uint8_t* __restrict__ vis, rt_hit* __restrict__ mirror,
    uint32_t* __restrict__ sstats, uint32_t* __restrict__ mstats, uint32_t* work, uint32_t num_tiles) {
    for (uint32_t tile = next_tile(work); tile < num_tiles; tile = next_tile(work)) {
        uint32_t i, j;
        const bool valid = tile_pixel(tile, threadIdx.x & 31, cam.width, cam.height, &i, &j);
        if (!valid) i = j = 0;
        secondary_pixel<STATS>(tr, soup, cam, lx, ly, lz, prim, vis, mirror, sstats, mstats, valid, i, j);
    }
}

template <bool STATS>
__global__ void __launch_bounds__(kTraceThreads) k_trace_rays(TreeRef tr, const rt_ray* __restrict__ rays, uint32_t n,
                                                              int any_hit, rt_hit* __restrict__ hits,
                                                              uint32_t* __restrict__ stats, uint32_t* work) {
    const uint32_t num_tiles = (n + 31) / 32;
    for (uint32_t tile = next_tile(work); tile < num_tiles; tile = next_tile(work)) {
        const uint32_t k = tile * 32 + (threadIdx.x & 31);
        const bool valid = k < n;
        float4 a = make_float4(0.f, 0.f, 0.f, __int_as_float(-1)), b = make_float4(0.f, 0.f, 1.f, 1.f);
        if (valid) {
            a = __ldg(reinterpret_cast<const float4*>(rays + k));
            b = __ldg(reinterpret_cast<const float4*>(rays + k) + 1);
        }
        const RayState r = make_ray(mk3(a.x, a.y, a.z), mk3(b.x, b.y, b.z), b.w, __float_as_int(a.w));
        uint32_t nb = 0, nt = 0;
        const Hit h = trace_ray<STATS>(r, valid, tr, any_hit != 0, &nb, &nt);
        if (valid) {
            store_hit(hits + k, h);
            if (STATS) {
                stats[2 * k] = nb;
                stats[2 * k + 1] = nt;
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

TreeRef tree_ref(const rt_ctx* ctx, const rt_lbvh* l) {
    TreeRef t;
    t.nodes = l->nodes;
    t.tris = l->sorted_tris;
    t.num_nodes = l->num_nodes;
    t.n = l->n;
    t.err = ctx->d_err;
    return t;
}

extern "C" rt_status rt_trace_primary(rt_ctx* ctx, const rt_lbvh* l, const rt_camera* cam, rt_hit* d_hits,
                                      uint32_t* d_stats) {
    rt_status s = check_trace_args(ctx, l, cam, "rt_trace_primary");
    if (s != RT_OK) return s;
    if (!d_hits) return rt_fail(ctx, RT_ERR_INVALID, "rt_trace_primary: null output");
    if ((s = reset_work(ctx, kWorkPrimary)) != RT_OK) return s;
    const uint32_t tiles = pixel_tiles(cam);
    uint32_t* work = ctx->d_work + kWorkPrimary;
    if (d_stats) {
        auto k = k_trace_primary<true>;
        k<<<persistent_blocks(ctx, k, kTraceThreads, tiles), kTraceThreads, 0, ctx->stream>>>(
            tree_ref(ctx, l), *cam, d_hits, d_stats, work, tiles);
    } else {
        auto k = k_trace_primary<false>;
        k<<<persistent_blocks(ctx, k, kTraceThreads, tiles), kTraceThreads, 0, ctx->stream>>>(
            tree_ref(ctx, l), *cam, d_hits, nullptr, work, tiles);
    }
    RT_CHECK_LAUNCH(ctx, "k_trace_primary");
    return RT_OK;
}

extern "C" rt_status rt_trace_shadow_mirror(rt_ctx* ctx, const rt_lbvh* l, const rt_camera* cam, const float light[3],
                                            const rt_hit* d_primary, uint8_t* d_vis, rt_hit* d_mirror,
                                            uint32_t* d_shadow_stats, uint32_t* d_mirror_stats) {
    rt_status s = check_trace_args(ctx, l, cam, "rt_trace_shadow_mirror");
    if (s != RT_OK) return s;
    if (!light || !d_primary) return rt_fail(ctx, RT_ERR_INVALID, "rt_trace_shadow_mirror: null argument");
    if (!l->src_tris) return rt_fail(ctx, RT_ERR_INVALID, "rt_trace_shadow_mirror: no triangle soup bound");
    if ((s = reset_work(ctx, kWorkSecondary)) != RT_OK) return s;
    const uint32_t tiles = pixel_tiles(cam);
    uint32_t* work = ctx->d_work + kWorkSecondary;
    if (d_shadow_stats || d_mirror_stats) {
        auto k = k_trace_secondary<true>;
        k<<<persistent_blocks(ctx, k, kTraceThreads, tiles), kTraceThreads, 0, ctx->stream>>>(
            tree_ref(ctx, l), l->src_tris, *cam, light[0], light[1], light[2], d_primary, d_vis, d_mirror,
            d_shadow_stats, d_mirror_stats, work, tiles);
    } else {
        auto k = k_trace_secondary<false>;
        k<<<persistent_blocks(ctx, k, kTraceThreads, tiles), kTraceThreads, 0, ctx->stream>>>(
            tree_ref(ctx, l), l->src_tris, *cam, light[0], light[1], light[2], d_primary, d_vis, d_mirror, nullptr,
            nullptr, work, tiles);
    }
    RT_CHECK_LAUNCH(ctx, "k_trace_secondary");
    return RT_OK;
}

extern "C" rt_status rt_trace_rays(rt_ctx* ctx, const rt_lbvh* l, const rt_ray* d_rays, uint32_t n, int any_hit,
                                   rt_hit* d_hits, uint32_t* d_stats) {
    if (!ctx) return RT_ERR_INVALID;
    if (!l || !d_rays || !d_hits) return rt_fail(ctx, RT_ERR_INVALID, "rt_trace_rays: null argument");
    if (l->n == 0) return rt_fail(ctx, RT_ERR_INVALID, "rt_trace_rays: the LBVH has not been built");
    if (n == 0) return RT_OK;
    rt_status s = reset_work(ctx, kWorkRays);
    if (s != RT_OK) return s;
    const uint32_t tiles = (n + 31) / 32;
    uint32_t* work = ctx->d_work + kWorkRays;
    if (d_stats) {
        auto k = k_trace_rays<true>;
        k<<<persistent_blocks(ctx, k, kTraceThreads, tiles), kTraceThreads, 0, ctx->stream>>>(
            tree_ref(ctx, l), d_rays, n, any_hit, d_hits, d_stats, work);
    } else {
        auto k = k_trace_rays<false>;
        k<<<persistent_blocks(ctx, k, kTraceThreads, tiles), kTraceThreads, 0, ctx->stream>>>(
            tree_ref(ctx, l), d_rays, n, any_hit, d_hits, nullptr, work);
    }
    RT_CHECK_LAUNCH(ctx, "k_trace_rays");
    return RT_OK;
}

extern "C" rt_status rt_render_frame_host(rt_ctx* ctx, rt_lbvh* l, const float* h_tris, uint32_t n,
                                          const rt_camera* cam, const float light[3], rt_hit* h_primary,
                                          uint8_t* h_vis, rt_hit* h_mirror) {
    if (!ctx) return RT_ERR_INVALID;
    if (!l || !h_tris || !cam || !light) return rt_fail(ctx, RT_ERR_INVALID, "rt_render_frame_host: null argument");
    const size_t px = (size_t)cam->width * cam->height;
    if (px == 0 || px > (1ull << 31)) return rt_fail(ctx, RT_ERR_INVALID, "rt_render_frame_host: bad image size");
    if (px > l->f_pixels) {  // frame buffers grow on the first call at a new size
        RT_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (l->f_primary) cudaFree(l->f_primary);
        if (l->f_mirror) cudaFree(l->f_mirror);
        if (l->f_vis) cudaFree(l->f_vis);
        l->f_primary = nullptr; l->f_mirror = nullptr; l->f_vis = nullptr; l->f_pixels = 0;
        RT_CHECK_CUDA(ctx, cudaMalloc((void**)&l->f_primary, sizeof(rt_hit) * px));
        RT_CHECK_CUDA(ctx, cudaMalloc((void**)&l->f_mirror, sizeof(rt_hit) * px));
        RT_CHECK_CUDA(ctx, cudaMalloc((void**)&l->f_vis, px));
        l->f_pixels = px;
    }
    rt_status s = rt_lbvh_build_host(ctx, l, h_tris, n, 0);
    if (s != RT_OK) return s;
    s = rt_trace_primary(ctx, l, cam, l->f_primary, nullptr);
    if (s != RT_OK) return s;
    s = rt_trace_shadow_mirror(ctx, l, cam, light, l->f_primary, h_vis ? l->f_vis : nullptr,
                               h_mirror ? l->f_mirror : nullptr, nullptr, nullptr);
    if (s != RT_OK) return s;
    cudaStream_t st = ctx->stream;
    if (h_primary) RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_primary, l->f_primary, sizeof(rt_hit) * px, cudaMemcpyDeviceToHost, st));
    if (h_vis) RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_vis, l->f_vis, px, cudaMemcpyDeviceToHost, st));
    if (h_mirror) RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_mirror, l->f_mirror, sizeof(rt_hit) * px, cudaMemcpyDeviceToHost, st));
    RT_CHECK_CUDA(ctx, cudaStreamSynchronize(st));
    return RT_OK;
}
