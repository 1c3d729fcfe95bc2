// rt_whitted.cu -- the ray-tracing colour stage with its bounce loop.
//
// RayTracerCS::Render without global illumination (RayTracerCS.cpp:284-295)
// runs CSGeneratePrimaryRays (CSPrimaryRays.hlsl:22-69), then bounces + 1
// times the intersection stage (CSIntersections.hlsl:18-39, LBVH_IntersectP
// restarted at the pixel's previous leaf) and the colour stage
// (CSComputeColorRT.hlsl:18-262).  Here one bounce is four passes over a
// list of the pixels whose rays are still alive, so rays that ended (a miss
// that took the environment colour) cost nothing in later bounces:
//
//   k_wh_trace<false>  closest hit of each live ray (persistent warps,
//                      32 rays per warp, walks restarted at the last leaf)
//   k_wh_setup         the shading geometry of each hit; pixels that cast a
//                      shadow ray are appended to the shadow list
//   k_wh_trace<true>   the shadow rays (first hit), restarted at the hit's leaf
//   k_wh_finish        colour, accumulation and result; the next ray (mirror
//                      or refracted) and the next bounce's list
//
// Without textures or normal maps; the environment cube map is a colour, and
// the random texture that chooses between the mirror and the refracted ray
// (:204-207) is a hash of (seed, pixel, bounce).  Every floating-point step
// is an IEEE operation in the reference's order (no contraction), normalize
// divides by the length and pow(x, 49) is x^32 x^16 x, so the oracle's
// restatement (or_render_whitted) gives the same bits.
#include <algorithm>

#include "rt_traverse.cuh"

using namespace rt;

namespace {

constexpr int kWhThreads = 128;
constexpr int kWhListThreads = 256;

// Work counters and list lengths (ctx->d_work slots).
enum : int { kWorkWhTrace = 10, kWorkWhShadow = 11, kWhCounts = 12 /* 3 words: list 0, list 1, shadow list */ };

// ray status (rf.w as int bits)
enum : int { kRayAlive = 0, kRayEnded = 1 };

struct WhBufs {
    float4* ro;       // origin.xyz, excluded triangle (int bits)
    float4* rd;       // direction.xyz, tmax
    float4* rf;       // reflective factor.xyz, status
    int4* hit;        // closest hit {id, u, v, t}
    uint32_t* leaf;   // the hit's leaf (iRoot)
    uint32_t* occl;   // shadow ray blocked
    uint32_t* list[3];
    uint32_t* counts; // 3 words
    uint32_t px;
};

struct ShadeArgs {
    const float* soup;       // by triangle id, 9 floats
    const float* normals;    // by triangle id, 9 floats (nullable)
    const int32_t* mat_ids;  // by triangle id (nullable)
    const rt_material* mats;
    uint32_t nmat;
    uint32_t n;
    float lx, ly, lz;
    int shadows, phong, gloss, env_flag;
    float env[3];
    uint32_t seed;
    uint32_t* err;
};

// List i of w (selects, so the kernel parameter is not copied to local memory).
__device__ __forceinline__ uint32_t* wlist(const WhBufs& w, int i) {
    return i == 0 ? w.list[0] : (i == 1 ? w.list[1] : w.list[2]);
}

__device__ __forceinline__ uint32_t lowbias32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// Uniform number in [0, 1) of the mirror / refraction choice.
__device__ __forceinline__ float wh_rand(uint32_t seed, uint32_t pixel, uint32_t bounce) {
    const uint32_t h = lowbias32(pixel ^ lowbias32(seed ^ (0x9e3779b9u * (bounce + 1u))));
    return fmul((float)(h >> 8), 1.0f / 16777216.0f);
}

__device__ __forceinline__ float pow49(float x) {
    const float x2 = fmul(x, x), x4 = fmul(x2, x2), x8 = fmul(x4, x4), x16 = fmul(x8, x8), x32 = fmul(x16, x16);
    return fmul(fmul(x32, x16), x);
}

__device__ __forceinline__ f3 ld3(const float* p) { return mk3(__ldg(p), __ldg(p + 1), __ldg(p + 2)); }

// Shading geometry of a hit (CSComputeColorRT.hlsl:57-147).
struct Geom {
    f3 N;      // vfNormal (flat or Phong), not flipped
    f3 NM;     // facing the ray
    f3 P;      // hit point
    f3 L;      // unit direction light -> hit point
    f3 R;      // normalize(reflect(d, NM))
    float dist;
    bool inverse;
    bool cast;  // light and ray on the same side of the surface
};

__device__ __forceinline__ Geom geom(const ShadeArgs& a, int id, float u, float v, float t, f3 o, f3 d) {
    Geom g;
    const float* tp = a.soup + 9 * (size_t)id;
    const f3 A = ld3(tp), B = ld3(tp + 3), C = ld3(tp + 6);
    g.N = normalize3(cross3(sub3(B, A), sub3(C, A)));  // :61-63, :75
    if (a.phong && a.normals) {                         // :68-70, Vec3BaryCentric
        const float* np = a.normals + 9 * (size_t)id;
        const f3 nA = ld3(np), nB = ld3(np + 3), nC = ld3(np + 6);
        const float w = fsub(1.0f, fadd(u, v));
        g.N = normalize3(mk3(fadd(fadd(fmul(nA.x, w), fmul(nB.x, u)), fmul(nC.x, v)),
                             fadd(fadd(fmul(nA.y, w), fmul(nB.y, u)), fmul(nC.y, v)),
                             fadd(fadd(fmul(nA.z, w), fmul(nB.z, u)), fmul(nC.z, v))));
    }
    g.NM = g.N;
    g.inverse = false;
    if (dot3(g.NM, d) > 0.0f) {  // :126-131
        g.NM = mk3(-g.N.x, -g.N.y, -g.N.z);
        g.inverse = true;
    }
    g.P = mk3(fadd(o.x, fmul(t, d.x)), fadd(o.y, fmul(t, d.y)), fadd(o.z, fmul(t, d.z)));  // :134-135
    f3 L = mk3(fsub(g.P.x, a.lx), fsub(g.P.y, a.ly), fsub(g.P.z, a.lz));                // :136
    g.dist = fsqrt(dot3(L, L));
    g.L = mk3(fdiv(L.x, g.dist), fdiv(L.y, g.dist), fdiv(L.z, g.dist));  // :137-138
    const float k = fmul(2.0f, dot3(d, g.NM));                            // :141-142
    g.R = normalize3(mk3(fsub(d.x, fmul(k, g.NM.x)), fsub(d.y, fmul(k, g.NM.y)), fsub(d.z, fmul(k, g.NM.z))));
    g.cast = fmul(dot3(g.N, g.L), dot3(g.N, d)) > 0.0f;  // :145-147
    return g;
}

__device__ __forceinline__ void append(bool take, uint32_t p, uint32_t* list, uint32_t cap, uint32_t* count) {
    const uint32_t m = __ballot_sync(0xffffffffu, take);
    if (!m) return;
    uint32_t base = 0;
    if ((threadIdx.x & 31) == 0) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    const uint32_t k = base + __popc(m & ((1u << (threadIdx.x & 31)) - 1u));
    if (take && k < cap) list[k] = p;
}

// Primary rays (CSPrimaryRays.hlsl:36-63) and the first list: every pixel
// in 8 x 4 tile order; accumulation and result cleared.
__global__ void __launch_bounds__(kWhListThreads) k_wh_init(rt_camera cam, WhBufs w, float4* __restrict__ accum,
                                                            float4* __restrict__ result, uint32_t num_tiles) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t t = warp; t < num_tiles; t += nwarps) {
        uint32_t i, j;
        const bool valid = tile_pixel(t, lane, cam.width, cam.height, &i, &j);
        const uint32_t p = j * cam.width + i;
        if (valid) {
            const f3 d = primary_dir(cam, i, j);
            w.ro[p] = make_float4(cam.eye[0], cam.eye[1], cam.eye[2], __int_as_float(-1));
            w.rd[p] = make_float4(d.x, d.y, d.z, 1e16f);
            w.rf[p] = make_float4(1.0f, 1.0f, 1.0f, __int_as_float(kRayAlive));
            w.leaf[p] = 1u;
            accum[p] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (result) result[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        append(valid, p, w.list[0], w.px, w.counts);
    }
}

// Closest hits of the listed rays (SHADOW = false) or the shadow rays of the
// listed hits (SHADOW = true).  Persistent warps, 32 list entries per step.
template <bool SHADOW>
__global__ void __launch_bounds__(kWhThreads) k_wh_trace(TreeRef tr, ShadeArgs a, WhBufs w, int src, uint32_t* work) {
    const uint32_t* list = wlist(w, src);
    const uint32_t n = min(w.counts[src], w.px);
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t c = next_tile(work); c * 32 < n; c = next_tile(work)) {
        const uint32_t k = c * 32 + lane;
        const bool valid = k < n;
        const uint32_t p = valid ? __ldg(list + k) : 0u;
        const float4 ro = valid ? w.ro[p] : make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
        const float4 rd = valid ? w.rd[p] : make_float4(0.f, 0.f, 1.f, 1.f);
        const uint32_t start = valid ? w.leaf[p] : 1u;
        uint32_t nb = 0, nt = 0;
        if (!SHADOW) {
            uint32_t leaf = 1;
            const RayState r = make_ray(mk3(ro.x, ro.y, ro.z), mk3(rd.x, rd.y, rd.z), rd.w, __float_as_int(ro.w));
            const Hit h = trace_ray<false>(r, valid, tr, false, &nb, &nt, nullptr, nullptr, start, &leaf);
            if (valid) {
                w.hit[p] = make_int4(h.id, __float_as_int(h.u), __float_as_int(h.v), __float_as_int(h.t));
                w.leaf[p] = leaf;
            }
        } else {
            RayState sr = make_ray(mk3(0.f, 0.f, 0.f), mk3(0.f, 0.f, 1.f), 1.0f, -1);
            int id = -1;
            if (valid) {
                const int4 h = w.hit[p];
                id = h.x;
                if (id >= 0 && (uint32_t)id < a.n) {
                    const Geom g = geom(a, id, __int_as_float(h.y), __int_as_float(h.z), __int_as_float(h.w),
                                        mk3(ro.x, ro.y, ro.z), mk3(rd.x, rd.y, rd.z));
                    // :149-153: from the hit point towards the light, up to the light
                    sr = make_ray(g.P, mk3(-g.L.x, -g.L.y, -g.L.z), g.dist, id);
                } else {
                    id = -1;
                }
            }
            const Hit h = trace_ray<false>(sr, valid && id >= 0, tr, true, &nb, &nt, nullptr, nullptr, start);
            if (valid) w.occl[p] = h.id >= 0 ? 1u : 0u;
        }
    }
}

// Pixels of the live list whose hit casts a shadow ray join the shadow list.
__global__ void __launch_bounds__(kWhListThreads) k_wh_setup(ShadeArgs a, WhBufs w, int src) {
    const uint32_t n = min(w.counts[src], w.px);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {  // uniform per warp
        const uint32_t k = base + threadIdx.x;
        bool take = false;
        uint32_t p = 0;
        if (k < n && a.shadows) {
            p = __ldg(wlist(w, src) + k);
            const int4 h = w.hit[p];
            if (h.x >= 0 && (uint32_t)h.x < a.n) {
                const float4 ro = w.ro[p], rd = w.rd[p];
                const Geom g = geom(a, h.x, __int_as_float(h.y), __int_as_float(h.z), __int_as_float(h.w),
                                    mk3(ro.x, ro.y, ro.z), mk3(rd.x, rd.y, rd.z));
                take = g.cast;
            }
        }
        append(take, p, w.list[2], w.px, w.counts + 2);
    }
}

// Colour of the live pixels (:29-256), the next ray and the next list.
__global__ void __launch_bounds__(kWhListThreads) k_wh_finish(ShadeArgs a, WhBufs w, int src, uint32_t bounce,
                                                              bool last, float4* __restrict__ accum,
                                                              float4* __restrict__ result) {
    const uint32_t n = min(w.counts[src], w.px);
    const int dst = src ^ 1;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {  // uniform per warp
        const uint32_t k = base + threadIdx.x;
        bool next = false;
        uint32_t p = 0;
        if (k < n) {
            p = __ldg(wlist(w, src) + k);
            const int4 h = w.hit[p];
            int id = h.x;
            if (id >= 0 && (uint32_t)id >= a.n) {
                atomicOr(a.err, RT_DEVERR_BOUNDS);
                id = -1;
            }
            if (id < a.env_flag) {  // :29-35: the same miss at every later bounce
                if (id > -2 && result) result[p] = make_float4(1.f, 1.f, 1.f, 1.f);
                w.rf[p].w = __int_as_float(kRayEnded);
            } else {
                float4 ro = w.ro[p], rd = w.rd[p], rf = w.rf[p];
                float fin[4] = {0.f, 0.f, 0.f, 1.f};
                if (id < 0) {  // :233-245: environment colour, the ray ends
                    fin[0] = fmul(rf.x, a.env[0]);
                    fin[1] = fmul(rf.y, a.env[1]);
                    fin[2] = fmul(rf.z, a.env[2]);
                    rf.w = __int_as_float(kRayEnded);
                } else {
                    const f3 o = mk3(ro.x, ro.y, ro.z), d = mk3(rd.x, rd.y, rd.z);
                    const Geom g = geom(a, id, __int_as_float(h.y), __int_as_float(h.z), __int_as_float(h.w), o, d);
                    float spec = 0.f, diff = 0.f, spec_w = 1.f, diff_w = 1.f;
                    if (g.cast && !(a.shadows && w.occl[p])) {  // :155-176
                        spec = pow49(fmaxf(0.0f, -dot3(g.L, g.R)));
                        diff = fmaxf(0.0f, -dot3(g.NM, g.L));
                        spec_w = spec;
                        diff_w = diff;
                    }
                    uint32_t m = a.mat_ids ? (uint32_t)__ldg(a.mat_ids + id) : 0u;
                    if (m >= a.nmat) {
                        atomicOr(a.err, RT_DEVERR_BOUNDS);
                        m = 0;
                    }
                    const float* mp = reinterpret_cast<const float*>(a.mats + m);
                    float amb[4], kd[4], ks[4];
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        amb[c] = __ldg(mp + c);
                        kd[c] = __ldg(mp + 4 + c);
                        ks[c] = __ldg(mp + 8 + c);
                    }
                    const float alpha = __ldg(mp + 13);
                    ks[3] = fmul(ks[3], (float)a.gloss);  // :194
                    const float dv[4] = {diff, diff, diff, diff_w}, sv[4] = {spec, spec, spec, spec_w};
#pragma unroll
                    for (int c = 0; c < 4; ++c) {  // :197-199
                        const float dc = fmul(fadd(amb[c], fmul(dv[c], kd[3])), kd[c]);
                        const float sc = fmul(fmul(sv[c], fsub(1.0f, kd[3])), ks[c]);
                        fin[c] = fadd(dc, sc);
                    }
                    fin[0] = fmul(fin[0], rf.x);  // :200
                    fin[1] = fmul(fin[1], rf.y);
                    fin[2] = fmul(fin[2], rf.z);
                    // :203-231: the next ray
                    f3 nd = g.R;
                    if (alpha >= wh_rand(a.seed, p, bounce)) {
                        rf.x = fmul(rf.x, ks[0]);
                        rf.y = fmul(rf.y, ks[1]);
                        rf.z = fmul(rf.z, ks[2]);
                    } else {
                        float eta = amb[3];
                        if (!g.inverse) eta = fdiv(1.0f, eta);
                        const float ci = dot3(g.NM, d);  // refract(d, NM, eta)
                        const float kk = fsub(1.0f, fmul(fmul(eta, eta), fsub(1.0f, fmul(ci, ci))));
                        f3 T = mk3(0.f, 0.f, 0.f);
                        if (!(kk < 0.0f)) {
                            const float sq = fadd(fmul(eta, ci), fsqrt(kk));
                            T = mk3(fsub(fmul(eta, d.x), fmul(sq, g.NM.x)), fsub(fmul(eta, d.y), fmul(sq, g.NM.y)),
                                    fsub(fmul(eta, d.z), fmul(sq, g.NM.z)));
                        }
                        const float tl = fsqrt(dot3(T, T));
                        if (!(tl < 0.000001f)) {
                            nd = mk3(fdiv(T.x, tl), fdiv(T.y, tl), fdiv(T.z, tl));
                            rf.x = fmul(rf.x, kd[0]);
                            rf.y = fmul(rf.y, kd[1]);
                            rf.z = fmul(rf.z, kd[2]);
                        }
                    }
                    ro = make_float4(g.P.x, g.P.y, g.P.z, __int_as_float(id));
                    rd = make_float4(nd.x, nd.y, nd.z, rd.w);
                    next = !last;
                }
                float4 acc = accum[p];  // :255-256
                acc.x = fadd(acc.x, fin[0]);
                acc.y = fadd(acc.y, fin[1]);
                acc.z = fadd(acc.z, fin[2]);
                acc.w = fadd(acc.w, fin[3]);
                accum[p] = acc;
                if (result) result[p] = acc;
                w.ro[p] = ro;
                w.rd[p] = rd;
                w.rf[p] = rf;
            }
        }
        append(next, p, wlist(w, dst), w.px, w.counts + dst);
    }
}

rt_status ensure_whitted(rt_ctx* ctx, rt_lbvh* l, size_t px) {
    if (px <= l->w_pixels) return RT_OK;
    RT_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (l->w_buf) cudaFree(l->w_buf);
    l->w_buf = nullptr;
    l->w_pixels = 0;
    // 3 float4 ray words + int4 hit + leaf + shadow flag + 3 lists, per pixel
    RT_CHECK_CUDA(ctx, cudaMalloc(&l->w_buf, px * (4 * 16 + 5 * 4)));
    l->w_pixels = px;
    return RT_OK;
}

WhBufs whitted_bufs(rt_ctx* ctx, const rt_lbvh* l, uint32_t px) {
    WhBufs w;
    char* b = static_cast<char*>(l->w_buf);
    const size_t cap = l->w_pixels;
    w.ro = reinterpret_cast<float4*>(b);
    w.rd = w.ro + cap;
    w.rf = w.rd + cap;
    w.hit = reinterpret_cast<int4*>(w.rf + cap);
    w.leaf = reinterpret_cast<uint32_t*>(w.hit + cap);
    w.occl = w.leaf + cap;
    w.list[0] = w.occl + cap;
    w.list[1] = w.list[0] + cap;
    w.list[2] = w.list[1] + cap;
    w.counts = ctx->d_work + kWhCounts;
    w.px = px;
    return w;
}

}  // namespace

extern "C" rt_status rt_render_whitted(rt_ctx* ctx, const rt_lbvh* l, const rt_camera* cam, const float light[3],
                                       const rt_shade_params* prm, const int32_t* d_material_ids,
                                       const rt_material* d_materials, uint32_t num_materials, const float* d_normals,
                                       float* d_accum, float* d_result) {
    if (!ctx) return RT_ERR_INVALID;
    if (!l || !cam || !light || !prm || !d_materials || !d_accum)
        return rt_fail(ctx, RT_ERR_INVALID, "rt_render_whitted: null argument");
    if (l->n == 0 || !l->src_tris) return rt_fail(ctx, RT_ERR_INVALID, "rt_render_whitted: the LBVH has not been built");
    if (num_materials == 0) return rt_fail(ctx, RT_ERR_INVALID, "rt_render_whitted: no materials");
    if (prm->bounces > 64) return rt_fail(ctx, RT_ERR_INVALID, "rt_render_whitted: at most 64 bounces");
    const size_t px = (size_t)cam->width * cam->height;
    if (px == 0 || px > (1ull << 30)) return rt_fail(ctx, RT_ERR_INVALID, "rt_render_whitted: bad image size");
    rt_lbvh* lm = const_cast<rt_lbvh*>(l);
    rt_status s = ensure_whitted(ctx, lm, px);
    if (s != RT_OK) return s;
    WhBufs w = whitted_bufs(ctx, l, (uint32_t)px);
    ShadeArgs a;
    a.soup = l->src_tris;
    a.normals = d_normals;
    a.mat_ids = d_material_ids;
    a.mats = d_materials;
    a.nmat = num_materials;
    a.n = l->n;
    a.lx = light[0];
    a.ly = light[1];
    a.lz = light[2];
    a.shadows = prm->shadows != 0;
    a.phong = prm->phong != 0;
    a.gloss = prm->gloss_mapping != 0;
    a.env_flag = prm->env_mapping;
    a.env[0] = prm->env_color[0];
    a.env[1] = prm->env_color[1];
    a.env[2] = prm->env_color[2];
    a.seed = prm->seed;
    a.err = ctx->d_err;
    // the walks restart at heap nodes: use the heap even when a compact layout exists
    TreeRef tr;
    tr.compact = false;
    tr.tri_base = 0;
    tr.nodes = l->nodes;
    tr.num_nodes = l->num_nodes;
    tr.tris = l->sorted_tris;
    tr.n = l->n;
    tr.err = ctx->d_err;
    cudaStream_t st = ctx->stream;
    float4* acc = reinterpret_cast<float4*>(d_accum);
    float4* res = reinterpret_cast<float4*>(d_result);
    const uint32_t tiles = (uint32_t)(((cam->width + 7) / 8) * ((cam->height + 3) / 4));
    RT_CHECK_CUDA(ctx, cudaMemsetAsync(w.counts, 0, 3 * sizeof(uint32_t), st));
    const uint32_t lblocks = (uint32_t)std::max(1, ctx->num_sms * 8);
    k_wh_init<<<std::min<uint32_t>(lblocks, (tiles + 7) / 8), kWhListThreads, 0, st>>>(*cam, w, acc, res, tiles);
    RT_CHECK_LAUNCH(ctx, "k_wh_init");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_wh_trace<false>, kWhThreads, 0) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    const uint32_t tblocks = (uint32_t)per_sm * ctx->num_sms;
    for (uint32_t b = 0; b <= prm->bounces; ++b) {
        const int src = (int)(b & 1u);
        // the next bounce's list and the shadow list start empty
        RT_CHECK_CUDA(ctx, cudaMemsetAsync(w.counts + (src ^ 1), 0, sizeof(uint32_t), st));
        RT_CHECK_CUDA(ctx, cudaMemsetAsync(w.counts + 2, 0, sizeof(uint32_t), st));
        if ((s = reset_work(ctx, kWorkWhTrace)) != RT_OK) return s;
        k_wh_trace<false><<<tblocks, kWhThreads, 0, st>>>(tr, a, w, src, ctx->d_work + kWorkWhTrace);
        RT_CHECK_LAUNCH(ctx, "k_wh_trace");
        if (a.shadows) {
            k_wh_setup<<<lblocks, kWhListThreads, 0, st>>>(a, w, src);
            RT_CHECK_LAUNCH(ctx, "k_wh_setup");
            if ((s = reset_work(ctx, kWorkWhShadow)) != RT_OK) return s;
            k_wh_trace<true><<<tblocks, kWhThreads, 0, st>>>(tr, a, w, 2, ctx->d_work + kWorkWhShadow);
            RT_CHECK_LAUNCH(ctx, "k_wh_trace_shadow");
        }
        k_wh_finish<<<lblocks, kWhListThreads, 0, st>>>(a, w, src, b, b == prm->bounces, acc, res);
        RT_CHECK_LAUNCH(ctx, "k_wh_finish");
    }
    return RT_OK;
}
