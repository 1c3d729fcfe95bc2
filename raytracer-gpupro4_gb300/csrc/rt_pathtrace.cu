// rt_pathtrace.cu -- path-traced GI and its adjoint on sm_103a.
//
// Forward: the GI branch of the reference (CSPrimaryRays.hlsl:23-34,63 and
// CSComputeColorGI.hlsl:19-238 with the progressive factors of
// cbGlobalIllumination, ConstantBuffers.h:85-110), one lane per pixel with
// its path state in registers (path regeneration, below) instead of a
// 48-byte ray / 24-byte hit round trip through global memory per segment.
// Per segment: closest hit, the walk started at the previous hit's leaf
// (CSIntersections.hlsl:32); on a hit acc += (1/(n+1) * beta) * Le,
// beta *= albedo, new direction
// cosine-distributed about the facing geometric normal; on a miss
// acc += (1/(n+1) * beta) * sky.  Sampling uses one PCG32 stream per
// (pixel, sample) and Malley's method, so every operation is an IEEE
// +,-,*,/ or sqrt and the image matches the CPU rendering bit for bit.
//
// Adjoint: the same paths are replayed (nothing is stored between the
// passes); for a path with throughputs beta_s, albedos a_s and radiances E_s,
// dC/da_j = beta_j * G_j with G_j = E_{j+1} + a_{j+1} * G_{j+1}.
#include "rt_traverse.cuh"

using namespace rt;

namespace {

constexpr int kPtThreads = 128;
constexpr int kMaxSeg = 16;

struct Pcg32 {
    uint64_t state, inc;
    __device__ __forceinline__ uint32_t next() {
        const uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((0u - rot) & 31u));
    }
    __device__ __forceinline__ void seed(uint64_t initstate, uint64_t initseq) {
        state = 0u;
        inc = (initseq << 1u) | 1u;
        next();
        state += initstate;
        next();
    }
    __device__ __forceinline__ float uniform() { return fmul((float)(next() >> 8), 1.0f / 16777216.0f); }
};

__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__device__ __forceinline__ void pt_seed(Pcg32& g, uint64_t seed, uint64_t pixel, uint32_t sample) {
    const uint64_t s = splitmix64(seed + 0x9E3779B97F4A7C15ULL * (pixel * 65536ULL + sample + 1ULL));
    g.seed(s, pixel);
}

// Malley's method + the orthonormal basis of Duff et al. (JCGT 2017).
__device__ __forceinline__ f3 cosine_dir(Pcg32& g, f3 n) {
    float x = 0.0f, y = 0.0f, r2 = 0.0f;
    for (int k = 0; k < 64; ++k) {
        x = fsub(fmul(2.0f, g.uniform()), 1.0f);
        y = fsub(fmul(2.0f, g.uniform()), 1.0f);
        r2 = fadd(fmul(x, x), fmul(y, y));
        if (r2 <= 1.0f) break;
        x = 0.0f; y = 0.0f; r2 = 0.0f;
    }
    const float z = fsqrt(fsub(1.0f, r2));
    const float sign = copysignf(1.0f, n.z);
    const float a = fdiv(-1.0f, fadd(sign, n.z));
    const float b = fmul(fmul(n.x, n.y), a);
    const f3 T = mk3(fadd(1.0f, fmul(fmul(fmul(sign, n.x), n.x), a)), fmul(sign, b), fmul(-sign, n.x));
    const f3 B = mk3(b, fadd(sign, fmul(fmul(n.y, n.y), a)), -n.y);
    return mk3(fadd(fadd(fmul(T.x, x), fmul(B.x, y)), fmul(n.x, z)),
               fadd(fadd(fmul(T.y, x), fmul(B.y, y)), fmul(n.y, z)),
               fadd(fadd(fmul(T.z, x), fmul(B.z, y)), fmul(n.z, z)));
}

__device__ __forceinline__ f3 facing_normal(const float* __restrict__ soup, int id, f3 d) {
    const float* tp = soup + 9 * (size_t)id;
    const f3 A = mk3(__ldg(tp), __ldg(tp + 1), __ldg(tp + 2));
    const f3 B = mk3(__ldg(tp + 3), __ldg(tp + 4), __ldg(tp + 5));
    const f3 C = mk3(__ldg(tp + 6), __ldg(tp + 7), __ldg(tp + 8));
    f3 N = normalize3(cross3(sub3(B, A), sub3(C, A)));
    if (dot3(N, d) > 0.0f) N = mk3(-N.x, -N.y, -N.z);
    return N;
}

struct PathParams {
    rt_camera cam;
    uint32_t spp, bounces;
    uint64_t seed;
    float sky[3];
    uint32_t n0;  // first sample index (samples 0 .. n0-1 are already in the image)
};

// Walk counts of the counting variant (rt_pathtrace_counted), per lane.
struct PathCounts {
    uint32_t segments = 0, boxes = 0, tris = 0, hits = 0;
};

// Path regeneration.  A warp's lanes each hold one pixel and trace its
// samples one segment at a time; every segment of every lane is one
// warp-wide traversal (trace_ray), whatever bounce each lane is at.  A lane
// whose sample ends begins the pixel's next sample, and a lane whose pixel
// is done takes the next pixel from the work counter as soon as
// kPtRefillLanes lanes of its warp are idle (the last pixels of the image
// leave lanes idle).  The pixels are handed out in 8 x 4 tiles, lanes of
// one grab taking consecutive pixels.  A pixel's samples stay on one lane
// and in order, so its progressive mean is the same sequence of fp32
// operations as a sample-by-sample loop.
constexpr int kPtRefillLanes = 16;

struct PathLane {
    bool live = false;           // holds a pixel
    uint32_t i = 0, j = 0;       // the pixel
    uint32_t n = 0;              // the sample being traced
    uint32_t s = 0;              // its segment
    Pcg32 g;
    f3 o, d;
    int exclude = -1;
    uint32_t start = 1u;         // restart node of the segment's walk
    float fact = 0.0f;           // 1 / (n + 1)
    float beta[3];
};

// Sample n of the lane's pixel: its stream and camera ray (the GI branch of
// CSPrimaryRays.hlsl:23-34 with a sub-pixel jitter).
__device__ __forceinline__ void begin_sample(PathLane& L, const PathParams& P) {
    pt_seed(L.g, P.seed, (uint64_t)L.j * P.cam.width + L.i, L.n);
    const float inv = fdiv(1.0f, (float)P.cam.height);
    const float jx = fsub(fmul(2.0f, L.g.uniform()), 1.0f);
    const float jy = fsub(fmul(2.0f, L.g.uniform()), 1.0f);
    const float x = fmul(fadd((float)(2 * (int)L.i + 1 - (int)P.cam.width), jx), inv);
    const float y = -fmul(fadd((float)(2 * (int)L.j + 1 - (int)P.cam.height), jy), inv);
    L.d = camera_dir(P.cam, x, y);
    L.o = mk3(P.cam.eye[0], P.cam.eye[1], P.cam.eye[2]);
    L.exclude = -1;
    L.start = 1u;
    L.s = 0;
    L.beta[0] = L.beta[1] = L.beta[2] = 1.0f;
}

// Next ray of a path that hit triangle `id` at t (not its last segment):
// origin at the hit, a cosine-distributed direction about the facing
// normal, the walk restarted at the hit's leaf.
__device__ __forceinline__ void bounce(PathLane& L, const float* __restrict__ soup, int id, float t, uint32_t leaf) {
    const f3 N = facing_normal(soup, id, L.d);
    L.o = mk3(fadd(L.o.x, fmul(t, L.d.x)), fadd(L.o.y, fmul(t, L.d.y)), fadd(L.o.z, fmul(t, L.d.z)));
    L.d = cosine_dir(L.g, N);
    L.exclude = id;
    L.start = leaf;
    ++L.s;
}

// Warp-aggregated grab of pixels for the idle lanes (all lanes call).
// Returns true for a lane that took a pixel inside the image.
__device__ __forceinline__ bool grab_pixel(PathLane& L, const PathParams& P, uint32_t* work, uint32_t total,
                                           bool& drained) {
    constexpr uint32_t kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t idle = __ballot_sync(kFull, !L.live);
    if (drained || !(idle == kFull || __popc(idle) >= kPtRefillLanes)) return false;
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(work, (uint32_t)__popc(idle));
    base = __shfl_sync(kFull, base, 0);
    if (base + (uint32_t)__popc(idle) >= total) drained = true;
    const uint32_t k = base + __popc(idle & ((1u << lane) - 1u));
    if (L.live || k >= total) return false;
    uint32_t i, j;
    if (!tile_pixel(k >> 5, k & 31u, P.cam.width, P.cam.height, &i, &j)) return false;
    L.i = i;
    L.j = j;
    L.n = P.n0;
    L.live = true;
    return true;
}

// At most 72 registers (seven blocks per SM).  Per segment: closest hit; on
// a hit acc += (1/(n+1) * beta) * Le, beta *= albedo; on a miss
// acc += (1/(n+1) * beta) * sky.  STATS: the counting variant, which also
// sums the walk counts into counts[4] (64-bit).
template <bool STATS>
__global__ void __launch_bounds__(kPtThreads, 7) k_pathtrace(TreeRef tr, const float* __restrict__ soup,
                                                          const float* __restrict__ albedo,
                                                          const float* __restrict__ emission, PathParams P,
                                                          float4* __restrict__ image, uint32_t* work,
                                                          uint32_t num_tiles, unsigned long long* counts) {
    constexpr uint32_t kFull = 0xffffffffu;
    const uint32_t total = num_tiles * 32u;
    PathCounts cnt;
    PathLane L;
    L.o = mk3(0.f, 0.f, 0.f);
    L.d = mk3(0.f, 0.f, 1.f);
    float acc[3] = {0.0f, 0.0f, 0.0f};
    bool drained = false;
    for (;;) {
        if (grab_pixel(L, P, work, total, drained)) {
            acc[0] = acc[1] = acc[2] = 0.0f;
            if (P.n0 > 0) {  // continue the progressive mean the image holds
                const float4 prev = image[(size_t)L.j * P.cam.width + L.i];
                acc[0] = prev.x;
                acc[1] = prev.y;
                acc[2] = prev.z;
            }
            const float fant = fdiv((float)L.n, (float)(L.n + 1));
            L.fact = fdiv(1.0f, (float)(L.n + 1));
            for (int c = 0; c < 3; ++c) acc[c] = fmul(acc[c], fant);
            begin_sample(L, P);
        }
        if (!__any_sync(kFull, L.live)) {
            if (drained) break;
            continue;
        }
        const RayState r = make_ray(L.o, L.d, 1e16f, L.exclude);
        uint32_t nb = 0, nt = 0, leaf = 1u;
        const Hit h = trace_ray<STATS>(r, L.live, tr, false, &nb, &nt, nullptr, nullptr, L.start, &leaf);
        if (!L.live) continue;
        if (STATS) {
            cnt.segments += 1;
            cnt.boxes += nb;
            cnt.tris += nt;
            cnt.hits += (h.id >= 0) ? 1u : 0u;
        }
        bool ended;
        if (h.id < 0) {
            for (int c = 0; c < 3; ++c) acc[c] = fadd(acc[c], fmul(fmul(L.fact, L.beta[c]), P.sky[c]));
            ended = true;
        } else {
            const float* le = emission + 3 * (size_t)h.id;
            const float* al = albedo + 3 * (size_t)h.id;
            for (int c = 0; c < 3; ++c) {
                acc[c] = fadd(acc[c], fmul(fmul(L.fact, L.beta[c]), __ldg(le + c)));
                L.beta[c] = fmul(L.beta[c], __ldg(al + c));
            }
            ended = L.s == P.bounces;
            if (!ended) bounce(L, soup, h.id, h.t, leaf);
        }
        if (ended) {
            if (++L.n == P.n0 + P.spp) {
                image[(size_t)L.j * P.cam.width + L.i] = make_float4(acc[0], acc[1], acc[2], 1.0f);
                L.live = false;
            } else {
                const float fant = fdiv((float)L.n, (float)(L.n + 1));
                L.fact = fdiv(1.0f, (float)(L.n + 1));
                for (int c = 0; c < 3; ++c) acc[c] = fmul(acc[c], fant);
                begin_sample(L, P);
            }
        }
    }
    if (STATS) {
        unsigned long long v[4] = {cnt.segments, cnt.boxes, cnt.tris, cnt.hits};
        for (int q = 0; q < 4; ++q) {
            for (int off = 16; off > 0; off >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], off);
            if ((threadIdx.x & 31) == 0 && v[q]) atomicAdd(counts + q, v[q]);
        }
    }
}

// Adjoint by path replay: the same paths as k_pathtrace (same streams, same
// walks); a lane records the triangles its sample hits, and when the sample
// ends runs the backward recurrence G_j = E_{j+1} + a_{j+1} G_{j+1} over
// them with the sample's weight in the final mean.
__global__ void __launch_bounds__(kPtThreads) k_pathtrace_adjoint(
    TreeRef tr, const float* __restrict__ soup,
    const float* __restrict__ albedo, const float* __restrict__ emission, PathParams P,
    const float4* __restrict__ dimage, float* __restrict__ dalbedo, float* __restrict__ demission, uint32_t* work,
    uint32_t num_tiles) {
    constexpr uint32_t kFull = 0xffffffffu;
    const uint32_t total = num_tiles * 32u;
    PathLane L;
    L.o = mk3(0.f, 0.f, 0.f);
    L.d = mk3(0.f, 0.f, 1.f);
    float dle[3] = {0.0f, 0.0f, 0.0f};
    float gimg[3] = {0.0f, 0.0f, 0.0f};
    int seg[kMaxSeg];
    int ns = 0;
    bool drained = false;
    for (;;) {
        if (grab_pixel(L, P, work, total, drained)) {
            const float4 g4 = __ldg(dimage + (size_t)L.j * P.cam.width + L.i);
            gimg[0] = g4.x;
            gimg[1] = g4.y;
            gimg[2] = g4.z;
            ns = 0;
            begin_sample(L, P);
        }
        if (!__any_sync(kFull, L.live)) {
            if (drained) break;
            continue;
        }
        const RayState r = make_ray(L.o, L.d, 1e16f, L.exclude);
        uint32_t nb = 0, nt = 0, leaf = 1u;
        const Hit h = trace_ray<false>(r, L.live, tr, false, &nb, &nt, nullptr, nullptr, L.start, &leaf);
        if (!L.live) continue;
        const bool missed = h.id < 0;
        if (!missed) seg[ns++] = h.id;
        const bool ended = missed || L.s == P.bounces;
        if (!ended) {
            bounce(L, soup, h.id, h.t, leaf);
            continue;
        }
        // weight of sample n in the progressive mean after the call
        float w = 1.0f / (float)(L.n + 1);
        for (uint32_t m = L.n + 1; m < P.n0 + P.spp; ++m) w *= (float)m / (float)(m + 1);
        float beta[kMaxSeg][3];
        beta[0][0] = beta[0][1] = beta[0][2] = 1.0f;
        for (int q = 0; q + 1 < ns; ++q)
            for (int c = 0; c < 3; ++c) beta[q + 1][c] = beta[q][c] * __ldg(albedo + 3 * (size_t)seg[q] + c);
        float G[3] = {0.0f, 0.0f, 0.0f};
        if (missed)
            for (int c = 0; c < 3; ++c) G[c] = P.sky[c];
        for (int q = ns - 1; q >= 0; --q) {
            const float* al = albedo + 3 * (size_t)seg[q];
            const float* le = emission + 3 * (size_t)seg[q];
            const float l0 = __ldg(le), l1 = __ldg(le + 1), l2 = __ldg(le + 2);
            const bool emitter = (l0 != 0.0f) || (l1 != 0.0f) || (l2 != 0.0f);
            const float lev[3] = {l0, l1, l2};
            for (int c = 0; c < 3; ++c) {
                const float gw = gimg[c] * w;
                const float da = gw * beta[q][c] * G[c];
                if (da != 0.0f) atomicAdd(dalbedo + 3 * (size_t)seg[q] + c, da);
                if (emitter) dle[c] += gw * beta[q][c];
                G[c] = lev[c] + __ldg(al + c) * G[c];
            }
        }
        ns = 0;
        if (++L.n == P.n0 + P.spp) L.live = false;
        else begin_sample(L, P);
    }
    // emitter gradient: warp reduction, one atomic per warp and channel
    for (int c = 0; c < 3; ++c) {
        float v = dle[c];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if ((threadIdx.x & 31) == 0 && v != 0.0f) atomicAdd(demission + c, v);
    }
}

rt_status pt_args(rt_ctx* ctx, const rt_lbvh* l, const float* a, const float* e, const rt_camera* cam,
                  const rt_pt_params* p, PathParams* out, const char* who) {
    if (!ctx) return RT_ERR_INVALID;
    if (!l || !a || !e || !cam || !p) return rt_fail(ctx, RT_ERR_INVALID, "%s: null argument", who);
    if (l->n == 0 || !l->src_tris) return rt_fail(ctx, RT_ERR_INVALID, "%s: the LBVH has not been built", who);
    if (cam->width == 0 || cam->height == 0) return rt_fail(ctx, RT_ERR_INVALID, "%s: empty image", who);
    if (p->spp == 0 || p->bounces + 1 > (uint32_t)kMaxSeg)
        return rt_fail(ctx, RT_ERR_INVALID, "%s: spp must be > 0 and bounces < %d", who, kMaxSeg);
    if ((uint64_t)p->first_sample + p->spp > 65535u)  // the per-pixel streams are seeded with pixel * 65536 + sample
        return rt_fail(ctx, RT_ERR_INVALID, "%s: first_sample + spp must stay below 65536", who);
    out->cam = *cam;
    out->spp = p->spp;
    out->bounces = p->bounces;
    out->seed = p->seed;
    out->n0 = p->first_sample;
    for (int c = 0; c < 3; ++c) out->sky[c] = p->sky[c];
    return RT_OK;
}

uint32_t px_tiles(const rt_camera* cam) {
    return (uint32_t)(((cam->width + 7) / 8) * ((cam->height + 3) / 4));
}

}  // namespace

TreeRef tree_ref(const rt_ctx* ctx, const rt_lbvh* l);

static rt_status launch_pathtrace(rt_ctx* ctx, const rt_lbvh* l, const float* d_albedo, const float* d_emission,
                                  const rt_camera* cam, const rt_pt_params* p, float* d_image,
                                  unsigned long long* d_counts, const char* who) {
    PathParams P;
    rt_status s = pt_args(ctx, l, d_albedo, d_emission, cam, p, &P, who);
    if (s != RT_OK) return s;
    if (!d_image) return rt_fail(ctx, RT_ERR_INVALID, "%s: null image", who);
    if ((s = reset_work(ctx, kWorkPath)) != RT_OK) return s;
    const uint32_t tiles = px_tiles(cam);
    if (d_counts) {
        k_pathtrace<true><<<persistent_blocks(ctx, k_pathtrace<true>, kPtThreads, tiles), kPtThreads, 0,
                            ctx->stream>>>(tree_ref(ctx, l), l->src_tris, d_albedo, d_emission, P,
                                           reinterpret_cast<float4*>(d_image), ctx->d_work + kWorkPath, tiles,
                                           d_counts);
    } else {
        k_pathtrace<false><<<persistent_blocks(ctx, k_pathtrace<false>, kPtThreads, tiles), kPtThreads, 0,
                             ctx->stream>>>(tree_ref(ctx, l), l->src_tris, d_albedo, d_emission, P,
                                            reinterpret_cast<float4*>(d_image), ctx->d_work + kWorkPath, tiles,
                                            nullptr);
    }
    RT_CHECK_LAUNCH(ctx, "k_pathtrace");
    return RT_OK;
}

extern "C" rt_status rt_pathtrace(rt_ctx* ctx, const rt_lbvh* l, const float* d_albedo, const float* d_emission,
                                  const rt_camera* cam, const rt_pt_params* p, float* d_image) {
    return launch_pathtrace(ctx, l, d_albedo, d_emission, cam, p, d_image, nullptr, "rt_pathtrace");
}

extern "C" rt_status rt_pathtrace_counted(rt_ctx* ctx, const rt_lbvh* l, const float* d_albedo,
                                          const float* d_emission, const rt_camera* cam, const rt_pt_params* p,
                                          float* d_image, unsigned long long* d_counts) {
    if (!d_counts) return ctx ? rt_fail(ctx, RT_ERR_INVALID, "rt_pathtrace_counted: null counts") : RT_ERR_INVALID;
    return launch_pathtrace(ctx, l, d_albedo, d_emission, cam, p, d_image, d_counts, "rt_pathtrace_counted");
}

extern "C" rt_status rt_pathtrace_adjoint(rt_ctx* ctx, const rt_lbvh* l, const float* d_albedo,
                                          const float* d_emission, const rt_camera* cam, const rt_pt_params* p,
                                          const float* d_dimage, float* d_dalbedo, float* d_demission) {
    PathParams P;
    rt_status s = pt_args(ctx, l, d_albedo, d_emission, cam, p, &P, "rt_pathtrace_adjoint");
    if (s != RT_OK) return s;
    if (!d_dimage || !d_dalbedo || !d_demission) return rt_fail(ctx, RT_ERR_INVALID, "rt_pathtrace_adjoint: null buffer");
    if ((s = reset_work(ctx, kWorkAdjoint)) != RT_OK) return s;
    const uint32_t tiles = px_tiles(cam);
    k_pathtrace_adjoint<<<persistent_blocks(ctx, k_pathtrace_adjoint, kPtThreads, tiles), kPtThreads, 0,
                          ctx->stream>>>(tree_ref(ctx, l), l->src_tris, d_albedo, d_emission, P,
                                         reinterpret_cast<const float4*>(d_dimage), d_dalbedo, d_demission,
                                         ctx->d_work + kWorkAdjoint, tiles);
    RT_CHECK_LAUNCH(ctx, "k_pathtrace_adjoint");
    return RT_OK;
}
