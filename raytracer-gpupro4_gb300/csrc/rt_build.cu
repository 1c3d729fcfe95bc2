// rt_build.cu -- per-frame LBVH build on sm_103a.
//
// Replaces LBVH::Build (AccelerationStructures/LBVH/LBVH.cpp:488-632) and the
// GPU stage StructureConstruction::GPUBuildStructure
// (RayTracerCS/StructureConstruction.cpp:86-131: LBVH_PreBuild, bitonic sort,
// one LBVH_Build dispatch per level, one LBVH_BuildAABB dispatch per level).
//
// Launch sequence of rt_lbvh_build (all on the context stream, no host
// synchronisation, programmatic dependent launch between kernels):
//   k_bounds        scene AABB (last-block reduction) + scratch reset
//   k_morton_hist   per-triangle centroid and 30-bit Morton code
//                   (LBVH.cpp:512, 520-553) + the four 8-bit digit histograms
//   k_onesweep x4   stable LSD radix sort of (code, id): warp-ballot digit
//                   ranks, grouped decoupled look-back over tiles,
//                   shared-memory staged scatter.  Result = qsort(cmpMorton)
//                   order (LBVH.cpp:21-38).
//   k_emit_tiles    per-tile aggregates of the boundary "record masks"
//   k_emit_prefix   tile prefixes (one block)
//   k_emit_units    per tile: each leaf's heap index and range, the triangle
//                   pre-gather in sorted order, the leaf records (boxes by a
//                   segmented scan) and the tile's leaves as ordered units
//   k_emit_chunks   shared-memory bottom-up over each tile's units
//   k_emit_merge    the same over groups of 32 chunks / groups, level after
//                   level to the root, in one launch
// The allocation-free build (rt_lbvh_build_noalloc) and the batched build
// keep the one-level look-back and the first emission form, k_emit_leaves +
// k_emit_refit (kb_emit_leaves + kb_emit_refit for a batch): leaf boxes,
// then an atomic bottom-up walk with epoch-tagged arrival words that writes
// every internal node (parent = h/2, sibling = h^1).
//
// Tree = the reference's: LBVH::build_recursive (LBVH.cpp:190-314) splits a
// sorted range at its highest differing Morton bit, keeps equal-code runs as
// one leaf, stores node i's children at 2i and 2i+1 and turns every node at
// heap index >= 2^(depth-1) into a leaf.  For boundary i between sorted
// elements i and i+1 let delta_i be its highest differing bit (-1 for equal
// codes).  The split bits on the root path of element k are exactly the
// "records" of delta seen from k (boundaries whose delta exceeds every delta
// between them and k), on both sides; a record mask (bit d set for a record
// with delta d) is an associative scan, so every element's heap index
// follows from two scans and its own code: depth = popcount(mask), index =
// 1 followed by the code's bits at the mask positions, high to low.
#include <algorithm>
#include <atomic>
#include <mutex>

#include "rt_internal.cuh"

namespace {

constexpr uint32_t kFull = 0xffffffffu;

__device__ __forceinline__ int hb(uint32_t x) { return 31 - __clz(x); }

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---------------------------------------------------------------------------
// Record-mask operators.  A segment's forward mask holds the deltas that are
// records when the segment is scanned from its right end; combining left
// segment A with right segment B keeps B and the records of A above max(B)
// (= highest bit of B).  The backward mask is the mirror image.
__device__ __forceinline__ uint32_t keep_above(uint32_t m, int b) {
    return (b < 0) ? m : (m & ~((2u << b) - 1u));
}
__device__ __forceinline__ uint32_t rec_fwd(uint32_t a, uint32_t b) {  // a left of b
    return b ? (b | keep_above(a, hb(b))) : a;
}
__device__ __forceinline__ uint32_t rec_bwd(uint32_t a, uint32_t b) {  // a left of b
    return a ? (a | keep_above(b, hb(a))) : b;
}

__device__ __forceinline__ int delta_of(uint32_t a, uint32_t b) { return (a == b) ? -1 : hb(a ^ b); }

// ---------------------------------------------------------------------------
// Morton quantisation (LBVH.cpp:538-540) and bit interleave (LBVH.cpp:541-552:
// z bit j -> 3j, y bit j -> 3j+1, x bit j -> 3j+2, ten bits per axis).
__device__ __forceinline__ uint32_t quantize(float c, float lo3, float f) {
    float v = fmul(fsub(c, lo3), f);
    if (!(v == v)) return 0u;                                   // NaN (flat axis)
    if (v >= 2147483648.0f || v <= -2147483649.0f) return 0u;   // outside int range
    return (uint32_t)__float2int_rz(v);
}
__device__ __forceinline__ uint32_t spread10(uint32_t x) {
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

// ---------------------------------------------------------------------------
// k_bounds: min/max over all vertices (LBVH.cpp:495-516), last block folds the
// per-block partials and derives the Morton parameters.  Also resets the
// build's scratch (histograms, tile tickets, look-back words, leaf count) and
// optionally writes the sentinel into every heap slot.
__global__ void __launch_bounds__(256) k_bounds(const float* __restrict__ tris, uint32_t n, SceneInfo* scene,
                                                float* partials, uint32_t* counters, uint32_t* hist,
                                                uint32_t* lookback, uint32_t lookback_words, rt_node* nodes,
                                                uint32_t num_nodes, int clear_nodes) {
    grid_dep_wait();
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t gstride = gridDim.x * blockDim.x;

    for (uint32_t i = gtid; i < 4 * 256; i += gstride) hist[i] = 0u;
    for (uint32_t i = gtid; i < lookback_words; i += gstride) lookback[i] = 0u;
    // counters: [0] bounds ticket (reset by the last block), [1..4] sort tile
    // tickets, [5] leaf count, [6] refit epoch (advanced once per build, so a
    // replayed CUDA graph of the build still tags every arrival afresh), [7]
    // spine-node count
    if ((gtid >= 1 && gtid < 6) || gtid == 7) counters[gtid] = 0u;
    if (gtid == 0) {
        uint32_t e = counters[6] + 1u;
        counters[6] = e ? e : 1u;  // 0 is the value of cleared arrival words
    }
    if (clear_nodes) {
        for (uint32_t i = gtid; i < num_nodes; i += gstride) {
            rt_node s;
            s.min[0] = s.min[1] = s.min[2] = 0.0f;
            s.max[0] = s.max[1] = s.max[2] = 0.0f;
            s.prim_count = RT_NODE_SENTINEL;
            s.prim_pos = RT_NODE_SENTINEL;
            nodes[i] = s;
        }
    }

    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    uint32_t bad = 0;
    auto acc = [&](float x, float y, float z) {
        bad |= !(isfinite(x) && isfinite(y) && isfinite(z));
        mn[0] = fminf(mn[0], x); mn[1] = fminf(mn[1], y); mn[2] = fminf(mn[2], z);
        mx[0] = fmaxf(mx[0], x); mx[1] = fmaxf(mx[1], y); mx[2] = fmaxf(mx[2], z);
    };
    const size_t nv = 3 * (size_t)n;
    size_t v0 = 0;
    if ((reinterpret_cast<uintptr_t>(tris) & 15u) == 0) {
        // 16-byte loads: 3 float4 = 4 vertices (x0 y0 z0 x1 | y1 z1 x2 y2 | z2 x3 y3 z3)
        const float4* t4 = reinterpret_cast<const float4*>(tris);
        const size_t ng = nv / 4;
#pragma unroll 2
        for (size_t g = gtid; g < ng; g += gstride) {
            const float4 a = __ldg(t4 + 3 * g), b = __ldg(t4 + 3 * g + 1), c = __ldg(t4 + 3 * g + 2);
            acc(a.x, a.y, a.z);
            acc(a.w, b.x, b.y);
            acc(b.z, b.w, c.x);
            acc(c.y, c.z, c.w);
        }
        v0 = ng * 4;
    }
    for (size_t v = v0 + gtid; v < nv; v += gstride)
        acc(__ldg(tris + 3 * v), __ldg(tris + 3 * v + 1), __ldg(tris + 3 * v + 2));
    for (int off = 16; off > 0; off >>= 1) {
        for (int c = 0; c < 3; ++c) {
            mn[c] = fminf(mn[c], __shfl_xor_sync(kFull, mn[c], off));
            mx[c] = fmaxf(mx[c], __shfl_xor_sync(kFull, mx[c], off));
        }
        bad |= __shfl_xor_sync(kFull, bad, off);
    }
    __shared__ float s_red[8][7];
    __shared__ bool s_last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        for (int c = 0; c < 3; ++c) { s_red[w][c] = mn[c]; s_red[w][3 + c] = mx[c]; }
        s_red[w][6] = bad ? 1.0f : 0.0f;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float r[7];
        for (int q = 0; q < 7; ++q) r[q] = s_red[0][q];
        for (int ww = 1; ww < 8; ++ww) {
            for (int c = 0; c < 3; ++c) { r[c] = fminf(r[c], s_red[ww][c]); r[3 + c] = fmaxf(r[3 + c], s_red[ww][3 + c]); }
            r[6] = fmaxf(r[6], s_red[ww][6]);
        }
        for (int q = 0; q < 7; ++q) partials[8 * blockIdx.x + q] = r[q];
        __threadfence();
        const uint32_t ticket = atomicAdd(&counters[0], 1u);
        s_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // the last block folds the per-block partials: strided over its threads,
    // then a warp / block reduction (order-free: min and max are exact)
    {
        float r[7];
        for (int c = 0; c < 3; ++c) { r[c] = INFINITY; r[3 + c] = -INFINITY; }
        r[6] = 0.0f;
        for (uint32_t b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
            for (int c = 0; c < 3; ++c) {
                r[c] = fminf(r[c], __ldcg(partials + 8 * b + c));
                r[3 + c] = fmaxf(r[3 + c], __ldcg(partials + 8 * b + 3 + c));
            }
            r[6] = fmaxf(r[6], __ldcg(partials + 8 * b + 6));
        }
        for (int off = 16; off > 0; off >>= 1) {
            for (int c = 0; c < 3; ++c) {
                r[c] = fminf(r[c], __shfl_xor_sync(kFull, r[c], off));
                r[3 + c] = fmaxf(r[3 + c], __shfl_xor_sync(kFull, r[3 + c], off));
            }
            r[6] = fmaxf(r[6], __shfl_xor_sync(kFull, r[6], off));
        }
        __syncthreads();
        if (lane == 0)
            for (int q = 0; q < 7; ++q) s_red[w][q] = r[q];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        float r[7];
        for (int q = 0; q < 7; ++q) r[q] = s_red[0][q];
        for (int ww = 1; ww < 8; ++ww) {
            for (int c = 0; c < 3; ++c) { r[c] = fminf(r[c], s_red[ww][c]); r[3 + c] = fmaxf(r[3 + c], s_red[ww][3 + c]); }
            r[6] = fmaxf(r[6], s_red[ww][6]);
        }
        SceneInfo s;
        for (int c = 0; c < 3; ++c) {
            s.bmin[c] = r[c];
            s.bmax[c] = r[3 + c];
            const float mx3 = fmul(3.0f, r[3 + c]);   // VertMax = 3.0f*VertMax (LBVH.cpp:521)
            s.lo3[c] = fmul(3.0f, r[c]);             // VertMin = 3.0f*VertMin (:522)
            s.f[c] = fdiv(1024.0f, fsub(mx3, s.lo3[c]));  // (:523-526)
        }
        s.nonfinite = r[6] != 0.0f;
        s.pad[0] = s.pad[1] = s.pad[2] = 0;
        *scene = s;
        counters[0] = 0u;
    }
}

// ---------------------------------------------------------------------------
// k_morton_hist: codes + ids, and the per-pass digit histograms for the
// radix sort (block-local shared-memory atomics, then one global add per
// bin; aggregating equal digits in the warp with match.any first was 5 %
// slower over the whole build).
constexpr int kMortonThreads = 512;

__global__ void __launch_bounds__(kMortonThreads) k_morton_hist(const float* __restrict__ tris, uint32_t n,
                                                                const SceneInfo* __restrict__ scene,
                                                                uint32_t* __restrict__ keys,
                                                                uint32_t* __restrict__ ids, uint32_t* hist,
                                                                uint32_t* err) {
    grid_dep_wait();
    __shared__ float s_tri[kMortonThreads * 9];
    __shared__ uint32_t s_hist[4][256];
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) (&s_hist[0][0])[i] = 0u;
    const SceneInfo sc = *scene;
    if (blockIdx.x == 0 && threadIdx.x == 0 && sc.nonfinite) atomicOr(err, RT_DEVERR_NONFINITE);
    __syncthreads();
    for (uint32_t base = blockIdx.x * kMortonThreads; base < n; base += gridDim.x * kMortonThreads) {
        const uint32_t cnt = min((uint32_t)kMortonThreads, n - base);
        const float* src = tris + 9 * (size_t)base;
        for (uint32_t q = threadIdx.x; q < 9 * cnt; q += kMortonThreads) s_tri[q] = __ldg(src + q);
        __syncthreads();
        const uint32_t i = base + threadIdx.x;
        const bool valid = threadIdx.x < cnt;
        uint32_t code = 0;
        if (valid) {
            const float* t = s_tri + 9 * threadIdx.x;
            uint32_t q[3];
            for (int c = 0; c < 3; ++c) {
                const float cen = fadd(fadd(t[c], t[3 + c]), t[6 + c]);  // (V0 + V1) + V2 (LBVH.cpp:512)
                q[c] = quantize(cen, sc.lo3[c], sc.f[c]);
            }
            code = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
            keys[i] = code;
            ids[i] = i;
        }
        if (valid) {
#pragma unroll
            for (int p = 0; p < kSortPasses; ++p) atomicAdd(&s_hist[p][(code >> (8 * p)) & 0xffu], 1u);
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) {
        const uint32_t v = (&s_hist[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

// ---------------------------------------------------------------------------
// Block-wide exclusive sum over 256 threads (one value each).
__device__ __forceinline__ uint32_t block_excl_sum_256(uint32_t v, uint32_t* s_tmp /*8*/) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) s_tmp[w] = x;
    __syncthreads();
    uint32_t wp = 0;
    for (int q = 0; q < w; ++q) wp += s_tmp[q];
    __syncthreads();
    return wp + x - v;
}

constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kFlagMask = 3u << 30;
constexpr uint32_t kValMask = (1u << 30) - 1u;
constexpr int kLookWidth = 4;  // predecessor words a look-back step reads at once
constexpr unsigned kLookSleepNs = 100;  // back-off before polling an unpublished word again

// k_onesweep: one LSD pass over 8 bits.  Each CTA takes the next tile ticket
// (so every tile it waits on belongs to a CTA that is already running),
// ranks its keys stably per digit with warp ballots, publishes its digit
// counts, looks back over earlier tiles for the global digit offsets, and
// scatters through shared memory so that each digit's run is written
// contiguously.  At most 64 registers, so four CTAs share an SM: the 513
// tiles of 2.1 M keys then run in one wave over 152 SMs (at three CTAs per
// SM, 57 tiles made a second wave; the cap costs a few spilled words).
//
// SCENE = true is the batched build's last pass: the digit is the scene of
// the element's triangle id (scene_off: S + 1 triangle offsets, S <= 256),
// which groups the scenes while keeping each scene's Morton order.
constexpr uint32_t kMaxBatchScenes = 256;

__device__ __forceinline__ uint32_t scene_of(const uint32_t* off, uint32_t S, uint32_t k) {
    uint32_t lo = 0, hi = S;  // off[lo] <= k < off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (off[mid] <= k) lo = mid; else hi = mid;
    }
    return lo;
}

template <bool SCENE>
__device__ __forceinline__ uint32_t sort_digit(uint32_t key, uint32_t id, int shift, const uint32_t* s_off, uint32_t S) {
    return SCENE ? scene_of(s_off, S, id) : ((key >> shift) & 0xffu);
}

// Grouped look-back (GROUPED = true, the single-scene build): the tiles form
// groups of kLookGroup consecutive tickets.  A tile publishes its digit
// counts, sums those of the earlier tiles of its group (one round of
// parallel loads), and the group's last tile publishes the group's
// aggregate, then, once it knows the prefix of all earlier groups, the
// group's inclusive prefix.  A tile's global offset is that group prefix,
// found by the usual look-back over the group words, plus its sum inside
// the group.  The chain of dependent L2 round trips runs over 17 group words
// instead of 513 tile words at 2.1 M keys.  Every wait is on a lower ticket,
// so no tile waits on one that may not have started.  The group words
// follow the tile words in `lookback` (256 per group).
constexpr uint32_t kLookGroup = 32;

__host__ __device__ constexpr uint32_t look_groups(uint32_t tiles) { return (tiles + kLookGroup - 1) / kLookGroup; }

template <bool SCENE, bool GROUPED = false>
__global__ void __launch_bounds__(kSortThreads, 4) k_onesweep(const uint32_t* __restrict__ keys_in,
                                                           const uint32_t* __restrict__ ids_in,
                                                           uint32_t* __restrict__ keys_out,
                                                           uint32_t* __restrict__ ids_out, uint32_t n, int pass,
                                                           const uint32_t* __restrict__ hist, uint32_t* lookback,
                                                           uint32_t* tile_counter, uint32_t* err,
                                                           const uint32_t* __restrict__ scene_off = nullptr,
                                                           uint32_t S = 0, uint32_t spin_limit = kSpinLimit) {
    grid_dep_wait();
    __shared__ uint32_t s_keys[kSortTile];
    __shared__ uint32_t s_ids[kSortTile];
    __shared__ uint32_t s_warp[kSortThreads / 32][256];
    __shared__ uint32_t s_lstart[256];
    __shared__ uint32_t s_gofs[256];
    __shared__ uint32_t s_tmp[8];
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_off[SCENE ? kMaxBatchScenes + 1 : 1];

    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    if (SCENE)
        for (uint32_t q = t; q <= S; q += kSortThreads) s_off[q] = scene_off[q];
    if (t == 0) s_tile = atomicAdd(tile_counter, 1u);
    for (int i = lane; i < 256; i += 32) s_warp[w][i] = 0u;
    const uint32_t gbase = block_excl_sum_256(hist[pass * 256 + t], s_tmp);  // includes __syncthreads
    const uint32_t tile = s_tile;
    const uint32_t base = tile * (uint32_t)kSortTile;
    const int shift = 8 * pass;

    uint32_t key[kSortItems], idv[kSortItems], rank[kSortItems];
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        const uint32_t idx = base + w * (32 * kSortItems) + i * 32 + lane;
        const bool valid = idx < n;
        key[i] = valid ? keys_in[idx] : 0xffffffffu;
        idv[i] = valid ? ids_in[idx] : 0u;
    }
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        const uint32_t idx = base + w * (32 * kSortItems) + i * 32 + lane;
        const bool valid = idx < n;
        const uint32_t d = sort_digit<SCENE>(key[i], idv[i], shift, s_off, S);
        uint32_t peers = __ballot_sync(kFull, valid);
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            const bool bit = (d >> b) & 1u;
            const uint32_t m = __ballot_sync(kFull, bit);
            peers &= bit ? m : ~m;
        }
        const uint32_t cnt = s_warp[w][d];
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) s_warp[w][d] = cnt + __popc(peers);
        rank[i] = cnt + __popc(peers & lt);
        __syncwarp();
    }
    __syncthreads();

    // digit t: per-warp exclusive prefixes and the tile count
    uint32_t run = 0;
#pragma unroll
    for (int ww = 0; ww < kSortThreads / 32; ++ww) {
        const uint32_t c = s_warp[ww][t];
        s_warp[ww][t] = run;
        run += c;
    }
    const uint32_t count = run;

    uint32_t excl = 0;
    if (GROUPED) {
        const uint32_t T = (n + kSortTile - 1) / kSortTile;  // the pass's tiles (the grid may start later)
        uint32_t* gwords = lookback + (size_t)T * 256;
        const uint32_t G = tile / kLookGroup, g0 = G * kLookGroup;
        const bool group_last = (tile - g0 == kLookGroup - 1) || (tile + 1 == T);
        st_relaxed(lookback + (size_t)tile * 256 + t, kFlagAgg | count);
        // sum of the earlier tiles of the group (published right after their
        // ranking; each word polled until it is)
        uint32_t pre = 0, spins = 0;
        for (uint32_t j0 = g0; j0 < tile; j0 += 8) {
            uint32_t v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = (j0 + q < tile) ? ld_relaxed(lookback + (size_t)(j0 + q) * 256 + t) : kFlagAgg;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                while ((v[q] & kFlagMask) == 0u) {
                    if (++spins > spin_limit) {
                        atomicOr(err, RT_DEVERR_TIMEOUT);
                        v[q] = kFlagAgg;
                        break;
                    }
                    __nanosleep(kLookSleepNs);
                    v[q] = ld_relaxed(lookback + (size_t)(j0 + q) * 256 + t);
                }
                pre += v[q] & kValMask;
            }
        }
        uint32_t* gw = gwords + (size_t)G * 256 + t;
        if (group_last) st_relaxed(gw, (G == 0 ? kFlagInc : kFlagAgg) | (pre + count));
        // prefix of the earlier groups: look-back over the group words
        uint32_t gex = 0;
        if (G > 0) {
            int p = (int)G - 1;
            bool done = false;
            while (!done && p >= 0) {
                uint32_t v[kLookWidth];
#pragma unroll
                for (int q = 0; q < kLookWidth; ++q)
                    v[q] = (p - q >= 0) ? ld_relaxed(gwords + (size_t)(p - q) * 256 + t) : 0u;
                int used = 0;
#pragma unroll
                for (int q = 0; q < kLookWidth; ++q) {
                    if (done || used < q || p - q < 0) continue;
                    const uint32_t f = v[q] & kFlagMask;
                    if (f == 0u) continue;  // not published yet: poll again from here
                    gex += v[q] & kValMask;
                    used = q + 1;
                    if (f == kFlagInc) done = true;
                }
                if (!done && used == 0) {
                    if (++spins > spin_limit) {
                        atomicOr(err, RT_DEVERR_TIMEOUT);
                        break;
                    }
                    __nanosleep(kLookSleepNs);
                }
                p -= used;
            }
            if (group_last) st_relaxed(gw, kFlagInc | (gex + pre + count));
        }
        excl = gex + pre;
    } else {
    // decoupled look-back (bounded)
    uint32_t* my = lookback + (size_t)tile * 256 + t;
    st_relaxed(my, (tile == 0 ? kFlagInc : kFlagAgg) | count);
    // Look-back over the predecessors' words for this digit, kLookWidth at a
    // time (the loads are in flight together): add aggregates until an
    // inclusive prefix; a word not yet published is polled again (bounded),
    // after a short sleep, so that the polls of waiting warps do not take
    // issue slots from the warps of the same SM that are still ranking.
    // (Reading 8 or 16 words a step was slower: the extra polls cost more
    // than the shorter chain of inclusive prefixes saved.)
    if (tile > 0) {
        int p = (int)tile - 1;
        uint32_t spins = 0;
        bool done = false;
        while (!done && p >= 0) {
            uint32_t v[kLookWidth];
#pragma unroll
            for (int q = 0; q < kLookWidth; ++q)
                v[q] = (p - q >= 0) ? ld_relaxed(lookback + (size_t)(p - q) * 256 + t) : 0u;
            int used = 0;
#pragma unroll
            for (int q = 0; q < kLookWidth; ++q) {
                if (done || used < q || p - q < 0) continue;
                const uint32_t f = v[q] & kFlagMask;
                if (f == 0u) continue;  // not published yet: poll again from here
                excl += v[q] & kValMask;
                used = q + 1;
                if (f == kFlagInc) done = true;
            }
            if (!done && used == 0) {
                if (++spins > spin_limit) {
                    atomicOr(err, RT_DEVERR_TIMEOUT);
                    break;
                }
                __nanosleep(kLookSleepNs);
            }
            p -= used;
        }
        st_relaxed(my, kFlagInc | (excl + count));
    }
    }

    const uint32_t lstart = block_excl_sum_256(count, s_tmp);
    s_lstart[t] = lstart;
    s_gofs[t] = gbase + excl - lstart;
    __syncthreads();

#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        const uint32_t idx = base + w * (32 * kSortItems) + i * 32 + lane;
        if (idx < n) {
            const uint32_t d = sort_digit<SCENE>(key[i], idv[i], shift, s_off, S);
            const uint32_t pos = s_lstart[d] + s_warp[w][d] + rank[i];
            if (pos < (uint32_t)kSortTile) {
                s_keys[pos] = key[i];
                s_ids[pos] = idv[i];
            } else {
                atomicOr(err, RT_DEVERR_BOUNDS);
            }
        }
    }
    __syncthreads();
    const uint32_t tile_n = (n - base < (uint32_t)kSortTile) ? (n - base) : (uint32_t)kSortTile;
    for (uint32_t j = t; j < tile_n; j += kSortThreads) {
        const uint32_t k = s_keys[j];
        const uint32_t gp = s_gofs[sort_digit<SCENE>(k, s_ids[j], shift, s_off, S)] + j;
        if (gp < n) {
            keys_out[gp] = k;
            ids_out[gp] = s_ids[j];
        } else {
            atomicOr(err, RT_DEVERR_BOUNDS);
        }
    }
}

// ---------------------------------------------------------------------------
// Ordered (non-commutative) reductions / scans of record masks.
template <bool FWD>
__device__ __forceinline__ uint32_t rec_op(uint32_t a, uint32_t b) {
    return FWD ? rec_fwd(a, b) : rec_bwd(a, b);
}

// Warp reduction in lane order; lane 0 receives op(v_0, v_1, ..., v_31).
template <bool FWD>
__device__ __forceinline__ uint32_t warp_reduce_ordered(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t o = __shfl_down_sync(kFull, v, off);
        if (lane + off < 32) v = rec_op<FWD>(v, o);
    }
    return v;
}

// Block-wide exclusive prefix (fwd, from the left) and exclusive suffix
// (bwd, from the right) of one value pair per thread, 256 threads.
template <int THREADS = kEmitThreads>
__device__ __forceinline__ void block_scan_records(uint32_t vf, uint32_t vb, uint32_t* pre_f, uint32_t* suf_b,
                                                   uint32_t* s_f /*THREADS / 32*/, uint32_t* s_b /*THREADS / 32*/) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t xf = vf;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, xf, off);
        if (lane >= off) xf = rec_fwd(y, xf);
    }
    uint32_t xb = vb;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_down_sync(kFull, xb, off);
        if (lane + off < 32) xb = rec_bwd(xb, y);
    }
    if (lane == 31) s_f[w] = xf;  // inclusive fwd total of the warp
    if (lane == 0) s_b[w] = xb;   // inclusive bwd total of the warp
    __syncthreads();
    uint32_t wf = 0, wb = 0;
    for (int q = 0; q < w; ++q) wf = rec_fwd(wf, s_f[q]);
    for (int q = (THREADS / 32) - 1; q > w; --q) wb = rec_bwd(s_b[q], wb);
    __syncthreads();
    uint32_t ef = __shfl_up_sync(kFull, xf, 1);
    if (lane == 0) ef = 0;
    uint32_t eb = __shfl_down_sync(kFull, xb, 1);
    if (lane == 31) eb = 0;
    *pre_f = rec_fwd(wf, ef);
    *suf_b = rec_bwd(eb, wb);
}

// Loads the codes a thread needs and its boundary record bits.
struct EmitChunk {
    uint32_t c[kEmitItems + 1];  // codes of elements s .. s+8 (0 beyond n)
    uint32_t r[kEmitItems];      // record bit of boundaries s .. s+7
    int dl[kEmitItems + 1];      // delta of boundaries s-1 .. s+7 (dl[q] = delta_{s+q-1})
};

__device__ __forceinline__ void load_chunk(const uint32_t* __restrict__ keys, uint32_t n, uint32_t s, EmitChunk& e) {
    uint32_t prev = (s >= 1 && s - 1 < n) ? __ldg(keys + s - 1) : 0u;
#pragma unroll
    for (int q = 0; q <= kEmitItems; ++q) e.c[q] = (s + q < n) ? __ldg(keys + s + q) : 0u;
    e.dl[0] = (s >= 1 && s < n) ? delta_of(prev, e.c[0]) : -1;
#pragma unroll
    for (int q = 0; q < kEmitItems; ++q) {
        const uint32_t i = s + q;  // boundary i between i and i+1
        const int d = (i + 1 < n) ? delta_of(e.c[q], e.c[q + 1]) : -1;
        e.dl[q + 1] = d;
        e.r[q] = (d >= 0) ? (1u << d) : 0u;
    }
}

// k_emit_tiles: per-tile fwd/bwd aggregates of the boundary record masks.
__global__ void __launch_bounds__(kEmitThreads) k_emit_tiles(const uint32_t* __restrict__ keys, uint32_t n,
                                                             uint32_t* scan, uint32_t* arrive, uint32_t arrive_words,
                                                             const uint32_t* epoch_word) {
    grid_dep_wait();
    // epoch 1 means the first build or a wrapped epoch counter: the refit's
    // arrival words may hold any old epoch and are cleared before k_emit_refit
    if (*epoch_word == 1u)
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < arrive_words; i += gridDim.x * blockDim.x)
            arrive[i] = 0u;
    __shared__ uint32_t s_f[8], s_b[8];
    const uint32_t s = blockIdx.x * kEmitTile + threadIdx.x * kEmitItems;
    EmitChunk e;
    load_chunk(keys, n, s, e);
    uint32_t af = 0, ab = 0;
#pragma unroll
    for (int q = 0; q < kEmitItems; ++q) af = rec_fwd(af, e.r[q]);
#pragma unroll
    for (int q = kEmitItems - 1; q >= 0; --q) ab = rec_bwd(e.r[q], ab);
    af = warp_reduce_ordered<true>(af);
    ab = warp_reduce_ordered<false>(ab);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { s_f[w] = af; s_b[w] = ab; }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t tf = 0, tb = 0;
        for (int q = 0; q < kEmitThreads / 32; ++q) tf = rec_fwd(tf, s_f[q]);
        for (int q = kEmitThreads / 32 - 1; q >= 0; --q) tb = rec_bwd(s_b[q], tb);
        scan[4 * blockIdx.x + 0] = tf;
        scan[4 * blockIdx.x + 1] = tb;
    }
}

// k_emit_prefix: exclusive fwd prefix / bwd suffix over the tiles (one block
// of 1024 threads, each over a contiguous run of tiles).
constexpr int kPrefixThreads = 1024;

__global__ void __launch_bounds__(kPrefixThreads) k_emit_prefix(uint32_t* scan, uint32_t tiles) {
    grid_dep_wait();
    __shared__ uint32_t s_f[kPrefixThreads / 32], s_b[kPrefixThreads / 32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const uint32_t per = (tiles + kPrefixThreads - 1) / kPrefixThreads;
    const uint32_t lo = min(tiles, (uint32_t)t * per), hi = min(tiles, lo + per);
    uint32_t af = 0, ab = 0;
    for (uint32_t q = lo; q < hi; ++q) af = rec_fwd(af, scan[4 * q + 0]);
    for (uint32_t q = hi; q > lo; --q) ab = rec_bwd(scan[4 * (q - 1) + 1], ab);
    uint32_t xf = af, xb = ab;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, xf, off);
        if (lane >= off) xf = rec_fwd(y, xf);
        const uint32_t z = __shfl_down_sync(kFull, xb, off);
        if (lane + off < 32) xb = rec_bwd(xb, z);
    }
    if (lane == 31) s_f[w] = xf;  // inclusive fwd total of the warp
    if (lane == 0) s_b[w] = xb;   // inclusive bwd total of the warp
    __syncthreads();
    uint32_t wf = 0, wb = 0;
    for (int q = 0; q < w; ++q) wf = rec_fwd(wf, s_f[q]);
    for (int q = kPrefixThreads / 32 - 1; q > w; --q) wb = rec_bwd(s_b[q], wb);
    uint32_t ef = __shfl_up_sync(kFull, xf, 1);
    if (lane == 0) ef = 0;
    uint32_t eb = __shfl_down_sync(kFull, xb, 1);
    if (lane == 31) eb = 0;
    uint32_t run = rec_fwd(wf, ef);
    for (uint32_t q = lo; q < hi; ++q) {
        const uint32_t a = scan[4 * q + 0];
        scan[4 * q + 2] = run;
        run = rec_fwd(run, a);
    }
    run = rec_bwd(eb, wb);
    for (uint32_t q = hi; q > lo; --q) {
        const uint32_t a = scan[4 * (q - 1) + 1];
        scan[4 * (q - 1) + 3] = run;
        run = rec_bwd(a, run);
    }
}

// k_emit_leaves: for every sorted element k, the heap index of the leaf that
// holds it (capped at depth-1), whether it opens / closes that leaf's range,
// and the triangle pre-gather in sorted order.
__global__ void __launch_bounds__(kEmitThreads) k_emit_leaves(const uint32_t* __restrict__ keys,
                                                              const uint32_t* __restrict__ ids,
                                                              const float* __restrict__ tris, uint32_t n,
                                                              uint32_t depth, const uint32_t* __restrict__ scan,
                                                              rt_node* nodes, float4* __restrict__ sorted_tris,
                                                              uint32_t* leaf_list, uint32_t* leaf_count,
                                                              uint32_t* err) {
    grid_dep_wait();
    __shared__ uint32_t s_f[8], s_b[8];
    const uint32_t s = blockIdx.x * kEmitTile + threadIdx.x * kEmitItems;
    EmitChunk e;
    load_chunk(keys, n, s, e);
    uint32_t af = 0, ab = 0;
#pragma unroll
    for (int q = 0; q < kEmitItems; ++q) af = rec_fwd(af, e.r[q]);
#pragma unroll
    for (int q = kEmitItems - 1; q >= 0; --q) ab = rec_bwd(e.r[q], ab);
    uint32_t pre, suf;
    block_scan_records(af, ab, &pre, &suf, s_f, s_b);
    const uint32_t tile_pre = scan[4 * blockIdx.x + 2];
    const uint32_t tile_suf = scan[4 * blockIdx.x + 3];
    uint32_t L[kEmitItems + 1], R[kEmitItems + 1];
    L[0] = rec_fwd(tile_pre, pre);   // records of boundaries 0 .. s-1
    R[kEmitItems] = rec_bwd(suf, tile_suf);  // records of boundaries s+8 .. n-2
#pragma unroll
    for (int q = 0; q < kEmitItems; ++q) L[q + 1] = rec_fwd(L[q], e.r[q]);
#pragma unroll
    for (int q = kEmitItems - 1; q >= 0; --q) R[q] = rec_bwd(e.r[q], R[q + 1]);

    const int leaf_depth = (int)depth - 1;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int q = 0; q < kEmitItems; ++q) {
        const uint32_t k = s + q;
        const bool valid = k < n;
        bool head = false;
        uint32_t h = 0;
        if (valid) {
            const uint32_t anc = L[q] | R[q];
            const uint32_t code = e.c[q];
            int dep = __popc(anc);
            uint32_t m = anc;
            while (dep > leaf_depth) { m &= m - 1u; --dep; }
            h = 1u;
            while (m) {
                const int b = hb(m);
                h = (h << 1) | ((code >> b) & 1u);
                m ^= 1u << b;
            }
            const int dprev = e.dl[q], dcur = e.dl[q + 1];
            head = (k == 0) || (dprev >= 0 && __popc(keep_above(anc, dprev)) < leaf_depth);
            const bool tail = (k == n - 1) || (dcur >= 0 && __popc(keep_above(anc, dcur)) < leaf_depth);
            if (head) nodes[h].prim_pos = (int32_t)k;
            if (tail) nodes[h].prim_count = (int32_t)k;  // range end; k_emit_refit finalises the field
        }
        // warp-aggregated append of the leaves opened here
        const uint32_t hm = __ballot_sync(kFull, head);
        uint32_t basei = 0;
        if (lane == 0 && hm) basei = atomicAdd(leaf_count, (uint32_t)__popc(hm));
        basei = __shfl_sync(kFull, basei, 0);
        if (head) leaf_list[basei + __popc(hm & lanemask_lt())] = h;
    }
    // pre-gather in sorted order (A.xyz,id | B.xyz,0 | C.xyz,0), lane-contiguous
    // so that the 48-byte records of a warp are written as one contiguous run
    const uint32_t tbase = blockIdx.x * kEmitTile;
#pragma unroll 4
    for (int q = 0; q < kEmitItems; ++q) {
        const uint32_t k = tbase + q * kEmitThreads + threadIdx.x;
        if (k < n) {
            uint32_t id = __ldg(ids + k);
            if (id >= n) {  // only after a failed sort (look-back timeout)
                atomicOr(err, RT_DEVERR_BOUNDS);
                id = 0;
            }
            const float* tp = tris + 9 * (size_t)id;
            float v[9];
#pragma unroll
            for (int c = 0; c < 9; ++c) v[c] = __ldg(tp + c);
            sorted_tris[3 * (size_t)k + 0] = make_float4(v[0], v[1], v[2], __int_as_float((int)id));
            sorted_tris[3 * (size_t)k + 1] = make_float4(v[3], v[4], v[5], 0.0f);
            sorted_tris[3 * (size_t)k + 2] = make_float4(v[6], v[7], v[8], 0.0f);
        }
    }
}

// k_emit_refit: leaf fields and boxes (LBVH.cpp:194-208 / LBVH.hlsl:240-258),
// then the bottom-up walk: the second of two siblings to arrive at a parent
// writes it (LBVH.cpp:310-313 / LBVH.hlsl:260-269).  Arrival words carry the
// build epoch (counters[6], advanced by k_bounds), so they never need clearing.
//
// A warp takes 32 leaves at a time.  Their boxes are computed together: the
// (leaf, triangle) pairs are numbered by a prefix sum of the leaf sizes and
// reduced 32 at a time with a segmented min / max, so a 200-triangle leaf
// costs 7 coalesced warp steps instead of 200 dependent loads on one thread.
// Then every lane writes its leaf and walks up.

// Checked range [pos, end] of the leaf at heap slot h of a tree of n
// triangles (fields written by the emission).  A child below the root has a
// sibling range beside it: pos > 0 for a right child, end + 1 < n for a left
// one (the axis reads that key).
__device__ __forceinline__ bool leaf_range(uint32_t h, const rt_node* nodes, uint32_t n, uint32_t depth,
                                           int32_t* pos, int32_t* end) {
    if (h >= (1u << depth)) return false;
    *pos = __ldcg(&nodes[h].prim_pos);
    *end = __ldcg(&nodes[h].prim_count);
    return !(*pos < 0 || *end < *pos || (uint32_t)*end >= n ||
             (h > 1u && ((h & 1u) ? *pos == 0 : (uint32_t)*end + 1u >= n)));
}

// Boxes of the lanes' leaves: lane i's triangles are sorted positions
// [gpos, gpos + cnt) of sorted_tris (cnt = 0: no leaf).  All 32 lanes call.
__device__ __forceinline__ void leaf_boxes(int64_t gpos, int cnt, const float4* __restrict__ sorted_tris,
                                           float mn[3], float mx[3]) {
    const int lane = threadIdx.x & 31;
    for (int c = 0; c < 3; ++c) {
        mn[c] = INFINITY;
        mx[c] = -INFINITY;
    }
    uint32_t incl = (uint32_t)cnt;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += y;
    }
    const uint32_t total = __shfl_sync(kFull, incl, 31);
    const uint32_t excl = incl - (uint32_t)cnt;
    const uint32_t glo = (uint32_t)gpos, ghi = (uint32_t)(gpos >> 32);
    // owner of pair p and the address of its triangle
    auto locate = [&](uint32_t p, int* owner) -> const float4* {
        int o = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const uint32_t v = __shfl_sync(kFull, incl, o + step - 1);
            if (v <= p) o += step;
        }
        const uint32_t o_excl = __shfl_sync(kFull, excl, o);
        const int64_t o_gpos =
            (int64_t)(((uint64_t)__shfl_sync(kFull, ghi, o) << 32) | __shfl_sync(kFull, glo, o));
        *owner = o;
        return sorted_tris + 3 * (o_gpos + (int64_t)(p - o_excl));
    };
    // software pipelined: the next batch's triangles are loaded while the
    // current batch is reduced
    int on = 0;
    float4 na = make_float4(0.f, 0.f, 0.f, 0.f), nb = na, nc = na;
    if (total > 0) {
        const float4* tp = locate(lane, &on);
        if ((uint32_t)lane < total) {
            na = __ldg(tp);
            nb = __ldg(tp + 1);
            nc = __ldg(tp + 2);
        }
    }
    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t p = base + lane;
        const int o = on;
        const float4 a = na, b = nb, c = nc;
        if (base + 32 < total) {
            const float4* tp = locate(p + 32, &on);
            if (p + 32 < total) {
                na = __ldg(tp);
                nb = __ldg(tp + 1);
                nc = __ldg(tp + 2);
            }
        }
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        if (p < total) {
            // gMinVertices / gMaxVertices (LBVH.cpp:505-509): min(V0, min(V1, V2))
            lo[0] = smin(a.x, smin(b.x, c.x)); hi[0] = smax(a.x, smax(b.x, c.x));
            lo[1] = smin(a.y, smin(b.y, c.y)); hi[1] = smax(a.y, smax(b.y, c.y));
            lo[2] = smin(a.z, smin(b.z, c.z)); hi[2] = smax(a.z, smax(b.z, c.z));
        }
        // segmented min / max (lanes of one owner are contiguous); afterwards
        // the first lane of each owner's run holds the run's box
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int o2 = __shfl_down_sync(kFull, o, off);
            const bool take = lane + off < 32 && o2 == o;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float l2 = __shfl_down_sync(kFull, lo[c], off);
                const float h2 = __shfl_down_sync(kFull, hi[c], off);
                if (take) {  // lane + off holds later triangles of the same leaf
                    lo[c] = smin(lo[c], l2);
                    hi[c] = smax(hi[c], h2);
                }
            }
        }
        const bool mine = cnt > 0 && excl < base + 32 && incl > base;
        const int head = mine ? (int)(max(excl, base) - base) : lane;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float l2 = __shfl_sync(kFull, lo[c], head);
            const float h2 = __shfl_sync(kFull, hi[c], head);
            if (mine) {  // earlier batches first, as the leaf loop of LBVH.cpp:202-206 runs
                mn[c] = smin(mn[c], l2);
                mx[c] = smax(mx[c], h2);
            }
        }
    }
}

// The leaf node at h of a tree (keys / nodes / arrive are the tree's own,
// scene-offset arrays) and the walk to the root.
__device__ __forceinline__ void refit_walk(uint32_t h, int32_t pos, int32_t end, const float mn_in[3],
                                           const float mx_in[3], const uint32_t* __restrict__ keys, uint32_t n,
                                           uint32_t depth, rt_node* nodes, uint32_t* arrive, uint32_t epoch,
                                           uint32_t* err, uint32_t* inner = nullptr) {
    const int32_t count = end - pos + 1;
    // leaf axis = the reference's round-robin counter at the call that made
    // the leaf: entry with bit (d_parent - 1) -> (31 - d_parent) % 3; a run
    // of equal codes recursed down to bit 0 -> 1; the root enters at bit 30.
    const int dh = 31 - __clz(h);
    int axis;
    if (dh == 0) {
        axis = (count <= 1 || depth <= 1) ? 0 : 1;
    } else if (count == 1 || dh == (int)depth - 1) {
        const uint32_t a = (h & 1u) ? __ldg(keys + pos - 1) : __ldg(keys + end);
        const uint32_t b = (h & 1u) ? __ldg(keys + pos) : __ldg(keys + end + 1);
        axis = (31 - hb(a ^ b)) % 3;
    } else {
        axis = 1;
    }
    rt_node nd;
    for (int q = 0; q < 3; ++q) { nd.min[q] = mn_in[q]; nd.max[q] = mx_in[q]; }
    nd.prim_count = (count << 3) | 4 | axis;
    nd.prim_pos = pos;
    nodes[h] = nd;
    while (h > 1) {
        // release our node, acquire the sibling's: one acq_rel exchange per level
        uint32_t old;
        asm volatile("atom.acq_rel.gpu.global.exch.b32 %0, [%1], %2;"
                     : "=r"(old)
                     : "l"(arrive + (h >> 1)), "r"(epoch)
                     : "memory");
        if (old != epoch) break;  // first of the two children: the sibling finishes the parent
        const uint32_t sib = h ^ 1u;
        const float4 s0 = __ldcg(reinterpret_cast<const float4*>(&nodes[sib]));
        const float4 s1 = __ldcg(reinterpret_cast<const float4*>(&nodes[sib]) + 1);
        const float smn[3] = {s0.x, s0.y, s0.z}, smx[3] = {s0.w, s1.x, s1.y};
        const int32_t scount = __float_as_int(s1.z) >> 3, spos = __float_as_int(s1.w);
        const int32_t lpos = (h & 1u) ? spos : nd.prim_pos;
        const int32_t rpos = (h & 1u) ? nd.prim_pos : spos;
        const int32_t pcount = (nd.prim_count >> 3) + scount;
        if (rpos < 1 || (uint32_t)rpos >= n) {
            atomicOr(err, RT_DEVERR_BOUNDS);
            break;
        }
        const int d = hb(__ldg(keys + rpos - 1) ^ __ldg(keys + rpos));
        // minBox / maxBox(left, right) (LBVH.cpp:312-313): the left child's
        // bound is kept on a tie, which decides the sign of a zero bound
        if (h & 1u) {
            for (int q = 0; q < 3; ++q) { nd.min[q] = smin(smn[q], nd.min[q]); nd.max[q] = smax(smx[q], nd.max[q]); }
        } else {
            for (int q = 0; q < 3; ++q) { nd.min[q] = smin(nd.min[q], smn[q]); nd.max[q] = smax(nd.max[q], smx[q]); }
        }
        nd.prim_count = (pcount << 3) | ((30 - d) % 3);
        nd.prim_pos = lpos;
        h >>= 1;
        nodes[h] = nd;
        if (inner) atomicOr(inner + (h >> 5), 1u << (h & 31));
    }
}

__global__ void __launch_bounds__(256) k_emit_refit(const uint32_t* __restrict__ keys, const float4* sorted_tris,
                                                    uint32_t n, uint32_t depth, rt_node* nodes,
                                                    const uint32_t* __restrict__ leaf_list,
                                                    const uint32_t* leaf_count, uint32_t* arrive,
                                                    const uint32_t* epoch_word, uint32_t* err,
                                                    uint32_t* inner = nullptr) {
    grid_dep_wait();
    const uint32_t nleaves = min(*leaf_count, n);
    const uint32_t epoch = *epoch_word;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t base = warp * 32; base < nleaves; base += nwarps * 32) {
        const uint32_t li = base + lane;
        uint32_t h = 0;
        int32_t pos = 0, end = -1;
        bool ok = false;
        if (li < nleaves) {
            h = leaf_list[li];
            ok = leaf_range(h, nodes, n, depth, &pos, &end);
            if (!ok) atomicOr(err, RT_DEVERR_BOUNDS);
        }
        float mn[3], mx[3];
        leaf_boxes(pos, ok ? end - pos + 1 : 0, sorted_tris, mn, mx);
        if (ok) refit_walk(h, pos, end, mn, mx, keys, n, depth, nodes, arrive, epoch, err, inner);
    }
}

// ---------------------------------------------------------------------------
// Emission and refit without global atomics (the single-scene build).
//
// k_emit_units handles one tile of kEmitTile sorted elements:
//   1. per element: ancestor record mask (two scans), head / tail of its
//      leaf's range, and at heads and tails the mask capped at the leaf depth
//      and the leaf's heap index; the tile's leaves become "units" in sorted
//      order;
//   0. the triangles gathered in sorted order (sorted_tris), striped so that
//      a warp takes 32 consecutive elements at a time: they leave through a
//      per-warp staging buffer as 512-byte runs, and their boxes go to
//      shared memory;
//   2. the boxes folded per leaf, each thread over its own eight consecutive
//      elements (a segmented scan carries a leaf that spans threads, with its
//      head); the leaf records are stored;
//   3. a leaf that began in an earlier tile and ends in this one is finished
//      here: its start is found by scanning back over the codes and its
//      earlier triangles are folded in from the soup.
// k_emit_merge then runs a shared-memory bottom-up (unit_bottom_up) over one
// tile's units per CTA; a node whose parent's split boundary lies outside
// the units becomes an "item" for the next level, and k_emit_merge runs
// again over the items of kMergeGroup consecutive tiles (groups) per CTA,
// level after level, until one CTA forms the root.  No node waits on another
// CTA, and nothing needs a global arrival word.
//
// The parent's split bit is the lowest bit of a node's remaining ancestor
// mask, so no walk reads a Morton code.  Boxes are min / max in the
// reference's operand order (left before right, earlier triangle first),
// which fixes the sign of a zero bound; a node's box is the ordered fold of
// its triangles' boxes, whatever the grouping.
constexpr uint32_t kHeadBit = 1u << 30;
constexpr uint32_t kTailBit = 1u << 31;
constexpr uint32_t kMaskBits = kHeadBit - 1u;
constexpr int kUnitCap = kEmitTile;  // units of one CTA: the leaves of a tile, the items of a group
constexpr int kChunkUnits = 512;     // units of one CTA of the tile level (a tile's leaves in chunks)
constexpr int kTileChunks = kUnitCap / kChunkUnits;
constexpr int kItemCap = 64;         // items one tile or group hands on (2 x depth + 2 <= 54)
constexpr int kMergeGroup = 32;      // tiles (groups) per CTA of the next level
constexpr int kUnitWords = 12;       // shared words per unit
constexpr size_t kUnitSmem = (size_t)kUnitWords * kUnitCap * sizeof(uint32_t) + 16;
constexpr size_t kChunkSmem = (size_t)kUnitWords * kChunkUnits * sizeof(uint32_t) + 16;
// k_emit_units: the tile's triangle boxes, six planes of kBoxStride floats
// (element e at e + e / 32, so that a warp reading eight consecutive
// elements per lane hits 32 different banks), then one staging buffer of
// 32 triangles (96 float4) per warp
constexpr int kBoxStride = kEmitTile + kEmitTile / 32;
constexpr int kGatherBatch = 4;  // triangles a thread has in flight in the gather
constexpr size_t kEmitUnitsSmem = 6 * kBoxStride * sizeof(float) + (kEmitThreads / 32) * 96 * sizeof(float4);
static_assert((6 * kBoxStride) % 4 == 0, "staging buffer must start 16-byte aligned");
static_assert(kEmitItems % kGatherBatch == 0, "gather batches must tile a thread's elements");

// Triangle `id` of a soup of n triangles (9 floats each): three 16-byte
// loads of the 12 floats starting at float 9 id - (id mod 4), which is 16-byte
// aligned when the soup is (9 id = id mod 4, mod 4), then a shift by id mod 4.
// The last triangles, whose 12 floats would run past the soup, and an
// unaligned soup take scalar loads.
__device__ __forceinline__ void load_tri(const float* __restrict__ tris, uint32_t id, uint32_t n, bool aligned,
                                         float v[9]) {
    const uint32_t r = id & 3u;
    const size_t f0 = 9 * (size_t)id - r;
    if (aligned && f0 + 12 <= 9 * (size_t)n) {
        const float4* p = reinterpret_cast<const float4*>(tris + f0);
        const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
        const float w[12] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w};
#pragma unroll
        for (int k = 0; k < 9; ++k) v[k] = r == 0 ? w[k] : r == 1 ? w[k + 1] : r == 2 ? w[k + 2] : w[k + 3];
    } else {
        const float* tp = tris + 9 * (size_t)id;
#pragma unroll
        for (int k = 0; k < 9; ++k) v[k] = __ldg(tp + k);
    }
}

// Leaf axis field: the reference's round-robin counter at the call that made
// the leaf (see refit_walk), with the parent's split bit = the lowest bit of
// the leaf's capped ancestor mask m (depth = popcount of m).
__device__ __forceinline__ int leaf_axis_of(uint32_t m, int32_t count, uint32_t depth) {
    const int dh = __popc(m);
    if (dh == 0) return (count <= 1 || depth <= 1) ? 0 : 1;
    if (count == 1 || dh == (int)depth - 1) return (31 - (__ffs(m) - 1)) % 3;
    return 1;
}

__device__ __forceinline__ void store_node(rt_node* nodes, uint32_t h, const float mn[3], const float mx[3],
                                           int32_t prim_count, int32_t prim_pos) {
    float4* p = reinterpret_cast<float4*>(nodes + h);
    p[0] = make_float4(mn[0], mn[1], mn[2], mx[0]);
    p[1] = make_float4(mx[1], mx[2], __int_as_float(prim_count), __int_as_float(prim_pos));
}

// Ordered union of two boxes (a holds the earlier triangles).
struct Box {
    float lo[3], hi[3];
};
__device__ __forceinline__ Box box_union(const Box& a, const Box& b) {
    Box r;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        r.lo[c] = smin(a.lo[c], b.lo[c]);
        r.hi[c] = smax(a.hi[c], b.hi[c]);
    }
    return r;
}
__device__ __forceinline__ Box empty_box() {
    Box r;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        r.lo[c] = INFINITY;
        r.hi[c] = -INFINITY;
    }
    return r;
}
// gMinVertices / gMaxVertices (LBVH.cpp:505-509): min(V0, min(V1, V2))
__device__ __forceinline__ Box tri_box(const float v[9]) {
    Box r;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        r.lo[c] = smin(v[c], smin(v[3 + c], v[6 + c]));
        r.hi[c] = smax(v[c], smax(v[3 + c], v[6 + c]));
    }
    return r;
}
__device__ __forceinline__ Box shfl_up_box(const Box& b, int off) {
    Box r;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        r.lo[c] = __shfl_up_sync(kFull, b.lo[c], off);
        r.hi[c] = __shfl_up_sync(kFull, b.hi[c], off);
    }
    return r;
}

// Shared-memory view of a CTA's units (capacity cap): unit i covers elements
// [pos[i], pos[i + 1]) and is the node (h[i], m[i]) with box lo/hi[i];
// arrivals of the bottom-up reuse the box slots and aext / am.
struct Units {
    int cap;
    float* lo;      // [3][cap]
    float* hi;      // [3][cap]
    int32_t* pos;   // [cap + 1]
    uint32_t* h;    // [cap]
    uint32_t* m;    // [cap]
    int32_t* aext;  // [cap] arrival: the far unit index of the arriving node
    uint32_t* am;   // [cap] arrival: the arriving node's remaining mask
    uint32_t* arr;  // [cap] arrival bits of the boundary after unit i (1 left child, 2 right child)
    uint32_t* n_items;
};
__device__ __forceinline__ Units units_of(uint32_t* smem, int cap) {
    Units u;
    u.cap = cap;
    u.lo = reinterpret_cast<float*>(smem);
    u.hi = u.lo + 3 * cap;
    u.pos = reinterpret_cast<int32_t*>(u.hi + 3 * cap);
    u.h = reinterpret_cast<uint32_t*>(u.pos + cap + 4);
    u.m = u.h + cap;
    u.aext = reinterpret_cast<int32_t*>(u.m + cap);
    u.am = reinterpret_cast<uint32_t*>(u.aext + cap);
    u.arr = u.am + cap;
    u.n_items = u.arr + cap;
    return u;
}
__device__ __forceinline__ void set_box(const Units& u, int i, const Box& b) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        u.lo[c * u.cap + i] = b.lo[c];
        u.hi[c * u.cap + i] = b.hi[c];
    }
}
__device__ __forceinline__ Box get_box(const Units& u, int i) {
    Box b;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        b.lo[c] = u.lo[c * u.cap + i];
        b.hi[c] = u.hi[c * u.cap + i];
    }
    return b;
}

__device__ __forceinline__ void push_item(const Units& u, uint2* items, uint32_t h, uint32_t m, uint32_t* err) {
    const uint32_t slot = atomicAdd(u.n_items, 1u);
    if (slot < (uint32_t)kItemCap) items[slot] = make_uint2(h, m);
    else atomicOr(err, RT_DEVERR_BOUNDS);
}

// Bottom-up over units 0 .. U-1 (arr[] zero, every unit's box, pos, h, m
// set, pos[U] = one past the last unit's last element, *n_items zero).  Each
// node arrives at the boundary between its parent's two children: a left
// child leaves its box, far unit and mask at its last unit's slot, a right
// child at its first unit's slot, then sets its bit; the second arrival
// forms the parent and carries on.  Nodes whose parent boundary lies outside
// the units, and arrivals whose sibling never came, become items.
template <int THREADS>
__device__ void unit_bottom_up(const Units& u, int U, rt_node* nodes, uint2* items, uint32_t* err,
                               uint32_t* inner) {
#pragma unroll 1
    for (int i = threadIdx.x; i < U; i += THREADS) {
        Box b = get_box(u, i);
        uint32_t h = u.h[i], m = u.m[i];
        int li = i, ri = i;
        while (h > 1) {
            const bool left = (h & 1u) == 0;
            const int k = left ? ri : li - 1;  // the parent's split boundary, after unit k
            if (k < 0 || k + 1 >= U) {
                push_item(u, items, h, m, err);
                break;
            }
            const int area = left ? ri : li;
            set_box(u, area, b);
            u.aext[area] = left ? li : ri;
            u.am[area] = m;
            __threadfence_block();
            const uint32_t old = atomicOr(&u.arr[k], left ? 1u : 2u);
            if (old == 0u) break;  // first: the sibling forms the parent
            __threadfence_block();
            const int sarea = left ? k + 1 : k;
            const Box sb = get_box(u, sarea);
            b = left ? box_union(b, sb) : box_union(sb, b);
            if (left) ri = u.aext[sarea]; else li = u.aext[sarea];
            const int d = __ffs(m) - 1;  // the parent's split bit
            m &= m - 1u;
            h >>= 1;
            const int32_t pos = u.pos[li], end = u.pos[ri + 1] - 1;
            store_node(nodes, h, b.lo, b.hi, ((end - pos + 1) << 3) | ((30 - d) % 3), pos);
            if (inner) atomicOr(inner + (h >> 5), 1u << (h & 31));
        }
    }
    __syncthreads();
    // arrivals whose sibling lies outside the units: their node is an item
    for (int k = threadIdx.x; k + 1 < U; k += THREADS) {
        const uint32_t v = u.arr[k];
        if (v != 1u && v != 2u) continue;
        const int area = v == 1u ? k : k + 1;
        const int li = v == 1u ? u.aext[area] : area;
        const uint32_t m = u.am[area];
        const int up = __popc(u.m[li]) - __popc(m);
        if (up < 0) {
            atomicOr(err, RT_DEVERR_BOUNDS);
            continue;
        }
        push_item(u, items, u.h[li] >> up, m, err);
    }
}

// The capped mask and heap index of an element with ancestor mask anc: the
// highest `cap` bits of anc (its ancestors down to the leaf depth), and 1
// followed by the code's bits at those positions, high to low.  Taken a run
// of consecutive mask bits at a time rather than bit by bit (a balanced
// region's mask is one run).
__device__ __forceinline__ uint32_t heap_index_capped(uint32_t code, uint32_t anc, int cap, uint32_t* m_out) {
    uint32_t h = 1u, m = 0u;
    int left = cap;
    while (anc != 0u && left > 0) {
        const int top = hb(anc);
        const int len = min(__clz(~(anc << (31 - top))), left);  // the run from top down, at most `left` bits
        const int lo = top - len + 1;
        const uint32_t ones = (len >= 32) ? ~0u : ((1u << len) - 1u);
        h = (h << len) | ((code >> lo) & ones);
        m |= ones << lo;
        anc &= ~(ones << lo);
        left -= len;
    }
    *m_out = m;
    return h;
}

// The open segment at a thread's end for the segmented scan of leaf boxes:
// its box and the position of its head (-1: it began before the tile).
struct Seg {
    Box b;
    int32_t head;
};

template <int THREADS>
__global__ void __launch_bounds__(THREADS) k_emit_units(const uint32_t* __restrict__ keys,
                                                        const uint32_t* __restrict__ ids,
                                                        const float* __restrict__ tris, uint32_t n, uint32_t depth,
                                                        const uint32_t* __restrict__ scan, rt_node* nodes,
                                                        float4* __restrict__ sorted_tris, uint2* units,
                                                        uint32_t* unit_counts, uint32_t* err) {
    __shared__ uint32_t s_f[THREADS / 32], s_b[THREADS / 32], s_tmp[THREADS / 32];
    __shared__ uint32_t s_first_head, s_first_tail, s_last_head, s_last_tail, s_cont_tail;
    __shared__ float s_red[THREADS / 32][6];
    __shared__ int32_t s_rhead[THREADS / 32];
    __shared__ int s_found;
    __shared__ float s_cont_box[6];
    static_assert(THREADS == kEmitThreads, "the shared-memory layout is sized for kEmitThreads");
    extern __shared__ float4 emit_smem[];
    float* s_box = reinterpret_cast<float*>(emit_smem);  // [6][kBoxStride]: lo xyz, hi xyz

    grid_dep_wait();
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const uint32_t tbase = blockIdx.x * (uint32_t)kEmitTile;
    uint2* my_units = units + (size_t)blockIdx.x * kUnitCap;
    if (t == 0) {
        s_first_head = s_first_tail = kEmitTile;
        s_last_head = s_last_tail = 0u;
    }

    // 0. pre-gather in sorted order (A.xyz,id | B.xyz,0 | C.xyz,0): element
    // tbase + b * THREADS + t, a batch of loads in flight per thread; the
    // warp's 32 triangles are staged and stored as three 512-byte runs
    {
        float4* stage = emit_smem + (6 * kBoxStride) / 4 + w * 96;
        const bool soup_aligned = (reinterpret_cast<uintptr_t>(tris) & 15u) == 0;
#pragma unroll 1
        for (int g = 0; g < kEmitItems; g += kGatherBatch) {
            uint32_t idv[kGatherBatch];
            float v[kGatherBatch][9];
#pragma unroll
            for (int b = 0; b < kGatherBatch; ++b) {
                const uint32_t k = tbase + (uint32_t)((g + b) * THREADS + t);
                uint32_t id = k < n ? __ldg(ids + k) : 0u;
                if (id >= n) {  // only after a failed sort (look-back timeout)
                    atomicOr(err, RT_DEVERR_BOUNDS);
                    id = 0;
                }
                idv[b] = id;
            }
#pragma unroll
            for (int b = 0; b < kGatherBatch; ++b) load_tri(tris, idv[b], n, soup_aligned, v[b]);
#pragma unroll
            for (int b = 0; b < kGatherBatch; ++b) {
                const uint32_t e0 = (uint32_t)((g + b) * THREADS + w * 32);  // the warp's first element
                const uint32_t el = e0 + lane;
                const Box tb = tri_box(v[b]);
                const uint32_t pb = el + (el >> 5);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    s_box[c * kBoxStride + pb] = tb.lo[c];
                    s_box[(3 + c) * kBoxStride + pb] = tb.hi[c];
                }
                stage[3 * lane + 0] = make_float4(v[b][0], v[b][1], v[b][2], __int_as_float((int)idv[b]));
                stage[3 * lane + 1] = make_float4(v[b][3], v[b][4], v[b][5], 0.0f);
                stage[3 * lane + 2] = make_float4(v[b][6], v[b][7], v[b][8], 0.0f);
                __syncwarp();
                const uint32_t kw = tbase + e0;
                const uint32_t live = kw < n ? min(32u, n - kw) : 0u;  // the run's elements inside the soup
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    const uint32_t f = (uint32_t)(lane + 32 * j);
                    if (f < 3 * live) sorted_tris[3 * (size_t)kw + f] = stage[f];
                }
                __syncwarp();
            }
        }
    }

    // 1. capped mask, head and tail of this thread's elements; heap index at
    // heads and tails (the elements between them share their leaf's)
    const uint32_t s = tbase + (uint32_t)t * kEmitItems;
    EmitChunk e;
    load_chunk(keys, n, s, e);
    uint32_t af = 0, ab = 0;
#pragma unroll
    for (int q = 0; q < kEmitItems; ++q) af = rec_fwd(af, e.r[q]);
#pragma unroll
    for (int q = kEmitItems - 1; q >= 0; --q) ab = rec_bwd(e.r[q], ab);
    uint32_t pre, suf;
    block_scan_records<THREADS>(af, ab, &pre, &suf, s_f, s_b);  // includes __syncthreads
    uint32_t L[kEmitItems + 1], R[kEmitItems + 1];
    L[0] = rec_fwd(scan[4 * blockIdx.x + 2], pre);
    R[kEmitItems] = rec_bwd(suf, scan[4 * blockIdx.x + 3]);
#pragma unroll
    for (int q = 0; q < kEmitItems; ++q) L[q + 1] = rec_fwd(L[q], e.r[q]);
#pragma unroll
    for (int q = kEmitItems - 1; q >= 0; --q) R[q] = rec_bwd(e.r[q], R[q + 1]);
    const int leaf_depth = (int)depth - 1;
    uint32_t hm[kEmitItems], hh[kEmitItems];  // capped mask | head | tail; heap index (heads, tails)
    uint32_t heads = 0u, tails = 0u;
#pragma unroll
    for (int q = 0; q < kEmitItems; ++q) {
        const uint32_t k = s + q;
        hm[q] = 0u;
        hh[q] = 0u;
        if (k < n) {
            const uint32_t anc = L[q] | R[q];
            const int dprev = e.dl[q], dcur = e.dl[q + 1];
            const bool head = (k == 0) || (dprev >= 0 && __popc(keep_above(anc, dprev)) < leaf_depth);
            const bool tail = (k == n - 1) || (dcur >= 0 && __popc(keep_above(anc, dcur)) < leaf_depth);
            if (head || tail) {
                // the capped mask and heap index: at heads, and at a tail that
                // may close a leaf whose head is in an earlier thread (a tail
                // after a head of this thread shares that head's)
                uint32_t m = 0u;
                if (head || heads == 0u) hh[q] = heap_index_capped(e.c[q], anc, leaf_depth, &m);
                hm[q] = m | (head ? kHeadBit : 0u) | (tail ? kTailBit : 0u);
                if (head) heads |= 1u << q;
                if (tail) tails |= 1u << q;
            }
        }
    }
    {  // the tile's first / last head and tail: warp reductions, one shared atomic per warp
        const uint32_t j0 = (uint32_t)t * kEmitItems;
        const uint32_t fh = __reduce_min_sync(kFull, heads ? j0 + __ffs(heads) - 1 : (uint32_t)kEmitTile);
        const uint32_t lh = __reduce_max_sync(kFull, heads ? j0 + (32 - __clz(heads)) : 0u);
        const uint32_t ft = __reduce_min_sync(kFull, tails ? j0 + __ffs(tails) - 1 : (uint32_t)kEmitTile);
        const uint32_t lt = __reduce_max_sync(kFull, tails ? j0 + (32 - __clz(tails)) : 0u);
        if (lane == 0) {
            atomicMin(&s_first_head, fh);
            atomicMax(&s_last_head, lh);
            atomicMin(&s_first_tail, ft);
            atomicMax(&s_last_tail, lt);
        }
    }
    const uint32_t hbase = block_excl_sum_256(__popc(heads), s_tmp);  // includes __syncthreads
    // units: the leaf that began in an earlier tile and ends here (unit 0),
    // then every leaf with its head and tail in the tile; a last leaf that
    // runs past the tile is the next tile's
    const uint32_t first_head = s_first_head, first_tail = s_first_tail;
    const uint32_t cont = (first_tail < kEmitTile && first_tail < first_head) ? 1u : 0u;
    const bool last_open = s_last_head > s_last_tail;  // the last head's leaf has no tail in the tile

    // 2. the leaf boxes: each thread folds its own elements' boxes (gathered
    // in step 0, ordered by the scans' barriers); a leaf spanning threads is
    // carried by a segmented scan that also carries the leaf's head position
    Box part = empty_box();  // elements before the thread's first head (or all of them)
    Box run = empty_box();   // the current leaf since its head in this thread
    bool seen_head = false, closed = false;
    int first_tail_q = -1;
    uint32_t ft_h = 0u, ft_m = 0u;  // heap index and mask of the first segment's tail
    uint32_t ord = 0;
    int32_t run_pos = -1;
    uint32_t run_h = 0u, run_m = 0u;  // heap index and mask of the current leaf
#pragma unroll
    for (int q = 0; q < kEmitItems; ++q) {
        const uint32_t k = s + q;
        if (k >= n) break;
        const uint32_t el = (uint32_t)t * kEmitItems + q, pb = el + (el >> 5);
        Box tb;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            tb.lo[c] = s_box[c * kBoxStride + pb];
            tb.hi[c] = s_box[(3 + c) * kBoxStride + pb];
        }
        const bool head = (hm[q] & kHeadBit) != 0, tail = (hm[q] & kTailBit) != 0;
        if (head) {
            const uint32_t idx = cont + hbase + ord++;
            const uint32_t j = t * kEmitItems + q;
            run_h = hh[q];
            run_m = hm[q] & kMaskBits;
            if (idx < (uint32_t)kUnitCap && !(last_open && j + 1 == s_last_head)) my_units[idx] = make_uint2(run_h, run_m);
            run = tb;
            seen_head = true;
            run_pos = (int32_t)k;
        } else if (!seen_head && !closed) {
            part = box_union(part, tb);
        } else if (seen_head) {
            run = box_union(run, tb);
        }
        if (tail) {
            if (seen_head) {  // a leaf with head and tail in this thread
                const int32_t count = (int32_t)k - run_pos + 1;
                store_node(nodes, run_h, run.lo, run.hi, (count << 3) | 4 | leaf_axis_of(run_m, count, depth), run_pos);
                seen_head = false;  // the next element is a head
            } else {
                first_tail_q = q;
                ft_h = hh[q];
                ft_m = hm[q] & kMaskBits;
            }
            closed = true;
        }
    }
    // segmented exclusive scan of the open segment at each thread's end;
    // reset = the thread holds a head or a tail
    const bool reset = heads != 0u || closed;
    Seg x;
    x.b = seen_head ? run : (closed ? empty_box() : part);
    x.head = seen_head ? run_pos : -1;
    {
        bool r = reset;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const Box yb = shfl_up_box(x.b, off);
            const int32_t yh = __shfl_up_sync(kFull, x.head, off);
            const bool ry = __shfl_up_sync(kFull, r, off);
            if (lane >= off && !r) {
                x.b = box_union(yb, x.b);
                x.head = yh;
                r = ry;
            }
        }
        if (lane == 31) {
            for (int c = 0; c < 3; ++c) { s_red[w][c] = x.b.lo[c]; s_red[w][3 + c] = x.b.hi[c]; }
            s_rhead[w] = x.head;
            s_tmp[w] = r ? 1u : 0u;
        }
        __syncthreads();
        Seg wp;  // the open segment entering this warp
        wp.b = empty_box();
        wp.head = -1;
        for (int ww = w - 1; ww >= 0; --ww) {
            Box y;
            for (int c = 0; c < 3; ++c) { y.lo[c] = s_red[ww][c]; y.hi[c] = s_red[ww][3 + c]; }
            wp.b = box_union(y, wp.b);
            wp.head = s_rhead[ww];
            if (s_tmp[ww]) break;
        }
        Seg ex;
        ex.b = shfl_up_box(x.b, 1);
        ex.head = __shfl_up_sync(kFull, x.head, 1);
        const bool rex = __shfl_up_sync(kFull, r, 1);
        if (lane == 0) {
            ex = wp;
        } else if (!rex) {
            ex.b = box_union(wp.b, ex.b);
            ex.head = wp.head;
        }
        x = ex;  // the open segment entering this thread
    }
    if (first_tail_q >= 0) {  // the segment entering this thread ends here
        const Box fin = box_union(x.b, part);
        const uint32_t j = t * kEmitItems + first_tail_q;
        if (x.head >= 0) {  // its head is in an earlier thread of this tile
            const int32_t count = (int32_t)(tbase + j) - x.head + 1;
            store_node(nodes, ft_h, fin.lo, fin.hi, (count << 3) | 4 | leaf_axis_of(ft_m, count, depth), x.head);
        } else {  // it began before the tile: finished in step 3
            for (int c = 0; c < 3; ++c) { s_cont_box[c] = fin.lo[c]; s_cont_box[3 + c] = fin.hi[c]; }
            s_cont_tail = tbase + j;
            my_units[0] = make_uint2(ft_h, ft_m);
        }
    }
    __syncthreads();

    // 3. the leaf that began in an earlier tile: its start (the nearest
    // boundary where the codes differ at or above its parent's split bit) and
    // the boxes of its triangles before this tile, folded in order with the rest
    if (cont) {
        const uint32_t m0 = my_units[0].y;
        const int dpar = m0 ? __ffs(m0) - 1 : 31;  // a root leaf starts at 0
        if (t == 0) s_found = 0;
        __syncthreads();
        int32_t start = 0;
        for (int64_t hi = (int64_t)tbase; hi > 0; hi -= THREADS) {
            const int64_t q = hi - t;  // candidate start: boundary (q - 1, q)
            bool hit = false;
            if (q >= 1) {
                const uint32_t a = __ldg(keys + q - 1), c = __ldg(keys + q);
                hit = a != c && hb(a ^ c) >= dpar;
            }
            if (__syncthreads_or(hit)) {
                if (hit) atomicMax(&s_found, (int)q);
                __syncthreads();
                start = s_found;
                break;
            }
        }
        Box before = empty_box();
        for (int64_t c0 = start; c0 < (int64_t)tbase; c0 += THREADS) {
            const int64_t k = c0 + t;
            Box tb = empty_box();
            if (k < (int64_t)tbase) {
                uint32_t id = __ldg(ids + k);
                if (id >= n) id = 0;
                const float* tp = tris + 9 * (size_t)id;
                float v[9];
                for (int c = 0; c < 9; ++c) v[c] = __ldg(tp + c);
                tb = tri_box(v);
            }
            // ordered block reduction of the chunk: lanes, then warps, in order
            for (int off = 1; off < 32; off <<= 1) {
                const Box y = shfl_up_box(tb, off);
                if (lane >= off) tb = box_union(y, tb);
            }
            if (lane == 31)
                for (int c = 0; c < 3; ++c) { s_red[w][c] = tb.lo[c]; s_red[w][3 + c] = tb.hi[c]; }
            __syncthreads();
            if (t == 0) {
                for (int ww = 0; ww < THREADS / 32; ++ww) {
                    Box y;
                    for (int c = 0; c < 3; ++c) { y.lo[c] = s_red[ww][c]; y.hi[c] = s_red[ww][3 + c]; }
                    before = box_union(before, y);
                }
            }
            __syncthreads();
        }
        if (t == 0) {
            Box in_tile;
            for (int c = 0; c < 3; ++c) { in_tile.lo[c] = s_cont_box[c]; in_tile.hi[c] = s_cont_box[3 + c]; }
            const Box fin = box_union(before, in_tile);
            const int32_t count = (int32_t)s_cont_tail - start + 1;
            const uint2 u0 = my_units[0];
            store_node(nodes, u0.x, fin.lo, fin.hi, (count << 3) | 4 | leaf_axis_of(u0.y, count, depth), start);
        }
    }
    if (t == THREADS - 1) {  // units: cont + heads, less an open last leaf
        const uint32_t total_heads = hbase + __popc(heads);
        unit_counts[blockIdx.x] = min((uint32_t)kUnitCap, cont + total_heads - (last_open ? 1u : 0u));
    }
}

// merge_group: the shared-memory bottom-up over the units of `ng` consecutive
// tiles (groups) of a level, whose stored records give each unit's box and
// range: at the tile level one tile (its leaves, in order), above it up to
// kMergeGroup groups (their items, each group's sorted by first element).
// The nodes that cannot be formed here are written to `out` sorted by first
// element, their number to *out_count.
template <int THREADS>
__device__ void merge_group(const Units& u, const uint2* in_items, const uint32_t* in_counts, int fixed_count,
                            uint32_t in_stride, uint32_t ng, uint32_t depth, rt_node* nodes, uint2* out,
                            uint32_t* out_count, uint32_t* err, uint32_t* inner, uint32_t* s_off, uint2* s_items,
                            int32_t* s_ipos) {
    const int t = threadIdx.x;
    if (t < 32) {  // unit offsets of the groups: one warp, a prefix sum over <= 32 counts
        const uint32_t c = (uint32_t)t < ng ? min(fixed_count >= 0 ? (uint32_t)fixed_count : __ldcg(in_counts + t),
                                                  in_stride)
                                            : 0u;
        uint32_t incl = c;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, incl, off);
            if (t >= off) incl += y;
        }
        if ((uint32_t)t < ng) s_off[t] = incl - c;
        if ((uint32_t)t == ng - 1) s_off[ng] = incl;
        if (t == 0) *u.n_items = 0u;
    }
    for (int i = t; i < u.cap; i += THREADS) u.arr[i] = 0u;
    __syncthreads();
    const int U = (int)min(s_off[ng], (uint32_t)u.cap);
    // every group's units are in order (tile leaves, or items sorted by the
    // CTA that made them), so their concatenation is sorted
    for (int i = t; i < U; i += THREADS) {
        uint32_t g = 0;
        while (g + 1 < ng && s_off[g + 1] <= (uint32_t)i) ++g;
        uint2 it = __ldcg(in_items + (size_t)g * in_stride + (i - s_off[g]));
        if (it.x < 1u || it.x >= (1u << depth)) {
            atomicOr(err, RT_DEVERR_BOUNDS);
            it = make_uint2(1u, 0u);  // a root stops the walk
        }
        const float4 a = __ldcg(reinterpret_cast<const float4*>(nodes + it.x));
        const float4 b = __ldcg(reinterpret_cast<const float4*>(nodes + it.x) + 1);
        u.h[i] = it.x;
        u.m[i] = it.y;
        u.lo[0 * u.cap + i] = a.x;
        u.lo[1 * u.cap + i] = a.y;
        u.lo[2 * u.cap + i] = a.z;
        u.hi[0 * u.cap + i] = a.w;
        u.hi[1 * u.cap + i] = b.x;
        u.hi[2 * u.cap + i] = b.y;
        u.pos[i] = __float_as_int(b.w);
        if (i == U - 1) u.pos[U] = __float_as_int(b.w) + (__float_as_int(b.z) >> 3);
    }
    __syncthreads();
    unit_bottom_up<THREADS>(u, U, nodes, s_items, err, inner);
    __syncthreads();
    // the items, sorted by first element (their records are stored)
    const uint32_t ni = min(*u.n_items, (uint32_t)kItemCap);
    for (uint32_t i = t; i < ni; i += THREADS) s_ipos[i] = __ldcg(&nodes[s_items[i].x].prim_pos);
    __syncthreads();
    for (uint32_t i = t; i < ni; i += THREADS) {
        uint32_t rank = 0;
        for (uint32_t o = 0; o < ni; ++o) rank += (s_ipos[o] < s_ipos[i] || (s_ipos[o] == s_ipos[i] && o < i)) ? 1u : 0u;
        out[rank] = s_items[i];
    }
    if (t == 0) *out_count = ni;
}

// k_emit_chunks: the tile level.  A tile's leaves are merged in chunks of
// kChunkUnits consecutive leaves, one CTA per chunk (kTileChunks chunk slots
// per tile, most of them empty for tiles with big leaves), so that the
// shared-memory units of eight CTAs fit an SM.  Chunk slot c's items go to
// items + c * kItemCap, their number to counts[c].
template <int THREADS>
__global__ void __launch_bounds__(THREADS) k_emit_chunks(const uint2* __restrict__ tile_units,
                                                         const uint32_t* __restrict__ tile_counts, uint32_t depth,
                                                         rt_node* nodes, uint2* items, uint32_t* counts, uint32_t* err,
                                                         uint32_t* inner) {
    extern __shared__ __align__(16) uint32_t smem[];
    const Units u = units_of(smem, kChunkUnits);
    __shared__ uint32_t s_off[kMergeGroup + 1];
    __shared__ uint2 s_items[kItemCap];
    __shared__ int32_t s_ipos[kItemCap];
    grid_dep_wait();
    const uint32_t c = blockIdx.x, tile = c / kTileChunks, chunk = c % kTileChunks;
    const uint32_t tc = min(__ldcg(tile_counts + tile), (uint32_t)kUnitCap);
    const int cnt = (int)min((uint32_t)kChunkUnits, tc > chunk * kChunkUnits ? tc - chunk * kChunkUnits : 0u);
    if (cnt == 0) {
        if (threadIdx.x == 0) counts[c] = 0u;
        return;
    }
    merge_group<THREADS>(u, tile_units + (size_t)tile * kUnitCap + (size_t)chunk * kChunkUnits, nullptr, cnt,
                         (uint32_t)kChunkUnits, 1u, depth, nodes, items + (size_t)c * kItemCap, counts + c, err, inner,
                         s_off, s_items, s_ipos);
}

// k_emit_merge: the levels above.  One CTA per kMergeGroup consecutive units
// of the level below (chunk slots, then groups) merges their items; then,
// level by level, the last CTA to finish among kMergeGroup consecutive groups
// merges their items (a ticket per group, taken after the CTA's items are
// stored and fenced; the last taker resets it for the next build), until one
// group covers the whole tree and forms the root.  No CTA waits on another.
// The first level's items are at out_items + g * kItemCap (counts at
// out_counts + g), each next level's after the previous one's.
template <int THREADS>
__global__ void __launch_bounds__(THREADS) k_emit_merge(const uint2* __restrict__ in_items,
                                                        const uint32_t* __restrict__ in_counts, uint32_t n_in,
                                                        uint32_t depth, rt_node* nodes, uint2* out_items,
                                                        uint32_t* out_counts, uint32_t* tickets, uint32_t* err,
                                                        uint32_t* inner) {
    extern __shared__ __align__(16) uint32_t smem[];
    const Units u = units_of(smem, kUnitCap);
    __shared__ uint32_t s_off[kMergeGroup + 1];
    __shared__ uint2 s_items[kItemCap];
    __shared__ int32_t s_ipos[kItemCap];
    __shared__ int s_last;
    grid_dep_wait();
    const int t = threadIdx.x;
    uint32_t g = blockIdx.x;
    uint32_t n_lev = (n_in + kMergeGroup - 1) / kMergeGroup;
    merge_group<THREADS>(u, in_items + (size_t)g * kMergeGroup * kItemCap, in_counts + (size_t)g * kMergeGroup, -1,
                         (uint32_t)kItemCap, min((uint32_t)kMergeGroup, n_in - g * kMergeGroup), depth, nodes,
                         out_items + (size_t)g * kItemCap, out_counts + g, err, inner, s_off, s_items, s_ipos);
    size_t ioff = 0, coff = 0, toff = 0;
    while (n_lev > 1) {
        const uint32_t parent = g / kMergeGroup;
        const uint32_t gs = min((uint32_t)kMergeGroup, n_lev - parent * kMergeGroup);
        const uint32_t n_next = (n_lev + kMergeGroup - 1) / kMergeGroup;
        __threadfence();  // this CTA's items, count and records before its ticket
        __syncthreads();
        if (t == 0) {
            const uint32_t k = atomicAdd(tickets + toff + parent, 1u);
            s_last = (k + 1 == gs) ? 1 : 0;
            if (s_last) tickets[toff + parent] = 0u;
        }
        __syncthreads();
        if (!s_last) return;
        __threadfence();  // the other CTAs' items and records after their tickets
        const size_t pioff = ioff + (size_t)parent * kMergeGroup * kItemCap;
        const size_t pcoff = coff + (size_t)parent * kMergeGroup;
        ioff += (size_t)n_lev * kItemCap;
        coff += n_lev;
        merge_group<THREADS>(u, out_items + pioff, out_counts + pcoff, -1, (uint32_t)kItemCap, gs, depth, nodes,
                             out_items + ioff + (size_t)parent * kItemCap, out_counts + coff + parent, err, inner,
                             s_off, s_items, s_ipos);
        toff += n_next;
        g = parent;
        n_lev = n_next;
    }
}

// Compact layout (rt_lbvh.cnodes) from the heap: inner_rank = exclusive
// popcount prefix of the internal-node bitmap (one block), then every
// reachable internal node x writes its two children at slots 2 rank(x) + 2
// and + 3, an internal child's PrimPos replaced by the slot of its own pair.
constexpr int kRankThreads = 1024;

__global__ void __launch_bounds__(kRankThreads) k_inner_rank(const uint32_t* __restrict__ inner, uint32_t words,
                                                             uint32_t* __restrict__ rank) {
    __shared__ uint32_t s_w[kRankThreads / 32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const uint32_t per = (words + kRankThreads - 1) / kRankThreads;
    const uint32_t lo = min(words, (uint32_t)t * per), hi = min(words, lo + per);
    uint32_t sum = 0;
    for (uint32_t q = lo; q < hi; ++q) sum += __popc(inner[q]);
    uint32_t incl = sum;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += y;
    }
    if (lane == 31) s_w[w] = incl;
    __syncthreads();
    uint32_t run = incl - sum;
    for (int q = 0; q < w; ++q) run += s_w[q];
    for (uint32_t q = lo; q < hi; ++q) {
        rank[q] = run;
        run += __popc(inner[q]);
    }
}

__device__ __forceinline__ uint32_t inner_slot(const uint32_t* inner, const uint32_t* rank, uint32_t x) {
    return 2u * (rank[x >> 5] + __popc(inner[x >> 5] & ((1u << (x & 31)) - 1u))) + 2u;
}

__global__ void __launch_bounds__(256) k_compact(const rt_node* __restrict__ nodes, const uint32_t* __restrict__ inner,
                                                 const uint32_t* __restrict__ rank, uint32_t words, uint32_t num_nodes,
                                                 rt_node* __restrict__ cnodes, uint32_t ccap, uint32_t* err) {
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
    if (gtid == 0) {  // the root at slot 1
        rt_node root = nodes[1];
        if (inner[0] & 2u) root.prim_pos = 2;
        cnodes[1] = root;
    }
    for (uint32_t w = gtid; w < words; w += gs) {
        uint32_t m = inner[w];
        while (m) {
            const uint32_t b = __ffs(m) - 1;
            m &= m - 1u;
            const uint32_t x = w * 32 + b;
            const uint32_t slot = inner_slot(inner, rank, x);
            if (2 * x + 1 >= num_nodes || slot + 1 >= ccap) {
                atomicOr(err, RT_DEVERR_BOUNDS);
                continue;
            }
#pragma unroll
            for (uint32_t q = 0; q < 2; ++q) {
                const uint32_t y = 2 * x + q;
                rt_node nd = nodes[y];
                if (!(nd.prim_count & 4)) nd.prim_pos = (int32_t)inner_slot(inner, rank, y);
                cnodes[slot + q] = nd;
            }
        }
    }
}


// Pre-gather for imported trees (ids + soup uploaded from the host).
__global__ void k_gather_tris(const uint32_t* __restrict__ ids, const float* __restrict__ tris, uint32_t n,
                              float4* __restrict__ sorted_tris) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t id = ids[k];
        const float* tp = tris + 9 * (size_t)id;
        sorted_tris[3 * (size_t)k + 0] = make_float4(tp[0], tp[1], tp[2], __int_as_float((int)id));
        sorted_tris[3 * (size_t)k + 1] = make_float4(tp[3], tp[4], tp[5], 0.0f);
        sorted_tris[3 * (size_t)k + 2] = make_float4(tp[6], tp[7], tp[8], 0.0f);
    }
}

uint32_t ceil_div(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

}  // namespace

// ===========================================================================
// C ABI
extern "C" rt_status rt_lbvh_create(rt_ctx* ctx, uint32_t max_tris, uint32_t depth, rt_lbvh** out) {
    if (!ctx || !out) return RT_ERR_INVALID;
    *out = nullptr;
    if (max_tris == 0 || max_tris > kMaxTris)
        return rt_fail(ctx, RT_ERR_INVALID, "rt_lbvh_create: max_tris must be in [1, %u]", kMaxTris);
    if (depth < 1 || depth > (uint32_t)kMaxDepth)
        return rt_fail(ctx, RT_ERR_INVALID, "rt_lbvh_create: depth must be in [1, %d]", kMaxDepth);
    RT_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
    rt_lbvh* l = new rt_lbvh();
    l->cap = max_tris;
    l->depth = depth;
    l->num_nodes = 1u << depth;
    l->sort_tiles_cap = ceil_div(max_tris, kSortTile);
    l->emit_tiles_cap = ceil_div(max_tris, kEmitTile);
    l->bounds_blocks = std::max(1u, std::min(ceil_div(3ull * max_tris, 256), (uint32_t)ctx->num_sms * 4));
    const size_t cap = max_tris;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    alloc((void**)&l->nodes, sizeof(rt_node) * l->num_nodes);
    alloc((void**)&l->keys, 4 * cap);
    alloc((void**)&l->ids, 4 * cap);
    // one block for both ping-pong buffers: after the sort it holds the
    // emission's per-tile unit lists (8 bytes per element)
    alloc((void**)&l->keys_alt, 8 * cap);
    if (e == cudaSuccess) l->ids_alt = l->keys_alt + cap;
    alloc((void**)&l->sorted_tris, sizeof(float4) * 3 * cap);
    l->ccap = (uint32_t)std::min<uint64_t>((uint64_t)l->num_nodes + 2, 2ull * cap + 2);
    alloc((void**)&l->cnodes, sizeof(rt_node) * l->ccap);
    alloc((void**)&l->inner, sizeof(uint32_t) * std::max(1u, l->num_nodes / 32));
    alloc((void**)&l->inner_rank, sizeof(uint32_t) * std::max(1u, l->num_nodes / 32));
    alloc((void**)&l->tris, sizeof(float) * 9 * cap);
    alloc((void**)&l->scene, sizeof(SceneInfo));
    alloc((void**)&l->partials, sizeof(float) * 8 * l->bounds_blocks);
    alloc((void**)&l->counters, sizeof(uint32_t) * 8);
    alloc((void**)&l->hist, sizeof(uint32_t) * 4 * 256);
    // per radix pass: 256 look-back words per tile, then 256 per tile group
    alloc((void**)&l->lookback,
          sizeof(uint32_t) * kSortPasses * 256 * ((size_t)l->sort_tiles_cap + look_groups(l->sort_tiles_cap)));
    alloc((void**)&l->scan, sizeof(uint32_t) * 4 * (size_t)l->emit_tiles_cap);
    alloc((void**)&l->leaf_list, 4 * cap);
    alloc((void**)&l->arrive, sizeof(uint32_t) * std::max(1u, l->num_nodes >> 1));
    // items and item counts of every merge level (chunk slots = 4 x tiles, then
    // the groups above: < 6 x tiles in all), the tiles' unit counts (tiles),
    // the merge tickets (tiles, zero between builds)
    alloc((void**)&l->items, sizeof(uint2) * 6 * (size_t)kItemCap * l->emit_tiles_cap);
    alloc((void**)&l->item_counts, sizeof(uint32_t) * 8 * (size_t)l->emit_tiles_cap);
    if (e == cudaSuccess) e = cudaMemset(l->counters, 0, sizeof(uint32_t) * 8);
    if (e == cudaSuccess) e = cudaMemset(l->arrive, 0, sizeof(uint32_t) * std::max(1u, l->num_nodes >> 1));
    if (e == cudaSuccess) e = cudaMemset(l->nodes, 0, sizeof(rt_node) * l->num_nodes);
    if (e == cudaSuccess) e = cudaMemset(l->item_counts, 0, sizeof(uint32_t) * 8 * (size_t)l->emit_tiles_cap);
    if (e != cudaSuccess) {
        rt_lbvh_destroy(l);
        return rt_fail(ctx, RT_ERR_CUDA, "rt_lbvh_create: allocation failed: %s", cudaGetErrorString(e));
    }
    *out = l;
    return RT_OK;
}

extern "C" rt_status rt_lbvh_destroy(rt_lbvh* l) {
    if (!l) return RT_OK;
    if (l->graph_refs > 0) {  // a captured frame still points into l: the last frame destroy frees it
        l->destroy_pending = true;
        return RT_OK;
    }
    free_lbvh(l);
    return RT_OK;
}

void free_lbvh(rt_lbvh* l) {
    void* ptrs[] = {l->nodes,    l->keys,     l->ids,      l->keys_alt,  nullptr,    l->sorted_tris,
                    l->tris,     l->scene,    l->partials, l->counters,  l->hist,    l->lookback,
                    l->scan,     l->leaf_list, l->arrive,  l->f_primary, l->f_mirror, l->f_vis,
                    l->s_lists,  l->cnodes,   l->inner,    l->inner_rank, l->w_buf, l->s_rays,
                    l->items,    l->item_counts};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete l;
}

static rt_status launch_build(rt_ctx* ctx, rt_lbvh* l, const float* d_tris, uint32_t n, uint32_t flags) {
    cudaStream_t st = ctx->stream;
    l->n = n;
    l->src_tris = d_tris;
    const uint32_t sort_tiles = ceil_div(n, kSortTile);
    const uint32_t emit_tiles = ceil_div(n, kEmitTile);
    const uint32_t lb_pass = 256 * (sort_tiles + look_groups(sort_tiles));  // tile words, group words
    const uint32_t lb_words = kSortPasses * lb_pass;
    const uint32_t bblocks = std::max(1u, std::min(ceil_div(3ull * n, 256), l->bounds_blocks));
    launch_pdl(k_bounds, bblocks, 256, 0, st, d_tris, n, l->scene, l->partials, l->counters, l->hist, l->lookback,
                                      lb_words, l->nodes, l->num_nodes, (flags & RT_BUILD_CLEAR_UNREACHED) ? 1 : 0);
    RT_CHECK_LAUNCH(ctx, "k_bounds");
    const uint32_t mblocks = std::max(1u, std::min(ceil_div(n, kMortonThreads), (uint32_t)ctx->num_sms * 4));
    launch_pdl(k_morton_hist, mblocks, kMortonThreads, 0, st, d_tris, n, l->scene, l->keys, l->ids, l->hist, ctx->d_err);
    RT_CHECK_LAUNCH(ctx, "k_morton_hist");
    uint32_t *kin = l->keys, *iin = l->ids, *kout = l->keys_alt, *iout = l->ids_alt;
    for (int p = 0; p < kSortPasses; ++p) {
        launch_pdl(k_onesweep<false, true>, sort_tiles, kSortThreads, 0, st, (const uint32_t*)kin, (const uint32_t*)iin,
                   kout, iout, n, p, (const uint32_t*)l->hist, l->lookback + (size_t)p * lb_pass,
                   l->counters + 1 + p, ctx->d_err, (const uint32_t*)nullptr, 0u, kSpinLimit);
        RT_CHECK_LAUNCH(ctx, "k_onesweep");
        std::swap(kin, kout);
        std::swap(iin, iout);
    }
    // four passes: sorted pairs are back in keys / ids
    launch_pdl(k_emit_tiles, emit_tiles, kEmitThreads, 0, st, l->keys, n, l->scan, l->arrive, std::max(1u, l->num_nodes >> 1),
                                                      l->counters + 6);
    RT_CHECK_LAUNCH(ctx, "k_emit_tiles");
    launch_pdl(k_emit_prefix, 1, kPrefixThreads, 0, st, l->scan, emit_tiles);
    RT_CHECK_LAUNCH(ctx, "k_emit_prefix");
    const bool compact = (flags & RT_BUILD_COMPACT) != 0;
    const uint32_t words = std::max(1u, l->num_nodes / 32);
    if (compact) RT_CHECK_CUDA(ctx, cudaMemsetAsync(l->inner, 0, sizeof(uint32_t) * words, st));
    // emission, pre-gather, leaf boxes and every node inside a tile in one
    // pass; the nodes above the tiles by k_emit_merge, level after level
    RT_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_emit_merge<kEmitThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)kUnitSmem));
    RT_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_emit_units<kEmitThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)kEmitUnitsSmem));
    uint32_t* inner = compact ? l->inner : nullptr;
    // the sort's ping-pong buffers are free again: they hold the tiles' unit lists
    uint2* tile_units = reinterpret_cast<uint2*>(l->keys_alt);
    const size_t cap = l->emit_tiles_cap;
    uint32_t* tile_counts = l->item_counts + 6 * cap;
    launch_pdl(k_emit_units<kEmitThreads>, emit_tiles, kEmitThreads, kEmitUnitsSmem, st, (const uint32_t*)l->keys,
               (const uint32_t*)l->ids, d_tris, n, l->depth, (const uint32_t*)l->scan, l->nodes, l->sorted_tris,
               tile_units, tile_counts, ctx->d_err);
    RT_CHECK_LAUNCH(ctx, "k_emit_units");
    const uint32_t chunks = emit_tiles * kTileChunks;
    launch_pdl(k_emit_chunks<kEmitThreads>, chunks, kEmitThreads, kChunkSmem, st, (const uint2*)tile_units,
               (const uint32_t*)tile_counts, l->depth, l->nodes, l->items, l->item_counts, ctx->d_err, inner);
    RT_CHECK_LAUNCH(ctx, "k_emit_chunks");
    launch_pdl(k_emit_merge<kEmitThreads>, ceil_div(chunks, kMergeGroup), kEmitThreads, kUnitSmem, st,
               (const uint2*)l->items, (const uint32_t*)l->item_counts, chunks, l->depth, l->nodes,
               l->items + (size_t)chunks * kItemCap, l->item_counts + chunks, l->item_counts + 7 * cap, ctx->d_err,
               inner);
    RT_CHECK_LAUNCH(ctx, "k_emit_merge");
    if (compact) {
        k_inner_rank<<<1, kRankThreads, 0, st>>>(l->inner, words, l->inner_rank);
        RT_CHECK_LAUNCH(ctx, "k_inner_rank");
        k_compact<<<std::max(1u, std::min(ceil_div(words, 256), (uint32_t)ctx->num_sms * 8)), 256, 0, st>>>(
            l->nodes, l->inner, l->inner_rank, words, l->num_nodes, l->cnodes, l->ccap, ctx->d_err);
        RT_CHECK_LAUNCH(ctx, "k_compact");
    }
    l->built_keys = true;
    l->compact_valid = compact;
    return RT_OK;
}

extern "C" rt_status rt_lbvh_build(rt_ctx* ctx, rt_lbvh* l, const float* d_tris, uint32_t n, uint32_t flags) {
    if (!ctx || !l || !d_tris) return ctx ? rt_fail(ctx, RT_ERR_INVALID, "rt_lbvh_build: null argument") : RT_ERR_INVALID;
    if (n == 0) return rt_fail(ctx, RT_ERR_INVALID, "rt_lbvh_build: n must be > 0");
    if (n > l->cap) return rt_fail(ctx, RT_ERR_CAPACITY, "rt_lbvh_build: n=%u exceeds capacity %u", n, l->cap);
    return launch_build(ctx, l, d_tris, n, flags);
}

extern "C" rt_status rt_lbvh_build_host(rt_ctx* ctx, rt_lbvh* l, const float* h_tris, uint32_t n, uint32_t flags) {
    if (!ctx || !l || !h_tris) return ctx ? rt_fail(ctx, RT_ERR_INVALID, "rt_lbvh_build_host: null argument") : RT_ERR_INVALID;
    if (n == 0) return rt_fail(ctx, RT_ERR_INVALID, "rt_lbvh_build_host: n must be > 0");
    if (n > l->cap) return rt_fail(ctx, RT_ERR_CAPACITY, "rt_lbvh_build_host: n=%u exceeds capacity %u", n, l->cap);
    RT_CHECK_CUDA(ctx, cudaMemcpyAsync(l->tris, h_tris, sizeof(float) * 9 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
    return launch_build(ctx, l, l->tris, n, flags);
}

extern "C" rt_status rt_lbvh_import_host(rt_ctx* ctx, rt_lbvh* l, const rt_node* h_nodes, const uint32_t* h_ids,
                                         const float* h_tris, uint32_t n) {
    if (!ctx || !l || !h_nodes || !h_ids || !h_tris)
        return ctx ? rt_fail(ctx, RT_ERR_INVALID, "rt_lbvh_import_host: null argument") : RT_ERR_INVALID;
    if (n == 0) return rt_fail(ctx, RT_ERR_INVALID, "rt_lbvh_import_host: n must be > 0");
    if (n > l->cap) return rt_fail(ctx, RT_ERR_CAPACITY, "rt_lbvh_import_host: n=%u exceeds capacity %u", n, l->cap);
    cudaStream_t st = ctx->stream;
    RT_CHECK_CUDA(ctx, cudaMemcpyAsync(l->nodes, h_nodes, sizeof(rt_node) * l->num_nodes, cudaMemcpyHostToDevice, st));
    RT_CHECK_CUDA(ctx, cudaMemcpyAsync(l->ids, h_ids, 4 * (size_t)n, cudaMemcpyHostToDevice, st));
    RT_CHECK_CUDA(ctx, cudaMemcpyAsync(l->tris, h_tris, sizeof(float) * 9 * (size_t)n, cudaMemcpyHostToDevice, st));
    const uint32_t blocks = std::max(1u, std::min(ceil_div(n, 256), (uint32_t)ctx->num_sms * 8));
    k_gather_tris<<<blocks, 256, 0, st>>>(l->ids, l->tris, n, l->sorted_tris);
    RT_CHECK_LAUNCH(ctx, "k_gather_tris");
    l->n = n;
    l->src_tris = l->tris;
    l->built_keys = false;
    l->compact_valid = false;  // an imported tree is traversed in its heap layout
    return RT_OK;
}

extern "C" rt_status rt_lbvh_view_get(const rt_lbvh* l, rt_lbvh_view* v) {
    if (!l || !v) return RT_ERR_INVALID;
    v->nodes = l->nodes;
    v->ids = l->ids;
    v->keys = l->built_keys ? l->keys : nullptr;
    v->sorted_tris = reinterpret_cast<const float*>(l->sorted_tris);
    v->n = l->n;
    v->depth = l->depth;
    v->num_nodes = l->num_nodes;
    v->node_size = (uint32_t)sizeof(rt_node);
    return RT_OK;
}

extern "C" rt_status rt_lbvh_compact_get(const rt_lbvh* l, const rt_node** d_nodes, uint32_t* slots) {
    if (!l || !d_nodes || !slots) return RT_ERR_INVALID;
    if (!l->compact_valid) return RT_ERR_INVALID;
    *d_nodes = l->cnodes;
    *slots = l->ccap;
    return RT_OK;
}

extern "C" rt_status rt_lbvh_world_bound(rt_ctx* ctx, const rt_lbvh* l, float out[6]) {
    if (!ctx || !l || !out) return ctx ? rt_fail(ctx, RT_ERR_INVALID, "rt_lbvh_world_bound: null argument") : RT_ERR_INVALID;
    rt_node root;
    RT_CHECK_CUDA(ctx, cudaMemcpyAsync(&root, l->nodes + 1, sizeof(rt_node), cudaMemcpyDeviceToHost, ctx->stream));
    RT_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int c = 0; c < 3; ++c) { out[c] = root.min[c]; out[3 + c] = root.max[c]; }
    return RT_OK;
}

extern "C" rt_status rt_lbvh_download(rt_ctx* ctx, const rt_lbvh* l, rt_node* h_nodes, uint32_t* h_ids,
                                      uint32_t* h_keys) {
    if (!ctx || !l) return ctx ? rt_fail(ctx, RT_ERR_INVALID, "rt_lbvh_download: null argument") : RT_ERR_INVALID;
    cudaStream_t st = ctx->stream;
    if (h_nodes) RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_nodes, l->nodes, sizeof(rt_node) * l->num_nodes, cudaMemcpyDeviceToHost, st));
    if (h_ids) RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_ids, l->ids, 4 * (size_t)l->n, cudaMemcpyDeviceToHost, st));
    if (h_keys) {
        if (!l->built_keys) return rt_fail(ctx, RT_ERR_INVALID, "rt_lbvh_download: keys exist only after rt_lbvh_build");
        RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_keys, l->keys, 4 * (size_t)l->n, cudaMemcpyDeviceToHost, st));
    }
    RT_CHECK_CUDA(ctx, cudaStreamSynchronize(st));
    return RT_OK;
}

// ===========================================================================
// Allocation-free LBVH build.
//
// Some callers cannot call cudaMalloc at the moment they need a rebuild: an
// engine whose device memory is owned by its own allocator (a caching pool
// that has already reserved the free memory, or a budgeted heap that must
// account for every byte) and must not be touched behind its back, or a
// real-time loop that cannot afford the implicit device-wide
// synchronisation of an allocation.  rt_lbvh_build_noalloc serves them: the
// caller passes the soup and every output buffer, and all of the build's
// scratch (sort ping-pong buffers, digit histograms, look-back words, tile
// scans, leaf list, refit arrival words) lives in the fixed array below,
// which the CUDA module reserves on every GPU that loads this library and
// keeps until the process exits.
//
// Limits: at most RT_NOALLOC_MAX_TRIS triangles (the 512 x 512 = 262,144
// primitives the reference's own GPU rebuild handles, BitonicSort.cpp:20-27)
// and depth at most RT_NOALLOC_MAX_DEPTH (the reference default, conf.ini).
// The array is shared by every call: a call clears what has to start at
// zero, so consecutive calls are independent, but calls that overlap on the
// GPU (two streams, two threads) race on it and must be serialised by the
// caller.
namespace {

constexpr uint32_t kNoAllocTiles = (RT_NOALLOC_MAX_TRIS + kSortTile - 1) / kSortTile;
constexpr uint32_t kNoAllocEmitTiles = (RT_NOALLOC_MAX_TRIS + kEmitTile - 1) / kEmitTile;
constexpr uint32_t kNoAllocBoundsBlocks = 2048;
// word offsets inside the scratch array
constexpr size_t kNaScene = 0;                                                      // SceneInfo (16 words)
constexpr size_t kNaCounters = kNaScene + 16;                                       // 8 words
constexpr size_t kNaHist = kNaCounters + 16;                                        // 4 x 256
constexpr size_t kNaPartials = kNaHist + 4 * 256;                                   // 8 floats per bounds block
constexpr size_t kNaLookback = kNaPartials + 8 * kNoAllocBoundsBlocks;              // 4 x 256 per sort tile
constexpr size_t kNaScan = kNaLookback + (size_t)kSortPasses * 256 * kNoAllocTiles;  // 4 per emission tile
constexpr size_t kNaLeaves = kNaScan + 4 * (size_t)kNoAllocEmitTiles;               // one per triangle
constexpr size_t kNaKeysAlt = kNaLeaves + RT_NOALLOC_MAX_TRIS;
constexpr size_t kNaIdsAlt = kNaKeysAlt + RT_NOALLOC_MAX_TRIS;
constexpr size_t kNaArrive = kNaIdsAlt + RT_NOALLOC_MAX_TRIS;                       // 1 << (depth - 1)
constexpr size_t kNaErr = kNaArrive + ((size_t)1 << (RT_NOALLOC_MAX_DEPTH - 1));   // error word (ctx == NULL)
constexpr size_t kNaWords = kNaErr + 64;
static_assert(kNaWords * sizeof(uint32_t) == 5577088, "the documented size of the fixed scratch");

static __device__ __align__(256) uint32_t g_noalloc_scratch[kNaWords];

// Device address of g_noalloc_scratch and the SM count, per device.  The
// first call on a device fills them under g_noalloc_mutex, with that device
// current, and publishes `scratch` last (release); later calls read it
// without the lock (acquire), so a non-null address always comes with its
// SM count.
struct NoAllocDevice {
    std::atomic<uint32_t*> scratch{nullptr};
    int num_sms = 0;
};
constexpr int kNoAllocMaxDevices = 64;
NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];
std::mutex g_noalloc_mutex;

rt_status noalloc_setup(rt_ctx* ctx, int dev, NoAllocDevice& D, uint32_t** out) {
    uint32_t* S = D.scratch.load(std::memory_order_acquire);
    if (S) {
        *out = S;
        return RT_OK;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    S = D.scratch.load(std::memory_order_acquire);
    if (!S) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return rt_fail(ctx, RT_ERR_CUDA, "rt_lbvh_build_noalloc: cudaGetSymbolAddress failed: %s",
                           cudaGetErrorString(e));
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess || sms < 1)
            return rt_fail(ctx, RT_ERR_CUDA, "rt_lbvh_build_noalloc: cudaDeviceGetAttribute failed: %s",
                           cudaGetErrorString(e));
        D.num_sms = sms;
        S = static_cast<uint32_t*>(p);
        D.scratch.store(S, std::memory_order_release);
    }
    *out = S;
    return RT_OK;
}

}  // namespace

extern "C" rt_status rt_lbvh_build_noalloc(rt_ctx* ctx, void* stream, const float* d_tris, uint32_t n, uint32_t depth,
                                           uint32_t flags, rt_node* d_nodes, uint32_t* d_ids, uint32_t* d_keys,
                                           float* d_sorted_tris) {
    if (!d_tris || !d_nodes || !d_ids || !d_keys || !d_sorted_tris)
        return rt_fail(ctx, RT_ERR_INVALID, "rt_lbvh_build_noalloc: null buffer");
    if (n == 0 || depth == 0) return rt_fail(ctx, RT_ERR_INVALID, "rt_lbvh_build_noalloc: n and depth must be > 0");
    if (flags & ~RT_BUILD_CLEAR_UNREACHED)
        return rt_fail(ctx, RT_ERR_INVALID,
                       "rt_lbvh_build_noalloc: flags 0x%x: only RT_BUILD_CLEAR_UNREACHED is supported "
                       "(the compact layout needs allocated buffers)", flags);
    if (n > RT_NOALLOC_MAX_TRIS || depth > RT_NOALLOC_MAX_DEPTH)
        return rt_fail(ctx, RT_ERR_CAPACITY,
                       "rt_lbvh_build_noalloc: n=%u depth=%u exceeds the fixed scratch (at most %u triangles, depth %u)",
                       n, depth, RT_NOALLOC_MAX_TRIS, RT_NOALLOC_MAX_DEPTH);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices)
        return rt_fail(ctx, RT_ERR_CUDA, "rt_lbvh_build_noalloc: no usable current device");
    if (ctx && ctx->device != dev)
        return rt_fail(ctx, RT_ERR_INVALID, "rt_lbvh_build_noalloc: ctx is bound to device %d, the current device is %d",
                       ctx->device, dev);
    NoAllocDevice& D = g_noalloc_dev[dev];
    uint32_t* S = nullptr;
    rt_status rs = noalloc_setup(ctx, dev, D, &S);
    if (rs != RT_OK) return rs;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SceneInfo* scene = reinterpret_cast<SceneInfo*>(S + kNaScene);
    uint32_t* counters = S + kNaCounters;
    uint32_t* hist = S + kNaHist;
    float* partials = reinterpret_cast<float*>(S + kNaPartials);
    uint32_t* lookback = S + kNaLookback;
    uint32_t* scan = S + kNaScan;
    uint32_t* leaves = S + kNaLeaves;
    uint32_t* keys_alt = S + kNaKeysAlt;
    uint32_t* ids_alt = S + kNaIdsAlt;
    uint32_t* arrive = S + kNaArrive;
    // device-side errors go to the context's error word (read and cleared by
    // rt_ctx_check); without a context to a word of the array, cleared below
    uint32_t* err = ctx ? ctx->d_err : S + kNaErr;
    const uint32_t num_nodes = 1u << depth;
    // what must start at zero: the bounds ticket, the refit epoch (k_bounds
    // advances it to 1), the refit arrival words and the array's error word;
    // the other counters, histograms and look-back words are reset by k_bounds
    e = cudaMemsetAsync(counters, 0, 8 * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(arrive, 0, sizeof(uint32_t) * std::max(1u, num_nodes >> 1), st);
    if (e == cudaSuccess && !ctx) e = cudaMemsetAsync(S + kNaErr, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess)
        return rt_fail(ctx, RT_ERR_CUDA, "rt_lbvh_build_noalloc: cudaMemsetAsync failed: %s", cudaGetErrorString(e));
    const uint32_t sort_tiles = ceil_div(n, kSortTile);
    const uint32_t emit_tiles = ceil_div(n, kEmitTile);
    const uint32_t lb_words = kSortPasses * 256 * sort_tiles;
    const uint32_t bblocks =
        std::max(1u, std::min({ceil_div(3ull * n, 256), (uint32_t)D.num_sms * 4, kNoAllocBoundsBlocks}));
    k_bounds<<<bblocks, 256, 0, st>>>(d_tris, n, scene, partials, counters, hist, lookback, lb_words, d_nodes,
                                      num_nodes, (flags & RT_BUILD_CLEAR_UNREACHED) ? 1 : 0);
    const uint32_t mblocks = std::max(1u, std::min(ceil_div(n, kMortonThreads), (uint32_t)D.num_sms * 4));
    k_morton_hist<<<mblocks, kMortonThreads, 0, st>>>(d_tris, n, scene, d_keys, d_ids, hist, err);
    uint32_t *kin = d_keys, *iin = d_ids, *kout = keys_alt, *iout = ids_alt;
    for (int p = 0; p < kSortPasses; ++p) {
        k_onesweep<false><<<sort_tiles, kSortThreads, 0, st>>>(kin, iin, kout, iout, n, p, hist,
                                                        lookback + (size_t)p * 256 * sort_tiles, counters + 1 + p, err);
        std::swap(kin, kout);
        std::swap(iin, iout);
    }
    k_emit_tiles<<<emit_tiles, kEmitThreads, 0, st>>>(d_keys, n, scan, arrive, std::max(1u, num_nodes >> 1), counters + 6);
    k_emit_prefix<<<1, kPrefixThreads, 0, st>>>(scan, emit_tiles);
    k_emit_leaves<<<emit_tiles, kEmitThreads, 0, st>>>(d_keys, d_ids, d_tris, n, depth, scan, d_nodes,
                                                       reinterpret_cast<float4*>(d_sorted_tris), leaves, counters + 5, err);
    const uint32_t rblocks = std::max(1u, std::min(ceil_div(n, 256), (uint32_t)D.num_sms * 8));
    k_emit_refit<<<rblocks, 256, 0, st>>>(d_keys, reinterpret_cast<const float4*>(d_sorted_tris), n, depth, d_nodes,
                                          leaves, counters + 5, arrive, counters + 6, err);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return rt_fail(ctx, RT_ERR_CUDA, "rt_lbvh_build_noalloc: launch failed: %s", cudaGetErrorString(e));
    return RT_OK;
}

// ===========================================================================
// The sort stage on its own (rt_radix_sort): the four onesweep passes of the
// build over caller-given (key, value) pairs with caller-owned scratch.
// Scratch words: [0, 16) tile tickets (pass p at 1 + p), [16, 1040) the
// four digit histograms, then the look-back words (per pass 256 per tile and
// 256 per group of tiles: the build's grouped look-back), then the ping-pong
// keys and values (n each, 16-byte aligned).
namespace {

constexpr size_t kRsHist = 16;
constexpr size_t kRsLookback = kRsHist + 4 * 256;

size_t rs_tiles(uint32_t n) { return ((size_t)n + kSortTile - 1) / kSortTile; }
size_t rs_pass_words(uint32_t n) { return 256 * (rs_tiles(n) + look_groups((uint32_t)rs_tiles(n))); }
size_t rs_alt_offset(uint32_t n) { return kRsLookback + (size_t)kSortPasses * rs_pass_words(n); }
size_t rs_words(uint32_t n) { return rs_alt_offset(n) + 2 * (((size_t)n + 3) & ~(size_t)3); }

// Digit histograms of the four passes (block-local shared-memory atomics,
// one global add per bin and block).
__global__ void __launch_bounds__(512) k_sort_hist(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* hist) {
    __shared__ uint32_t s_hist[4 * 256];
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) s_hist[i] = 0u;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = __ldg(keys + i);
#pragma unroll
        for (int p = 0; p < kSortPasses; ++p) atomicAdd(&s_hist[p * 256 + ((k >> (8 * p)) & 0xffu)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x)
        if (s_hist[i]) atomicAdd(&hist[i], s_hist[i]);
}

__global__ void k_set_word(uint32_t* p, uint32_t v) { *p = v; }

rt_status rs_prepare(rt_ctx* ctx, const uint32_t* d_keys, const uint32_t* d_values, uint32_t n, void* d_scratch,
                     size_t scratch_bytes, const char* who, uint32_t** S) {
    if (!ctx) return RT_ERR_INVALID;
    if (!d_keys || !d_values || !d_scratch) return rt_fail(ctx, RT_ERR_INVALID, "%s: null buffer", who);
    if ((reinterpret_cast<uintptr_t>(d_scratch) & 15u) != 0)
        return rt_fail(ctx, RT_ERR_INVALID, "%s: the scratch must be 16-byte aligned", who);
    if (n > kMaxTris) return rt_fail(ctx, RT_ERR_INVALID, "%s: n=%u exceeds %u", who, n, kMaxTris);
    if (scratch_bytes < rs_words(n) * sizeof(uint32_t))
        return rt_fail(ctx, RT_ERR_CAPACITY, "%s: scratch of %zu bytes, %zu needed", who, scratch_bytes,
                       rs_words(n) * sizeof(uint32_t));
    *S = static_cast<uint32_t*>(d_scratch);
    // tile tickets, histograms and look-back words start at zero
    RT_CHECK_CUDA(ctx, cudaMemsetAsync(*S, 0, sizeof(uint32_t) * rs_alt_offset(n), ctx->stream));
    const uint32_t hb_blocks = std::max(1u, std::min(ceil_div(n, 512), (uint32_t)ctx->num_sms * 4));
    k_sort_hist<<<hb_blocks, 512, 0, ctx->stream>>>(d_keys, n, *S + kRsHist);
    RT_CHECK_LAUNCH(ctx, "k_sort_hist");
    return RT_OK;
}

}  // namespace

extern "C" size_t rt_radix_sort_scratch_bytes(uint32_t n) { return rs_words(n) * sizeof(uint32_t); }

extern "C" rt_status rt_radix_sort(rt_ctx* ctx, uint32_t* d_keys, uint32_t* d_values, uint32_t n, void* d_scratch,
                                   size_t scratch_bytes) {
    if (!ctx) return RT_ERR_INVALID;
    if (n == 0) return RT_OK;
    uint32_t* S = nullptr;
    rt_status s = rs_prepare(ctx, d_keys, d_values, n, d_scratch, scratch_bytes, "rt_radix_sort", &S);
    if (s != RT_OK) return s;
    const uint32_t tiles = (uint32_t)rs_tiles(n);
    uint32_t* kalt = S + rs_alt_offset(n);
    uint32_t* valt = kalt + (((size_t)n + 3) & ~(size_t)3);
    uint32_t *kin = d_keys, *iin = d_values, *kout = kalt, *iout = valt;
    for (int p = 0; p < kSortPasses; ++p) {
        k_onesweep<false, true><<<tiles, kSortThreads, 0, ctx->stream>>>(kin, iin, kout, iout, n, p, S + kRsHist,
                                                                         S + kRsLookback + (size_t)p * rs_pass_words(n),
                                                                         S + 1 + p, ctx->d_err);
        RT_CHECK_LAUNCH(ctx, "k_onesweep");
        std::swap(kin, kout);
        std::swap(iin, iout);
    }
    return RT_OK;  // four passes: the sorted pairs are back in d_keys / d_values
}

extern "C" rt_status rt_radix_sort_stall_test(rt_ctx* ctx, const uint32_t* d_keys, const uint32_t* d_values,
                                              uint32_t n, void* d_scratch, size_t scratch_bytes,
                                              uint32_t spin_limit) {
    if (!ctx) return RT_ERR_INVALID;
    if (n <= (uint32_t)kSortTile)
        return rt_fail(ctx, RT_ERR_INVALID, "rt_radix_sort_stall_test: n must exceed %d (two tiles)", kSortTile);
    if (spin_limit == 0) return rt_fail(ctx, RT_ERR_INVALID, "rt_radix_sort_stall_test: spin_limit must be > 0");
    uint32_t* S = nullptr;
    rt_status s = rs_prepare(ctx, d_keys, d_values, n, d_scratch, scratch_bytes, "rt_radix_sort_stall_test", &S);
    if (s != RT_OK) return s;
    const uint32_t tiles = (uint32_t)rs_tiles(n);
    uint32_t* kalt = S + rs_alt_offset(n);
    uint32_t* valt = kalt + (((size_t)n + 3) & ~(size_t)3);
    // the pass's tile tickets start at 1: tiles 1 .. tiles-1 run and tile 0
    // never publishes its digit counts, so the other tiles of its group give
    // up waiting for them after spin_limit polls (the grouped look-back of
    // rt_radix_sort and the build; the group's last tile then publishes a
    // group prefix, and later groups finish)
    k_set_word<<<1, 1, 0, ctx->stream>>>(S + 1, 1u);
    RT_CHECK_LAUNCH(ctx, "k_set_word");
    k_onesweep<false, true><<<tiles - 1, kSortThreads, 0, ctx->stream>>>(d_keys, d_values, kalt, valt, n, 0,
                                                                         S + kRsHist, S + kRsLookback, S + 1,
                                                                         ctx->d_err, nullptr, 0u, spin_limit);
    RT_CHECK_LAUNCH(ctx, "k_onesweep");
    return RT_OK;
}

// ===========================================================================
// Batched build: S independent scenes (S <= 256) built by one pass of the
// build kernels over their concatenated soups.  Scene s's triangles are
// [tri_off[s], tri_off[s+1]); its tree is the single-scene tree of those
// triangles, stored in its own heap of 1 << depth slots at node_off[s], with
// PrimPos and the ordered ids local to the scene.
//   kb_init          per-scene bounds reset, scratch reset, epoch
//   kb_bounds        per-scene bounds over host-made one-scene chunks
//   kb_morton_hist   codes with each scene's own Morton parameters
//   k_onesweep x4+1  four code passes, then a stable pass on the scene
//   kb_emit_tiles / k_emit_prefix / kb_emit_leaves
//                    the record scans with a separator record (bit 31) at
//                    every scene boundary, so no scan crosses two scenes
//   kb_emit_refit    the per-leaf refit walk in each scene's heap
namespace {

constexpr uint32_t kChunkTris = 4096;
constexpr int kSepBit = 31;

__device__ __forceinline__ void atomic_min_f(float* a, float v) {
    v = fadd(v, 0.0f);  // -0 -> +0
    if (v >= 0.0f) atomicMin(reinterpret_cast<int*>(a), __float_as_int(v));
    else atomicMax(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float* a, float v) {
    v = fadd(v, 0.0f);
    if (v >= 0.0f) atomicMax(reinterpret_cast<int*>(a), __float_as_int(v));
    else atomicMin(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}

__global__ void kb_init(float* sbounds, uint32_t S, const uint32_t* __restrict__ tri_off, uint32_t* counters,
                        uint32_t* hist, uint32_t* lookback, uint32_t lb_words, rt_node* nodes, uint32_t num_nodes,
                        int clear_nodes) {
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
    for (uint32_t i = gtid; i < 8 * S; i += gs) {
        const uint32_t c = i & 7u;
        sbounds[i] = c < 3 ? INFINITY : (c < 6 ? -INFINITY : 0.0f);
    }
    for (uint32_t i = gtid; i < 5 * 256; i += gs) {
        const uint32_t s = i - 4 * 256;
        hist[i] = (i >= 4 * 256 && s < S) ? tri_off[s + 1] - tri_off[s] : 0u;  // pass 4: scene sizes
    }
    for (uint32_t i = gtid; i < lb_words; i += gs) lookback[i] = 0u;
    if (gtid < 6) counters[gtid] = 0u;
    if (gtid == 6) {
        const uint32_t e = counters[6] + 1u;
        counters[6] = e ? e : 1u;
    }
    if (clear_nodes)
        for (uint32_t i = gtid; i < num_nodes; i += gs) {
            rt_node s;
            s.min[0] = s.min[1] = s.min[2] = 0.0f;
            s.max[0] = s.max[1] = s.max[2] = 0.0f;
            s.prim_count = RT_NODE_SENTINEL;
            s.prim_pos = RT_NODE_SENTINEL;
            nodes[i] = s;
        }
}

__global__ void __launch_bounds__(256) kb_bounds(const float* __restrict__ tris, const uint32_t* __restrict__ chunks,
                                                 float* sbounds, uint32_t* err) {
    const uint32_t s = chunks[3 * blockIdx.x], beg = chunks[3 * blockIdx.x + 1], end = chunks[3 * blockIdx.x + 2];
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    uint32_t bad = 0;
    for (size_t v = 3 * (size_t)beg + threadIdx.x; v < 3 * (size_t)end; v += blockDim.x) {
        const float x = __ldg(tris + 3 * v), y = __ldg(tris + 3 * v + 1), z = __ldg(tris + 3 * v + 2);
        bad |= !(isfinite(x) && isfinite(y) && isfinite(z));
        mn[0] = fminf(mn[0], x); mn[1] = fminf(mn[1], y); mn[2] = fminf(mn[2], z);
        mx[0] = fmaxf(mx[0], x); mx[1] = fmaxf(mx[1], y); mx[2] = fmaxf(mx[2], z);
    }
    for (int off = 16; off > 0; off >>= 1) {
        for (int c = 0; c < 3; ++c) {
            mn[c] = fminf(mn[c], __shfl_xor_sync(kFull, mn[c], off));
            mx[c] = fmaxf(mx[c], __shfl_xor_sync(kFull, mx[c], off));
        }
        bad |= __shfl_xor_sync(kFull, bad, off);
    }
    __shared__ float s_red[8][6];
    __shared__ uint32_t s_bad[8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        for (int c = 0; c < 3; ++c) { s_red[w][c] = mn[c]; s_red[w][3 + c] = mx[c]; }
        s_bad[w] = bad;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int c = threadIdx.x;
        float r = s_red[0][c];
        for (int ww = 1; ww < (int)(blockDim.x / 32); ++ww) r = c < 3 ? fminf(r, s_red[ww][c]) : fmaxf(r, s_red[ww][c]);
        if (c < 3) atomic_min_f(sbounds + 8 * s + c, r);
        else atomic_max_f(sbounds + 8 * s + c, r);
    }
    if (threadIdx.x == 6) {
        uint32_t b = 0;
        for (int ww = 0; ww < (int)(blockDim.x / 32); ++ww) b |= s_bad[ww];
        if (b) atomicOr(err, RT_DEVERR_NONFINITE);
    }
}

__global__ void __launch_bounds__(256) kb_morton_hist(const float* __restrict__ tris, const uint32_t* __restrict__ chunks,
                                                      const float* __restrict__ sbounds, uint32_t* __restrict__ keys,
                                                      uint32_t* __restrict__ ids, uint32_t* hist) {
    __shared__ uint32_t s_hist[4][256];
    __shared__ float s_par[6];
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) (&s_hist[0][0])[i] = 0u;
    const uint32_t s = chunks[3 * blockIdx.x], beg = chunks[3 * blockIdx.x + 1], end = chunks[3 * blockIdx.x + 2];
    if (threadIdx.x < 3) {  // the scene's Morton parameters, as k_bounds derives them (LBVH.cpp:521-526)
        const int c = threadIdx.x;
        const float lo3 = fmul(3.0f, sbounds[8 * s + c]);
        const float mx3 = fmul(3.0f, sbounds[8 * s + 3 + c]);
        s_par[c] = lo3;
        s_par[3 + c] = fdiv(1024.0f, fsub(mx3, lo3));
    }
    __syncthreads();
    for (uint32_t base = beg; base < end; base += blockDim.x) {
        const uint32_t k = base + threadIdx.x;
        const bool valid = k < end;
        uint32_t code = 0;
        if (valid) {
            const float* t = tris + 9 * (size_t)k;
            uint32_t q[3];
            for (int c = 0; c < 3; ++c) {
                const float cen = fadd(fadd(__ldg(t + c), __ldg(t + 3 + c)), __ldg(t + 6 + c));
                q[c] = quantize(cen, s_par[c], s_par[3 + c]);
            }
            code = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
            keys[k] = code;
            ids[k] = k;
        }
        if (valid) {
#pragma unroll
            for (int p = 0; p < kSortPasses; ++p) atomicAdd(&s_hist[p][(code >> (8 * p)) & 0xffu], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) {
        const uint32_t v = (&s_hist[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

// Boundary deltas of a thread's chunk with a separator record at each
// scene boundary (off: S + 1 scene offsets in shared memory).
__device__ __forceinline__ void load_chunk_b(const uint32_t* __restrict__ keys, uint32_t n, uint32_t s,
                                             const uint32_t* off, uint32_t S, EmitChunk& e) {
    const uint32_t prev = (s >= 1 && s - 1 < n) ? __ldg(keys + s - 1) : 0u;
#pragma unroll
    for (int q = 0; q <= kEmitItems; ++q) e.c[q] = (s + q < n) ? __ldg(keys + s + q) : 0u;
    uint32_t sc = scene_of(off, S, s < n ? s : n - 1);
    e.dl[0] = (s >= 1 && s < n) ? (s == off[sc] ? kSepBit : delta_of(prev, e.c[0])) : -1;
    uint32_t nb = off[sc + 1];
#pragma unroll
    for (int q = 0; q < kEmitItems; ++q) {
        const uint32_t i = s + q;
        int d = -1;
        if (i + 1 < n) {
            if (i + 1 == nb) {
                d = kSepBit;
                ++sc;
                nb = off[sc + 1];
            } else {
                d = delta_of(e.c[q], e.c[q + 1]);
            }
        }
        e.dl[q + 1] = d;
        e.r[q] = (d >= 0) ? (1u << d) : 0u;
    }
}

__global__ void __launch_bounds__(kEmitThreads) kb_emit_tiles(const uint32_t* __restrict__ keys, uint32_t n,
                                                              const uint32_t* __restrict__ tri_off, uint32_t S,
                                                              uint32_t* scan, uint32_t* arrive, uint32_t arrive_words,
                                                              const uint32_t* epoch_word) {
    __shared__ uint32_t s_f[8], s_b[8];
    __shared__ uint32_t s_off[kMaxBatchScenes + 1];
    for (uint32_t q = threadIdx.x; q <= S; q += blockDim.x) s_off[q] = tri_off[q];
    if (*epoch_word == 1u)
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < arrive_words; i += gridDim.x * blockDim.x)
            arrive[i] = 0u;
    __syncthreads();
    const uint32_t s = blockIdx.x * kEmitTile + threadIdx.x * kEmitItems;
    EmitChunk e;
    load_chunk_b(keys, n, s, s_off, S, e);
    uint32_t af = 0, ab = 0;
#pragma unroll
    for (int q = 0; q < kEmitItems; ++q) af = rec_fwd(af, e.r[q]);
#pragma unroll
    for (int q = kEmitItems - 1; q >= 0; --q) ab = rec_bwd(e.r[q], ab);
    af = warp_reduce_ordered<true>(af);
    ab = warp_reduce_ordered<false>(ab);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { s_f[w] = af; s_b[w] = ab; }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t tf = 0, tb = 0;
        for (int q = 0; q < kEmitThreads / 32; ++q) tf = rec_fwd(tf, s_f[q]);
        for (int q = kEmitThreads / 32 - 1; q >= 0; --q) tb = rec_bwd(s_b[q], tb);
        scan[4 * blockIdx.x + 0] = tf;
        scan[4 * blockIdx.x + 1] = tb;
    }
}

__global__ void __launch_bounds__(kEmitThreads) kb_emit_leaves(
    const uint32_t* __restrict__ keys, const uint32_t* __restrict__ ids, const float* __restrict__ tris, uint32_t n,
    const uint32_t* __restrict__ tri_off, uint32_t S, uint32_t depth, const uint32_t* __restrict__ scan,
    rt_node* nodes, float4* __restrict__ sorted_tris, uint32_t* __restrict__ ids_local, uint32_t* leaf_list,
    uint32_t* leaf_count, uint32_t* err) {
    __shared__ uint32_t s_f[8], s_b[8];
    __shared__ uint32_t s_off[kMaxBatchScenes + 1];
    for (uint32_t q = threadIdx.x; q <= S; q += blockDim.x) s_off[q] = tri_off[q];
    __syncthreads();
    const uint32_t s = blockIdx.x * kEmitTile + threadIdx.x * kEmitItems;
    EmitChunk e;
    load_chunk_b(keys, n, s, s_off, S, e);
    uint32_t af = 0, ab = 0;
#pragma unroll
    for (int q = 0; q < kEmitItems; ++q) af = rec_fwd(af, e.r[q]);
#pragma unroll
    for (int q = kEmitItems - 1; q >= 0; --q) ab = rec_bwd(e.r[q], ab);
    uint32_t pre, suf;
    block_scan_records(af, ab, &pre, &suf, s_f, s_b);
    uint32_t L[kEmitItems + 1], R[kEmitItems + 1];
    L[0] = rec_fwd(scan[4 * blockIdx.x + 2], pre);
    R[kEmitItems] = rec_bwd(suf, scan[4 * blockIdx.x + 3]);
#pragma unroll
    for (int q = 0; q < kEmitItems; ++q) L[q + 1] = rec_fwd(L[q], e.r[q]);
#pragma unroll
    for (int q = kEmitItems - 1; q >= 0; --q) R[q] = rec_bwd(e.r[q], R[q + 1]);

    const int leaf_depth = (int)depth - 1;
    const int lane = threadIdx.x & 31;
    uint32_t sc = scene_of(s_off, S, s < n ? s : n - 1);
#pragma unroll
    for (int q = 0; q < kEmitItems; ++q) {
        const uint32_t k = s + q;
        const bool valid = k < n;
        bool head = false;
        uint32_t h = 0;
        if (valid) {
            while (k >= s_off[sc + 1]) ++sc;
            const uint32_t first = s_off[sc], last = s_off[sc + 1] - 1;
            const uint32_t anc = (L[q] | R[q]) & 0x3fffffffu;  // drop the separator record
            const uint32_t code = e.c[q];
            int dep = __popc(anc);
            uint32_t m = anc;
            while (dep > leaf_depth) { m &= m - 1u; --dep; }
            h = 1u;
            while (m) {
                const int b = hb(m);
                h = (h << 1) | ((code >> b) & 1u);
                m ^= 1u << b;
            }
            const int dprev = e.dl[q], dcur = e.dl[q + 1];
            head = (k == first) || (dprev >= 0 && __popc(keep_above(anc, dprev)) < leaf_depth);
            const bool tail = (k == last) || (dcur >= 0 && __popc(keep_above(anc, dcur)) < leaf_depth);
            rt_node* tree = nodes + ((size_t)sc << depth);
            if (head) tree[h].prim_pos = (int32_t)(k - first);
            if (tail) tree[h].prim_count = (int32_t)(k - first);
            h |= sc << 23;  // leaf entry: scene and heap slot
        }
        const uint32_t hm = __ballot_sync(kFull, head);
        uint32_t basei = 0;
        if (lane == 0 && hm) basei = atomicAdd(leaf_count, (uint32_t)__popc(hm));
        basei = __shfl_sync(kFull, basei, 0);
        if (head) leaf_list[basei + __popc(hm & lanemask_lt())] = h;
    }
    const uint32_t tbase = blockIdx.x * kEmitTile;
#pragma unroll 2
    for (int q = 0; q < kEmitItems; ++q) {
        const uint32_t k = tbase + q * kEmitThreads + threadIdx.x;
        if (k < n) {
            uint32_t id = __ldg(ids + k);
            const uint32_t sk = scene_of(s_off, S, k);
            if (id < s_off[sk] || id >= s_off[sk + 1]) {  // only after a failed sort (look-back timeout)
                atomicOr(err, RT_DEVERR_BOUNDS);
                id = s_off[sk];
            }
            const uint32_t local = id - s_off[sk];
            const float* tp = tris + 9 * (size_t)id;
            float v[9];
#pragma unroll
            for (int c = 0; c < 9; ++c) v[c] = __ldg(tp + c);
            sorted_tris[3 * (size_t)k + 0] = make_float4(v[0], v[1], v[2], __int_as_float((int)local));
            sorted_tris[3 * (size_t)k + 1] = make_float4(v[3], v[4], v[5], 0.0f);
            sorted_tris[3 * (size_t)k + 2] = make_float4(v[6], v[7], v[8], 0.0f);
            ids_local[k] = local;
        }
    }
}

__global__ void __launch_bounds__(256) kb_emit_refit(const uint32_t* __restrict__ keys, const float4* sorted_tris,
                                                     const uint32_t* __restrict__ tri_off, uint32_t depth,
                                                     rt_node* nodes, const uint32_t* __restrict__ leaf_list,
                                                     const uint32_t* leaf_count, uint32_t n, uint32_t* arrive,
                                                     const uint32_t* epoch_word, uint32_t* err) {
    const uint32_t nleaves = min(*leaf_count, n);
    const uint32_t epoch = *epoch_word;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t base = warp * 32; base < nleaves; base += nwarps * 32) {
        const uint32_t li = base + lane;
        uint32_t sc = 0, h = 0, toff = 0, ns = 0;
        int32_t pos = 0, end = -1;
        bool ok = false;
        if (li < nleaves) {
            const uint32_t e = leaf_list[li];
            sc = e >> 23;
            h = e & ((1u << 23) - 1u);
            toff = __ldg(tri_off + sc);
            ns = __ldg(tri_off + sc + 1) - toff;
            ok = leaf_range(h, nodes + ((size_t)sc << depth), ns, depth, &pos, &end);
            if (!ok) atomicOr(err, RT_DEVERR_BOUNDS);
        }
        float mn[3], mx[3];
        leaf_boxes((int64_t)toff + pos, ok ? end - pos + 1 : 0, sorted_tris, mn, mx);
        if (ok)
            refit_walk(h, pos, end, mn, mx, keys + toff, ns, depth, nodes + ((size_t)sc << depth),
                       arrive + ((size_t)sc << (depth - 1)), epoch, err);
    }
}

}  // namespace

extern "C" rt_status rt_batch_destroy(rt_batch* b) {
    if (!b) return RT_OK;
    if (b->graph_refs > 0) {  // a captured frame still points into b: the last frame destroy frees it
        b->destroy_pending = true;
        return RT_OK;
    }
    free_batch(b);
    return RT_OK;
}

void free_batch(rt_batch* b) {
    void* ptrs[] = {b->tri_off, b->node_off, b->chunks, b->nodes, b->keys, b->ids, b->keys_alt, b->ids_alt,
                    b->ids_local, b->sorted_tris, b->sbounds, b->counters, b->hist, b->lookback, b->scan,
                    b->leaf_list, b->arrive, b->cams, b->lights, b->s_lists, b->s_rays};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete b;
}

extern "C" rt_status rt_batch_create(rt_ctx* ctx, uint32_t n_scenes, const uint32_t* h_tri_counts, uint32_t depth,
                                     rt_batch** out) {
    if (!ctx || !out) return RT_ERR_INVALID;
    *out = nullptr;
    if (!h_tri_counts) return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_create: null counts");
    if (n_scenes == 0 || n_scenes > RT_BATCH_MAX_SCENES)
        return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_create: 1 to %u scenes", RT_BATCH_MAX_SCENES);
    if (depth < 1 || depth > RT_BATCH_MAX_DEPTH)
        return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_create: depth must be in [1, %u]", RT_BATCH_MAX_DEPTH);
    uint64_t total = 0;
    for (uint32_t s = 0; s < n_scenes; ++s) {
        if (h_tri_counts[s] == 0) return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_create: scene %u is empty", s);
        total += h_tri_counts[s];
    }
    if (total > kMaxTris) return rt_fail(ctx, RT_ERR_CAPACITY, "rt_batch_create: %llu triangles in all", (unsigned long long)total);
    RT_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
    rt_batch* b = new rt_batch();
    b->S = n_scenes;
    b->depth = depth;
    b->total = (uint32_t)total;
    b->h_tri_off.resize(n_scenes + 1);
    std::vector<uint32_t> node_off(n_scenes + 1), chunks;
    b->h_tri_off[0] = 0;
    for (uint32_t s = 0; s < n_scenes; ++s) {
        b->h_tri_off[s + 1] = b->h_tri_off[s] + h_tri_counts[s];
        for (uint32_t c = b->h_tri_off[s]; c < b->h_tri_off[s + 1]; c += kChunkTris) {
            chunks.push_back(s);
            chunks.push_back(c);
            chunks.push_back(std::min(c + kChunkTris, b->h_tri_off[s + 1]));
        }
    }
    for (uint32_t s = 0; s <= n_scenes; ++s) node_off[s] = s << depth;
    b->nchunks = (uint32_t)(chunks.size() / 3);
    const size_t n = total;
    const size_t num_nodes = (size_t)n_scenes << depth;
    const uint32_t sort_tiles = ceil_div(n, kSortTile), emit_tiles = ceil_div(n, kEmitTile);
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    alloc((void**)&b->tri_off, 4 * (n_scenes + 1));
    alloc((void**)&b->node_off, 4 * (n_scenes + 1));
    alloc((void**)&b->chunks, 4 * chunks.size());
    alloc((void**)&b->nodes, sizeof(rt_node) * num_nodes);
    alloc((void**)&b->keys, 4 * n);
    alloc((void**)&b->ids, 4 * n);
    alloc((void**)&b->keys_alt, 4 * n);
    alloc((void**)&b->ids_alt, 4 * n);
    alloc((void**)&b->ids_local, 4 * n);
    alloc((void**)&b->sorted_tris, sizeof(float4) * 3 * n);
    alloc((void**)&b->sbounds, sizeof(float) * 8 * n_scenes);
    alloc((void**)&b->counters, sizeof(uint32_t) * 8);
    alloc((void**)&b->hist, sizeof(uint32_t) * 5 * 256);
    alloc((void**)&b->lookback, sizeof(uint32_t) * 5 * 256 * (size_t)sort_tiles);
    alloc((void**)&b->scan, sizeof(uint32_t) * 4 * (size_t)emit_tiles);
    alloc((void**)&b->leaf_list, 4 * n);
    alloc((void**)&b->arrive, sizeof(uint32_t) * (num_nodes >> 1));
    alloc((void**)&b->cams, sizeof(rt_camera) * n_scenes);
    alloc((void**)&b->lights, sizeof(float) * 3 * n_scenes);
    if (e == cudaSuccess) e = cudaMemcpy(b->tri_off, b->h_tri_off.data(), 4 * (n_scenes + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->node_off, node_off.data(), 4 * (n_scenes + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->chunks, chunks.data(), 4 * chunks.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(b->counters, 0, sizeof(uint32_t) * 8);
    if (e == cudaSuccess) e = cudaMemset(b->arrive, 0, sizeof(uint32_t) * (num_nodes >> 1));
    if (e == cudaSuccess) e = cudaMemset(b->nodes, 0, sizeof(rt_node) * num_nodes);
    if (e != cudaSuccess) {
        rt_batch_destroy(b);
        return rt_fail(ctx, RT_ERR_CUDA, "rt_batch_create: allocation failed: %s", cudaGetErrorString(e));
    }
    *out = b;
    return RT_OK;
}

extern "C" rt_status rt_batch_build(rt_ctx* ctx, rt_batch* b, const float* d_tris, uint32_t flags) {
    if (!ctx) return RT_ERR_INVALID;
    if (!b || !d_tris) return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_build: null argument");
    cudaStream_t st = ctx->stream;
    const uint32_t n = b->total, S = b->S;
    const uint32_t sort_tiles = ceil_div(n, kSortTile), emit_tiles = ceil_div(n, kEmitTile);
    const uint32_t lb_words = 5 * 256 * sort_tiles;
    const uint32_t num_nodes = S << b->depth;
    kb_init<<<std::max(1u, std::min(ceil_div(std::max(lb_words, num_nodes), 256), (uint32_t)ctx->num_sms * 8)), 256, 0,
              st>>>(b->sbounds, S, b->tri_off, b->counters, b->hist, b->lookback, lb_words, b->nodes, num_nodes,
                    (flags & RT_BUILD_CLEAR_UNREACHED) ? 1 : 0);
    RT_CHECK_LAUNCH(ctx, "kb_init");
    kb_bounds<<<b->nchunks, 256, 0, st>>>(d_tris, b->chunks, b->sbounds, ctx->d_err);
    RT_CHECK_LAUNCH(ctx, "kb_bounds");
    kb_morton_hist<<<b->nchunks, 256, 0, st>>>(d_tris, b->chunks, b->sbounds, b->keys, b->ids, b->hist);
    RT_CHECK_LAUNCH(ctx, "kb_morton_hist");
    uint32_t *kin = b->keys, *iin = b->ids, *kout = b->keys_alt, *iout = b->ids_alt;
    for (int p = 0; p < 5; ++p) {
        uint32_t* lbp = b->lookback + (size_t)p * 256 * sort_tiles;
        if (p < 4)
            k_onesweep<false><<<sort_tiles, kSortThreads, 0, st>>>(kin, iin, kout, iout, n, p, b->hist, lbp,
                                                                   b->counters + p, ctx->d_err);
        else
            k_onesweep<true><<<sort_tiles, kSortThreads, 0, st>>>(kin, iin, kout, iout, n, p, b->hist, lbp,
                                                                  b->counters + p, ctx->d_err, b->tri_off, S);
        RT_CHECK_LAUNCH(ctx, "k_onesweep");
        std::swap(kin, kout);
        std::swap(iin, iout);
    }
    b->res_keys = kin;  // five passes: the sorted pairs are in the alternate buffers
    b->res_ids = iin;
    kb_emit_tiles<<<emit_tiles, kEmitThreads, 0, st>>>(kin, n, b->tri_off, S, b->scan, b->arrive, num_nodes >> 1,
                                                       b->counters + 6);
    RT_CHECK_LAUNCH(ctx, "kb_emit_tiles");
    k_emit_prefix<<<1, kPrefixThreads, 0, st>>>(b->scan, emit_tiles);
    RT_CHECK_LAUNCH(ctx, "k_emit_prefix");
    kb_emit_leaves<<<emit_tiles, kEmitThreads, 0, st>>>(kin, iin, d_tris, n, b->tri_off, S, b->depth, b->scan, b->nodes,
                                                        b->sorted_tris, b->ids_local, b->leaf_list, b->counters + 5,
                                                        ctx->d_err);
    RT_CHECK_LAUNCH(ctx, "kb_emit_leaves");
    // one thread per leaf at most (no persistent cap), in blocks of two warps:
    // a warp's time is its longest climb, and fresh warps then take the SM
    // slots of finished ones instead of each thread walking ~40 leaves in
    // turn (256 random-soup scenes, 11.5 M triangles: 3.89 -> 3.31 ms a
    // batched build with 256-thread blocks, 3.15 ms with 64)
    const uint32_t rblocks = std::max(1u, ceil_div(n, 64));
    kb_emit_refit<<<rblocks, 64, 0, st>>>(kin, b->sorted_tris, b->tri_off, b->depth, b->nodes, b->leaf_list,
                                           b->counters + 5, n, b->arrive, b->counters + 6, ctx->d_err);
    RT_CHECK_LAUNCH(ctx, "kb_emit_refit");
    b->src_tris = d_tris;
    b->built = true;
    return RT_OK;
}

extern "C" rt_status rt_batch_view_get(const rt_batch* b, uint32_t scene, rt_lbvh_view* v) {
    if (!b || !v || scene >= b->S || !b->built) return RT_ERR_INVALID;
    const uint32_t off = b->h_tri_off[scene];
    v->nodes = b->nodes + ((size_t)scene << b->depth);
    v->ids = b->ids_local + off;
    v->keys = b->res_keys + off;
    v->sorted_tris = reinterpret_cast<const float*>(b->sorted_tris + 3 * (size_t)off);
    v->n = b->h_tri_off[scene + 1] - off;
    v->depth = b->depth;
    v->num_nodes = 1u << b->depth;
    v->node_size = (uint32_t)sizeof(rt_node);
    return RT_OK;
}

extern "C" uint32_t rt_batch_scene_count(const rt_batch* b) { return b ? b->S : 0u; }

extern "C" rt_status rt_batch_download(rt_ctx* ctx, const rt_batch* b, uint32_t scene, rt_node* h_nodes,
                                       uint32_t* h_ids, uint32_t* h_keys) {
    if (!ctx) return RT_ERR_INVALID;
    rt_lbvh_view v;
    if (rt_batch_view_get(b, scene, &v) != RT_OK)
        return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_download: no built scene %u", scene);
    cudaStream_t st = ctx->stream;
    if (h_nodes)
        RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_nodes, v.nodes, sizeof(rt_node) * v.num_nodes, cudaMemcpyDeviceToHost, st));
    if (h_ids) RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_ids, v.ids, 4 * (size_t)v.n, cudaMemcpyDeviceToHost, st));
    if (h_keys) RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_keys, v.keys, 4 * (size_t)v.n, cudaMemcpyDeviceToHost, st));
    RT_CHECK_CUDA(ctx, cudaStreamSynchronize(st));
    return RT_OK;
}
