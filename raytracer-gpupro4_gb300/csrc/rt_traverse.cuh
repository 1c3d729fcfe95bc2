// rt_traverse.cuh -- closest-hit / any-hit traversal of the heap-layout LBVH.
//
// Restates LBVH_IntersectP (RayTracerCS/Shaders/AccelerationStructures/
// LBVH.hlsl:363-440) and LBVH::IntersectP (LBVH.cpp:919-1039) as a
// stack-based depth-first walk: at an internal node both children (heap
// slots 2i, 2i+1: one 64-byte line) are box-tested, the near child is
// entered first and a hit far child is pushed with its entry distance; a
// popped node is entered only if that distance still does not exceed the
// closest hit (the reference's pruning, LBVH.cpp:992).  The near child is
// chosen by the ray direction on the node's split axis; the reference
// indexes signo[] with the stored axis field (LBVH.cpp:1033), which
// build_recursive sets one axis past the split axis, so it orders children
// arbitrarily.  Order changes only the number of tests, not the closest hit:
// ties at equal t keep the smaller triangle id.  The CPU oracle walks the
// same order and counts the same tests.
//
// Box test = RayBoxInterval (LBVH.cpp:634-659), triangle test =
// RayTriangleTest (AccelerationStructure.h:70-97), both in the reference's
// operation order without contraction.  The excluded triangle is skipped
// (LBVH.hlsl:415).
#pragma once
#include "rt_internal.cuh"

namespace rt {

constexpr int kStackSize = 32;  // > kMaxDepth
constexpr int kSerialLanes = 16;  // leaf phase: lanes that must share a serial step

// Bounds of the arrays a traversal may touch; an index outside them (only
// possible with a corrupt tree) sets RT_DEVERR_BOUNDS and stops that ray.
struct TreeRef {
    const rt_node* __restrict__ nodes;
    const float4* __restrict__ tris;
    uint32_t num_nodes;
    uint32_t n;
    uint32_t* err;
    // compact layout: the children of an internal node are the pair at
    // slots PrimPos, PrimPos + 1 (even), not at heap slots 2i, 2i + 1
    bool compact;
    // added to every leaf's PrimPos by the per-lane walk: one scene of a
    // batch read through the batch's whole sorted-triangle array (its
    // triangles are [tri_base, n)); 0 otherwise, and 0 for the warp- and
    // block-per-ray walks
    uint32_t tri_base;
};

// First slot of the children pair of internal node `node` whose record's
// fourth float4 lane (PrimPos) is pp.
__device__ __forceinline__ uint32_t child_pair(const TreeRef& tr, uint32_t node, float pp) {
    return tr.compact ? (uint32_t)__float_as_int(pp) : node << 1;
}

struct RayState {
    f3 o, d, inv;
    uint32_t sgn;  // bit c set when d[c] < 0 (signo[] of LBVH.cpp:983-985)
    int exclude;
    float tmax;
    bool exact;  // some 1/d is infinite: use the reference's NaN-sensitive min/max
};

__device__ __forceinline__ RayState make_ray(f3 o, f3 d, float tmax, int exclude) {
    RayState r;
    r.o = o;
    r.d = d;
    r.inv = mk3(fdiv(1.0f, d.x), fdiv(1.0f, d.y), fdiv(1.0f, d.z));
    r.sgn = (uint32_t)(d.x < 0.0f) | ((uint32_t)(d.y < 0.0f) << 1) | ((uint32_t)(d.z < 0.0f) << 2);
    r.exclude = exclude;
    r.tmax = tmax;
    r.exact = isinf(r.inv.x) || isinf(r.inv.y) || isinf(r.inv.z);
    return r;
}

template <bool EXACT>
__device__ __forceinline__ float vmin(float a, float b) { return EXACT ? smin(a, b) : fminf(a, b); }
template <bool EXACT>
__device__ __forceinline__ float vmax(float a, float b) { return EXACT ? smax(a, b) : fmaxf(a, b); }

// Returns true when the reference would enter the node: not (T1 < 0 or
// T0 > best_t) after the empty-interval reset.  With every 1/d finite no
// product is NaN and fminf/fmaxf equal std::min/std::max.
template <bool EXACT>
__device__ __forceinline__ bool box_enter(const RayState& r, float mnx, float mny, float mnz, float mxx, float mxy,
                                          float mxz, float best_t, float* t0out) {
    const float dMx = fmul(fsub(mxx, r.o.x), r.inv.x), dMy = fmul(fsub(mxy, r.o.y), r.inv.y),
                dMz = fmul(fsub(mxz, r.o.z), r.inv.z);
    const float dmx = fmul(fsub(mnx, r.o.x), r.inv.x), dmy = fmul(fsub(mny, r.o.y), r.inv.y),
                dmz = fmul(fsub(mnz, r.o.z), r.inv.z);
    float t0 = vmin<EXACT>(dmx, dMx);
    float t1 = vmax<EXACT>(dmx, dMx);
    t0 = vmax<EXACT>(t0, vmin<EXACT>(dmy, dMy));
    t1 = vmin<EXACT>(t1, vmax<EXACT>(dmy, dMy));
    t0 = vmax<EXACT>(t0, vmin<EXACT>(dmz, dMz));
    t1 = vmin<EXACT>(t1, vmax<EXACT>(dmz, dMz));
    if (t0 > t1) { t0 = -1.0f; t1 = -1.0f; }
    *t0out = t0;
    return !(t1 < 0.0f) && !(t0 > best_t);
}

struct Hit {
    int id;
    float u, v, t;
};

// Moller-Trumbore, AccelerationStructure.h:70-97.
__device__ __forceinline__ bool tri_test(const RayState& r, float4 a, float4 b, float4 c, float* u, float* v,
                                         float* t) {
    const f3 A = mk3(a.x, a.y, a.z);
    const f3 E1 = sub3(mk3(b.x, b.y, b.z), A);
    const f3 E2 = sub3(mk3(c.x, c.y, c.z), A);
    const f3 P = cross3(r.d, E2);
    float det = dot3(E1, P);
    det = __frcp_rn(det);  // 1.0f / det, correctly rounded
    const f3 T = sub3(r.o, A);
    const float uu = fmul(dot3(T, P), det);
    const f3 Q = cross3(T, E1);
    const float vv = fmul(dot3(r.d, Q), det);
    const float tt = fmul(dot3(E2, Q), det);
    *u = uu;
    *v = vv;
    *t = tt;
    return (uu >= 0.0f) && (uu <= 1.0f) && (vv >= 0.0f) && (fadd(uu, vv) <= 1.0f) && (tt >= 0.0f);
}

struct NodeBox {
    float4 a, b;  // a = min.xyz,max.x  b = max.yz,prim_count,prim_pos
};

__device__ __forceinline__ NodeBox load_node(const rt_node* __restrict__ nodes, uint32_t i) {
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    NodeBox nb;
    nb.a = __ldg(p);
    nb.b = __ldg(p + 1);
    return nb;
}

// Order key of a candidate hit: (t, id) as one unsigned 64-bit number, so
// the tie rule (smaller t, then smaller id) is an integer minimum.  Accepted
// hits have t >= 0; the sign bit is dropped so that -0 and +0 compare equal,
// as they do in the reference's float comparison.
__device__ __forceinline__ uint64_t hit_key(float t, int id) {
    return ((uint64_t)(__float_as_uint(t) & 0x7fffffffu) << 32) | (uint32_t)id;
}

__device__ __forceinline__ uint64_t shfl_u64(uint64_t v, int src) {
    const uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)v, src);
    const uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(v >> 32), src);
    return ((uint64_t)hi << 32) | lo;
}
__device__ __forceinline__ uint64_t shfl_down_u64(uint64_t v, int off) {
    const uint32_t lo = __shfl_down_sync(0xffffffffu, (uint32_t)v, off);
    const uint32_t hi = __shfl_down_sync(0xffffffffu, (uint32_t)(v >> 32), off);
    return ((uint64_t)hi << 32) | lo;
}

// Best accepted hit of one lane's ray (or of the part of a ray a lane works
// on): key = hit_key(t, id), or hit_key(tmax, 0) while nothing is accepted, so
// a candidate is accepted exactly when its key is smaller (t < tmax, and the
// tie rule at equal t).
struct Best {
    uint64_t key;
    float t, u, v;
    int id;
    uint32_t leaf;  // node whose triangles gave the hit (the reference's iRoot)
};

__device__ __forceinline__ float key_t(uint64_t key) { return __uint_as_float((uint32_t)(key >> 32)); }

// Leaf phase: the warp tests the triangles [pos, pos + cnt) of every lane's
// held leaf together.  The (lane, triangle) pairs are numbered by a prefix
// sum of the leaf sizes and processed 32 at a time, so consecutive lanes read
// consecutive triangles and a 200-triangle leaf costs 7 warp steps instead of
// 200.  A segmented minimum over hit_key gives each lane the closest accepted
// hit of its leaf; that is the result of testing the leaf's triangles in any
// order under the tie rule.  `bound` is the lane's acceptance key on entry;
// returns true when b (and the bound) improved.
template <bool STATS>
__device__ __forceinline__ bool leaf_phase(const TreeRef& tr_, const RayState& r, bool have, const NodeBox& cur,
                                           uint32_t node, uint64_t& bound, Best& b, uint32_t& ntri) {
    constexpr uint32_t kFull = 0xffffffffu;
    const float4* __restrict__ tris = tr_.tris;
    const int lane = threadIdx.x & 31;
    int cnt = 0, pos = 0;
    if (have) {
        cnt = __float_as_int(cur.b.z) >> 3;
        pos = __float_as_int(cur.b.w);
        if (pos < 0 || cnt < 0 || (uint32_t)pos + tr_.tri_base + (uint32_t)cnt > tr_.n) {
            atomicOr(tr_.err, RT_DEVERR_BOUNDS);
            cnt = 0;
        }
        pos += (int)tr_.tri_base;
    }
    ntri += (uint32_t)cnt;
    bool improved = false;
    // Serial part: while at least kSerialLanes lanes still have triangles,
    // each lane tests its own leaf's triangles (no exchange between lanes);
    // L = the largest count that many lanes reach.  The remainder of every
    // leaf (the long tails) is pooled below.
    int L = 0;
#pragma unroll
    for (int step = 32; step > 0; step >>= 1)
        if (__popc(__ballot_sync(kFull, cnt >= L + step)) >= kSerialLanes) L += step;
    if (L > 0) {
        const int ns = min(cnt, L);
        // software pipelined: the next triangle's loads are in flight while
        // the current one is tested
        const float4* tp = tris + 3 * (size_t)pos;
        float4 na = make_float4(0.f, 0.f, 0.f, 0.f), nb = na, nc = na;
        if (ns > 0) {
            na = __ldg(tp);
            nb = __ldg(tp + 1);
            nc = __ldg(tp + 2);
        }
        for (int j = 0; j < ns; ++j) {
            const float4 a = na, bb = nb, c = nc;
            if (j + 1 < ns) {
                tp += 3;
                na = __ldg(tp);
                nb = __ldg(tp + 1);
                nc = __ldg(tp + 2);
            }
            const int id = __float_as_int(a.w);
            float u, v, t;
            if (id != r.exclude && tri_test(r, a, bb, c, &u, &v, &t)) {
                const uint64_t k = hit_key(t, id);
                if (k < bound) {
                    bound = k;
                    b.key = k;
                    b.t = t;
                    b.u = u;
                    b.v = v;
                    b.id = id;
                    b.leaf = node;
                    improved = true;
                }
            }
        }
        pos += ns;
        cnt -= ns;
    }
    uint32_t incl = (uint32_t)cnt;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += y;
    }
    const uint32_t total = __shfl_sync(kFull, incl, 31);
    const uint32_t excl = incl - (uint32_t)cnt;
    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t p = base + lane;
        // owner of pair p: the first lane whose inclusive prefix exceeds p
        int o = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const uint32_t v = __shfl_sync(kFull, incl, o + step - 1);
            if (v <= p) o += step;
        }
        const uint32_t o_excl = __shfl_sync(kFull, excl, o);
        const int o_pos = __shfl_sync(kFull, pos, o);
        RayState ro;
        ro.o = mk3(__shfl_sync(kFull, r.o.x, o), __shfl_sync(kFull, r.o.y, o), __shfl_sync(kFull, r.o.z, o));
        ro.d = mk3(__shfl_sync(kFull, r.d.x, o), __shfl_sync(kFull, r.d.y, o), __shfl_sync(kFull, r.d.z, o));
        const int o_exclude = __shfl_sync(kFull, r.exclude, o);
        const uint64_t o_best = shfl_u64(bound, o);
        uint64_t key = ~0ull;
        float kt = 0.0f, ku = 0.0f, kv = 0.0f;
        if (p < total) {
            const float4* tp = tris + 3 * (size_t)(o_pos + (p - o_excl));
            const float4 a = __ldg(tp), bb = __ldg(tp + 1), c = __ldg(tp + 2);
            const int id = __float_as_int(a.w);
            float u, v, t;
            if (id != o_exclude && tri_test(ro, a, bb, c, &u, &v, &t)) {
                const uint64_t k = hit_key(t, id);
                if (k < o_best) {
                    key = k;
                    kt = t;
                    ku = u;
                    kv = v;
                }
            }
        }
        // segmented minimum of the key (lanes of one owner are contiguous),
        // carrying the lane that computed it; afterwards the first lane of
        // each owner's run holds the run's minimum and its source lane
        int src = lane;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint64_t k2 = shfl_down_u64(key, off);
            const int s2 = __shfl_down_sync(kFull, src, off);
            const int o2 = __shfl_down_sync(kFull, o, off);
            if (lane + off < 32 && o2 == o && k2 < key) {
                key = k2;
                src = s2;
            }
        }
        const bool mine = cnt > 0 && excl < base + 32 && incl > base;
        const int head = mine ? (int)(max(excl, base) - base) : lane;
        const uint64_t hk = shfl_u64(key, head);
        const int hs = __shfl_sync(kFull, src, head);
        const float ht = __shfl_sync(kFull, kt, hs);
        const float hu = __shfl_sync(kFull, ku, hs);
        const float hv = __shfl_sync(kFull, kv, hs);
        if (mine && hk < bound) {
            bound = hk;
            b.key = hk;
            b.t = ht;
            b.u = hu;
            b.v = hv;
            b.id = (int)(uint32_t)hk;
            b.leaf = node;
            improved = true;
        }
    }
    return improved;
}

// Descent of one lane from its held node to the next leaf: both children
// box-tested, the near one (by the ray direction on the node's split axis)
// entered, a hit far child pushed with its entry distance; a node with no
// hit child pops the next stacked node the bound does not prune (the far
// child is re-checked, LBVH.cpp:992).  The stack is a ring of kStackSize
// entries holding [base, sp); a depth-first walk never holds more than the
// tree depth.  Returns false when the lane has nothing left.
//
// CAPPED: at most max_steps internal nodes are expanded in this call; a lane
// that runs out keeps its place (returns true with *at_leaf false) and goes
// on at the next call.  The walk, and so every test, is the same.
template <bool EXACT, bool STATS, bool CAPPED = false>
__device__ __forceinline__ bool descend(const TreeRef& tr_, const RayState& r, float bt, uint32_t& node, NodeBox& cur,
                                        uint32_t* stack_node, float* stack_t0, uint32_t& sp, uint32_t base,
                                        uint32_t& nbox, int max_steps = 0, bool* at_leaf = nullptr) {
    const rt_node* __restrict__ nodes = tr_.nodes;
    int steps = 0;
    if (CAPPED) *at_leaf = false;
    while (!(__float_as_int(cur.b.z) & 4)) {
        if (CAPPED && steps++ >= max_steps) return true;
        const int pc = __float_as_int(cur.b.z);
        const uint32_t c0 = child_pair(tr_, node, cur.b.w);
        if (c0 + 1 >= tr_.num_nodes) {
            atomicOr(tr_.err, RT_DEVERR_BOUNDS);
            return false;
        }
        const float4* p = reinterpret_cast<const float4*>(nodes + c0);
        const float4 l0 = __ldg(p), l1 = __ldg(p + 1), r0 = __ldg(p + 2), r1 = __ldg(p + 3);
        float tl, tr;
        const bool hl = box_enter<EXACT>(r, l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, bt, &tl);
        const bool hr = box_enter<EXACT>(r, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, bt, &tr);
        nbox += 2;
        // near child by the split axis: the stored field is (30 - bit) % 3,
        // the axis the bit splits is (field + 2) % 3
        const int field = pc & 3;
        const int near_right = (r.sgn >> (field == 0 ? 2 : field - 1)) & 1;
        const bool hn = near_right ? hr : hl, hf = near_right ? hl : hr;
        const float tf = near_right ? tl : tr;
        const uint32_t nn = c0 | (uint32_t)near_right, nf = nn ^ 1u;
        if (hn) {
            if (hf) {
                if (sp - base >= (uint32_t)kStackSize) {
                    atomicOr(tr_.err, RT_DEVERR_BOUNDS);
                    return false;
                }
                stack_node[sp & (kStackSize - 1)] = nf;
                stack_t0[sp & (kStackSize - 1)] = tf;
                ++sp;
            }
            node = nn;
            cur.a = near_right ? r0 : l0;
            cur.b = near_right ? r1 : l1;
        } else if (hf) {
            node = nf;
            cur.a = near_right ? l0 : r0;
            cur.b = near_right ? l1 : r1;
        } else {
            bool got = false;
            while (sp != base) {
                --sp;
                if (!(stack_t0[sp & (kStackSize - 1)] > bt)) {
                    node = stack_node[sp & (kStackSize - 1)];
                    got = true;
                    break;
                }
            }
            if (!got) return false;
            cur = load_node(nodes, node);
        }
    }
    if (CAPPED) *at_leaf = true;
    return true;
}

__device__ __forceinline__ bool pop_node(const TreeRef& tr_, float bt, uint32_t& node, NodeBox& cur,
                                         const uint32_t* stack_node, const float* stack_t0, uint32_t& sp,
                                         uint32_t base) {
    while (sp != base) {
        --sp;
        if (!(stack_t0[sp & (kStackSize - 1)] > bt)) {
            node = stack_node[sp & (kStackSize - 1)];
            cur = load_node(tr_.nodes, node);
            return true;
        }
    }
    return false;
}

// Start of a walk at heap node `start` (<= 1: the root; see traverse): the
// siblings of start's ancestors are box-tested and stacked, then start's own
// box is tested; a missed start pops the stack.  Returns true when the lane
// holds a node to enter.
template <bool EXACT>
__device__ __forceinline__ bool start_walk(const RayState& r, const TreeRef& tr_, uint32_t start, float bt,
                                           uint32_t* stack_node, float* stack_t0, uint32_t& sp, uint32_t& node,
                                           NodeBox& cur, uint32_t& nbox) {
    // no t satisfies 0 <= t < tmax when tmax <= 0 or is NaN
    const bool live = r.tmax > 0.0f;
    node = 1;
    if (start > 1u && !tr_.compact) {
        if (start >= tr_.num_nodes) {
            atomicOr(tr_.err, RT_DEVERR_BOUNDS);
        } else {
            const int D = 31 - __clz(start);  // <= kMaxDepth < kStackSize
            for (int k = 1; k <= D; ++k) {
                const uint32_t sib = (start >> (D - k)) ^ 1u;
                const NodeBox sb = load_node(tr_.nodes, sib);
                ++nbox;
                float t0;
                if (live && box_enter<EXACT>(r, sb.a.x, sb.a.y, sb.a.z, sb.a.w, sb.b.x, sb.b.y, bt, &t0)) {
                    stack_node[sp & (kStackSize - 1)] = sib;
                    stack_t0[sp & (kStackSize - 1)] = t0;
                    ++sp;
                }
            }
            node = start;
        }
    }
    cur = load_node(tr_.nodes, node);
    ++nbox;
    float t0;
    bool have = live && box_enter<EXACT>(r, cur.a.x, cur.a.y, cur.a.z, cur.a.w, cur.b.x, cur.b.y, bt, &t0);
    if (!have) {
        while (sp != 0) {  // pop_node, declared below
            --sp;
            if (!(stack_t0[sp & (kStackSize - 1)] > bt)) {
                node = stack_node[sp & (kStackSize - 1)];
                cur = load_node(tr_.nodes, node);
                have = true;
                break;
            }
        }
    }
    return have;
}

// Hand-over of rays that exceed a work budget.  A lane whose ray has spent
// more than `budget` box + triangle tests takes a slot of the heavy-ray list
// (atomicAdd on *count) and stops; the caller records the ray in that slot,
// and a second kernel traces it with a whole warp (traverse_wide).  When the
// list is full the lane keeps going.  count == nullptr: no budget.
struct Spill {
    uint32_t* count;
    uint32_t cap;
    uint32_t budget;
    uint32_t* work;  // claim counter of the warp-per-ray pass (host side)
};

// Warp-cooperative traversal.  All 32 lanes of the warp call it together;
// lanes with active == false only help with the leaf phase.  Each round,
// every lane descends until it holds a leaf or has nothing left, then the
// warp tests the held leaves' triangles together.  Without a budget, hits and
// box / triangle test counts equal the oracle's.  *slot_out = the heavy-list
// slot of a ray handed over (its hit is then not valid), else -1.
//
// Restart (the iRoot argument of LBVH_IntersectP, LBVH.hlsl:363-376): with
// start > 1 the walk begins at heap node `start`.  The siblings of start's
// ancestors are box-tested first and stacked with their entry distances
// (the deepest on top), then start itself is entered; together they cover
// the heap, and since a parent's box admits every ray its children's boxes
// admit, the closest hit is the root walk's (except where two triangles are
// hit within an ulp and a rounded box entry lets the order decide, as it
// does between any two walk orders).  Only the heap layout can be
// restarted (with the compact layout the walk starts at the root).  start
// must be a node the build reached, e.g. a leaf a trace of the same tree
// reported through *leaf_out (1 when nothing was hit).
template <bool EXACT, bool STATS>
__device__ __forceinline__ Hit traverse(const RayState& r, bool active, const TreeRef& tr_, bool any_hit,
                                        uint32_t* nbox_out, uint32_t* ntri_out, const Spill* spill,
                                        int* slot_out, uint32_t start = 1u, uint32_t* leaf_out = nullptr) {
    constexpr uint32_t kFull = 0xffffffffu;
    Best b;
    b.key = hit_key(r.tmax, 0);
    b.id = -1;
    b.u = -1.0f;
    b.v = -1.0f;
    b.t = r.tmax;
    b.leaf = 1u;
    uint64_t bound = b.key;
    uint32_t nbox = 0, ntri = 0;
    uint32_t stack_node[kStackSize];
    float stack_t0[kStackSize];
    uint32_t sp = 0;
    NodeBox cur;
    cur.a = make_float4(0.f, 0.f, 0.f, 0.f);
    cur.b = cur.a;
    bool have = false;
    uint32_t node = 1;
    int slot = -1;
    bool budgeted = !STATS && spill != nullptr && spill->count != nullptr;
    if (active) have = start_walk<EXACT>(r, tr_, start, b.t, stack_node, stack_t0, sp, node, cur, nbox);
    while (__any_sync(kFull, have)) {
        if (have) have = descend<EXACT, STATS>(tr_, r, b.t, node, cur, stack_node, stack_t0, sp, 0u, nbox);
        __syncwarp();
        leaf_phase<STATS>(tr_, r, have, cur, node, bound, b, ntri);
        if (have) {
            if (any_hit && b.id >= 0) {
                have = false;
            } else {
                have = pop_node(tr_, b.t, node, cur, stack_node, stack_t0, sp, 0u);
                if (budgeted && have && nbox + ntri > spill->budget) {
                    const uint32_t s = atomicAdd(spill->count, 1u);
                    if (s < spill->cap) {
                        slot = (int)s;
                        have = false;
                    } else {
                        budgeted = false;  // list full: finish here
                    }
                }
            }
        }
    }
    if (nbox_out) *nbox_out = nbox;
    if (ntri_out) *ntri_out = ntri;
    if (slot_out) *slot_out = slot;
    if (leaf_out) *leaf_out = tr_.compact ? 1u : b.leaf;
    Hit h;
    h.id = b.id;
    h.u = b.u;
    h.v = b.v;
    h.t = b.t;
    return h;
}

__device__ __forceinline__ uint64_t warp_min_u64(uint64_t v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const uint64_t o = shfl_u64(v, (threadIdx.x & 31) ^ off);
        v = o < v ? o : v;
    }
    return v;
}

// One ray traced by the whole warp (every lane passes the same ray): a
// frontier walk.  The warp keeps a stack of the internal nodes the ray enters
// (as the slot of their children pair, with the entry distance) and a queue
// of leaves in shared memory.  Each step
// pops up to 32 nodes from the top (the deepest: the walk stays depth-first
// at the scale of a warp, which bounds the stack by 32 entries per level),
// tests both children of each, and pushes the entered internal children and
// queues the entered leaves.  When the queue holds 64 or more triangles, or
// the stack is empty, the queued leaves still in front of the closest hit are
// tested 32 (leaf, triangle) pairs at a time and the warp minimum of the
// (t, id) keys becomes the shared bound.  The closest hit under the tie rule
// does not depend on the order of the tests, so the hit equals traverse()'s.
// For any_hit the walk stops at the first accepted hit.
// Each step pops the newest 32 entries, so every group of pushed children
// leaves at most 32 entries behind, one group per tree level: a tree of
// depth D needs at most 32 (D + 1) entries, and wide_stack_entries adds one
// more group.  The stack lives in dynamic shared memory sized per launch.
constexpr int kWideStackMax = 1024;  // entries per warp for depth <= 29
constexpr int kWideQueue = 128;      // queued leaves per warp
constexpr int kWideWarps = 4;        // blocks of at most 128 threads

__host__ __device__ constexpr uint32_t wide_stack_entries(uint32_t depth) {
    return (depth + 2u) * 32u < (uint32_t)kWideStackMax ? (depth + 2u) * 32u : (uint32_t)kWideStackMax;
}

// Dynamic shared memory of a block running traverse_wide with `cap` stack
// entries per warp: stack nodes and entry distances, then the leaf queue.
__host__ __device__ constexpr size_t wide_smem_bytes(uint32_t cap) {
    return (size_t)kWideWarps * (cap * 8u + kWideQueue * 16u);
}

template <bool EXACT>
__device__ __forceinline__ Hit traverse_wide(const RayState& r, const TreeRef& tr_, bool any_hit, uint32_t cap) {
    constexpr uint32_t kFull = 0xffffffffu;
    extern __shared__ uint4 wide_dyn[];
    uint8_t* base8 = reinterpret_cast<uint8_t*>(wide_dyn);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    uint32_t* snode = reinterpret_cast<uint32_t*>(base8) + (size_t)wib * cap;
    float* st0 = reinterpret_cast<float*>(base8 + (size_t)kWideWarps * cap * 4u) + (size_t)wib * cap;
    uint8_t* qbase = base8 + (size_t)kWideWarps * cap * 8u;
    int32_t* qpos = reinterpret_cast<int32_t*>(qbase) + wib * kWideQueue;
    int32_t* qcnt = reinterpret_cast<int32_t*>(qbase) + (kWideWarps + wib) * kWideQueue;
    float* qt0 = reinterpret_cast<float*>(qbase) + (2 * kWideWarps + wib) * kWideQueue;
    uint32_t* qincl = reinterpret_cast<uint32_t*>(qbase) + (3 * kWideWarps + wib) * kWideQueue;
    const uint64_t init = hit_key(r.tmax, 0);
    uint64_t best = init;  // uniform across the warp
    float bu = -1.0f, bv = -1.0f, bt = r.tmax;
    int size = 0, nq = 0, qtris = 0;  // uniform
    bool stop = false;
    // root
    {
        const NodeBox root = load_node(tr_.nodes, 1);
        float t0;
        const bool enter = r.tmax > 0.0f &&
                           box_enter<EXACT>(r, root.a.x, root.a.y, root.a.z, root.a.w, root.b.x, root.b.y, r.tmax, &t0);
        if (enter) {
            if (__float_as_int(root.b.z) & 4) {
                if (lane == 0) {
                    qpos[0] = __float_as_int(root.b.w);
                    qcnt[0] = __float_as_int(root.b.z) >> 3;
                    qt0[0] = t0;
                }
                nq = 1;
                qtris = __float_as_int(root.b.z) >> 3;
            } else {
                if (lane == 0) {
                    snode[0] = child_pair(tr_, 1, root.b.w);  // the stack holds children-pair slots
                    st0[0] = t0;
                }
                size = 1;
            }
        }
    }
    __syncwarp();
    while (!stop && (size > 0 || nq > 0)) {
        // test the queued leaves
        if (nq > 0 && (size == 0 || qtris >= 64 || nq > kWideQueue - 64)) {
            const float bound_t = key_t(best);
            // drop leaves now behind the closest hit; prefix of the kept sizes
            uint32_t run = 0;
            for (int q0 = 0; q0 < nq; q0 += 32) {
                const int q = q0 + lane;
                int c = 0;
                if (q < nq) {
                    c = qcnt[q];
                    if (qt0[q] > bound_t || qpos[q] < 0 || c < 0 || (uint32_t)qpos[q] + (uint32_t)c > tr_.n) c = 0;
                }
                uint32_t incl = (uint32_t)c;
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const uint32_t y = __shfl_up_sync(kFull, incl, off);
                    if (lane >= off) incl += y;
                }
                if (q < nq) qincl[q] = run + incl;
                run += __shfl_sync(kFull, incl, 31);
            }
            __syncwarp();
            const uint32_t total = run;
            for (uint32_t base = 0; base < total; base += 32) {
                const uint32_t p = base + lane;
                uint64_t key = ~0ull;
                float kt = 0.0f, ku = 0.0f, kv = 0.0f;
                if (p < total) {
                    // queued leaf holding pair p: the first with inclusive prefix > p
                    int lo = 0, hi = nq - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1;
                        if (qincl[mid] > p) hi = mid; else lo = mid + 1;
                    }
                    const uint32_t ex = lo > 0 ? qincl[lo - 1] : 0u;
                    const float4* tp = tr_.tris + 3 * (size_t)(qpos[lo] + (int)(p - ex));
                    const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                    const int id = __float_as_int(a.w);
                    float u, v, t;
                    if (id != r.exclude && tri_test(r, a, b, c, &u, &v, &t)) {
                        const uint64_t k = hit_key(t, id);
                        if (k < best) {
                            key = k;
                            kt = t;
                            ku = u;
                            kv = v;
                        }
                    }
                }
                const uint64_t kmin = warp_min_u64(key);
                if (kmin < best) {
                    const int w = __ffs(__ballot_sync(kFull, key == kmin)) - 1;
                    best = kmin;
                    bt = __shfl_sync(kFull, kt, w);
                    bu = __shfl_sync(kFull, ku, w);
                    bv = __shfl_sync(kFull, kv, w);
                    if (any_hit) break;
                }
            }
            nq = 0;
            qtris = 0;
            __syncwarp();
            if (any_hit && best < init) stop = true;
            continue;
        }
        // pop up to 32 internal nodes from the top
        const int k = min(32, size);
        const float bound_t = key_t(best);
        uint32_t nd = 0;
        bool live = false;
        if (lane < k) {
            nd = snode[size - 1 - lane];
            live = !(st0[size - 1 - lane] > bound_t);
        }
        size -= k;
        __syncwarp();
        // children of each popped node
        bool push_l = false, push_r = false, leaf_l = false, leaf_r = false;
        float tl = 0.0f, tr = 0.0f;
        float4 l1 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = l1;
        uint32_t c0 = 0;
        if (live) {
            c0 = nd;
            if (c0 + 1 >= tr_.num_nodes) {
                atomicOr(tr_.err, RT_DEVERR_BOUNDS);
            } else {
                const float4* p = reinterpret_cast<const float4*>(tr_.nodes + c0);
                const float4 l0 = __ldg(p), r0 = __ldg(p + 2);
                l1 = __ldg(p + 1);
                r1 = __ldg(p + 3);
                push_l = box_enter<EXACT>(r, l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, bound_t, &tl);
                push_r = box_enter<EXACT>(r, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, bound_t, &tr);
                leaf_l = push_l && (__float_as_int(l1.z) & 4);
                leaf_r = push_r && (__float_as_int(r1.z) & 4);
            }
        }
        // internal children onto the stack, leaves into the queue
        const uint32_t lt = (1u << lane) - 1u;
        const int ni = (push_l && !leaf_l) + (push_r && !leaf_r);
        const int nl = leaf_l + leaf_r;
        const uint32_t ib0 = __ballot_sync(kFull, ni >= 1), ib1 = __ballot_sync(kFull, ni >= 2);
        const uint32_t lb0 = __ballot_sync(kFull, nl >= 1), lb1 = __ballot_sync(kFull, nl >= 2);
        const int ioff = size + __popc(ib0 & lt) + __popc(ib1 & lt);
        const int loff = nq + __popc(lb0 & lt) + __popc(lb1 & lt);
        const int itotal = __popc(ib0) + __popc(ib1), ltotal = __popc(lb0) + __popc(lb1);
        if (size + itotal > (int)cap) {  // cannot happen within the tree's depth; stop rather than overflow
            if (lane == 0) atomicOr(tr_.err, RT_DEVERR_BOUNDS);
            stop = true;
            break;
        }
        int io = ioff, lo_ = loff;
        if (push_l) {
            if (leaf_l) {
                qpos[lo_] = __float_as_int(l1.w);
                qcnt[lo_] = __float_as_int(l1.z) >> 3;
                qt0[lo_] = tl;
                ++lo_;
            } else {
                snode[io] = child_pair(tr_, c0, l1.w);
                st0[io] = tl;
                ++io;
            }
        }
        if (push_r) {
            if (leaf_r) {
                qpos[lo_] = __float_as_int(r1.w);
                qcnt[lo_] = __float_as_int(r1.z) >> 3;
                qt0[lo_] = tr;
            } else {
                snode[io] = child_pair(tr_, c0 | 1u, r1.w);
                st0[io] = tr;
            }
        }
        int lt_tris = (leaf_l ? (__float_as_int(l1.z) >> 3) : 0) + (leaf_r ? (__float_as_int(r1.z) >> 3) : 0);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) lt_tris += __shfl_xor_sync(kFull, lt_tris, off);
        size += itotal;
        nq += ltotal;
        qtris += lt_tris;
        __syncwarp();
    }
    Hit h;
    if (best < init) {
        h.id = (int)(uint32_t)best;
        h.t = bt;
        h.u = bu;
        h.v = bv;
    } else {
        h.id = -1;
        h.u = -1.0f;
        h.v = -1.0f;
        h.t = r.tmax;
    }
    __syncwarp();
    return h;
}

// One ray traced by a whole block of kTeamThreads threads: traverse_wide's
// frontier walk with the block as the team.  Each step pops up to
// kTeamThreads nodes (the deepest), tests their children, and pushes /
// queues them at offsets from a block-wide prefix sum; the queued leaves are
// tested kTeamThreads (leaf, triangle) pairs at a time, the block minimum of
// the (t, id) keys (a shared-memory atomicMin) becoming the shared bound.
// The hit is traverse_wide's (the tie rule makes it order-free); a ray whose
// frontier is wide (grazing rays with thousands of tests) finishes in a
// quarter of the steps.  Every thread of the block calls it with the same
// ray; it synchronises the block.  Stack bound as in traverse_wide with
// kTeamThreads entries per level.
constexpr int kTeamThreads = 128;
constexpr int kTeamQueue = 4 * kTeamThreads;

__host__ __device__ constexpr uint32_t team_stack_entries(uint32_t depth) {
    return (depth + 2u) * (uint32_t)kTeamThreads;
}

// Dynamic shared memory of traverse_team with `cap` stack entries.
__host__ __device__ constexpr size_t team_smem_bytes(uint32_t cap) {
    return (size_t)cap * 8u + (size_t)kTeamQueue * 16u;
}

struct TeamShared {
    unsigned long long best;
    float bt, bu, bv;
    uint32_t warp_sum[kTeamThreads / 32];
    int tris_sum[kTeamThreads / 32];
};

// Inclusive block-wide prefix sum of v (all threads call); *total = the sum.
__device__ __forceinline__ uint32_t team_scan(uint32_t v, TeamShared& ts, uint32_t* total) {
    constexpr uint32_t kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, x, off);
        if (lane >= off) x += y;
    }
    __syncthreads();
    if (lane == 31) ts.warp_sum[w] = x;
    __syncthreads();
    uint32_t before = 0, all = 0;
#pragma unroll
    for (int q = 0; q < kTeamThreads / 32; ++q) {
        const uint32_t t = ts.warp_sum[q];
        if (q < w) before += t;
        all += t;
    }
    *total = all;
    return before + x;
}

template <bool EXACT>
__device__ __forceinline__ Hit traverse_team(const RayState& r, const TreeRef& tr_, bool any_hit, uint32_t cap,
                                             TeamShared& ts) {
    constexpr uint32_t kFull = 0xffffffffu;
    extern __shared__ uint4 wide_dyn[];
    uint8_t* base8 = reinterpret_cast<uint8_t*>(wide_dyn);
    const int tid = threadIdx.x, lane = tid & 31;
    uint32_t* snode = reinterpret_cast<uint32_t*>(base8);
    float* st0 = reinterpret_cast<float*>(base8 + (size_t)cap * 4u);
    uint8_t* qbase = base8 + (size_t)cap * 8u;
    int32_t* qpos = reinterpret_cast<int32_t*>(qbase);
    int32_t* qcnt = qpos + kTeamQueue;
    float* qt0 = reinterpret_cast<float*>(qcnt + kTeamQueue);
    uint32_t* qincl = reinterpret_cast<uint32_t*>(qt0 + kTeamQueue);
    const uint64_t init = hit_key(r.tmax, 0);
    // uniform across the block (every thread keeps the same copy)
    uint64_t best = init;
    int size = 0, nq = 0, qtris = 0;
    bool stop = false;
    __syncthreads();  // the previous ray's readers of the shared state are done
    if (tid == 0) {
        ts.best = init;
        ts.bt = r.tmax;
        ts.bu = -1.0f;
        ts.bv = -1.0f;
    }
    {
        const NodeBox root = load_node(tr_.nodes, 1);
        float t0;
        const bool enter = r.tmax > 0.0f &&
                           box_enter<EXACT>(r, root.a.x, root.a.y, root.a.z, root.a.w, root.b.x, root.b.y, r.tmax, &t0);
        if (enter) {
            if (__float_as_int(root.b.z) & 4) {
                if (tid == 0) {
                    qpos[0] = __float_as_int(root.b.w);
                    qcnt[0] = __float_as_int(root.b.z) >> 3;
                    qt0[0] = t0;
                }
                nq = 1;
                qtris = __float_as_int(root.b.z) >> 3;
            } else {
                if (tid == 0) {
                    snode[0] = child_pair(tr_, 1, root.b.w);
                    st0[0] = t0;
                }
                size = 1;
            }
        }
    }
    __syncthreads();
    while (!stop && (size > 0 || nq > 0)) {
        if (nq > 0 && (size == 0 || qtris >= 2 * kTeamThreads || nq > kTeamQueue - 2 * kTeamThreads)) {
            const float bound_t = key_t(best);
            // drop leaves now behind the closest hit; prefix of the kept sizes
            uint32_t run = 0;
            for (int q0 = 0; q0 < nq; q0 += kTeamThreads) {
                const int q = q0 + tid;
                int c = 0;
                if (q < nq) {
                    c = qcnt[q];
                    if (qt0[q] > bound_t || qpos[q] < 0 || c < 0 || (uint32_t)qpos[q] + (uint32_t)c > tr_.n) c = 0;
                }
                uint32_t chunk = 0;
                const uint32_t incl = team_scan((uint32_t)c, ts, &chunk);
                if (q < nq) qincl[q] = run + incl;
                run += chunk;
            }
            __syncthreads();
            const uint32_t total = run;
            for (uint32_t base = 0; base < total; base += kTeamThreads) {
                const uint32_t p = base + tid;
                uint64_t key = ~0ull;
                float kt = 0.0f, ku = 0.0f, kv = 0.0f;
                if (p < total) {
                    int lo = 0, hi = nq - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1;
                        if (qincl[mid] > p) hi = mid; else lo = mid + 1;
                    }
                    const uint32_t ex = lo > 0 ? qincl[lo - 1] : 0u;
                    const float4* tp = tr_.tris + 3 * (size_t)(qpos[lo] + (int)(p - ex));
                    const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                    const int id = __float_as_int(a.w);
                    float u, v, t;
                    if (id != r.exclude && tri_test(r, a, b, c, &u, &v, &t)) {
                        const uint64_t k = hit_key(t, id);
                        if (k < best) {
                            key = k;
                            kt = t;
                            ku = u;
                            kv = v;
                        }
                    }
                }
                const uint64_t wmin = warp_min_u64(key);
                if (lane == 0 && wmin < best) atomicMin(&ts.best, (unsigned long long)wmin);
                __syncthreads();
                const uint64_t bmin = ts.best;
                if (bmin < best && key == bmin) {  // the one triangle with this (t, id): same t, u, v
                    ts.bt = kt;
                    ts.bu = ku;
                    ts.bv = kv;
                }
                best = bmin;
                __syncthreads();
                if (any_hit && best < init) break;
            }
            nq = 0;
            qtris = 0;
            if (any_hit && best < init) stop = true;
            continue;
        }
        // pop up to kTeamThreads internal nodes from the top
        const int k = min(kTeamThreads, size);
        const float bound_t = key_t(best);
        uint32_t nd = 0;
        bool live = false;
        if (tid < k) {
            nd = snode[size - 1 - tid];
            live = !(st0[size - 1 - tid] > bound_t);
        }
        size -= k;
        __syncthreads();
        bool push_l = false, push_r = false, leaf_l = false, leaf_r = false;
        float tl = 0.0f, tr = 0.0f;
        float4 l1 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = l1;
        uint32_t c0 = 0;
        if (live) {
            c0 = nd;
            if (c0 + 1 >= tr_.num_nodes) {
                atomicOr(tr_.err, RT_DEVERR_BOUNDS);
            } else {
                const float4* p = reinterpret_cast<const float4*>(tr_.nodes + c0);
                const float4 l0 = __ldg(p), r0 = __ldg(p + 2);
                l1 = __ldg(p + 1);
                r1 = __ldg(p + 3);
                push_l = box_enter<EXACT>(r, l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, bound_t, &tl);
                push_r = box_enter<EXACT>(r, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, bound_t, &tr);
                leaf_l = push_l && (__float_as_int(l1.z) & 4);
                leaf_r = push_r && (__float_as_int(r1.z) & 4);
            }
        }
        const uint32_t ni = (uint32_t)((push_l && !leaf_l) + (push_r && !leaf_r));
        const uint32_t nl = (uint32_t)(leaf_l + leaf_r);
        // one scan for both counts (internal in the low half, leaves in the high)
        uint32_t both = 0;
        const uint32_t incl = team_scan(ni | (nl << 16), ts, &both);
        const uint32_t excl = incl - (ni | (nl << 16));
        const int itotal = (int)(both & 0xffffu), ltotal = (int)(both >> 16);
        int lt_tris = (leaf_l ? (__float_as_int(l1.z) >> 3) : 0) + (leaf_r ? (__float_as_int(r1.z) >> 3) : 0);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) lt_tris += __shfl_xor_sync(kFull, lt_tris, off);
        if (lane == 0) ts.tris_sum[threadIdx.x >> 5] = lt_tris;
        if (size + itotal > (int)cap) {  // cannot happen within the tree's depth; stop rather than overflow
            if (tid == 0) atomicOr(tr_.err, RT_DEVERR_BOUNDS);
            stop = true;
            __syncthreads();
            break;
        }
        int io = size + (int)(excl & 0xffffu), lo_ = nq + (int)(excl >> 16);
        if (push_l) {
            if (leaf_l) {
                qpos[lo_] = __float_as_int(l1.w);
                qcnt[lo_] = __float_as_int(l1.z) >> 3;
                qt0[lo_] = tl;
                ++lo_;
            } else {
                snode[io] = child_pair(tr_, c0, l1.w);
                st0[io] = tl;
                ++io;
            }
        }
        if (push_r) {
            if (leaf_r) {
                qpos[lo_] = __float_as_int(r1.w);
                qcnt[lo_] = __float_as_int(r1.z) >> 3;
                qt0[lo_] = tr;
            } else {
                snode[io] = child_pair(tr_, c0 | 1u, r1.w);
                st0[io] = tr;
            }
        }
        __syncthreads();
        int tsum = 0;
#pragma unroll
        for (int q = 0; q < kTeamThreads / 32; ++q) tsum += ts.tris_sum[q];
        size += itotal;
        nq += ltotal;
        qtris += tsum;
    }
    Hit h;
    if (best < init) {
        h.id = (int)(uint32_t)best;
        h.t = ts.bt;
        h.u = ts.bu;
        h.v = ts.bv;
    } else {
        h.id = -1;
        h.u = -1.0f;
        h.v = -1.0f;
        h.t = r.tmax;
    }
    __syncthreads();
    return h;
}

__device__ __forceinline__ Hit trace_team(const RayState& r, const TreeRef& tr, bool any_hit, uint32_t cap,
                                          TeamShared& ts) {
    if (r.exact) return traverse_team<true>(r, tr, any_hit, cap, ts);
    return traverse_team<false>(r, tr, any_hit, cap, ts);
}

// Warp-uniform dispatch between the fast and the NaN-exact box test.  Must be
// called by all 32 lanes of the warp together (inactive lanes pass
// active == false).  spill / slot: see Spill (nullptr: no budget).
template <bool STATS>
__device__ __forceinline__ Hit trace_ray(const RayState& r, bool active, const TreeRef& tr, bool any_hit,
                                         uint32_t* nbox, uint32_t* ntri, const Spill* spill = nullptr,
                                         int* slot = nullptr, uint32_t start = 1u, uint32_t* leaf = nullptr) {
    if (__any_sync(0xffffffffu, active && r.exact))
        return traverse<true, STATS>(r, active, tr, any_hit, nbox, ntri, spill, slot, start, leaf);
    return traverse<false, STATS>(r, active, tr, any_hit, nbox, ntri, spill, slot, start, leaf);
}

// One ray traced by the whole warp; every lane passes the same ray.
__device__ __forceinline__ Hit trace_wide(const RayState& r, const TreeRef& tr, bool any_hit, uint32_t cap) {
    if (r.exact) return traverse_wide<true>(r, tr, any_hit, cap);
    return traverse_wide<false>(r, tr, any_hit, cap);
}

// Primary ray of pixel (i, j): CSPrimaryRays.hlsl:36-56 with the basis camera.
__device__ __forceinline__ f3 camera_dir(const rt_camera& cam, float x, float y) {
    const float dx = fmul(x, cam.tan_half_fovy), dy = fmul(y, cam.tan_half_fovy);
    f3 d;
    d.x = fadd(fadd(fmul(cam.right[0], dx), fmul(cam.up[0], dy)), cam.fwd[0]);
    d.y = fadd(fadd(fmul(cam.right[1], dx), fmul(cam.up[1], dy)), cam.fwd[1]);
    d.z = fadd(fadd(fmul(cam.right[2], dx), fmul(cam.up[2], dy)), cam.fwd[2]);
    return normalize3(d);
}

__device__ __forceinline__ f3 primary_dir(const rt_camera& cam, uint32_t i, uint32_t j) {
    const float inv = fdiv(1.0f, (float)cam.height);
    const float x = fmul((float)(2 * (int)i + 1 - (int)cam.width), inv);
    const float y = -fmul((float)(2 * (int)j + 1 - (int)cam.height), inv);
    return camera_dir(cam, x, y);
}

// Persistent warps: each warp takes the next 32-item tile from a work counter
// (reset before the launch), so heavy tiles never queue behind an idle SM.
__device__ __forceinline__ uint32_t next_tile(uint32_t* work) {
    uint32_t t = 0;
    if ((threadIdx.x & 31) == 0) t = atomicAdd(work, 1u);
    return __shfl_sync(0xffffffffu, t, 0);
}

// Pixel of lane `lane` of warp tile `tile`: 8 x 4 pixel tiles for coherence.
__device__ __forceinline__ bool tile_pixel(uint32_t tile, uint32_t lane, uint32_t w, uint32_t h, uint32_t* i,
                                           uint32_t* j) {
    const uint32_t tiles_x = (w + 7) / 8;
    const uint32_t tx = tile % tiles_x, ty = tile / tiles_x;
    *i = tx * 8 + (lane & 7);
    *j = ty * 4 + (lane >> 3);
    return *i < w && *j < h;
}

// Heavy-first tile order.  A trace call records the tiles whose rays spent
// more than kHeavyTileTests box + triangle tests in all (a list and a bitmap,
// written by call c into buffer w = parity); call c + 1 hands those tiles out
// first (buffer 1 - w), then every other tile in image order, skipping the
// ones already handed out.  Frames are coherent, so the tiles that made the
// last call's tail start first; the order changes no result, and a stale or
// foreign list (another image, another scene) only changes the order: every
// tile is still traced exactly once.  The parity word is flipped on the
// device (k_order_begin), so a replayed CUDA graph alternates too.
constexpr uint32_t kHeavyTileTests = 4096;

struct TileOrder {
    uint32_t* parity;      // device word: the buffer this call writes
    uint32_t* lists;       // 2 x cap tile indices
    uint32_t* counts;      // 2 words
    uint32_t* bits;        // 2 x (cap / 32) words
    uint32_t cap;
};

// Next tile of this warp (all lanes call; returns num_tiles when done).
__device__ __forceinline__ uint32_t next_ordered_tile(uint32_t* work, const TileOrder& ord, uint32_t rbuf,
                                                      uint32_t heavy, uint32_t num_tiles) {
    for (;;) {
        const uint32_t v = next_tile(work);
        if (v < heavy) {
            const uint32_t t = __ldg(ord.lists + (size_t)rbuf * ord.cap + v);
            if (t < num_tiles) return t;
            continue;  // a tile of another image
        }
        const uint32_t t = v - heavy;
        if (t >= num_tiles) return num_tiles;
        if (t < ord.cap && heavy > 0 && ((__ldg(ord.bits + (size_t)rbuf * (ord.cap / 32) + t / 32) >> (t % 32)) & 1u))
            continue;  // handed out first
        return t;
    }
}

// Records tile t as heavy for the next call when the warp's tests exceed the
// threshold (lane 0 of the warp).
__device__ __forceinline__ void record_tile_cost(const TileOrder& ord, uint32_t wbuf, uint32_t t, uint32_t tests) {
    uint32_t sum = tests;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
    if ((threadIdx.x & 31) == 0 && sum > kHeavyTileTests && t < ord.cap) {
        const uint32_t k = atomicAdd(ord.counts + wbuf, 1u);
        if (k < ord.cap) {
            ord.lists[(size_t)wbuf * ord.cap + k] = t;
            atomicOr(ord.bits + (size_t)wbuf * (ord.cap / 32) + t / 32, 1u << (t % 32));
        }
    }
}

// The shading rays of one pixel whose primary hit is ph (CSComputeColorRT.hlsl,
// flat normal, no textures): the shadow ray towards the point light, cast
// only when the light and the viewer are on the same side of the surface,
// and the mirror ray.  has = the primary ray hit something.
struct ShadeRays {
    RayState shadow, mirror;
    bool has, cast;
};

__device__ __forceinline__ ShadeRays shade_rays(const float* __restrict__ soup, const rt_camera& cam, float lx,
                                                float ly, float lz, int4 ph, bool valid, uint32_t i, uint32_t j,
                                                bool want_mirror) {
    ShadeRays s;
    const int id = valid ? ph.x : -1;
    s.has = valid && id >= 0;
    s.cast = false;
    f3 N = mk3(0.f, 0.f, 1.f), Nf = N, P = mk3(0.f, 0.f, 0.f), L = mk3(0.f, 0.f, 1.f), d = mk3(0.f, 0.f, 1.f);
    float dist = 1.0f;
    if (s.has) {
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
        s.cast = fmul(ls, rs) > 0.0f;                              // :147
    }
    s.shadow = make_ray(P, mk3(-L.x, -L.y, -L.z), dist, id);      // :149-153
    f3 R = mk3(0.f, 0.f, 1.f);
    if (want_mirror && s.has) {
        const float k = fmul(2.0f, dot3(d, Nf));                   // reflect(d, N) = d - 2*dot(d,N)*N
        R = normalize3(mk3(fsub(d.x, fmul(k, Nf.x)), fsub(d.y, fmul(k, Nf.y)), fsub(d.z, fmul(k, Nf.z))));
    }
    s.mirror = make_ray(P, R, 1e16f, id);
    return s;
}

__device__ __forceinline__ uint8_t vis_code(bool has, bool cast, bool occluded) {
    return !has ? 0 : (!cast ? 1 : (occluded ? 2 : 3));
}

}  // namespace rt
