/*
 * rt_oracle.c -- CPU restatement of the reference's LBVH hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker): used by tests/, by the smoke check
 * and by the CPU-baseline leg of bench.py.  The product path never calls it.
 *
 * Compiled with -O2 -ffp-contract=off -fopenmp.  All floating point is IEEE
 * binary32 in the reference's operation order (no fused multiply-add); the
 * adjoint accumulates in binary64.  Citations are paths inside the
 * elfrank/raytracer-gpupro4 checkout.
 */
#include "rt_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* std::min / std::max semantics used by the reference's CPU code
 * (LBVH.cpp:40-56, RayBoxInterval LBVH.cpp:634-659): min(a,b) = (b<a)?b:a. */
static inline float smin(float a, float b) { return (b < a) ? b : a; }
static inline float smax(float a, float b) { return (a < b) ? b : a; }

static inline int hb32(uint32_t x) { return 31 - __builtin_clz(x); } /* x != 0 */

/* ------------------------------------------------------------------------ */
/* Scene bounds: LBVH.cpp:495-516 (VertMin/VertMax over per-triangle boxes). */
void or_scene_bounds(const float* tris, uint32_t n, float out6[6]) {
    float mn[3], mx[3];
    for (int c = 0; c < 3; ++c) mn[c] = mx[c] = n ? tris[c] : 0.0f;
    for (uint32_t i = 0; i < n; ++i) {
        const float* t = tris + 9 * (size_t)i;
        for (int c = 0; c < 3; ++c) {
            /* gMinVertices[i] = minBox(V0, minBox(V1, V2)) (LBVH.cpp:505-506) */
            float lo = smin(t[c], smin(t[3 + c], t[6 + c]));
            float hi = smax(t[c], smax(t[3 + c], t[6 + c]));
            mn[c] = smin(mn[c], lo); /* VertMin = minBox(VertMin, gMin[i]) (:514) */
            mx[c] = smax(mx[c], hi);
        }
    }
    for (int c = 0; c < 3; ++c) { out6[c] = mn[c]; out6[3 + c] = mx[c]; }
}

/* Morton codes: LBVH.cpp:520-553 (GPU twin LBVH.hlsl:92-114).
 *   centroid = (V0 + V1) + V2           (:512, unscaled sum)
 *   VertMax *= 3, VertMin *= 3          (:521-522)
 *   f = 1024 / (VertMax - VertMin)      (:523-526)
 *   q = (unsigned)int((c - VertMin) * f) (:538-540), bits 0..9 only (:546)
 *   z_j -> bit 3j, y_j -> 3j+1, x_j -> 3j+2 (:541, :548-550) */
static inline uint32_t quantize(float c, float lo3, float f) {
    float v = (c - lo3) * f;
    /* int(v): C++ float->int truncation.  NaN (a flat scene axis gives
     * 0 * inf) and out-of-range values are undefined in C++; x86 yields
     * 0x80000000 whose low 10 bits are 0, CUDA yields 0 for NaN.  Both
     * keep 0 in the 10 bits that are used. */
    if (!(v == v)) return 0u;
    if (v >= 2147483648.0f || v <= -2147483649.0f) return 0u;
    return (uint32_t)(int32_t)v;
}

void or_morton(const float* tris, uint32_t n, const float b[6], uint32_t* keys) {
    float lo3[3], f[3];
    for (int c = 0; c < 3; ++c) {
        float mx3 = 3.0f * b[3 + c];
        lo3[c] = 3.0f * b[c];
        f[c] = 1024.f / (mx3 - lo3[c]);
    }
    for (uint32_t i = 0; i < n; ++i) {
        const float* t = tris + 9 * (size_t)i;
        uint32_t q[3];
        for (int c = 0; c < 3; ++c) {
            float cen = (t[c] + t[3 + c]) + t[6 + c];
            q[c] = quantize(cen, lo3[c], f[c]);
        }
        uint32_t code = (q[2] & 1u) | ((q[1] & 1u) << 1) | ((q[0] & 1u) << 2);
        uint32_t shift3 = 2, shift = 2;
        for (int j = 1; j < 10; ++j) {
            code |= (q[2] & shift) << (shift3++);
            code |= (q[1] & shift) << (shift3++);
            code |= (q[0] & shift) << (shift3);
            shift <<= 1;
        }
        keys[i] = code;
    }
}

/* Order of cmpMorton (LBVH.cpp:21-38): by code, then by id.  ids enter in
 * ascending order, so a stable sort by code gives exactly that order.
 * Two-pass LSD counting sort (15 + 15 bits). */
void or_sort_pairs(uint32_t* keys, uint32_t* ids, uint32_t n) {
    uint32_t* k2 = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    uint32_t* i2 = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    uint32_t* cnt = (uint32_t*)malloc(sizeof(uint32_t) * 32768);
    uint32_t *sk = keys, *si = ids, *dk = k2, *di = i2;
    for (int pass = 0; pass < 2; ++pass) {
        int sh = 15 * pass;
        memset(cnt, 0, sizeof(uint32_t) * 32768);
        for (uint32_t i = 0; i < n; ++i) cnt[(sk[i] >> sh) & 32767u]++;
        uint32_t s = 0;
        for (int d = 0; d < 32768; ++d) { uint32_t c = cnt[d]; cnt[d] = s; s += c; }
        for (uint32_t i = 0; i < n; ++i) {
            uint32_t p = cnt[(sk[i] >> sh) & 32767u]++;
            dk[p] = sk[i]; di[p] = si[i];
        }
        uint32_t* t;
        t = sk; sk = dk; dk = t;
        t = si; si = di; di = t;
    }
    /* two passes: result is back in keys/ids */
    free(k2); free(i2); free(cnt);
}

/* ------------------------------------------------------------------------ */
/* Node emission + refit: LBVH::build_recursive (LBVH.cpp:190-314) applied
 * to the already sorted pairs.  The reference partitions unsorted data in
 * place on each bit; on sorted data that partition is a split point, so
 * the topology, PrimPos/PrimCount/leaf/axis fields and the boxes are the
 * same.  The axis field is the reference's round-robin counter, which is
 * (30 - bit) % 3 for the bit being examined. */
typedef struct emit_ctx {
    const float* tris;
    const uint32_t* keys;
    const uint32_t* ids;
    or_node* nodes;
    uint8_t* reached;
    uint32_t num_nodes;
} emit_ctx;

static void leaf_box(const emit_ctx* e, int pos, int count, float mn[3], float mx[3]) {
    for (int j = 0; j < count; ++j) {
        const float* t = e->tris + 9 * (size_t)e->ids[pos + j];
        for (int c = 0; c < 3; ++c) {
            float lo = smin(t[c], smin(t[3 + c], t[6 + c]));
            float hi = smax(t[c], smax(t[3 + c], t[6 + c]));
            if (j == 0) { mn[c] = lo; mx[c] = hi; }
            else { mn[c] = smin(mn[c], lo); mx[c] = smax(mx[c], hi); }
        }
    }
}

/* bit == -1 stands for the reference's bit value 0 (all 30 bits consumed). */
static void emit_rec(const emit_ctx* e, int pos, int count, int bit, uint32_t node, int axis) {
    or_node* nd = &e->nodes[node];
    if (bit < 0 || count <= 1 || (node << 1) >= e->num_nodes) {
        nd->prim_count = (count << 3) | 4 | axis;
        nd->prim_pos = pos;
        leaf_box(e, pos, count, nd->mn, nd->mx);
        if (e->reached) e->reached[node] = 1;
        return;
    }
    const uint32_t m = 1u << bit;
    /* first element of the range with the bit set (data sorted) */
    int lo = pos, hi = pos + count;
    while (lo < hi) {
        int mid = lo + (hi - lo) / 2;
        if (e->keys[mid] & m) hi = mid; else lo = mid + 1;
    }
    int one = lo - pos;
    if (one == count || one == 0) { /* all 0 (:231-237) or all 1 (:260-266) */
        emit_rec(e, pos, count, bit - 1, node, (axis + 1) % 3);
        return;
    }
    emit_rec(e, pos, one, bit - 1, node << 1, (axis + 1) % 3);
    emit_rec(e, pos + one, count - one, bit - 1, (node << 1) | 1, (axis + 1) % 3);
    nd->prim_count = (count << 3) | axis;
    nd->prim_pos = pos;
    const or_node* l = &e->nodes[node << 1];
    const or_node* r = &e->nodes[(node << 1) | 1];
    for (int c = 0; c < 3; ++c) {
        nd->mx[c] = smax(l->mx[c], r->mx[c]);
        nd->mn[c] = smin(l->mn[c], r->mn[c]);
    }
    if (e->reached) e->reached[node] = 1;
}

void or_lbvh_emit(const float* tris, const uint32_t* keys, const uint32_t* ids, uint32_t n,
                  uint32_t depth, or_node* nodes, uint8_t* reached) {
    emit_ctx e = {tris, keys, ids, nodes, reached, 1u << depth};
    for (uint32_t i = 0; i < e.num_nodes; ++i) {
        or_node* nd = &nodes[i];
        nd->mn[0] = nd->mn[1] = nd->mn[2] = 0.0f;
        nd->mx[0] = nd->mx[1] = nd->mx[2] = 0.0f;
        nd->prim_count = OR_SENTINEL;
        nd->prim_pos = OR_SENTINEL;
    }
    if (reached) memset(reached, 0, e.num_nodes);
    if (n == 0) return;
    emit_rec(&e, 0, (int)n, 30, 1, 0);
}

void or_lbvh_build(const float* tris, uint32_t n, uint32_t depth, or_node* nodes, uint32_t* ids,
                   uint32_t* keys, uint8_t* reached) {
    float b[6];
    or_scene_bounds(tris, n, b);
    or_morton(tris, n, b, keys);
    for (uint32_t i = 0; i < n; ++i) ids[i] = i;
    or_sort_pairs(keys, ids, n);
    or_lbvh_emit(tris, keys, ids, n, depth, nodes, reached);
}

/* ------------------------------------------------------------------------ */
/* Ray/box interval: RayBoxInterval (LBVH.cpp:634-659) = IntersectBox
 * (Intersection.hlsl:18-42). */
static inline void box_interval(const or_node* nd, const float o[3], const float inv[3], float* T0,
                                float* T1) {
    float dmx[3], dmn[3];
    for (int c = 0; c < 3; ++c) {
        dmx[c] = (nd->mx[c] - o[c]) * inv[c];
        dmn[c] = (nd->mn[c] - o[c]) * inv[c];
    }
    float t0 = smin(dmn[0], dmx[0]);
    float t1 = smax(dmn[0], dmx[0]);
    t0 = smax(t0, smin(dmn[1], dmx[1]));
    t1 = smin(t1, smax(dmn[1], dmx[1]));
    t0 = smax(t0, smin(dmn[2], dmx[2]));
    t1 = smin(t1, smax(dmn[2], dmx[2]));
    if (t0 > t1) { t0 = t1 = -1.0f; }
    *T0 = t0; *T1 = t1;
}

/* Moller-Trumbore: RayTriangleTest (AccelerationStructure.h:70-97) with
 * Cross/Dot of Geometry.h (left-to-right sums). */
static inline int tri_test(const float* A, const float* B, const float* C, const float o[3],
                           const float d[3], float* u, float* v, float* t) {
    float E1[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
    float E2[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
    float P[3] = {(d[1] * E2[2]) - (d[2] * E2[1]), (d[2] * E2[0]) - (d[0] * E2[2]),
                  (d[0] * E2[1]) - (d[1] * E2[0])};
    float det = E1[0] * P[0] + E1[1] * P[1] + E1[2] * P[2];
    det = 1.0f / det;
    float T[3] = {o[0] - A[0], o[1] - A[1], o[2] - A[2]};
    float res = T[0] * P[0] + T[1] * P[1] + T[2] * P[2];
    float uu = res * det;
    float Q[3] = {(T[1] * E1[2]) - (T[2] * E1[1]), (T[2] * E1[0]) - (T[0] * E1[2]),
                  (T[0] * E1[1]) - (T[1] * E1[0])};
    float vv = d[0] * Q[0] + d[1] * Q[1] + d[2] * Q[2];
    vv *= det;
    float tt = E2[0] * Q[0] + E2[1] * Q[1] + E2[2] * Q[2];
    tt *= det;
    *u = uu; *v = vv; *t = tt;
    return (uu >= 0.0f) && (uu <= 1.0f) && (vv >= 0.0f) && ((uu + vv) <= 1.0f) && (tt >= 0.0f);
}

/* Closest hit over the implicit heap: LBVH_IntersectP (LBVH.hlsl:363-440) /
 * LBVH::IntersectP (LBVH.cpp:919-1039), with the same box test, the same
 * triangle test, the same pruning (a node is entered unless T1 < 0 or
 * T0 > closest t, LBVH.cpp:992 / LBVH.hlsl:390) and depth-first order.
 * Differences, none of which changes a result:
 *   - the excluded triangle is skipped without overwriting it (LBVH.hlsl:415;
 *     LBVH.cpp:1015 overwrites TriangleID, which only matters for rays that
 *     carry an exclusion);
 *   - ties at equal t keep the smaller triangle id, so the result does not
 *     depend on the order triangles are tested in;
 *   - the near child is chosen by the ray direction on the node's split
 *     axis.  The reference indexes signo[] with the stored axis field
 *     (LBVH.cpp:1033, LBVH.hlsl:432), which build_recursive sets to
 *     (30 - bit) % 3: one axis after the one the bit splits (bits 3k+2,
 *     3k+1, 3k split x, y, z).  The split axis is (field + 2) % 3.  Visiting
 *     order only changes how many nodes are tested, not the closest hit
 *     under the tie rule; the golden tests against LBVH::IntersectP pin it.
 * Walk: both children of an entered internal node (heap slots 2i, 2i+1) are
 * box-tested together, the near one is entered, a hit far one is pushed with
 * its entry distance and re-checked against the closest t when popped.
 * Box tests are counted as 1 (root) + 2 per entered internal node.
 *
 * Restart (the iRoot argument of LBVH_IntersectP, LBVH.hlsl:363-376, fed
 * from the previous intersection's leaf at CSIntersections.hlsl:32 and
 * CSComputeColorRT.hlsl:160): with start > 1 the walk begins at heap node
 * `start` instead of the root.  The reference's trail bits then visit
 * start, its sibling, the parent's sibling and so on up to level 1, which
 * together cover the whole heap; here the siblings of start's ancestors are
 * box-tested first (one test each, deepest on top of the stack) and start's
 * own box next.  A box that contains a child's box admits the child's rays
 * (the slab arithmetic is monotone in the bounds), so the closest hit is the
 * one a walk from the root finds, except where two triangles are hit within
 * an ulp of each other and a box entry distance rounded past the nearer one
 * lets the order decide (as between any two walk orders).  start must
 * be a node the build reached (a leaf a trace of the same tree returned).
 * *leaf_out = the heap node whose triangles gave the closest hit (the
 * reference's iRoot, LBVH.hlsl:422), or 1 when nothing was hit. */
static void trace_one_from(const or_node* nodes, const uint32_t* ids, const float* tris, const float* r,
                           or_hit* out, uint32_t* stats, int any_hit, uint32_t start, uint32_t* leaf_out) {
    const float o[3] = {r[0], r[1], r[2]};
    const float d[3] = {r[3], r[4], r[5]};
    const int exclude = (int)r[7];
    float inv[3] = {1.0f / d[0], 1.0f / d[1], 1.0f / d[2]};
    int sgn[3] = {d[0] < 0.0f, d[1] < 0.0f, d[2] < 0.0f};
    float best_t = r[6], best_u = -1.0f, best_v = -1.0f;
    int best_id = -1;
    uint32_t best_leaf = 1;
    uint32_t nbox = 1, ntri = 0;
    uint32_t stack_node[64];
    float stack_t0[64];
    int sp = 0;
    float T0, T1;
    uint32_t node = 1;
    if (start > 1) {
        const int D = hb32(start);
        for (int k = 1; k <= D; ++k) {
            const uint32_t sib = (start >> (D - k)) ^ 1u;
            box_interval(&nodes[sib], o, inv, &T0, &T1);
            ++nbox;
            if (r[6] > 0.0f && !(T1 < 0.0f) && !(T0 > best_t)) { stack_node[sp] = sib; stack_t0[sp] = T0; ++sp; }
        }
        node = start;
    }
    box_interval(&nodes[node], o, inv, &T0, &T1);
    /* no t satisfies 0 <= t < tmax when tmax <= 0 or is NaN */
    int have = r[6] > 0.0f && !(T1 < 0.0f) && !(T0 > best_t);
    for (;;) {
        if (have) {
            const or_node* nd = &nodes[node];
            if (nd->prim_count & 4) {
                int cnt = nd->prim_count >> 3;
                int pos = nd->prim_pos;
                for (int i = 0; i < cnt; ++i) {
                    ++ntri;
                    int id = (int)ids[pos + i];
                    if (id == exclude) continue;
                    const float* t = tris + 9 * (size_t)id;
                    float u, v, tt;
                    if (tri_test(t, t + 3, t + 6, o, d, &u, &v, &tt)) {
                        if (tt < best_t || (tt == best_t && best_id >= 0 && id < best_id)) {
                            best_t = tt; best_u = u; best_v = v; best_id = id; best_leaf = node;
                        }
                    }
                }
                if (any_hit && best_id >= 0) break;
            } else {
                const uint32_t c0 = node << 1;
                float tl, tr, t1l, t1r;
                box_interval(&nodes[c0], o, inv, &tl, &t1l);
                box_interval(&nodes[c0 + 1], o, inv, &tr, &t1r);
                nbox += 2;
                const int hl = !(t1l < 0.0f) && !(tl > best_t);
                const int hr = !(t1r < 0.0f) && !(tr > best_t);
                const int near_right = sgn[((nd->prim_count & 3) + 2) % 3];
                const int hn = near_right ? hr : hl, hf = near_right ? hl : hr;
                const float tf = near_right ? tl : tr;
                const uint32_t nn = c0 | (uint32_t)near_right, nf = nn ^ 1u;
                if (hn) {
                    if (hf) { stack_node[sp] = nf; stack_t0[sp] = tf; ++sp; }
                    node = nn;
                    continue;
                } else if (hf) {
                    node = nf;
                    continue;
                }
            }
        }
        int found = 0;
        while (sp > 0) {
            --sp;
            if (!(stack_t0[sp] > best_t)) { node = stack_node[sp]; found = 1; break; }
        }
        if (!found) break;
        have = 1;
    }
    out->id = best_id;
    out->u = best_u;
    out->v = best_v;
    out->t = best_t;
    if (stats) { stats[0] = nbox; stats[1] = ntri; }
    if (leaf_out) *leaf_out = best_leaf;
}

static void trace_one(const or_node* nodes, const uint32_t* ids, const float* tris, const float* r,
                      or_hit* out, uint32_t* stats, int any_hit) {
    trace_one_from(nodes, ids, tris, r, out, stats, any_hit, 1u, NULL);
}

void or_trace(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
              const float* rays, uint32_t nrays, or_hit* hits, uint32_t* stats, int any_hit,
              int nthreads) {
    (void)depth;
    if (nthreads <= 0) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long i = 0; i < (long)nrays; ++i)
        trace_one(nodes, ids, tris, rays + 8 * i, &hits[i], stats ? stats + 2 * i : NULL, any_hit);
}

void or_trace_from(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
                   const float* rays, uint32_t nrays, const uint32_t* starts, or_hit* hits, uint32_t* leaves,
                   uint32_t* stats, int any_hit, int nthreads) {
    (void)depth;
    if (nthreads <= 0) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long i = 0; i < (long)nrays; ++i)
        trace_one_from(nodes, ids, tris, rays + 8 * i, &hits[i], stats ? stats + 2 * i : NULL, any_hit,
                       starts ? starts[i] : 1u, leaves ? leaves + i : NULL);
}

/* ------------------------------------------------------------------------ */
/* Primary rays: CSPrimaryRays.hlsl:36-56 (RT branch).  Pixel centre
 * x = (2i + 1 - W) / H, y = -(2j + 1 - H) / H (the reference multiplies by
 * inverse = 1/N), camera-space direction (x*tan, y*tan, 1), origin = eye,
 * normalised as Normalize() in Geometry.h (divide by the length). */
static inline void camera_dir(const or_camera* cam, float x, float y, float d[3]) {
    float dx = x * cam->tan_half_fovy;
    float dy = y * cam->tan_half_fovy;
    for (int c = 0; c < 3; ++c) d[c] = (cam->right[c] * dx + cam->up[c] * dy) + cam->fwd[c];
    float len = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    d[0] /= len; d[1] /= len; d[2] /= len;
}

void or_primary_rays(const or_camera* cam, float* rays) {
    const float inv = 1.0f / (float)cam->height;
    for (uint32_t j = 0; j < cam->height; ++j)
        for (uint32_t i = 0; i < cam->width; ++i) {
            float* r = rays + 8 * ((size_t)j * cam->width + i);
            float x = (float)(2 * (int)i + 1 - (int)cam->width) * inv;
            float y = -((float)(2 * (int)j + 1 - (int)cam->height) * inv);
            float d[3];
            camera_dir(cam, x, y, d);
            r[0] = cam->eye[0]; r[1] = cam->eye[1]; r[2] = cam->eye[2];
            r[3] = d[0]; r[4] = d[1]; r[5] = d[2];
            r[6] = 1e16f;   /* ray.fMaxT (CSPrimaryRays.hlsl:50) */
            r[7] = -1.0f;   /* ray.iTriangleId (:53) */
        }
}

static inline float dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* Flat shading normal and the secondary rays of CSComputeColorRT.hlsl:
 *   N = normalize(cross(B - A, C - A))                  (:61-63, :75)
 *   Nf = -N if dot(N, d) > 0                            (:126-131)
 *   hit = o + t*d; L = hit - light; dist = |L|; L /= dist (:134-138)
 *   mirror = normalize(reflect(d, Nf)), reflect(i,n) = i - 2*dot(i,n)*n (:141-142)
 *   shadow ray cast iff dot(N,L) * dot(N,d) > 0 (unflipped N, :145-147),
 *   origin hit, direction -L, maxT dist, excluding the hit triangle (:149-153). */
static void secondary(const float* tris, const float* r, const or_hit* h, const float light[3],
                      float shadow[8], float mirror[8], int* cast) {
    const float* t = tris + 9 * (size_t)h->id;
    float E1[3] = {t[3] - t[0], t[4] - t[1], t[5] - t[2]};
    float E2[3] = {t[6] - t[0], t[7] - t[1], t[8] - t[2]};
    float N[3] = {(E1[1] * E2[2]) - (E1[2] * E2[1]), (E1[2] * E2[0]) - (E1[0] * E2[2]),
                  (E1[0] * E2[1]) - (E1[1] * E2[0])};
    float nl = sqrtf(dot3(N, N));
    N[0] /= nl; N[1] /= nl; N[2] /= nl;
    const float* d = r + 3;
    float Nf[3] = {N[0], N[1], N[2]};
    if (dot3(Nf, d) > 0.0f) { Nf[0] = -Nf[0]; Nf[1] = -Nf[1]; Nf[2] = -Nf[2]; }
    float P[3];
    for (int c = 0; c < 3; ++c) P[c] = r[c] + h->t * d[c];
    float L[3] = {P[0] - light[0], P[1] - light[1], P[2] - light[2]};
    float dist = sqrtf(dot3(L, L));
    L[0] /= dist; L[1] /= dist; L[2] /= dist;
    float k = 2.0f * dot3(d, Nf);
    float R[3] = {d[0] - k * Nf[0], d[1] - k * Nf[1], d[2] - k * Nf[2]};
    float rl = sqrtf(dot3(R, R));
    R[0] /= rl; R[1] /= rl; R[2] /= rl;
    float ls = dot3(N, L);
    float rs = dot3(N, d);
    *cast = (ls * rs) > 0.0f;
    shadow[0] = P[0]; shadow[1] = P[1]; shadow[2] = P[2];
    shadow[3] = -L[0]; shadow[4] = -L[1]; shadow[5] = -L[2];
    shadow[6] = dist; shadow[7] = (float)h->id;
    mirror[0] = P[0]; mirror[1] = P[1]; mirror[2] = P[2];
    mirror[3] = R[0]; mirror[4] = R[1]; mirror[5] = R[2];
    mirror[6] = r[6]; mirror[7] = (float)h->id;
}

void or_shadow_mirror(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
                      const or_camera* cam, const float light[3], const or_hit* prim, uint8_t* vis,
                      or_hit* mirror, uint32_t* shadow_stats, uint32_t* mirror_stats, int nthreads) {
    or_shadow_mirror_from(nodes, depth, ids, tris, cam, light, prim, NULL, vis, mirror, NULL, shadow_stats,
                          mirror_stats, nthreads);
}

/* The shading rays started at the primary hit's leaf (prim_leaves, the
 * iRoot the colour stage passes to LBVH_IntersectP, CSComputeColorRT.hlsl:160,
 * and the next intersection stage, CSIntersections.hlsl:32); NULL: the root.
 * mirror_leaves (nullable) receives the mirror hit's leaf. */
void or_shadow_mirror_from(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
                           const or_camera* cam, const float light[3], const or_hit* prim,
                           const uint32_t* prim_leaves, uint8_t* vis, or_hit* mirror, uint32_t* mirror_leaves,
                           uint32_t* shadow_stats, uint32_t* mirror_stats, int nthreads) {
    (void)depth;
    const long npx = (long)cam->width * cam->height;
    if (nthreads <= 0) nthreads = 1;
    const float inv = 1.0f / (float)cam->height;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long p = 0; p < npx; ++p) {
        uint32_t i = (uint32_t)(p % cam->width), j = (uint32_t)(p / cam->width);
        if (shadow_stats) { shadow_stats[2 * p] = 0; shadow_stats[2 * p + 1] = 0; }
        if (mirror_stats) { mirror_stats[2 * p] = 0; mirror_stats[2 * p + 1] = 0; }
        if (mirror_leaves) mirror_leaves[p] = 1;
        if (prim[p].id < 0) {
            vis[p] = 0;
            mirror[p].id = -2; mirror[p].u = -1.0f; mirror[p].v = -1.0f; mirror[p].t = 0.0f;
            continue;
        }
        const uint32_t start = prim_leaves ? prim_leaves[p] : 1u;
        float r[8];
        float x = (float)(2 * (int)i + 1 - (int)cam->width) * inv;
        float y = -((float)(2 * (int)j + 1 - (int)cam->height) * inv);
        camera_dir(cam, x, y, r + 3);
        r[0] = cam->eye[0]; r[1] = cam->eye[1]; r[2] = cam->eye[2];
        r[6] = 1e16f; r[7] = -1.0f;
        float sr[8], mr[8];
        int cast;
        secondary(tris, r, &prim[p], light, sr, mr, &cast);
        if (cast) {
            or_hit sh;
            trace_one_from(nodes, ids, tris, sr, &sh, shadow_stats ? shadow_stats + 2 * p : NULL, 1, start, NULL);
            vis[p] = (sh.id >= 0) ? 2 : 3;
        } else {
            vis[p] = 1;
        }
        trace_one_from(nodes, ids, tris, mr, &mirror[p], mirror_stats ? mirror_stats + 2 * p : NULL, 0, start,
                       mirror_leaves ? mirror_leaves + p : NULL);
    }
}

/* ------------------------------------------------------------------------ */
/* PCG32 (M. O'Neill, pcg32_random_r / pcg32_srandom_r, pcg-random.org). */
typedef struct { uint64_t state, inc; } pcg32;
static inline uint32_t pcg32_next(pcg32* g) {
    uint64_t old = g->state;
    g->state = old * 6364136223846793005ULL + g->inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((-rot) & 31u));
}
static inline void pcg32_seed(pcg32* g, uint64_t initstate, uint64_t initseq) {
    g->state = 0u;
    g->inc = (initseq << 1u) | 1u;
    pcg32_next(g);
    g->state += initstate;
    pcg32_next(g);
}
static inline float pcg32_float(pcg32* g) { return (float)(pcg32_next(g) >> 8) * (1.0f / 16777216.0f); }
static inline uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
/* One PCG32 stream per (pixel, sample): state from splitmix64, stream id =
 * pixel index. */
static inline void pt_seed(pcg32* g, uint64_t seed, uint64_t pixel, uint32_t sample) {
    uint64_t s = splitmix64(seed + 0x9E3779B97F4A7C15ULL * (pixel * 65536ULL + sample + 1ULL));
    pcg32_seed(g, s, pixel);
}

uint32_t or_pcg32_first(uint64_t initstate, uint64_t initseq, uint32_t count, uint32_t* out) {
    pcg32 g;
    pcg32_seed(&g, initstate, initseq);
    for (uint32_t i = 0; i < count; ++i) out[i] = pcg32_next(&g);
    return count;
}

/* Cosine-weighted direction about the unit normal n: Malley's method (a
 * uniform point of the unit disc by rejection, lifted to the hemisphere)
 * in the orthonormal basis of Duff et al., "Building an Orthonormal Basis,
 * Revisited" (JCGT 2017).  Only +,-,*,/ and sqrt, so CPU and GPU agree
 * bit for bit. */
static inline void cosine_dir(pcg32* g, const float n[3], float out[3]) {
    float x = 0.0f, y = 0.0f, r2 = 0.0f;
    for (int k = 0; k < 64; ++k) {
        x = 2.0f * pcg32_float(g) - 1.0f;
        y = 2.0f * pcg32_float(g) - 1.0f;
        r2 = x * x + y * y;
        if (r2 <= 1.0f) break;
        x = 0.0f; y = 0.0f; r2 = 0.0f;
    }
    float z = sqrtf(1.0f - r2);
    float sign = copysignf(1.0f, n[2]);
    float a = -1.0f / (sign + n[2]);
    float b = n[0] * n[1] * a;
    float T[3] = {1.0f + sign * n[0] * n[0] * a, sign * b, -sign * n[0]};
    float B[3] = {b, sign + n[1] * n[1] * a, -n[1]};
    for (int c = 0; c < 3; ++c) out[c] = (T[c] * x + B[c] * y) + n[c] * z;
}

/* Camera ray with a sub-pixel jitter in [-1,1) pixel half-widths
 * (the GI branch of CSPrimaryRays.hlsl:23-34). */
static inline void pt_camera_ray(const or_camera* cam, uint32_t i, uint32_t j, pcg32* g, float r[8]) {
    const float inv = 1.0f / (float)cam->height;
    float jx = 2.0f * pcg32_float(g) - 1.0f;
    float jy = 2.0f * pcg32_float(g) - 1.0f;
    float x = ((float)(2 * (int)i + 1 - (int)cam->width) + jx) * inv;
    float y = -(((float)(2 * (int)j + 1 - (int)cam->height) + jy) * inv);
    camera_dir(cam, x, y, r + 3);
    r[0] = cam->eye[0]; r[1] = cam->eye[1]; r[2] = cam->eye[2];
    r[6] = 1e16f; r[7] = -1.0f;
}

/* Facing geometric normal at a hit (CSComputeColorGI.hlsl:60-62, :126-130). */
static inline void facing_normal(const float* t, const float d[3], float N[3]) {
    float E1[3] = {t[3] - t[0], t[4] - t[1], t[5] - t[2]};
    float E2[3] = {t[6] - t[0], t[7] - t[1], t[8] - t[2]};
    N[0] = (E1[1] * E2[2]) - (E1[2] * E2[1]);
    N[1] = (E1[2] * E2[0]) - (E1[0] * E2[2]);
    N[2] = (E1[0] * E2[1]) - (E1[1] * E2[0]);
    float nl = sqrtf(dot3(N, N));
    N[0] /= nl; N[1] /= nl; N[2] /= nl;
    if (dot3(N, d) > 0.0f) { N[0] = -N[0]; N[1] = -N[1]; N[2] = -N[2]; }
}

#define OR_MAX_SEG 16

/* One path: returns the number of recorded hit segments, fills per-segment
 * triangle ids; *missed = 1 if the path left the scene after them. */
static int trace_path(const or_node* nodes, const uint32_t* ids, const float* tris,
                      const or_camera* cam, uint32_t i, uint32_t j, uint32_t sample,
                      const or_pt_params* p, int* seg_id, int* missed) {
    pcg32 g;
    uint64_t pixel = (uint64_t)j * cam->width + i;
    pt_seed(&g, p->seed, pixel, sample);
    float r[8];
    pt_camera_ray(cam, i, j, &g, r);
    int nseg = 0;
    *missed = 0;
    /* each bounce walks from the leaf of the previous hit, the iRoot of the
     * reference's intersection stage (CSIntersections.hlsl:32) */
    uint32_t start = 1u;
    for (uint32_t s = 0; s <= p->bounces && s < OR_MAX_SEG; ++s) {
        or_hit h;
        uint32_t leaf = 1u;
        trace_one_from(nodes, ids, tris, r, &h, NULL, 0, start, &leaf);
        if (h.id < 0) { *missed = 1; break; }
        start = leaf;
        seg_id[nseg++] = h.id;
        if (s == p->bounces) break;
        const float* t = tris + 9 * (size_t)h.id;
        float N[3], P[3], nd[3];
        facing_normal(t, r + 3, N);
        for (int c = 0; c < 3; ++c) P[c] = r[c] + h.t * r[3 + c];
        cosine_dir(&g, N, nd);
        r[0] = P[0]; r[1] = P[1]; r[2] = P[2];
        r[3] = nd[0]; r[4] = nd[1]; r[5] = nd[2];
        r[6] = 1e16f; r[7] = (float)h.id;
    }
    return nseg;
}

/* Progressive mean of CSComputeColorGI.hlsl:218,227 with the factors of
 * cbGlobalIllumination::Update (ConstantBuffers.h:102-109):
 *   acc *= n/(n+1)  (CSPrimaryRays.hlsl:63), then per segment
 *   acc += (1/(n+1) * beta) * Le,  beta *= albedo; a miss adds the sky. */
/* The window of the image a call covers (the whole image when win_w = 0). */
static void pt_window(const or_camera* cam, const or_pt_params* p, uint32_t* x0, uint32_t* y0, uint32_t* w,
                      uint32_t* h) {
    if (p->win_w == 0) {
        *x0 = 0; *y0 = 0; *w = cam->width; *h = cam->height;
    } else {
        *x0 = p->x0; *y0 = p->y0; *w = p->win_w; *h = p->win_h;
    }
}

void or_pathtrace(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
                  const float* albedo, const float* emission, const or_camera* cam,
                  const or_pt_params* p, float* image, int nthreads) {
    (void)depth;
    uint32_t wx0, wy0, ww, wh;
    pt_window(cam, p, &wx0, &wy0, &ww, &wh);
    const long npx = (long)ww * wh;
    const uint32_t n0 = p->first_sample;
    if (nthreads <= 0) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (long px = 0; px < npx; ++px) {
        uint32_t i = wx0 + (uint32_t)(px % ww), j = wy0 + (uint32_t)(px / ww);
        float acc[3] = {0.0f, 0.0f, 0.0f};
        if (n0 > 0) /* continue the progressive mean of samples 0 .. n0-1 */
            for (int c = 0; c < 3; ++c) acc[c] = image[4 * px + c];
        for (uint32_t n = n0; n < n0 + p->spp; ++n) {
            float fant = (float)n / (float)(n + 1);
            float fact = 1.0f / (float)(n + 1);
            for (int c = 0; c < 3; ++c) acc[c] *= fant;
            int seg[OR_MAX_SEG], missed;
            int ns = trace_path(nodes, ids, tris, cam, i, j, n, p, seg, &missed);
            float beta[3] = {1.0f, 1.0f, 1.0f};
            for (int s = 0; s < ns; ++s) {
                const float* le = emission + 3 * (size_t)seg[s];
                const float* al = albedo + 3 * (size_t)seg[s];
                for (int c = 0; c < 3; ++c) {
                    acc[c] += (fact * beta[c]) * le[c];
                    beta[c] = beta[c] * al[c];
                }
            }
            if (missed)
                for (int c = 0; c < 3; ++c) acc[c] += (fact * beta[c]) * p->sky[c];
        }
        float* o = image + 4 * px;
        o[0] = acc[0]; o[1] = acc[1]; o[2] = acc[2]; o[3] = 1.0f;
    }
}

/* Adjoint by path replay.  For one path with hit albedos a_s, radiances E_s
 * (E of a trailing miss = sky) and throughputs beta_0 = 1,
 * beta_{s+1} = beta_s * a_s, the contribution is C = sum_s beta_s * E_s, so
 *   dC/da_j = beta_j * G_j,  G_j = E_{j+1} + a_{j+1} * G_{j+1}
 *   dC/dLe  = sum over emitting hits of beta_s
 * with the per-sample weight of the progressive mean. */
void or_pathtrace_adjoint(const or_node* nodes, uint32_t depth, const uint32_t* ids,
                          const float* tris, const float* albedo, const float* emission,
                          const or_camera* cam, const or_pt_params* p, const float* d_image,
                          double* d_albedo, double* d_emission_scale, int nthreads) {
    (void)depth;
    uint32_t wx0, wy0, ww, wh;
    pt_window(cam, p, &wx0, &wy0, &ww, &wh);
    const long npx = (long)ww * wh;
    if (nthreads <= 0) nthreads = 1;
    /* weight of sample n0 + k in the progressive mean after the call */
    double wsample[64];
    const uint32_t n0 = p->first_sample;
    uint32_t spp = p->spp < 64 ? p->spp : 64;
    for (uint32_t k = 0; k < spp; ++k) {
        uint32_t n = n0 + k;
        double w = (double)(1.0f / (float)(n + 1));
        for (uint32_t m = n + 1; m < n0 + spp; ++m) w *= (double)((float)m / (float)(m + 1));
        wsample[k] = w;
    }
    double dle[3] = {0.0, 0.0, 0.0};
#pragma omp parallel num_threads(nthreads)
    {
        double dle_local[3] = {0.0, 0.0, 0.0};
#pragma omp for schedule(dynamic, 16)
        for (long px = 0; px < npx; ++px) {
            uint32_t i = wx0 + (uint32_t)(px % ww), j = wy0 + (uint32_t)(px / ww);
            const float* g = d_image + 4 * px;
            for (uint32_t k = 0; k < spp; ++k) {
                const uint32_t n = k;  /* wsample index; the stream is sample n0 + k */
                int seg[OR_MAX_SEG], missed;
                int ns = trace_path(nodes, ids, tris, cam, i, j, n0 + k, p, seg, &missed);
                double beta[OR_MAX_SEG + 1][3];
                beta[0][0] = beta[0][1] = beta[0][2] = 1.0;
                for (int s = 0; s < ns; ++s)
                    for (int c = 0; c < 3; ++c)
                        beta[s + 1][c] = beta[s][c] * (double)albedo[3 * (size_t)seg[s] + c];
                double G[3] = {0.0, 0.0, 0.0};
                if (missed)
                    for (int c = 0; c < 3; ++c) G[c] = (double)p->sky[c];
                for (int s = ns - 1; s >= 0; --s) {
                    const float* al = albedo + 3 * (size_t)seg[s];
                    const float* le = emission + 3 * (size_t)seg[s];
                    int emitter = (le[0] != 0.0f) || (le[1] != 0.0f) || (le[2] != 0.0f);
                    for (int c = 0; c < 3; ++c) {
                        double gw = (double)g[c] * wsample[n];
                        double da = gw * beta[s][c] * G[c];
                        if (da != 0.0) {
#pragma omp atomic
                            d_albedo[3 * (size_t)seg[s] + c] += da;
                        }
                        if (emitter) dle_local[c] += gw * beta[s][c];
                        G[c] = (double)le[c] + (double)al[c] * G[c];
                    }
                }
            }
        }
#pragma omp critical
        {
            for (int c = 0; c < 3; ++c) dle[c] += dle_local[c];
        }
    }
    for (int c = 0; c < 3; ++c) d_emission_scale[c] = dle[c];
}

/* ------------------------------------------------------------------------ */
/* The ray-tracing colour stage and its bounce loop: RayTracerCS::Render
 * (RayTracerCS.cpp:284-295) runs CSGeneratePrimaryRays, then bounces + 1
 * times CSComputeIntersections (CSIntersections.hlsl:18-39) and
 * CSComputeColor (CSComputeColorRT.hlsl:18-262), without textures or normal
 * maps.  Per pixel, in the reference's operation order:
 *   N   = normalize(cross(B-A, C-A)), or with Phong normalize(nA*w + nB*u +
 *         nC*v), w = 1 - (u+v) (Vec3BaryCentric, Intersection.hlsl:98-108)
 *   NM  = -N if dot(N, d) > 0                              (:126-131)
 *   P = o + t d; L = (P - light) / |P - light|             (:134-138)
 *   R   = normalize(reflect(d, NM))                        (:141-142)
 *   lit when dot(N,L)*dot(N,d) > 0 and (shadows off or the shadow ray from P
 *   towards the light, excluding the hit triangle, restarted at the hit's
 *   leaf, reaches the light)                               (:145-169)
 *   spec = max(0, -dot(L, R))^49, diff = max(0, -dot(NM, L))  (:164-175)
 *   colour = (amb + diff*kd.w)*kd + spec*(1 - kd.w)*ks', ks'.w = ks.w*gloss,
 *   times (factor, 1)                                      (:183-200)
 *   next ray: from P; with probability alpha the mirror ray R and factor *=
 *   ks.xyz, else refract(d, NM, eta) with eta = amb.w (1/amb.w entering),
 *   normalised, factor *= kd.xyz, or R on total internal reflection (:203-231)
 *   a miss: colour = (factor * env, 1) and the ray ends (:233-245)
 *   accumulation += colour, result = accumulation          (:255-256)
 * A pixel whose intersection id is below the environment flag (a miss with
 * the flag 0) gets result 1 and keeps its ray, so every later bounce finds
 * the same miss (:29-35).  The random texture sample of :204-207 is a hash
 * of (seed, pixel, bounce); normalize divides by the length (as Geometry.h
 * does) and pow(x, 49) is x^32 * x^16 * x, so the CUDA kernels can match
 * these values bit for bit. */
static inline uint32_t lowbias32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

float or_whitted_rand(uint32_t seed, uint32_t pixel, uint32_t bounce) {
    const uint32_t h = lowbias32(pixel ^ lowbias32(seed ^ (0x9e3779b9U * (bounce + 1U))));
    return (float)(h >> 8) * (1.0f / 16777216.0f);
}

static inline float pow49(float x) {
    float x2 = x * x, x4 = x2 * x2, x8 = x4 * x4, x16 = x8 * x8, x32 = x16 * x16;
    return (x32 * x16) * x;
}

static inline void normalize3v(float v[3]) {
    float l = sqrtf(dot3(v, v));
    v[0] /= l; v[1] /= l; v[2] /= l;
}

static void whitted_pixel(const or_node* nodes, const uint32_t* ids, const float* tris, const float* normals,
                          const int32_t* mat_ids, const or_material* mats, uint32_t nmat, const or_camera* cam,
                          const float light[3], const or_shade_params* sp, uint32_t i, uint32_t j, float acc[4],
                          float res[4]) {
    const uint32_t pixel = j * cam->width + i;
    const float inv = 1.0f / (float)cam->height;
    float o[3] = {cam->eye[0], cam->eye[1], cam->eye[2]}, d[3];
    float x = (float)(2 * (int)i + 1 - (int)cam->width) * inv;
    float y = -((float)(2 * (int)j + 1 - (int)cam->height) * inv);
    camera_dir(cam, x, y, d);
    float factor[3] = {1.0f, 1.0f, 1.0f};
    int exclude = -1;
    uint32_t start = 1;
    for (int c = 0; c < 4; ++c) { acc[c] = 0.0f; res[c] = 0.0f; }
    for (uint32_t b = 0; b <= sp->bounces; ++b) {
        float r[8] = {o[0], o[1], o[2], d[0], d[1], d[2], 1e16f, (float)exclude};
        or_hit h;
        uint32_t leaf = 1;
        trace_one_from(nodes, ids, tris, r, &h, NULL, 0, start, &leaf);
        const int id = h.id;
        if (id < sp->env_mapping) {
            if (id > -2) for (int c = 0; c < 4; ++c) res[c] = 1.0f;
            return;  /* the same miss at every later bounce */
        }
        float fin[4] = {0.0f, 0.0f, 0.0f, 1.0f};
        if (id < 0) {
            for (int c = 0; c < 3; ++c) fin[c] = factor[c] * sp->env_color[c];
            for (int c = 0; c < 4; ++c) acc[c] += fin[c];
            for (int c = 0; c < 4; ++c) res[c] = acc[c];
            return;  /* the ray ends */
        }
        const float* t = tris + 9 * (size_t)id;
        float E1[3] = {t[3] - t[0], t[4] - t[1], t[5] - t[2]};
        float E2[3] = {t[6] - t[0], t[7] - t[1], t[8] - t[2]};
        float N[3] = {(E1[1] * E2[2]) - (E1[2] * E2[1]), (E1[2] * E2[0]) - (E1[0] * E2[2]),
                      (E1[0] * E2[1]) - (E1[1] * E2[0])};
        normalize3v(N);
        if (sp->phong && normals) {
            const float* nn = normals + 9 * (size_t)id;
            const float w = 1.0f - (h.u + h.v);
            for (int c = 0; c < 3; ++c) N[c] = (nn[c] * w + nn[3 + c] * h.u) + nn[6 + c] * h.v;
            normalize3v(N);
        }
        float NM[3] = {N[0], N[1], N[2]};
        int inverse = 0;
        if (dot3(NM, d) > 0.0f) { NM[0] = -NM[0]; NM[1] = -NM[1]; NM[2] = -NM[2]; inverse = 1; }
        float P[3], L[3];
        for (int c = 0; c < 3; ++c) P[c] = o[c] + h.t * d[c];
        for (int c = 0; c < 3; ++c) L[c] = P[c] - light[c];
        const float dist = sqrtf(dot3(L, L));
        L[0] /= dist; L[1] /= dist; L[2] /= dist;
        const float k2 = 2.0f * dot3(d, NM);
        float R[3] = {d[0] - k2 * NM[0], d[1] - k2 * NM[1], d[2] - k2 * NM[2]};
        normalize3v(R);
        const float ls = dot3(N, L), rs = dot3(N, d);
        float spec = 0.0f, diff = 0.0f, spec_w = 1.0f, diff_w = 1.0f;
        if (ls * rs > 0.0f) {
            int lit = 1;
            if (sp->shadows) {
                float s[8] = {P[0], P[1], P[2], -L[0], -L[1], -L[2], dist, (float)id};
                or_hit sh;
                trace_one_from(nodes, ids, tris, s, &sh, NULL, 1, leaf, NULL);
                lit = sh.id < 0;
            }
            if (lit) {
                spec = pow49(fmaxf(0.0f, -dot3(L, R)));
                diff = fmaxf(0.0f, -dot3(NM, L));
                spec_w = spec;
                diff_w = diff;
            }
        }
        uint32_t m = mat_ids ? (uint32_t)mat_ids[id] : 0u;
        if (m >= nmat) m = 0;
        const or_material* mt = &mats[m];
        float ks[4] = {mt->specular[0], mt->specular[1], mt->specular[2], mt->specular[3] * (float)sp->gloss_mapping};
        const float* amb = mt->ambient;
        const float* kd = mt->diffuse;
        const float dv[4] = {diff, diff, diff, diff_w}, sv[4] = {spec, spec, spec, spec_w};
        for (int c = 0; c < 4; ++c) {
            const float dc = (amb[c] + dv[c] * kd[3]) * kd[c];
            const float sc = (sv[c] * (1.0f - kd[3])) * ks[c];
            fin[c] = dc + sc;
        }
        for (int c = 0; c < 3; ++c) fin[c] *= factor[c];
        for (int c = 0; c < 4; ++c) acc[c] += fin[c];
        for (int c = 0; c < 4; ++c) res[c] = acc[c];
        /* the next ray */
        float nd[3] = {R[0], R[1], R[2]};
        if (mt->alpha >= or_whitted_rand(sp->seed, pixel, b)) {
            for (int c = 0; c < 3; ++c) factor[c] *= ks[c];
        } else {
            float eta = amb[3];
            if (!inverse) eta = 1.0f / eta;
            const float ci = dot3(NM, d);
            const float kk = 1.0f - (eta * eta) * (1.0f - ci * ci);
            float T[3] = {0.0f, 0.0f, 0.0f};
            if (!(kk < 0.0f)) {
                const float sq = eta * ci + sqrtf(kk);
                for (int c = 0; c < 3; ++c) T[c] = eta * d[c] - sq * NM[c];
            }
            const float tl = sqrtf(dot3(T, T));
            if (!(tl < 0.000001f)) {
                for (int c = 0; c < 3; ++c) nd[c] = T[c] / tl;
                for (int c = 0; c < 3; ++c) factor[c] *= kd[c];
            }
        }
        for (int c = 0; c < 3; ++c) { o[c] = P[c]; d[c] = nd[c]; }
        exclude = id;
        start = leaf;
    }
}

void or_render_whitted(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
                       const float* normals, const int32_t* mat_ids, const or_material* mats, uint32_t nmat,
                       const or_camera* cam, const float light[3], const or_shade_params* sp, float* accum,
                       float* result, int nthreads) {
    (void)depth;
    const long npx = (long)cam->width * cam->height;
    if (nthreads <= 0) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long p = 0; p < npx; ++p)
        whitted_pixel(nodes, ids, tris, normals, mat_ids, mats, nmat, cam, light, sp, (uint32_t)(p % cam->width),
                      (uint32_t)(p / cam->width), accum + 4 * p, result + 4 * p);
}

/* ------------------------------------------------------------------------ */
/* Closest hit over the reference's flattened SAH BVH (LinearBVHNode array of
 * BVH::FlattenBVHTree, bvh.cpp:272-293; the same 32-byte record as the LBVH
 * node: bounds, nPrimitives, offset): BVH_IntersectP (BVH.hlsl:124-217).
 * A visited node's box is tested (IntersectBox) and pruned when T1 < 0 or
 * T0 > closest t; a leaf (nPrimitives > 0) tests its triangles ids[offset ..
 * offset + nPrimitives); an interior node (nPrimitives = -split axis) goes
 * to its second child (offset) first when the ray direction is negative on
 * the split axis, else to its first child (the next record), and stacks the
 * other.  Box tests count visited nodes.  Differences from the shader, none
 * of which changes a closest hit: a leaf's triangles are all tested (the
 * shader tests its first one nPrimitives + 1 times, which is the same for
 * the one-primitive leaves it supports), and equal-t ties keep the smaller
 * id.  Rays with tmax <= 0 or NaN walk nothing. */
static void bvh_trace_one(const or_node* nodes, uint32_t num_nodes, const uint32_t* ids, uint32_t n,
                          const float* tris, const float* r, or_hit* out, uint32_t* stats, int any_hit) {
    const float o[3] = {r[0], r[1], r[2]};
    const float d[3] = {r[3], r[4], r[5]};
    const int exclude = (int)r[7];
    float inv[3] = {1.0f / d[0], 1.0f / d[1], 1.0f / d[2]};
    float best_t = r[6], best_u = -1.0f, best_v = -1.0f;
    int best_id = -1;
    uint32_t nbox = 0, ntri = 0;
    uint32_t stack[128];
    int sp = 0;
    uint32_t node = 0;
    int live = r[6] > 0.0f && num_nodes > 0;
    while (live) {
        const or_node* nd = &nodes[node];
        float T0, T1;
        box_interval(nd, o, inv, &T0, &T1);
        ++nbox;
        int next = 0;
        if (!(T1 < 0.0f) && !(T0 > best_t)) {
            if (nd->prim_count > 0) {
                for (int i = 0; i < nd->prim_count; ++i) {
                    const uint32_t k = (uint32_t)nd->prim_pos + (uint32_t)i;
                    if (k >= n) break;
                    ++ntri;
                    const int id = (int)ids[k];
                    if (id == exclude) continue;
                    const float* t = tris + 9 * (size_t)id;
                    float u, v, tt;
                    if (tri_test(t, t + 3, t + 6, o, d, &u, &v, &tt)) {
                        if (tt < best_t || (tt == best_t && best_id >= 0 && id < best_id)) {
                            best_t = tt; best_u = u; best_v = v; best_id = id;
                        }
                    }
                }
                if (any_hit && best_id >= 0) break;
            } else {
                const int axis = -nd->prim_count;
                const int neg = (axis >= 0 && axis < 3) ? (inv[axis] < 0.0f) : 0;
                const uint32_t first = node + 1, second = (uint32_t)nd->prim_pos;
                if (sp >= 128 || first >= num_nodes || second >= num_nodes) break;
                stack[sp++] = neg ? first : second;
                node = neg ? second : first;
                next = 1;
            }
        }
        if (!next) {
            if (sp == 0) break;
            node = stack[--sp];
        }
    }
    out->id = best_id;
    out->u = best_u;
    out->v = best_v;
    out->t = best_t;
    if (stats) { stats[0] = nbox; stats[1] = ntri; }
}

void or_bvh_trace(const or_node* nodes, uint32_t num_nodes, const uint32_t* ids, uint32_t n, const float* tris,
                  const float* rays, uint32_t nrays, or_hit* hits, uint32_t* stats, int any_hit, int nthreads) {
    if (nthreads <= 0) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long i = 0; i < (long)nrays; ++i)
        bvh_trace_one(nodes, num_nodes, ids, n, tris, rays + 8 * i, &hits[i], stats ? stats + 2 * i : NULL, any_hit);
}

/* or_shadow_mirror over the BVH: the same shading rays, traced by
 * bvh_trace_one. */
void or_bvh_shadow_mirror(const or_node* nodes, uint32_t num_nodes, const uint32_t* ids, uint32_t n,
                          const float* tris, const or_camera* cam, const float light[3], const or_hit* prim,
                          uint8_t* vis, or_hit* mirror, uint32_t* shadow_stats, uint32_t* mirror_stats,
                          int nthreads) {
    const long npx = (long)cam->width * cam->height;
    if (nthreads <= 0) nthreads = 1;
    const float inv = 1.0f / (float)cam->height;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long p = 0; p < npx; ++p) {
        uint32_t i = (uint32_t)(p % cam->width), j = (uint32_t)(p / cam->width);
        if (shadow_stats) { shadow_stats[2 * p] = 0; shadow_stats[2 * p + 1] = 0; }
        if (mirror_stats) { mirror_stats[2 * p] = 0; mirror_stats[2 * p + 1] = 0; }
        if (prim[p].id < 0) {
            vis[p] = 0;
            mirror[p].id = -2; mirror[p].u = -1.0f; mirror[p].v = -1.0f; mirror[p].t = 0.0f;
            continue;
        }
        float r[8];
        float x = (float)(2 * (int)i + 1 - (int)cam->width) * inv;
        float y = -((float)(2 * (int)j + 1 - (int)cam->height) * inv);
        camera_dir(cam, x, y, r + 3);
        r[0] = cam->eye[0]; r[1] = cam->eye[1]; r[2] = cam->eye[2];
        r[6] = 1e16f; r[7] = -1.0f;
        float sr[8], mr[8];
        int cast;
        secondary(tris, r, &prim[p], light, sr, mr, &cast);
        if (cast) {
            or_hit sh;
            bvh_trace_one(nodes, num_nodes, ids, n, tris, sr, &sh, shadow_stats ? shadow_stats + 2 * p : NULL, 1);
            vis[p] = (sh.id >= 0) ? 2 : 3;
        } else {
            vis[p] = 1;
        }
        bvh_trace_one(nodes, num_nodes, ids, n, tris, mr, &mirror[p], mirror_stats ? mirror_stats + 2 * p : NULL, 0);
    }
}

/* ------------------------------------------------------------------------ */
/* The reference's own walk, LBVH_IntersectP (LBVH.hlsl:363-440): a stackless
 * walk over the heap driven by a trail word (the `iRoot` restart sets
 * trail = 1 << firstbithigh(node), as if every ancestor had been entered by
 * its first child), one box test per visited node (IntersectBox), the child
 * picked by dirIsNeg[axis field] entered first, each visited leaf's
 * triangles tested in order, a candidate accepted when it is not the
 * excluded triangle, passes RayTriangleTest and is strictly nearer (so on
 * an exact tie the first one tested stays), and fMaxT lowered to it.  It is
 * a closest-hit walk for every ray, shadow rays included
 * (CSComputeColorRT.hlsl:160).  stats = {visited nodes, triangle tests}: the
 * two halves of the shader's iVisitedNodes counter (result++ per node,
 * += 65536 per triangle, :389, :404). */
static void hlsl_walk(const or_node* nodes, const uint32_t* ids, const float* tris, const float* r,
                      uint32_t node, or_hit* out, uint32_t* stats, uint32_t* leaf_out) {
    const float o[3] = {r[0], r[1], r[2]};
    const float d[3] = {r[3], r[4], r[5]};
    const int exclude = (int)r[7];
    const float inv[3] = {1.0f / d[0], 1.0f / d[1], 1.0f / d[2]};
    const int neg[3] = {inv[0] < 0.0f, inv[1] < 0.0f, inv[2] < 0.0f};
    float best_t = r[6], best_u = -1.0f, best_v = -1.0f;
    int best_id = -1;
    uint32_t root = 1, visits = 0, ntri = 0;
    if (node < 1) node = 1;
    uint32_t trail = 1u << hb32(node);
    do {
        float T0, T1;
        box_interval(&nodes[node], o, inv, &T0, &T1);
        const int p = __builtin_ctz(trail + 1u);
        ++visits;
        if (T0 > best_t || T1 < 0.0f) {
            trail = (trail >> p) + 1u;
            node = (node >> p) ^ 1u;
        } else if (nodes[node].prim_count & 4) {
            const int cnt = nodes[node].prim_count >> 3, pos = nodes[node].prim_pos;
            for (int i = 0; i < cnt; ++i) {
                ++ntri;
                const int id = (int)ids[pos + i];
                const float* t = tris + 9 * (size_t)id;
                float u, v, tt;
                if (id != exclude && tri_test(t, t + 3, t + 6, o, d, &u, &v, &tt) && tt < best_t) {
                    best_t = tt; best_u = u; best_v = v; best_id = id; root = node;
                }
            }
            trail = (trail >> p) + 1u;
            node = (node >> p) ^ 1u;
        } else {
            trail <<= 1;
            node = (node << 1) | (uint32_t)neg[nodes[node].prim_count & 3];
        }
    } while (trail > 1u);
    out->id = best_id; out->u = best_u; out->v = best_v; out->t = best_t;
    if (stats) { stats[0] = visits; stats[1] = ntri; }
    if (leaf_out) *leaf_out = root;
}

void or_trace_hlsl(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
                   const float* rays, uint32_t nrays, const uint32_t* starts, or_hit* hits, uint32_t* leaves,
                   uint32_t* stats, int nthreads) {
    (void)depth;
    if (nthreads <= 0) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long i = 0; i < (long)nrays; ++i)
        hlsl_walk(nodes, ids, tris, rays + 8 * i, starts ? starts[i] : 1u, &hits[i], stats ? stats + 2 * i : NULL,
                  leaves ? leaves + i : NULL);
}

/* The shading rays of or_shadow_mirror traced with the reference's own walk
 * (hlsl_walk), restarted at the primary hit's leaf from or_trace_hlsl; the
 * shadow ray is a closest-hit walk as CSComputeColorRT.hlsl:160 issues it. */
void or_shadow_mirror_hlsl(const or_node* nodes, uint32_t depth, const uint32_t* ids, const float* tris,
                           const or_camera* cam, const float light[3], const or_hit* prim, const uint32_t* prim_leaves,
                           uint8_t* vis, or_hit* mirror, uint32_t* shadow_stats, uint32_t* mirror_stats,
                           int nthreads) {
    (void)depth;
    const long npx = (long)cam->width * cam->height;
    if (nthreads <= 0) nthreads = 1;
    const float inv = 1.0f / (float)cam->height;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long p = 0; p < npx; ++p) {
        uint32_t i = (uint32_t)(p % cam->width), j = (uint32_t)(p / cam->width);
        if (shadow_stats) { shadow_stats[2 * p] = 0; shadow_stats[2 * p + 1] = 0; }
        if (mirror_stats) { mirror_stats[2 * p] = 0; mirror_stats[2 * p + 1] = 0; }
        if (prim[p].id < 0) {
            vis[p] = 0;
            mirror[p].id = -2; mirror[p].u = -1.0f; mirror[p].v = -1.0f; mirror[p].t = 0.0f;
            continue;
        }
        float r[8];
        float x = (float)(2 * (int)i + 1 - (int)cam->width) * inv;
        float y = -((float)(2 * (int)j + 1 - (int)cam->height) * inv);
        camera_dir(cam, x, y, r + 3);
        r[0] = cam->eye[0]; r[1] = cam->eye[1]; r[2] = cam->eye[2];
        r[6] = 1e16f; r[7] = -1.0f;
        float sr[8], mr[8];
        int cast;
        secondary(tris, r, &prim[p], light, sr, mr, &cast);
        const uint32_t start = prim_leaves[p];
        if (cast) {
            or_hit sh;
            hlsl_walk(nodes, ids, tris, sr, start, &sh, shadow_stats ? shadow_stats + 2 * p : NULL, NULL);
            vis[p] = (sh.id >= 0) ? 2 : 3;
        } else {
            vis[p] = 1;
        }
        hlsl_walk(nodes, ids, tris, mr, start, &mirror[p], mirror_stats ? mirror_stats + 2 * p : NULL, NULL);
    }
}
