"""Helpers for comparing hits with the reference's own LBVH::IntersectP.

intersect_t: Moller-Trumbore of AccelerationStructure.h:70-97 in numpy
float32 (no fused multiply-add).

assert_matches_reference: hit ids must equal the reference's except on
near-ties -- rays where the reference's triangle and ours are both hit within
the contract's 1e-6 relative t tolerance.  On those rays the reference's own
answer depends on its visit order (strict '<' over leaves in its order, and
a box whose rounded entry distance exceeds a contained hit's t by an ulp is
pruned), so its CPU and GPU paths can disagree too.
"""
import numpy as np

f = np.float32
T_REL_TOL = 1e-6


def intersect_t(ray, tri):
    o = ray[0:3].astype(f)
    d = ray[3:6].astype(f)
    A, B, C = (tri[0:3].astype(f), tri[3:6].astype(f), tri[6:9].astype(f))
    E1 = B - A
    E2 = C - A
    P = np.array([d[1] * E2[2] - d[2] * E2[1], d[2] * E2[0] - d[0] * E2[2], d[0] * E2[1] - d[1] * E2[0]], f)
    det = f(f(E1[0] * P[0] + E1[1] * P[1]) + E1[2] * P[2])
    det = f(f(1.0) / det)
    T = o - A
    Q = np.array([T[1] * E1[2] - T[2] * E1[1], T[2] * E1[0] - T[0] * E1[2], T[0] * E1[1] - T[1] * E1[0]], f)
    t = f(f(f(E2[0] * Q[0] + E2[1] * Q[1]) + E2[2] * Q[2]) * det)
    return t


def assert_matches_reference(hit_id, hit_t, ref_id, ref_t, rays, tris, max_near_tie_frac=0.01):
    hit_id = np.asarray(hit_id)
    hit_t = np.asarray(hit_t)
    assert np.array_equal(hit_id >= 0, ref_id >= 0), "hit / miss differs from the reference"
    h = ref_id >= 0
    rel = np.abs(hit_t[h].astype(np.float64) - ref_t[h]) / np.abs(ref_t[h].astype(np.float64))
    assert rel.max(initial=0.0) <= T_REL_TOL, f"t differs by {rel.max()} relative"
    diff = np.nonzero(hit_id != ref_id)[0]
    near = 0
    for k in diff:  # both triangles are hit at (almost) the same distance
        tr = intersect_t(rays[k], tris[ref_id[k]])
        to = intersect_t(rays[k], tris[hit_id[k]])
        assert tr == ref_t[k] and to == hit_t[k]
        assert abs(float(to) - float(tr)) <= T_REL_TOL * abs(float(tr)), (k, to, tr)
        if to == tr:
            assert hit_id[k] < ref_id[k]  # exact tie: the smaller id is kept
        else:
            near += 1
    assert near <= max_near_tie_frac * len(ref_id), f"{near} ulp-apart id differences"
    return near
