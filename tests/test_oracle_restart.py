"""The oracle's restart walk (iRoot of LBVH_IntersectP, LBVH.hlsl:363-376):
started at any node the build reached, it returns the closest hits of a walk
from the root, and on the golden fixtures those are the reference's own
LBVH::IntersectP hits.  The one exception is the one every walk order has:
two triangles hit within an ulp of each other, where a box entry distance
rounded past the nearer one lets the order decide (the coplanar flat_z
case); there the hits match the reference to the same tolerance the root
walk does.  CPU only."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden
import tri_np


def reached_nodes(nodes, depth):
    from oracle import reachable_mask
    return np.nonzero(reachable_mask(nodes))[0].astype(np.uint32)


@pytest.mark.parametrize("case", golden_cases())
def test_restart_from_hit_leaves_equals_reference(oracle_mod, case):
    g = load_golden(case)
    tris, depth, rays = g["tris"], int(g["depth"]), g["rays"]
    nodes, ids, _, _ = oracle_mod.lbvh_build(tris, depth)
    h0, leaves = oracle_mod.trace_from(nodes, depth, ids, tris, rays)
    assert np.array_equal(h0, oracle_mod.trace(nodes, depth, ids, tris, rays))
    # a leaf reported for a hit holds the hit triangle
    hit = h0["id"] >= 0
    for k in np.nonzero(hit)[0][:200]:
        nd = nodes[leaves[k]]
        assert nd["prim_count"] & 4
        pos, cnt = nd["prim_pos"], nd["prim_count"] >> 3
        assert h0["id"][k] in ids[pos:pos + cnt]
    assert np.all(leaves[~hit] == 1)
    # the same rays restarted at those leaves, and at random reached nodes
    rng = np.random.default_rng(7)
    for starts in (leaves, rng.choice(reached_nodes(nodes, depth), size=len(rays))):
        h1, l1 = oracle_mod.trace_from(nodes, depth, ids, tris, rays, starts=starts)
        near = tri_np.assert_matches_reference(h1["id"], h1["t"], g["hit_id"], g["hit_t"], rays, tris)
        if case != "flat_z":
            assert np.array_equal(h1, h0) and np.array_equal(l1, leaves) and near == 0


def test_restart_shading_rays_equal_root_walk(oracle_mod):
    from rtgpu import scenes
    tris = scenes.torus(96, 48)
    nodes, ids, _, _ = oracle_mod.lbvh_build(tris, 16)
    cam = scenes.torus_camera(160, 120)
    prim, leaves = oracle_mod.trace_from(nodes, 16, ids, tris, oracle_mod.primary_rays(cam))
    vis, mir, ss, ms = oracle_mod.shadow_mirror(nodes, 16, ids, tris, cam, scenes.TORUS_LIGHT, prim, stats=True)
    v2, m2, ml, ss2, ms2 = oracle_mod.shadow_mirror_from(nodes, 16, ids, tris, cam, scenes.TORUS_LIGHT, prim, leaves,
                                                         stats=True)
    assert np.array_equal(vis, v2) and np.array_equal(mir, m2)
    # fewer box tests: the walk does not descend again through the origin's ancestors
    assert ss2[:, 0].sum() < ss[:, 0].sum() and ms2[:, 0].sum() < ms[:, 0].sum()


@pytest.mark.parametrize("case", golden_cases())
def test_reference_walk_restatement_matches_reference(oracle_mod, case):
    """or_trace_hlsl restates the shader's own walk (LBVH.hlsl:363-440): on
    the golden fixtures its t equals the reference's LBVH::IntersectP t bit
    for bit, and its ids differ only where two triangles are hit at the same
    t (the shader keeps the first it tests)."""
    g = load_golden(case)
    tris, depth, rays = g["tris"], int(g["depth"]), g["rays"]
    nodes, ids, _, _ = oracle_mod.lbvh_build(tris, depth)
    h, leaves, st = oracle_mod.trace_hlsl(nodes, depth, ids, tris, rays)
    assert np.array_equal(h["t"], g["hit_t"])
    diff = np.nonzero(h["id"] != g["hit_id"])[0]
    for k in diff:
        assert tri_np.intersect_t(rays[k], tris[h["id"][k]]) == tri_np.intersect_t(rays[k], tris[g["hit_id"][k]])
    assert (st[:, 0] >= 1).all()
    # the closest hit of the shader's walk equals this project's walk up to the tie rule
    o = oracle_mod.trace(nodes, depth, ids, tris, rays)
    assert np.array_equal(o["t"], h["t"]) or case == "flat_z"
