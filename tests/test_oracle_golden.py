"""The CPU oracle against the golden fixtures produced by the reference's own
LBVH::Build / LBVH::IntersectP (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from conftest import camera_from_array, golden_cases, load_golden
import tri_np  # noqa: E402
from bitcmp import assert_nodes_match_reference, same_bits


@pytest.mark.parametrize("case", golden_cases())
def test_build_matches_reference(oracle_mod, case):
    g = load_golden(case)
    nodes, ids, keys, reached = oracle_mod.lbvh_build(g["tris"], int(g["depth"]))
    idx = g["node_index"]
    # reachable slots are the same set
    assert np.array_equal(np.nonzero(oracle_mod.reachable_mask(nodes))[0], idx)
    assert np.array_equal(np.nonzero(reached)[0], idx)
    a, b = nodes[idx], g["nodes"]
    assert np.array_equal(a["prim_count"], b["prim_count"])  # count, leaf bit, axis
    assert np.array_equal(a["prim_pos"], b["prim_pos"])
    # boxes bit for bit (a zero bound's sign may differ only where the
    # reference lists a leaf's triangles in its unstable partition order)
    assert_nodes_match_reference(nodes, ids, b, g["ids"], idx, case)
    if case != "signed_zero":
        assert same_bits(a, b)
    # ordered ids: the reference partitions in place (unstable), so ids agree
    # as a set inside every leaf and the oracle's order is cmpMorton order
    leaf = (b["prim_count"] & 4) != 0
    for pos, cnt in zip(b["prim_pos"][leaf], b["prim_count"][leaf] >> 3):
        assert set(ids[pos:pos + cnt].tolist()) == set(g["ids"][pos:pos + cnt].tolist())
    order = np.lexsort((np.arange(len(keys)), oracle_mod.morton(g["tris"])))
    assert np.array_equal(order.astype(np.uint32), ids)
    # WorldBound() = root box
    assert np.array_equal(nodes[1]["min"], g["world_bound"][:3]) and np.array_equal(nodes[1]["max"], g["world_bound"][3:])


@pytest.mark.parametrize("case", golden_cases())
def test_trace_matches_reference(oracle_mod, case):
    g = load_golden(case)
    depth = int(g["depth"])
    nodes, ids, _, _ = oracle_mod.lbvh_build(g["tris"], depth)
    cam = camera_from_array(g["camera"])
    rays = g["rays"]
    # the stored rays start with the camera's primary rays (restated ray generation)
    npx = cam.width * cam.height
    assert np.array_equal(oracle_mod.primary_rays(cam), rays[:npx])
    hits = oracle_mod.trace(nodes, depth, ids, g["tris"], rays, nthreads=2)
    ref_id, ref_t = g["hit_id"], g["hit_t"]
    # ids equal except on near-ties (equal t: the reference keeps the first
    # triangle it tests, the oracle the smallest id; ulp-apart t: order-dependent
    # pruning), t within 1e-6 relative
    near = tri_np.assert_matches_reference(hits["id"], hits["t"], ref_id, ref_t, rays, g["tris"])
    if case != "flat_z":  # coplanar overlapping triangles
        assert np.array_equal(hits["t"], ref_t)
        assert near == 0
