"""The oracle against the reference's own CPU code run live (only where the
reference checkout was built into oracle/_ref; skipped elsewhere): larger
scenes than the committed golden fixtures."""
import numpy as np
import pytest

import tri_np


@pytest.fixture(scope="module")
def ref_mod(oracle_mod):
    oracle_mod.build_reference()
    if not oracle_mod.ref_available():
        pytest.skip("reference CPU code not built here")
    return oracle_mod


@pytest.mark.parametrize("scene", ["torus", "soup"])
def test_build_and_trace_vs_live_reference(ref_mod, scene):
    from rtgpu import scenes
    O = ref_mod
    if scene == "torus":
        tris, depth, cam = scenes.torus(), 20, scenes.torus_camera(256, 256)
    else:
        tris, depth, cam = scenes.random_soup(60000, seed=77), 18, scenes.look_at((0.5, 0.5, -1.2), (0.5, 0.5, 0.5), width=256, height=256)
    ref = O.RefStructure(tris, "lbvh", depth)
    rn = ref.nodes()
    nodes, ids, keys, reached = O.lbvh_build(tris, depth)
    m = O.reachable_mask(rn)
    assert np.array_equal(m, reached)
    assert np.array_equal(rn[m], nodes[m])
    rays = O.primary_rays(cam)
    hid, ht, _, _ = ref.intersect(rays)
    hits = O.trace(nodes, depth, ids, tris, rays)
    near = tri_np.assert_matches_reference(hits["id"], hits["t"], hid, ht, rays, tris)
    assert near == 0 and np.array_equal(hits["t"], ht)
    ref.close()
