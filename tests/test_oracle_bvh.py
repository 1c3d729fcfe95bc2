"""The oracle's BVH_IntersectP restatement (or_bvh_trace) against the
reference's own BVH::IntersectP over the reference's SAH trees: the golden
fixtures in tests/golden/bvh/ (made by tests/golden/make_bvh.py), and live
where oracle/_ref was built.  The shader's IntersectBox and the CPU's PBRT
slab test round differently, so ids may differ only on near-ties; t is
bit-exact.  CPU only."""
from pathlib import Path

import numpy as np
import pytest

import tri_np

BVH_DIR = Path(__file__).resolve().parent / "golden" / "bvh"


def bvh_cases():
    return sorted(p.stem for p in BVH_DIR.glob("*.npz"))


def load_bvh(name):
    return dict(np.load(BVH_DIR / f"{name}.npz"))


@pytest.mark.parametrize("case", bvh_cases())
def test_oracle_bvh_matches_reference_fixture(oracle_mod, case):
    g = load_bvh(case)
    hits = oracle_mod.bvh_trace(g["nodes"], g["ids"], g["tris"], g["rays"], nthreads=2)
    near = tri_np.assert_matches_reference(hits["id"], hits["t"], g["hit_id"], g["hit_t"], g["rays"], g["tris"])
    assert near == 0 and np.array_equal(hits["t"], g["hit_t"])


def test_oracle_bvh_any_hit_agrees_with_closest(oracle_mod):
    g = load_bvh("torus_96x48")
    closest = oracle_mod.bvh_trace(g["nodes"], g["ids"], g["tris"], g["rays"])
    anyh = oracle_mod.bvh_trace(g["nodes"], g["ids"], g["tris"], g["rays"], any_hit=True)
    assert np.array_equal(closest["id"] >= 0, anyh["id"] >= 0)


def test_oracle_bvh_vs_live_reference(oracle_mod):
    from rtgpu import scenes
    oracle_mod.build_reference()
    if not oracle_mod.ref_available():
        pytest.skip("reference CPU code not built here")
    tris = scenes.torus(256, 128)
    ref = oracle_mod.RefStructure(tris, "bvh", 20, max_prims=1)
    cam = scenes.torus_camera(192, 192)
    rays = oracle_mod.primary_rays(cam)
    hid, ht, _, _ = ref.intersect(rays)
    hits = oracle_mod.bvh_trace(ref.nodes(), ref.ids(), tris, rays)
    near = tri_np.assert_matches_reference(hits["id"], hits["t"], hid, ht, rays, tris)
    assert near == 0 and np.array_equal(hits["t"], ht)
    ref.close()
