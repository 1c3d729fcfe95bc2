"""Generates the SAH BVH fixtures in tests/golden/bvh/ from the reference's
OWN CPU code (AccelerationStructures/BVH/bvh.cpp: BVH::Build with the SAH
split and its flattened LinearBVHNode array, BVH::IntersectP), compiled from
the reference checkout by oracle/ref/build_ref.sh.

Run from the repository root where the reference checkout is present:
    python tests/golden/make_bvh.py
Each case stores its soup, the reference's nodes and ordered ids, a ray set
(primary rays of a camera plus rays through sampled triangle centroids) and
the reference's closest hits (id, t).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "raytracer-gpupro4_gb300"))
sys.path.insert(0, str(Path(__file__).resolve().parent))

import oracle as O  # noqa: E402
from rtgpu import scenes  # noqa: E402
from make_golden import centroid_rays  # noqa: E402

OUT = Path(__file__).resolve().parent / "bvh"


def cases():
    # name, soup, bvh_max_prims_node (conf.ini: 1), camera
    yield "torus_96x48", scenes.torus(96, 48, seed=1), 1, scenes.torus_camera(96, 64)
    yield "soup_5000", scenes.random_soup(5000, seed=31), 1, scenes.look_at((0.5, 0.5, -1.5), (0.5, 0.5, 0.5),
                                                                             width=64, height=64)
    soup = scenes.random_soup(2000, seed=32)
    dup = np.concatenate([soup, soup[:300]])
    yield "soup_duplicates", np.ascontiguousarray(dup), 1, scenes.look_at((0.5, 0.5, -1.5), (0.5, 0.5, 0.5),
                                                                          width=48, height=48)
    yield "soup_4_per_leaf", scenes.random_soup(3000, seed=33), 4, scenes.look_at((0.5, 0.5, -1.5),
                                                                                   (0.5, 0.5, 0.5), width=48,
                                                                                   height=48)
    yield "single", scenes.random_soup(1, seed=34), 1, scenes.look_at((0.5, 0.5, -1.5), (0.5, 0.5, 0.5), width=16,
                                                                       height=16)


def main():
    O.build_oracle()
    if O.build_reference() is None:
        raise SystemExit("reference checkout not found; set RT_REFERENCE_DIR")
    OUT.mkdir(exist_ok=True)
    for name, tris, max_prims, cam in cases():
        tris = np.ascontiguousarray(tris, np.float32)
        ref = O.RefStructure(tris, "bvh", 20, max_prims=max_prims)
        nodes, ids = ref.nodes(), ref.ids()
        rays = np.concatenate([O.primary_rays(cam), centroid_rays(tris)])
        hid, ht, _, _ = ref.intersect(rays, nthreads=1)
        cam_arr = np.array([*cam.eye, *cam.right, *cam.up, *cam.fwd, cam.tan_half_fovy, cam.width, cam.height],
                           np.float64)
        np.savez_compressed(OUT / f"{name}.npz", tris=tris, max_prims=np.int32(max_prims), nodes=nodes, ids=ids,
                            camera=cam_arr, rays=rays, hit_id=hid, hit_t=ht)
        ref.close()
        leaves = int((nodes["prim_count"] > 0).sum())
        print(f"{name}: n={len(tris)} nodes={len(nodes)} leaves={leaves} rays={len(rays)} hits={(hid >= 0).sum()}")


if __name__ == "__main__":
    main()
