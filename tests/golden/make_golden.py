"""Generates the golden fixtures in this folder from the reference's OWN CPU
code (AccelerationStructures/LBVH/LBVH.cpp: LBVH::Build, LBVH::IntersectP),
compiled from the reference checkout by oracle/ref/build_ref.sh.

Run from the repository root where the reference checkout is present:
    python tests/golden/make_golden.py [case ...]
Each case stores its input soup, the reference's reachable nodes (index +
record; unreached heap slots are uninitialised in the reference), its
ordered ids, world bound, and its closest hits (id, t) for a ray set.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "raytracer-gpupro4_gb300"))

import oracle as O  # noqa: E402
from rtgpu import scenes  # noqa: E402

OUT = Path(__file__).resolve().parent


def cases():
    yield "torus_64x32", scenes.torus(64, 32, seed=1), 14, scenes.torus_camera(96, 64)
    soup = scenes.random_soup(3000, seed=11)
    dup = np.concatenate([soup, soup[:400], soup[100:300] + np.float32(1e-6)])
    yield "soup_duplicates", np.ascontiguousarray(dup), 16, scenes.look_at((0.5, 0.5, -1.5), (0.5, 0.5, 0.5), width=64, height=64)
    yield "soup_capped_depth8", scenes.random_soup(5000, seed=12), 8, scenes.look_at((0.5, 0.5, -1.5), (0.5, 0.5, 0.5), width=64, height=64)
    flat = scenes.random_soup(1000, seed=13)
    flat[:, 2::3] = np.float32(0.5)
    yield "flat_z", flat, 12, scenes.look_at((0.5, 0.5, -1.5), (0.5, 0.5, 0.5), width=48, height=48)
    yield "single", scenes.random_soup(1, seed=14), 10, scenes.look_at((0.5, 0.5, -1.5), (0.5, 0.5, 0.5), width=16, height=16)
    three = scenes.random_soup(1, seed=15)
    yield "three_equal", np.ascontiguousarray(np.repeat(three, 3, axis=0)), 10, scenes.look_at((0.5, 0.5, -1.5), (0.5, 0.5, 0.5), width=16, height=16)
    yield "depth1_root_leaf", scenes.random_soup(64, seed=16), 1, scenes.look_at((0.5, 0.5, -1.5), (0.5, 0.5, 0.5), width=16, height=16)
    yield "signed_zero", signed_zero_soup(2000, seed=17), 12, scenes.look_at((0.3, 0.4, -2.5), (0.0, 0.0, 0.0), width=48, height=48)


def signed_zero_soup(n, seed):
    """Triangles on either side of the coordinate planes with many vertex
    coordinates exactly +0.0 or -0.0: box bounds of 0 are ties between the
    two zeros, whose sign only the order of the reference's min / max
    (std::min / std::max keep their first argument on a tie) decides."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = np.abs(scenes.random_soup(n, seed)).reshape(n, 3, 3)
    side = rng.choice(np.array([-1.0, 1.0], np.float32), size=(n, 1, 3))
    t = t * side
    zero = rng.random((n, 3, 3)) < 0.3
    sign = rng.choice(np.array([-0.0, 0.0], np.float32), size=(n, 3, 3))
    t = np.where(zero, sign, t).astype(np.float32)
    return np.ascontiguousarray(t.reshape(n, 9))


def centroid_rays(tris, count=256, seed=5):
    """Rays from a fixed origin through the centroids of sampled triangles."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pick = rng.choice(len(tris), size=min(count, len(tris)), replace=False)
    c = tris[pick].reshape(-1, 3, 3).astype(np.float64).mean(axis=1)
    o = np.array([0.41, 0.47, -1.3])
    d = c - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return O.rays_array(o.astype(np.float32), d.astype(np.float32), 1e16, -1)


def main():
    O.build_oracle()
    if O.build_reference() is None:
        raise SystemExit("reference checkout not found; set RT_REFERENCE_DIR")
    only = set(sys.argv[1:])  # optional case names: regenerate only those
    for name, tris, depth, cam in cases():
        if only and name not in only:
            continue
        tris = np.ascontiguousarray(tris, np.float32)
        ref = O.RefStructure(tris, "lbvh", depth)
        nodes = ref.nodes()
        reach = O.reachable_mask(nodes)
        idx = np.nonzero(reach)[0].astype(np.int32)
        rays = np.concatenate([O.primary_rays(cam), centroid_rays(tris)])
        hid, ht, hu, hv = ref.intersect(rays, nthreads=1)
        cam_arr = np.array([*cam.eye, *cam.right, *cam.up, *cam.fwd, cam.tan_half_fovy, cam.width, cam.height],
                           np.float64)
        np.savez_compressed(OUT / f"{name}.npz", tris=tris, depth=np.int32(depth), node_index=idx,
                            nodes=nodes[idx], ids=ref.ids(), world_bound=ref.world_bound(), camera=cam_arr, rays=rays,
                            hit_id=hid, hit_t=ht)
        ref.close()
        print(f"{name}: n={len(tris)} depth={depth} reachable={len(idx)} rays={len(rays)} hits={(hid >= 0).sum()}")


if __name__ == "__main__":
    main()
