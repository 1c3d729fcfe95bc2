"""Traversal restart (the iRoot of LBVH_IntersectP, LBVH.hlsl:363-376) on
the GPU through the C ABI: the leaves a trace reports, shading rays started
at the primary leaves, and generic rays started at given nodes, all against
the oracle walking the same order: hits, leaves and per-ray test counts
bit-exact.  Visibility (any hit) does not depend on the walk order at all."""
import numpy as np
import pytest

from test_gpu_trace import assert_hits_equal, build_both

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sphere(gpu_ctx, oracle_mod):
    from rtgpu import scenes
    tris = np.ascontiguousarray(scenes.icosphere(60).frame(0), np.float32)
    lb, dt, nodes, ids = build_both(gpu_ctx, oracle_mod, tris, 18)
    return tris, lb, nodes, ids


def test_primary_leaves_and_shading_rays_from_leaves(gpu_ctx, oracle_mod, sphere):
    from rtgpu import scenes
    from rtgpu.api import RayTracer, hits_to_numpy
    tris, lb, nodes, ids = sphere
    cam = scenes.sphere_camera(320, 180)
    light = scenes.TORUS_LIGHT
    rt = RayTracer(gpu_ctx)
    hits, leaves, pst = rt.primary_leaves(lb, cam, stats=True)
    vis, mir, ml, ss, ms = rt.shadow_mirror_from(lb, cam, light, hits, leaves, stats=True)
    gpu_ctx.check()
    oh, ol, opst = oracle_mod.trace_from(nodes, 18, ids, tris, oracle_mod.primary_rays(cam), stats=True)
    assert_hits_equal(hits_to_numpy(hits), oh, "primary")
    assert np.array_equal(leaves.cpu().numpy().astype(np.uint32), ol)
    assert np.array_equal(pst.cpu().numpy().astype(np.uint32), opst)
    ovis, omir, oml, oss, oms = oracle_mod.shadow_mirror_from(nodes, 18, ids, tris, cam, light, oh, ol, stats=True)
    assert np.array_equal(vis.cpu().numpy(), ovis)
    assert set(np.unique(ovis)) >= {0, 2, 3}
    assert_hits_equal(hits_to_numpy(mir), omir, "mirror")
    assert np.array_equal(ml.cpu().numpy().astype(np.uint32), oml)
    assert np.array_equal(ss.cpu().numpy().astype(np.uint32), oss)
    assert np.array_equal(ms.cpu().numpy().astype(np.uint32), oms)
    # visibility equals the root walk's; the restart tests fewer boxes
    rvis, _, rss, rms = oracle_mod.shadow_mirror(nodes, 18, ids, tris, cam, light, oh, stats=True)
    assert np.array_equal(rvis, ovis)
    assert oss[:, 0].sum() < rss[:, 0].sum() and oms[:, 0].sum() < rms[:, 0].sum()


@pytest.mark.parametrize("block", [0, 2])
@pytest.mark.parametrize("budget", [0, 24, 384])
def test_production_shading_rays_from_leaves(gpu_ctx, oracle_mod, sphere, budget, block):
    """The compacted production pass (k_shade_setup + k_trace_shade) with
    and without the heavy-ray hand-over (its second pass a warp or, with
    block, a block per ray): vis and mirror hits equal the
    oracle's restart walk; leaves too, except for rays the warp-per-ray pass
    traced, which report the root."""
    from rtgpu import scenes
    from rtgpu.api import RayTracer, hits_to_numpy
    tris, lb, nodes, ids = sphere
    cam = scenes.look_at((0.4, 2.0, 2.2), (0.0, 0.0, 0.0), width=400, height=300)
    light = scenes.TORUS_LIGHT
    rt = RayTracer(gpu_ctx)
    gpu_ctx.set_trace_budget(budget)
    gpu_ctx.set_heavy_block(block)
    try:
        hits, leaves = rt.primary_leaves(lb, cam)
        vis, mir, ml = rt.shadow_mirror_from(lb, cam, light, hits, leaves)
        gpu_ctx.check()
    finally:
        gpu_ctx.set_trace_budget(None)
        gpu_ctx.set_heavy_block(None)
    oh, ol = oracle_mod.trace_from(nodes, 18, ids, tris, oracle_mod.primary_rays(cam))
    ovis, omir, oml = oracle_mod.shadow_mirror_from(nodes, 18, ids, tris, cam, light, oh, ol)
    assert_hits_equal(hits_to_numpy(hits), oh, "primary")
    assert np.array_equal(vis.cpu().numpy(), ovis)
    assert_hits_equal(hits_to_numpy(mir), omir, "mirror")
    gl, gml = leaves.cpu().numpy().astype(np.uint32), ml.cpu().numpy().astype(np.uint32)
    if budget == 0:
        assert np.array_equal(gl, ol) and np.array_equal(gml, oml)
    else:
        assert np.all((gl == ol) | (gl == 1)) and np.all((gml == oml) | (gml == 1))


@pytest.mark.parametrize("any_hit", [False, True])
def test_generic_rays_from_start_nodes(gpu_ctx, oracle_mod, any_hit):
    """Rays leaving triangles of a soup, started at the leaf of the triangle
    they leave and at random reached nodes: hits, leaves and counts equal the
    oracle's; an out-of-range start is reported as a device error."""
    import torch
    from oracle import reachable_mask
    from rtgpu import scenes
    from rtgpu.api import RayTracer, hits_to_numpy, rays_tensor
    tris = scenes.random_soup(40000, seed=61)
    lb, dt, nodes, ids = build_both(gpu_ctx, oracle_mod, tris, 17)
    rng = np.random.default_rng(62)
    n = 30000
    src = rng.integers(0, len(tris), n)
    o = tris[src].reshape(n, 3, 3).mean(axis=1).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    excl = src.astype(np.int32)
    tmax = np.where(np.arange(n) % 3 == 0, 0.05, 1e16).astype(np.float32)
    # the leaf holding each source triangle
    leaf_of = np.zeros(len(tris), np.uint32)
    for h in np.nonzero(reachable_mask(nodes) & ((nodes["prim_count"] & 4) != 0))[0]:
        pos, cnt = nodes["prim_pos"][h], nodes["prim_count"][h] >> 3
        leaf_of[ids[pos:pos + cnt]] = h
    reached = np.nonzero(reachable_mask(nodes))[0].astype(np.uint32)
    rt = RayTracer(gpu_ctx)
    orays = oracle_mod.rays_array(o, d, tmax, excl)
    for starts in (leaf_of[src], rng.choice(reached, size=n)):
        dr = rays_tensor(o, d, tmax, excl, "cuda")
        ds = torch.from_numpy(starts.astype(np.int32)).cuda()
        hits, leaves, st = rt.rays_from(lb, dr, ds, any_hit=any_hit, stats=True)
        gpu_ctx.check()
        oh, ol, ost = oracle_mod.trace_from(nodes, 17, ids, tris, orays, starts=starts, any_hit=any_hit, stats=True)
        g = hits_to_numpy(hits)
        if any_hit:
            assert np.array_equal(g["id"], oh["id"])
        else:
            assert_hits_equal(g, oh, "rays")
        assert np.array_equal(leaves.cpu().numpy().astype(np.uint32), ol)
        assert np.array_equal(st.cpu().numpy().astype(np.uint32), ost)
    # a start outside the heap: flagged, and the ray walks from the root
    bad = torch.full((n,), 1 << 30, dtype=torch.int32, device="cuda")
    rt.rays_from(lb, rays_tensor(o, d, tmax, excl, "cuda"), bad)
    with pytest.raises(Exception):
        gpu_ctx.check()
