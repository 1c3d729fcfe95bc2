"""GPU traversal parity against the oracle's restatement of LBVH_IntersectP
(LBVH.hlsl:363-440) and the shading rays of CSComputeColorRT.hlsl:
closest-hit ids bit-exact, t / u / v bit-exact (tolerance stated by the
contract: 1e-6 relative), per-ray box/triangle test counts equal."""
import numpy as np
import pytest

from conftest import camera_from_array, golden_cases, load_golden
import tri_np
from bitcmp import same_bits

pytestmark = pytest.mark.gpu


def build_both(ctx, oracle_mod, tris, depth):
    import torch
    from rtgpu.api import LBVH
    lb = LBVH(ctx, len(tris), depth)
    dt = torch.from_numpy(np.ascontiguousarray(tris)).cuda()
    lb.Build(dt)
    nodes, ids, keys, _ = oracle_mod.lbvh_build(tris, depth)
    return lb, dt, nodes, ids


def assert_hits_equal(gpu, ref, what):
    assert np.array_equal(gpu["id"], ref["id"]), f"{what}: {np.sum(gpu['id'] != ref['id'])} id mismatches"
    hit = ref["id"] >= 0
    t_rel = np.abs(gpu["t"][hit] - ref["t"][hit]) / np.maximum(np.abs(ref["t"][hit]), 1e-30)
    assert t_rel.max(initial=0.0) <= 1e-6, what
    # the kernels evaluate the reference's operation order without contraction: equal bits
    assert same_bits(gpu["t"], ref["t"]) and same_bits(gpu["u"], ref["u"]) and same_bits(gpu["v"], ref["v"]), what


@pytest.fixture(scope="module")
def torus_scene(gpu_ctx, oracle_mod):
    from rtgpu import scenes
    tris = scenes.torus()
    lb, dt, nodes, ids = build_both(gpu_ctx, oracle_mod, tris, 20)
    return tris, lb, dt, nodes, ids


def test_primary_torus_512(gpu_ctx, oracle_mod, torus_scene):
    from rtgpu import scenes
    from rtgpu.api import RayTracer, hits_to_numpy
    tris, lb, dt, nodes, ids = torus_scene
    cam = scenes.torus_camera()
    hits, st = RayTracer(gpu_ctx).primary(lb, cam, stats=True)
    gpu_ctx.check()
    oh, ost = oracle_mod.trace(nodes, 20, ids, tris, oracle_mod.primary_rays(cam), stats=True)
    assert_hits_equal(hits_to_numpy(hits), oh, "primary")
    assert np.array_equal(st.cpu().numpy().astype(np.uint32), ost)
    assert (oh["id"] >= 0).mean() > 0.2


def test_shadow_mirror_torus_512(gpu_ctx, oracle_mod, torus_scene):
    from rtgpu import scenes
    from rtgpu.api import RayTracer, hits_to_numpy
    tris, lb, dt, nodes, ids = torus_scene
    cam = scenes.torus_camera()
    rt = RayTracer(gpu_ctx)
    hits = rt.primary(lb, cam)
    vis, mirror, ss, ms = rt.shadow_mirror(lb, cam, scenes.TORUS_LIGHT, hits, stats=True)
    gpu_ctx.check()
    oh = oracle_mod.trace(nodes, 20, ids, tris, oracle_mod.primary_rays(cam))
    ovis, omir, oss, oms = oracle_mod.shadow_mirror(nodes, 20, ids, tris, cam, scenes.TORUS_LIGHT, oh, stats=True)
    assert np.array_equal(vis.cpu().numpy(), ovis)
    assert set(np.unique(ovis)) >= {0, 2, 3}
    assert_hits_equal(hits_to_numpy(mirror), omir, "mirror")
    assert np.array_equal(ss.cpu().numpy().astype(np.uint32), oss)
    assert np.array_equal(ms.cpu().numpy().astype(np.uint32), oms)


@pytest.mark.parametrize("any_hit", [False, True])
def test_generic_rays_with_exclusion(gpu_ctx, oracle_mod, any_hit):
    """Random rays inside a triangle soup, half leaving from a triangle they
    must exclude, some with axis-aligned directions (infinite 1/d: the
    reference's NaN-sensitive std::min/std::max path)."""
    import torch
    from rtgpu import scenes
    from rtgpu.api import RayTracer, hits_to_numpy, rays_tensor
    tris = scenes.random_soup(50000, seed=51)
    lb, dt, nodes, ids = build_both(gpu_ctx, oracle_mod, tris, 18)
    rng = np.random.default_rng(52)
    n = 40000
    src = rng.integers(0, len(tris), n)
    o = tris[src].reshape(n, 3, 3).mean(axis=1).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d[: n // 8, rng.integers(0, 3)] = 0.0           # exact zero components
    d[n // 8: n // 4, :2] = 0.0
    d[n // 8: n // 4, 2] = 1.0
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    excl = np.where(np.arange(n) % 2 == 0, src, -1).astype(np.int32)
    tmax = np.where(np.arange(n) % 3 == 0, 0.05, 1e16).astype(np.float32)
    hits, st = RayTracer(gpu_ctx).rays(lb, rays_tensor(o, d, tmax, excl, "cuda"), any_hit=any_hit, stats=True)
    gpu_ctx.check()
    orays = oracle_mod.rays_array(o, d, tmax, excl)
    oh, ost = oracle_mod.trace(nodes, 18, ids, tris, orays, any_hit=any_hit, stats=True)
    g = hits_to_numpy(hits)
    if any_hit:
        assert np.array_equal(g["id"] >= 0, oh["id"] >= 0)
        assert np.array_equal(g["id"], oh["id"])
    else:
        assert_hits_equal(g, oh, "rays")
    assert np.array_equal(st.cpu().numpy().astype(np.uint32), ost)


@pytest.mark.parametrize("case", golden_cases())
def test_trace_on_reference_tree(gpu_ctx, case):
    """The reference's own CPU-built tree (golden fixture) imported through
    rt_lbvh_import_host and traced on the GPU: hits equal the reference's
    LBVH::IntersectP up to its tie order (t bit-exact)."""
    import torch
    from rtgpu._lib import NODE_DTYPE, RT_NODE_SENTINEL
    from rtgpu.api import LBVH, RayTracer, hits_to_numpy, rays_tensor
    g = load_golden(case)
    depth = int(g["depth"])
    nodes = np.zeros(1 << depth, NODE_DTYPE)
    nodes["prim_count"] = RT_NODE_SENTINEL
    nodes["prim_pos"] = RT_NODE_SENTINEL
    nodes[g["node_index"]] = g["nodes"].astype(NODE_DTYPE)
    lb = LBVH(gpu_ctx, len(g["tris"]), depth).Import(nodes, g["ids"], g["tris"])
    r = g["rays"]
    hits = hits_to_numpy(RayTracer(gpu_ctx).rays(lb, rays_tensor(r[:, 0:3], r[:, 3:6], r[:, 6], r[:, 7].astype(np.int32), "cuda")))
    gpu_ctx.check()
    tri_np.assert_matches_reference(hits["id"], hits["t"], g["hit_id"], g["hit_t"], r, g["tris"])


def test_render_frame_host_equals_device_path(gpu_ctx, torus_scene):
    from rtgpu import scenes
    from rtgpu._lib import HIT_DTYPE
    from rtgpu.api import LBVH, RayTracer, hits_to_numpy
    tris, lb, dt, nodes, ids = torus_scene
    cam = scenes.torus_camera(320, 200)
    rt = RayTracer(gpu_ctx)
    # the frame call starts the shading rays at the primary leaves
    hits, leaves = rt.primary_leaves(lb, cam)
    vis, mirror, _ = rt.shadow_mirror_from(lb, cam, scenes.TORUS_LIGHT, hits, leaves)
    lb2 = LBVH(gpu_ctx, len(tris), 20)
    hp = np.zeros(cam.width * cam.height, HIT_DTYPE)
    hv = np.zeros(cam.width * cam.height, np.uint8)
    hm = np.zeros(cam.width * cam.height, HIT_DTYPE)
    rt.render_frame_host(lb2, tris, cam, scenes.TORUS_LIGHT, hp, hv, hm)
    assert np.array_equal(hp, hits_to_numpy(hits))
    assert np.array_equal(hv, vis.cpu().numpy())
    assert np.array_equal(hm, hits_to_numpy(mirror))


def test_shared_traversal_matches_oracle(gpu_ctx, oracle_mod, torus_scene):
    """The production traversal (no counters: serial and pooled leaf parts,
    rays over the work budget handed to the warp-per-ray pass) gives the
    oracle's hits bit for bit."""
    from rtgpu import scenes
    from rtgpu.api import RayTracer, hits_to_numpy
    tris, lb, dt, nodes, ids = torus_scene
    rt = RayTracer(gpu_ctx)
    for cam in (scenes.torus_camera(), scenes.look_at((2.2, 0.3, 0.4), (0.0, 0.0, 0.0), width=640, height=360)):
        hits = rt.primary(lb, cam)
        vis, mirror = rt.shadow_mirror(lb, cam, scenes.TORUS_LIGHT, hits)
        gpu_ctx.check()
        oh = oracle_mod.trace(nodes, 20, ids, tris, oracle_mod.primary_rays(cam))
        ovis, omir = oracle_mod.shadow_mirror(nodes, 20, ids, tris, cam, scenes.TORUS_LIGHT, oh)
        assert_hits_equal(hits_to_numpy(hits), oh, "primary")
        assert np.array_equal(vis.cpu().numpy(), ovis)
        assert_hits_equal(hits_to_numpy(mirror), omir, "mirror")


@pytest.mark.parametrize("any_hit", [False, True])
def test_shared_traversal_generic_rays(gpu_ctx, oracle_mod, any_hit):
    """Random rays in a soup (exclusions, axis-aligned directions, short and
    non-positive tmax) through the production traversal: closest hits equal
    the oracle's; any-hit rays report occlusion exactly as the oracle does
    (which occluder is reported depends on the walk order)."""
    from rtgpu import scenes
    from rtgpu.api import RayTracer, hits_to_numpy, rays_tensor
    tris = scenes.random_soup(50000, seed=61)
    lb, dt, nodes, ids = build_both(gpu_ctx, oracle_mod, tris, 18)
    rng = np.random.default_rng(62)
    n = 40000
    src = rng.integers(0, len(tris), n)
    o = tris[src].reshape(n, 3, 3).mean(axis=1).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d[: n // 8, rng.integers(0, 3)] = 0.0
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    excl = np.where(np.arange(n) % 2 == 0, src, -1).astype(np.int32)
    tmax = np.where(np.arange(n) % 3 == 0, 0.05, 1e16).astype(np.float32)
    tmax[::97] = 0.0
    tmax[1::97] = -1.0
    hits = RayTracer(gpu_ctx).rays(lb, rays_tensor(o, d, tmax, excl, "cuda"), any_hit=any_hit)
    gpu_ctx.check()
    oh = oracle_mod.trace(nodes, 18, ids, tris, oracle_mod.rays_array(o, d, tmax, excl), any_hit=any_hit)
    g = hits_to_numpy(hits)
    assert not (g["id"][::97] >= 0).any() and not (g["id"][1::97] >= 0).any()
    if any_hit:
        assert np.array_equal(g["id"] >= 0, oh["id"] >= 0)
    else:
        assert_hits_equal(g, oh, "rays")


@pytest.mark.parametrize("block", [0, 7])
@pytest.mark.parametrize("budget", [1, 24, 0])
def test_heavy_ray_handover_matches_oracle(gpu_ctx, oracle_mod, torus_scene, budget, block):
    """Rays over the work budget are re-traced by the second pass (a warp per
    ray, or with `block` a block of 128 threads per ray); with a budget of 1
    nearly every ray is, with 0 none is: hits, visibility and mirror hits
    equal the oracle's either way."""
    from rtgpu import scenes
    from rtgpu.api import RayTracer, hits_to_numpy
    tris, lb, dt, nodes, ids = torus_scene
    rt = RayTracer(gpu_ctx)
    cam = scenes.look_at((2.2, 0.3, 0.4), (0.0, 0.0, 0.0), width=320, height=200)
    gpu_ctx.set_trace_budget(budget)
    gpu_ctx.set_heavy_block(block)
    try:
        hits = rt.primary(lb, cam)
        vis, mirror = rt.shadow_mirror(lb, cam, scenes.TORUS_LIGHT, hits)
        gpu_ctx.check()
    finally:
        gpu_ctx.set_trace_budget(None)
        gpu_ctx.set_heavy_block(None)
    oh = oracle_mod.trace(nodes, 20, ids, tris, oracle_mod.primary_rays(cam))
    ovis, omir = oracle_mod.shadow_mirror(nodes, 20, ids, tris, cam, scenes.TORUS_LIGHT, oh)
    assert_hits_equal(hits_to_numpy(hits), oh, "primary")
    assert np.array_equal(vis.cpu().numpy(), ovis)
    assert_hits_equal(hits_to_numpy(mirror), omir, "mirror")


@pytest.mark.parametrize("block", [0, 4])
@pytest.mark.parametrize("any_hit", [False, True])
def test_heavy_ray_handover_generic_rays(gpu_ctx, oracle_mod, any_hit, block):
    from rtgpu import scenes
    from rtgpu.api import RayTracer, hits_to_numpy, rays_tensor
    tris = scenes.random_soup(30000, seed=71)
    lb, dt, nodes, ids = build_both(gpu_ctx, oracle_mod, tris, 16)
    rng = np.random.default_rng(72)
    n = 20000
    src = rng.integers(0, len(tris), n)
    o = tris[src].reshape(n, 3, 3).mean(axis=1).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d[: n // 8, rng.integers(0, 3)] = 0.0
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    excl = np.where(np.arange(n) % 2 == 0, src, -1).astype(np.int32)
    tmax = np.where(np.arange(n) % 3 == 0, 0.05, 1e16).astype(np.float32)
    gpu_ctx.set_trace_budget(2)
    gpu_ctx.set_heavy_block(block)
    try:
        hits = RayTracer(gpu_ctx).rays(lb, rays_tensor(o, d, tmax, excl, "cuda"), any_hit=any_hit)
        gpu_ctx.check()
    finally:
        gpu_ctx.set_trace_budget(None)
        gpu_ctx.set_heavy_block(None)
    oh = oracle_mod.trace(nodes, 16, ids, tris, oracle_mod.rays_array(o, d, tmax, excl), any_hit=any_hit)
    g = hits_to_numpy(hits)
    if any_hit:
        assert np.array_equal(g["id"] >= 0, oh["id"] >= 0)
    else:
        assert_hits_equal(g, oh, "rays")


def test_render_frame_host_async_two_streams(gpu_ctx, torus_scene):
    """rt_render_frame_host_async on two contexts / streams, alternate frames,
    gives the synchronous call's results."""
    import torch
    from rtgpu import scenes
    from rtgpu._lib import HIT_DTYPE
    from rtgpu.api import LBVH, Context, RayTracer
    tris, lb, dt, nodes, ids = torus_scene
    cam = scenes.torus_camera(256, 160)
    npx = cam.width * cam.height
    rt = RayTracer(gpu_ctx)
    lbs = LBVH(gpu_ctx, len(tris), 20)
    ref = [np.zeros(npx, HIT_DTYPE), np.zeros(npx, np.uint8), np.zeros(npx, HIT_DTYPE)]
    rt.render_frame_host(lbs, tris, cam, scenes.TORUS_LIGHT, *ref)
    lanes = []
    for _ in range(2):
        ctx = Context(0, stream=torch.cuda.Stream())
        outs = [torch.empty(npx * 4, dtype=torch.int32).pin_memory(), torch.empty(npx, dtype=torch.uint8).pin_memory(),
                torch.empty(npx * 4, dtype=torch.int32).pin_memory()]
        lanes.append((ctx, LBVH(ctx, len(tris), 20), RayTracer(ctx), outs))
    soup = torch.from_numpy(tris).pin_memory().numpy()
    for k in range(4):
        ctx, lbq, rtq, outs = lanes[k % 2]
        ctx.sync()
        rtq.render_frame_host(lbq, soup, cam, scenes.TORUS_LIGHT, outs[0].numpy().view(HIT_DTYPE), outs[1].numpy(),
                              outs[2].numpy().view(HIT_DTYPE), wait=False)
    for ctx, lbq, rtq, outs in lanes:
        ctx.check()
        assert np.array_equal(outs[0].numpy().view(HIT_DTYPE), ref[0])
        assert np.array_equal(outs[1].numpy(), ref[1])
        assert np.array_equal(outs[2].numpy().view(HIT_DTYPE), ref[2])


def test_heavy_first_tile_order_keeps_results(gpu_ctx, oracle_mod, torus_scene):
    """With the heavy-first order on for every kind, calls that follow calls
    on other images (a foreign tile list) and on the same image (its own list)
    still give the oracle's results."""
    from rtgpu import scenes
    from rtgpu.api import RayTracer, hits_to_numpy
    tris, lb, dt, nodes, ids = torus_scene
    rt = RayTracer(gpu_ctx)
    gpu_ctx.set_tile_order(7)
    try:
        big = scenes.torus_camera(512, 512)
        rt.shadow_mirror(lb, big, scenes.TORUS_LIGHT, rt.primary(lb, big))
        cam = scenes.look_at((2.2, 0.3, 0.4), (0.0, 0.0, 0.0), width=320, height=200)
        for _ in range(3):
            hits = rt.primary(lb, cam)
            vis, mirror = rt.shadow_mirror(lb, cam, scenes.TORUS_LIGHT, hits)
        gpu_ctx.check()
    finally:
        gpu_ctx.set_tile_order(1)
    oh = oracle_mod.trace(nodes, 20, ids, tris, oracle_mod.primary_rays(cam))
    ovis, omir = oracle_mod.shadow_mirror(nodes, 20, ids, tris, cam, scenes.TORUS_LIGHT, oh)
    assert_hits_equal(hits_to_numpy(hits), oh, "primary")
    assert np.array_equal(vis.cpu().numpy(), ovis)
    assert_hits_equal(hits_to_numpy(mirror), omir, "mirror")


def test_compact_layout_traversal(gpu_ctx, oracle_mod):
    """RT_BUILD_COMPACT: the heap export is unchanged, the compact layout is
    reported, and the traversal over it gives the oracle's hits."""
    import ctypes as C
    import torch
    from rtgpu import _lib as L
    from rtgpu import scenes
    from rtgpu.api import LBVH, RayTracer, hits_to_numpy
    tris = scenes.torus(128, 64)
    lb = LBVH(gpu_ctx, len(tris), 18).Build(torch.from_numpy(tris).cuda(), L.RT_BUILD_COMPACT)
    ptr, slots = C.c_void_p(), C.c_uint32()
    assert L.lib().rt_lbvh_compact_get(lb.h, C.byref(ptr), C.byref(slots)) == L.RT_OK
    assert ptr.value and slots.value >= 2
    nodes, ids, keys = lb.download(True, True, True)
    onodes, oids, okeys, reached = oracle_mod.lbvh_build(tris, 18)
    r = np.nonzero(reached)[0]
    assert np.array_equal(nodes[r], onodes[r]) and np.array_equal(ids, oids)
    cam = scenes.look_at((2.2, 0.3, 0.4), (0.0, 0.0, 0.0), width=320, height=200)
    rt = RayTracer(gpu_ctx)
    hits = rt.primary(lb, cam)
    vis, mirror = rt.shadow_mirror(lb, cam, scenes.TORUS_LIGHT, hits)
    gpu_ctx.check()
    oh = oracle_mod.trace(onodes, 18, oids, tris, oracle_mod.primary_rays(cam))
    ovis, omir = oracle_mod.shadow_mirror(onodes, 18, oids, tris, cam, scenes.TORUS_LIGHT, oh)
    assert_hits_equal(hits_to_numpy(hits), oh, "primary")
    assert np.array_equal(vis.cpu().numpy(), ovis)
    assert_hits_equal(hits_to_numpy(mirror), omir, "mirror")
    # a build without the flag reports no compact layout
    lb.Build(torch.from_numpy(tris).cuda())
    assert L.lib().rt_lbvh_compact_get(lb.h, C.byref(ptr), C.byref(slots)) == L.RT_ERR_INVALID
