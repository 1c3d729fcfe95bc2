"""Batched build + trace (rt_batch_*) parity: every scene of a batch gets
the tree the oracle builds for that scene alone (codes, permutation and all
reachable nodes bit-exact, ids scene-local), and the batched primary and
shadow rays equal the oracle's per scene."""
import numpy as np
import pytest

from test_gpu_trace import assert_hits_equal
from bitcmp import same_bits

pytestmark = pytest.mark.gpu


def make_batch(gpu_ctx, sizes, depth, seed_base):
    import torch
    from rtgpu import scenes
    from rtgpu.api import Batch
    soups = [scenes.random_soup(int(n), seed_base + i) for i, n in enumerate(sizes)]
    b = Batch(gpu_ctx, [len(s) for s in soups], depth)
    dt = torch.from_numpy(np.ascontiguousarray(np.concatenate(soups))).cuda()
    b.build(dt)
    return b, dt, soups


def check_trees(gpu_ctx, oracle_mod, b, soups, depth, scenes_to_check=None):
    gpu_ctx.check()
    for s in (scenes_to_check if scenes_to_check is not None else range(len(soups))):
        nodes, ids, keys = b.download(s)
        onodes, oids, okeys, reached = oracle_mod.lbvh_build(soups[s], depth)
        assert np.array_equal(keys, okeys), f"scene {s}: codes"
        assert np.array_equal(ids, oids), f"scene {s}: permutation"
        r = np.nonzero(reached)[0]
        assert same_bits(nodes[r], onodes[r]), f"scene {s}: nodes"


def test_batch_build_mixed_sizes(gpu_ctx, oracle_mod):
    sizes = [1, 2, 3, 4096, 4097, 700, 1, 12000, 33, 5000]
    b, dt, soups = make_batch(gpu_ctx, sizes, 14, 300)
    check_trees(gpu_ctx, oracle_mod, b, soups, 14)
    # a rebuild of the same batch (epoch-tagged refit words) gives the same trees
    b.build(dt)
    check_trees(gpu_ctx, oracle_mod, b, soups, 14, [0, 3, 7])


def test_batch_build_256_scenes_with_duplicates(gpu_ctx, oracle_mod):
    import torch
    from rtgpu import scenes
    from rtgpu.api import Batch
    rng = np.random.default_rng(9)
    soups = []
    for s in range(256):
        t = scenes.random_soup(int(rng.integers(1, 400)), 2000 + s)
        if s % 5 == 0:  # equal codes: repeated triangles
            t = np.ascontiguousarray(np.concatenate([t, t[: max(1, len(t) // 3)]]))
        soups.append(t)
    b = Batch(gpu_ctx, [len(t) for t in soups], 10)
    b.build(torch.from_numpy(np.ascontiguousarray(np.concatenate(soups))).cuda())
    check_trees(gpu_ctx, oracle_mod, b, soups, 10)


def test_batch_equals_single_scene_builds(gpu_ctx):
    """Scene s of a batch and rt_lbvh_build of scene s alone: identical heaps
    (sentinels included when both clear unreached slots)."""
    import torch
    from rtgpu import _lib as L
    from rtgpu.api import LBVH
    sizes = [900, 20000, 3]
    b, dt, soups = make_batch(gpu_ctx, sizes, 16, 400)
    b.build(dt, L.RT_BUILD_CLEAR_UNREACHED)
    for s, soup in enumerate(soups):
        lb = LBVH(gpu_ctx, len(soup), 16).Build(torch.from_numpy(soup).cuda(), L.RT_BUILD_CLEAR_UNREACHED)
        n1, i1, k1 = lb.download(True, True, True)
        n2, i2, k2 = b.download(s)
        assert np.array_equal(n1.view(np.uint8), n2.view(np.uint8)) and np.array_equal(i1, i2) and np.array_equal(k1, k2)


def test_batch_trace_primary_shadow(gpu_ctx, oracle_mod):
    from rtgpu import scenes
    from rtgpu.api import hits_to_numpy
    sizes = [5000, 1, 800, 30000, 64]
    depth = 16
    b, dt, soups = make_batch(gpu_ctx, sizes, depth, 600)
    cams, lights = scenes.batch_views(len(sizes), 96, 64)
    b.set_views(cams, lights)
    for order in (0, 1):
        for grab in (1, 3):
            b.tuning = {"threads": 128 if order else 64, "grab": grab, "order": order}
            hits, vis = b.alloc_outputs()
            b.trace(hits, vis)
            gpu_ctx.check()
            H = hits_to_numpy(hits).reshape(len(sizes), -1)
            V = vis.cpu().numpy().reshape(len(sizes), -1)
            for s, soup in enumerate(soups):
                nodes, ids, _, _ = oracle_mod.lbvh_build(soup, depth)
                oh = oracle_mod.trace(nodes, depth, ids, soup, oracle_mod.primary_rays(cams[s]))
                assert_hits_equal(H[s], oh, f"scene {s} primary")
                ovis, _ = oracle_mod.shadow_mirror(nodes, depth, ids, soup, cams[s], lights[s], oh)[:2]
                assert np.array_equal(V[s], ovis), f"scene {s} shadow"
    assert (H[3]["id"] >= 0).mean() > 0.1


def test_batch_graph_and_primary_only(gpu_ctx):
    import torch
    from rtgpu import scenes
    from rtgpu.api import BatchFrame
    sizes = [3000, 200, 9000]
    b, dt, soups = make_batch(gpu_ctx, sizes, 15, 700)
    cams, lights = scenes.batch_views(len(sizes), 64, 48)
    b.set_views(cams, lights)
    hits, vis = b.alloc_outputs()
    b.trace(hits, vis)
    ref_h, ref_v = hits.clone(), vis.clone()
    h2, _ = b.alloc_outputs(shadow=False)
    b.trace(h2, None)
    f = BatchFrame(gpu_ctx, b, dt, hits, vis)
    assert f.nodes >= 10
    hits.zero_(); vis.zero_()
    for _ in range(3):
        f.launch()
    gpu_ctx.check()
    assert torch.equal(hits, ref_h) and torch.equal(vis, ref_v) and torch.equal(h2, ref_h)


def test_batch_rejects_bad_arguments(gpu_ctx):
    from rtgpu import _lib as L
    from rtgpu import scenes
    from rtgpu.api import Batch
    with pytest.raises(L.RtError):
        Batch(gpu_ctx, [10, 0, 5], 12)
    with pytest.raises(L.RtError):
        Batch(gpu_ctx, [10] * 257, 12)
    with pytest.raises(L.RtError):
        Batch(gpu_ctx, [10], 24)
    b = Batch(gpu_ctx, [10, 20], 8)
    cams, lights = scenes.batch_views(2, 16, 16)
    cams[1] = scenes.batch_views(2, 16, 8)[0][1]
    with pytest.raises(L.RtError):
        b.set_views(cams, lights)
    with pytest.raises(L.RtError):
        b.tuning = {"threads": 96, "grab": 1, "order": 0}
    with pytest.raises(L.RtError):
        b.tuning = {"threads": 64, "grab": 17, "order": 0}
