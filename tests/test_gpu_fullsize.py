"""Parity at the full size of the per-frame workload: the 2,099,520-triangle
displaced icosphere rebuilt at depth 20 (two frames), traced at 1920x1080
with primary, shadow and mirror rays through the production path (heavy-ray
hand-over, heavy-first tile order, compacted shading rays) and through the
captured frame graph, all against the oracle."""
import numpy as np
import pytest

from test_gpu_trace import assert_hits_equal
from bitcmp import same_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def frames():
    from rtgpu import scenes
    s = scenes.icosphere(324)
    return [s.frame(0), s.frame(1)]


def test_full_frame_build_and_trace(gpu_ctx, oracle_mod, frames):
    import torch
    from rtgpu import scenes
    from rtgpu.api import LBVH, Frame, RayTracer, hits_to_numpy
    cam = scenes.sphere_camera()
    light = scenes.TORUS_LIGHT
    npx = cam.width * cam.height
    lb = LBVH(gpu_ctx, len(frames[0]), 20)
    rt = RayTracer(gpu_ctx)
    dev = [torch.from_numpy(f).cuda() for f in frames]
    for k, tris in enumerate(frames):
        lb.Build(dev[k])
        # twice, so the second call runs with the first call's tile order
        for _ in range(2):
            hits = rt.primary(lb, cam)
            vis, mirror = rt.shadow_mirror(lb, cam, light, hits)
        gpu_ctx.check()
        nodes, ids, keys = lb.download(True, True, True)
        onodes, oids, okeys, reached = oracle_mod.lbvh_build(tris, 20)
        assert np.array_equal(keys, okeys) and np.array_equal(ids, oids)
        r = np.nonzero(reached)[0]
        assert same_bits(nodes[r], onodes[r])
        oh = oracle_mod.trace(onodes, 20, oids, tris, oracle_mod.primary_rays(cam))
        ovis, omir = oracle_mod.shadow_mirror(onodes, 20, oids, tris, cam, light, oh)
        assert_hits_equal(hits_to_numpy(hits), oh, "primary")
        assert np.array_equal(vis.cpu().numpy(), ovis)
        assert_hits_equal(hits_to_numpy(mirror), omir, "mirror")
        assert (oh["id"] >= 0).sum() > 300_000 and (ovis == 3).sum() > 100_000
    # the shading rays started at the primary leaves (the frame path's walk)
    hits, leaves = rt.primary_leaves(lb, cam)
    vis, mirror, _ = rt.shadow_mirror_from(lb, cam, light, hits, leaves)
    gpu_ctx.check()
    oh, ol = oracle_mod.trace_from(onodes, 20, oids, tris, oracle_mod.primary_rays(cam))
    ovis, omir, _ = oracle_mod.shadow_mirror_from(onodes, 20, oids, tris, cam, light, oh, ol)
    assert np.array_equal(vis.cpu().numpy(), ovis)
    assert_hits_equal(hits_to_numpy(mirror), omir, "mirror from leaves")
    # the captured frame (rebuild + both passes in one graph) gives the same images
    h2 = torch.empty((npx, 4), dtype=torch.int32, device="cuda")
    v2 = torch.empty(npx, dtype=torch.uint8, device="cuda")
    m2 = torch.empty((npx, 4), dtype=torch.int32, device="cuda")
    f = Frame(gpu_ctx, lb, dev[1], cam, light, h2, v2, m2)
    for _ in range(3):
        f.launch()
    gpu_ctx.check()
    assert torch.equal(h2, hits) and torch.equal(v2, vis) and torch.equal(m2, mirror)
    f.close()
