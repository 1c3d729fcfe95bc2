"""rt_trace_frame_shader_order: a frame traced in the reference shader's own
walk order (LBVH_IntersectP, LBVH.hlsl:363-440) on the GPU, against the
oracle's restatement of that walk: hits (exact ties resolved as the shader
resolves them), visibility, mirror hits and the per-ray iVisitedNodes counts
bit-exact."""
import numpy as np
import pytest

from conftest import camera_from_array, load_golden
from bitcmp import same_bits

pytestmark = pytest.mark.gpu


def run_both(gpu_ctx, oracle_mod, tris, depth, cam, light):
    import torch
    from rtgpu.api import LBVH, RayTracer, hits_to_numpy
    lb = LBVH(gpu_ctx, len(tris), depth).Build(torch.from_numpy(np.ascontiguousarray(tris)).cuda())
    prim, vis, mir, pst, sst, mst = RayTracer(gpu_ctx).frame_shader_order(lb, cam, light, stats=True)
    gpu_ctx.check()
    nodes, ids, _, _ = oracle_mod.lbvh_build(tris, depth)
    o = oracle_mod.frame_hlsl(nodes, depth, ids, tris, cam, light)
    g = (hits_to_numpy(prim), vis.cpu().numpy(), hits_to_numpy(mir),
         *(x.cpu().numpy().astype(np.uint32) for x in (pst, sst, mst)))
    return g, o


@pytest.mark.parametrize("scene", ["torus", "duplicates"])
def test_frame_shader_order_matches_oracle(gpu_ctx, oracle_mod, scene):
    from rtgpu import scenes
    if scene == "torus":
        tris, depth, cam = scenes.torus(), 20, scenes.torus_camera(256, 256)
    else:  # every triangle three times: exact ties everywhere
        g = load_golden("soup_duplicates")
        tris, depth, cam = g["tris"], int(g["depth"]), camera_from_array(g["camera"])
    light = scenes.TORUS_LIGHT
    (gp, gv, gm, gps, gss, gms), (op, ov, om, ops, oss, oms) = run_both(gpu_ctx, oracle_mod, tris, depth, cam, light)
    assert same_bits(gp, op) and np.array_equal(gv, ov) and same_bits(gm, om)
    assert np.array_equal(gps, ops) and np.array_equal(gss, oss) and np.array_equal(gms, oms)
    assert (op["id"] >= 0).sum() > 100


def test_frame_shader_order_vs_production_path(gpu_ctx, oracle_mod):
    """Same scene through the production calls: identical t and visibility,
    ids equal except where the two tie rules pick different triangles."""
    import torch
    from rtgpu import scenes
    from rtgpu.api import LBVH, RayTracer, hits_to_numpy
    tris = np.ascontiguousarray(scenes.icosphere(80).frame(0), np.float32)
    cam = scenes.sphere_camera(480, 270)
    lb = LBVH(gpu_ctx, len(tris), 18).Build(torch.from_numpy(tris).cuda())
    rt = RayTracer(gpu_ctx)
    sp, sv, sm = rt.frame_shader_order(lb, cam, scenes.TORUS_LIGHT)
    pp, leaves = rt.primary_leaves(lb, cam)
    pv, pm, _ = rt.shadow_mirror_from(lb, cam, scenes.TORUS_LIGHT, pp, leaves)
    gpu_ctx.check()
    a, b = hits_to_numpy(sp), hits_to_numpy(pp)
    assert same_bits(a["t"], b["t"])
    same = a["id"] == b["id"]
    assert same.mean() > 0.999
    assert np.array_equal(sv.cpu().numpy()[same], pv.cpu().numpy()[same])
