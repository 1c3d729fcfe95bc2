"""The reference's SAH BVH traced on the GPU (rt_bvh: BVH_IntersectP,
BVH.hlsl:124-217) through the C ABI, over the reference's own trees from
the golden fixtures: hits and per-ray box / triangle test counts bit-exact
against the oracle's restatement, and the reference's own BVH::IntersectP
hits matched up to near-ties (t bit-exact)."""
import numpy as np
import pytest

import tri_np
from test_gpu_trace import assert_hits_equal
from test_oracle_bvh import bvh_cases, load_bvh
from bitcmp import same_bits

pytestmark = pytest.mark.gpu


def import_bvh(ctx, g):
    from rtgpu.api import BVH
    return BVH(ctx, len(g["nodes"]), len(g["tris"])).Import(g["nodes"], g["ids"], g["tris"])


@pytest.mark.parametrize("case", bvh_cases())
@pytest.mark.parametrize("any_hit", [False, True])
def test_bvh_rays_fixture(gpu_ctx, oracle_mod, case, any_hit):
    from rtgpu.api import RayTracer, hits_to_numpy, rays_tensor
    g = load_bvh(case)
    b = import_bvh(gpu_ctx, g)
    r = g["rays"]
    hits, st = RayTracer(gpu_ctx).rays(b, rays_tensor(r[:, 0:3], r[:, 3:6], r[:, 6], r[:, 7].astype(np.int32), "cuda"),
                                       any_hit=any_hit, stats=True)
    gpu_ctx.check()
    oh, ost = oracle_mod.bvh_trace(g["nodes"], g["ids"], g["tris"], r, any_hit=any_hit, stats=True)
    gh = hits_to_numpy(hits)
    if any_hit:
        assert np.array_equal(gh["id"], oh["id"])
        assert np.array_equal(gh["id"] >= 0, g["hit_id"] >= 0)
    else:
        assert_hits_equal(gh, oh, case)
        tri_np.assert_matches_reference(gh["id"], gh["t"], g["hit_id"], g["hit_t"], r, g["tris"])
        assert same_bits(gh["t"], g["hit_t"])
    assert np.array_equal(st.cpu().numpy().astype(np.uint32), ost)
    b.close()


def test_bvh_primary_shadow_mirror(gpu_ctx, oracle_mod):
    from conftest import camera_from_array
    from rtgpu import scenes
    from rtgpu.api import RayTracer, hits_to_numpy
    g = load_bvh("torus_96x48")
    b = import_bvh(gpu_ctx, g)
    cam = scenes.look_at((2.0, -1.6, 1.4), (0.0, 0.0, 0.0), width=240, height=160)
    rt = RayTracer(gpu_ctx)
    hits, pst = rt.primary(b, cam, stats=True)
    vis, mir, ss, ms = rt.shadow_mirror(b, cam, scenes.TORUS_LIGHT, hits, stats=True)
    gpu_ctx.check()
    oh, opst = oracle_mod.bvh_trace(g["nodes"], g["ids"], g["tris"], oracle_mod.primary_rays(cam), stats=True)
    assert_hits_equal(hits_to_numpy(hits), oh, "primary")
    assert np.array_equal(pst.cpu().numpy().astype(np.uint32), opst)
    ovis, omir, oss, oms = oracle_mod.bvh_shadow_mirror(g["nodes"], g["ids"], g["tris"], cam, scenes.TORUS_LIGHT, oh,
                                                        stats=True)
    assert np.array_equal(vis.cpu().numpy(), ovis)
    assert set(np.unique(ovis)) >= {0, 2, 3}
    assert_hits_equal(hits_to_numpy(mir), omir, "mirror")
    assert np.array_equal(ss.cpu().numpy().astype(np.uint32), oss)
    assert np.array_equal(ms.cpu().numpy().astype(np.uint32), oms)
    # the LBVH over the same soup (a different tree) finds the same closest
    # hits, up to near-ties
    import torch
    from rtgpu.api import LBVH
    lb = LBVH(gpu_ctx, len(g["tris"]), 18).Build(torch.from_numpy(g["tris"]).cuda())
    lh = hits_to_numpy(rt.primary(lb, cam))
    gpu_ctx.check()
    gh = hits_to_numpy(hits)
    tri_np.assert_matches_reference(lh["id"], lh["t"], gh["id"], gh["t"], oracle_mod.primary_rays(cam), g["tris"])
    b.close()


def test_bvh_import_rejects_malformed_trees(gpu_ctx):
    from rtgpu._lib import RtError
    from rtgpu.api import BVH
    g = load_bvh("soup_5000")
    nodes, ids, tris = g["nodes"].copy(), g["ids"].copy(), g["tris"]
    b = BVH(gpu_ctx, len(nodes), len(tris))
    interior = np.nonzero(nodes["prim_count"] <= 0)[0]
    leaf = np.nonzero(nodes["prim_count"] > 0)[0]
    bad = []
    x = nodes.copy(); x["prim_pos"][interior[0]] = len(nodes) + 5; bad.append((x, ids))        # child outside
    x = nodes.copy(); x["prim_pos"][interior[3]] = interior[3]; bad.append((x, ids))            # child before itself
    x = nodes.copy(); x["prim_pos"][interior[1]] = x["prim_pos"][interior[2]]; bad.append((x, ids))  # shared child
    x = nodes.copy(); x["prim_count"][interior[0]] = -3; bad.append((x, ids))                   # axis 3
    x = nodes.copy(); x["prim_pos"][leaf[0]] = len(tris); bad.append((x, ids))                  # leaf range
    y = ids.copy(); y[7] = len(tris); bad.append((nodes, y))                                    # id
    for bn, bi in bad:
        with pytest.raises(RtError):
            b.Import(bn, bi, tris)
    b.Import(nodes, ids, tris)  # the unmodified tree still imports
    gpu_ctx.check()
    b.close()
