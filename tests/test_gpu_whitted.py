"""The colour stage with its bounce loop (rt_render_whitted: CSComputeColorRT
.hlsl with RayTracerCS::Render's loop) against the oracle's restatement
(or_render_whitted): accumulation and result images bit-exact.  The
contract's tolerance for this floating-point stage is 1e-5 relative per
channel; the kernels evaluate the same IEEE operations in the same order, so
the test asks for equality."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def materials(seed=3, m=6):
    rng = np.random.default_rng(seed)
    rows = np.zeros((m, 14), np.float32)
    rows[:, 0:3] = rng.uniform(0.0, 0.3, (m, 3))
    rows[:, 3] = rng.choice([1.0, 1.5, 0.7], m)          # ambient.w: refraction index
    rows[:, 4:7] = rng.uniform(0.2, 1.0, (m, 3))
    rows[:, 7] = rng.choice([1.0, 0.6, 0.25], m)         # diffuse.w weighs diffuse against specular
    rows[:, 8:11] = rng.uniform(0.0, 0.9, (m, 3))
    rows[:, 11] = 1.0
    rows[:, 12] = rng.uniform(0.0, 1.0, m)
    rows[:, 13] = rng.choice([1.0, 0.5, 0.0], m)         # alpha: mirror probability
    rows[0, 13] = 1.0
    return rows


def close_enough(g, o):
    assert np.all(np.isfinite(o))
    rel = np.abs(g.astype(np.float64) - o) / np.maximum(np.abs(o.astype(np.float64)), 1e-30)
    assert rel.max(initial=0.0) <= 1e-5
    assert np.array_equal(g, o)


@pytest.fixture(scope="module")
def torus(gpu_ctx, oracle_mod):
    import torch
    from rtgpu import scenes
    from rtgpu.api import LBVH
    tris = scenes.torus(128, 64)
    lb = LBVH(gpu_ctx, len(tris), 16).Build(torch.from_numpy(tris).cuda())
    nodes, ids, _, _ = oracle_mod.lbvh_build(tris, 16)
    rng = np.random.default_rng(11)
    mids = rng.integers(0, 6, len(tris)).astype(np.int32)
    # per-corner normals: away from the ring centre, slightly perturbed
    c = tris.reshape(-1, 3, 3).astype(np.float64)
    ring = c.copy()
    ring[..., 2] = 0.0
    ring /= np.linalg.norm(ring, axis=2, keepdims=True)
    nrm = c - ring + rng.normal(0, 0.02, c.shape)
    nrm = (nrm / np.linalg.norm(nrm, axis=2, keepdims=True)).astype(np.float32).reshape(-1, 9)
    return tris, lb, nodes, ids, mids, nrm


CASES = [
    dict(bounces=0, shadows=True, phong=False, gloss_mapping=False, env_mapping=-1),
    dict(bounces=3, shadows=True, phong=True, gloss_mapping=True, env_mapping=-1, seed=5),
    dict(bounces=2, shadows=False, phong=False, gloss_mapping=False, env_mapping=0, seed=9),
    dict(bounces=5, shadows=True, phong=True, gloss_mapping=False, env_mapping=0, env_color=(0.3, 0.5, 0.9)),
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_whitted_torus(gpu_ctx, oracle_mod, torus, case):
    import torch
    from rtgpu import scenes
    from rtgpu.api import RayTracer
    tris, lb, nodes, ids, mids, nrm = torus
    kw = dict(CASES[case])
    cam = scenes.look_at((2.0, -1.6, 1.4), (0.0, 0.0, 0.0), width=200, height=150)
    light = (1.5, 2.5, 3.0)
    mats = materials()
    acc, res = RayTracer(gpu_ctx).whitted(lb, cam, light, mats, torch.from_numpy(mids).cuda(),
                                          torch.from_numpy(nrm).cuda(), **kw)
    gpu_ctx.check()
    oacc, ores = oracle_mod.render_whitted(nodes, 16, ids, tris, cam, light, mats, mids, nrm, **kw)
    close_enough(acc.cpu().numpy(), oacc)
    close_enough(res.cpu().numpy(), ores)
    assert oacc[:, :3].max() > 0.1
    if kw["env_mapping"] == 0:  # a miss shows 1 and leaves the accumulation alone
        assert (ores == 1.0).all(axis=1).sum() > 100


def test_whitted_model_file(gpu_ctx, oracle_mod):
    """A model file's soup, material ids and MTL colours (rt_model_load)
    through the colour stage."""
    import torch
    from conftest import GOLDEN
    from rtgpu import model, scenes
    from rtgpu.api import LBVH, RayTracer
    from rtgpu import build
    build.build_host()
    m = model.load(GOLDEN / "models" / "torus.OBJ")
    mats = np.stack([x.row() for x in m.materials])
    lb = LBVH(gpu_ctx, len(m.soup), 12).Build(torch.from_numpy(m.soup).cuda())
    cam = scenes.look_at((0.3, -1.2, 0.9), (0.0, 0.0, 0.0), width=160, height=120)
    light = (1.0, 1.0, 1.0)
    acc, res = RayTracer(gpu_ctx).whitted(lb, cam, light, mats, torch.from_numpy(m.material_ids).cuda(),
                                          bounces=2)
    gpu_ctx.check()
    nodes, ids, _, _ = oracle_mod.lbvh_build(m.soup, 12)
    oacc, ores = oracle_mod.render_whitted(nodes, 12, ids, m.soup, cam, light, mats, m.material_ids, bounces=2)
    close_enough(acc.cpu().numpy(), oacc)
    close_enough(res.cpu().numpy(), ores)
