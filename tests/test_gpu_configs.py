"""Parity at the workloads' full sizes, through the C ABI, against the oracle.

  * Path-traced GI: the closed box with 262,144 random triangles (262,158 in
    all) built at depth 20, rendered at 1024 x 1024, 4 spp, 4 bounces on the
    GPU; the oracle renders a 128 x 128 crop of the same image (same pixels,
    same per-pixel sample streams): RMSE <= 1e-4 per channel, and equal bits.
  * Differentiable: the same scene at 512 x 512, 8 spp, 3 bounces, target
    rendered with albedo + U(+-0.1) clamped to [0, 1], L2 image loss.  The
    GPU adjoint gradients against central finite differences (h = 1e-3) on
    64 sampled parameters (63 albedo channels and the emitter radiance), and
    against the oracle's FP64 adjoint on a 128 x 128 crop (dL/dI outside the
    crop set to zero on both sides).
  * Batched: the 256-scene batch of 1,000 - 200,000 triangles each
    (11,549,566 in all) at depth 20 and 256 x 256 per scene; the ten largest
    scenes' trees, primary hits and shadow visibility against the oracle's
    build and trace of each scene alone.
"""
import numpy as np
import pytest

from bitcmp import same_bits
from test_gpu_trace import assert_hits_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gi_full(gpu_ctx, oracle_mod):
    import torch
    from rtgpu import scenes
    from rtgpu.api import LBVH
    sc = scenes.gi_box(262144, seed=3)
    depth = 20
    lb = LBVH(gpu_ctx, len(sc.tris), depth)
    lb.Build(torch.from_numpy(sc.tris).cuda())
    gpu_ctx.check()
    nodes, ids, keys, reached = oracle_mod.lbvh_build(sc.tris, depth)
    return sc, lb, depth, nodes, ids, keys, reached


def _crop(img, width, x0, y0, w, h):
    return img.reshape(-1, width, 4)[y0:y0 + h, x0:x0 + w].reshape(-1, 4)


def test_gi_box_build_at_full_size(gpu_ctx, gi_full):
    sc, lb, depth, nodes, ids, keys, reached = gi_full
    assert len(sc.tris) == 262158
    gn, gi, gk = lb.download(True, True, True)
    assert np.array_equal(gk, keys) and np.array_equal(gi, ids)
    r = np.nonzero(reached)[0]
    assert same_bits(gn[r], nodes[r])


def test_pathtrace_1024_4spp_4bounces_crop(gpu_ctx, oracle_mod, gi_full):
    import torch
    from rtgpu import scenes
    from rtgpu.api import RayTracer
    sc, lb, depth, nodes, ids, _, _ = gi_full
    cam = scenes.gi_camera(1024, 1024)
    img = RayTracer(gpu_ctx).pathtrace(lb, torch.from_numpy(sc.albedo).cuda(), torch.from_numpy(sc.emission).cuda(),
                                       cam, spp=4, bounces=4, seed=1000).cpu().numpy()
    gpu_ctx.check()
    win = (448, 448, 128, 128)
    ref = oracle_mod.pathtrace(nodes, depth, ids, sc.tris, sc.albedo, sc.emission, cam, 4, 4, 1000, window=win)
    got = _crop(img, 1024, *win)
    rmse = np.sqrt(np.mean((got[:, :3].astype(np.float64) - ref[:, :3]) ** 2, axis=0))
    assert np.all(rmse <= 1e-4), rmse
    assert same_bits(got, ref)
    # the soup is dense (262,144 triangles in the unit cube): few paths reach
    # the emitter within 4 bounces, so the image is dark but not black
    assert (got[:, :3] > 0).any() and (img[:, :3] > 0).sum() > 1000 and np.isfinite(img).all()


def test_adjoint_512_8spp_3bounces_fd64_and_fp64(gpu_ctx, oracle_mod, gi_full):
    import torch
    from rtgpu import scenes
    from rtgpu.api import RayTracer
    from rtgpu.autograd import render
    sc, lb, depth, nodes, ids, _, _ = gi_full
    W = H = 512
    spp, bounces, seed = 8, 3, 12345
    cam = scenes.gi_camera(W, H)
    rt = RayTracer(gpu_ctx)
    mask = torch.from_numpy((sc.emission[:, 0] > 0).astype(np.float32)).cuda()
    rng = np.random.Generator(np.random.PCG64(7))
    talb = np.clip(sc.albedo + rng.uniform(-0.1, 0.1, sc.albedo.shape), 0, 1).astype(np.float32)
    le = torch.tensor([10.0, 10.0, 10.0], device="cuda")
    with torch.no_grad():
        target = render(torch.from_numpy(talb).cuda(), le, mask, rt, lb, cam, spp, bounces, seed)[:, :3].double()
    alb = torch.from_numpy(sc.albedo).cuda().requires_grad_(True)
    le_p = le.clone().requires_grad_(True)
    img = render(alb, le_p, mask, rt, lb, cam, spp, bounces, seed)
    loss = ((img[:, :3] - target.float()) ** 2).mean()
    loss.backward()
    gpu_ctx.check()
    g_alb = alb.grad.cpu().numpy().astype(np.float64).ravel()
    g_le = le_p.grad.cpu().numpy().astype(np.float64)
    nz = np.nonzero(g_alb)[0]
    assert len(nz) > 100  # only triangles on paths that reach the emitter get a gradient

    # forward crop equals the oracle bit for bit
    win = (192, 192, 128, 128)
    ref_img = oracle_mod.pathtrace(nodes, depth, ids, sc.tris, sc.albedo, sc.emission, cam, spp, bounces, seed,
                                   window=win)
    assert same_bits(_crop(img.detach().cpu().numpy(), W, *win), ref_img)

    # FP64 oracle adjoint on the crop against the GPU adjoint of the same crop
    d_img = np.zeros((W * H, 4), np.float32)
    d_img[:, :3] = (2.0 / (W * H * 3)) * (img.detach()[:, :3].double() - target).cpu().numpy()
    d_crop = np.zeros_like(d_img)
    d_crop.reshape(-1, W, 4)[win[1]:win[1] + win[3], win[0]:win[0] + win[2]] = \
        d_img.reshape(-1, W, 4)[win[1]:win[1] + win[3], win[0]:win[0] + win[2]]
    emission = np.ascontiguousarray(sc.emission)
    ga, gl = rt.pathtrace_adjoint(lb, torch.from_numpy(sc.albedo).cuda(), torch.from_numpy(emission).cuda(), cam, spp,
                                  bounces, seed, torch.from_numpy(d_crop).cuda())
    gpu_ctx.check()
    ra, rl = oracle_mod.pathtrace_adjoint(nodes, depth, ids, sc.tris, sc.albedo, emission, cam, spp, bounces, seed,
                                          np.ascontiguousarray(_crop(d_img, W, *win)), window=win)
    scale = np.abs(ra).max()
    assert scale > 0
    assert np.abs(ga.cpu().numpy().astype(np.float64) - ra).max() <= 1e-4 * scale
    assert np.allclose(gl.cpu().numpy().astype(np.float64), rl, rtol=1e-4, atol=1e-4 * np.abs(rl).max())

    # central differences (h = 1e-3) on 64 sampled parameters
    order = nz[np.argsort(-np.abs(g_alb[nz]))]
    pick = list(order[:32]) + list(rng.choice(order[32:], size=31, replace=False))
    alb0 = torch.from_numpy(sc.albedo).cuda()

    def loss_at(a, radiance):
        with torch.no_grad():
            im = render(a, radiance, mask, rt, lb, cam, spp, bounces, seed)
            return float(((im[:, :3].double() - target) ** 2).mean())

    h = 1e-3
    gmax = np.abs(g_alb).max()
    for k in pick:
        a_p = alb0.clone()
        a_m = alb0.clone()
        a_p.view(-1)[k] += h
        a_m.view(-1)[k] -= h
        h_eff = (float(a_p.view(-1)[k]) - float(a_m.view(-1)[k])) / 2.0  # the fp32 step actually taken
        fd = (loss_at(a_p, le) - loss_at(a_m, le)) / (2.0 * h_eff)
        assert abs(fd - g_alb[k]) <= 1e-2 * abs(g_alb[k]) + 1e-5 * gmax, (k, fd, g_alb[k])
    # the 64th: the emitter radiance (its red channel)
    l_p = le.clone()
    l_m = le.clone()
    l_p[0] += h
    l_m[0] -= h
    h_eff = (float(l_p[0]) - float(l_m[0])) / 2.0
    fd = (loss_at(alb0, l_p) - loss_at(alb0, l_m)) / (2.0 * h_eff)
    assert abs(fd - g_le[0]) <= 1e-2 * abs(g_le[0]) + 1e-9, (fd, g_le[0])


def test_batch_256_scenes_largest_ten(gpu_ctx, oracle_mod):
    import torch
    from rtgpu import scenes
    from rtgpu.api import Batch, hits_to_numpy
    sizes = scenes.batch_sizes(256)
    soup = scenes.batch_scene(sizes)
    assert int(sizes.sum()) == 11_549_566 and sizes.max() <= 200_000
    off = np.concatenate([[0], np.cumsum(sizes)])
    depth = 20
    cams, lights = scenes.batch_views(len(sizes), 256, 256)
    b = Batch(gpu_ctx, sizes, depth)
    b.set_views(cams, lights)
    b.build(torch.from_numpy(soup).cuda())
    hits, vis = b.alloc_outputs()
    b.trace(hits, vis)
    gpu_ctx.check()
    H = hits_to_numpy(hits).reshape(len(sizes), -1)
    V = vis.cpu().numpy().reshape(len(sizes), -1)
    for s in np.argsort(-sizes)[:10]:
        tris = soup[off[s]:off[s + 1]]
        nodes, ids, keys = b.download(int(s))
        onodes, oids, okeys, reached = oracle_mod.lbvh_build(tris, depth)
        assert np.array_equal(keys, okeys) and np.array_equal(ids, oids), f"scene {s}"
        r = np.nonzero(reached)[0]
        assert same_bits(nodes[r], onodes[r]), f"scene {s}: nodes"
        oh = oracle_mod.trace(onodes, depth, oids, tris, oracle_mod.primary_rays(cams[s]))
        assert_hits_equal(H[s], oh, f"scene {s} primary")
        ovis, _ = oracle_mod.shadow_mirror(onodes, depth, oids, tris, cams[s], lights[s], oh)[:2]
        assert np.array_equal(V[s], ovis), f"scene {s} shadow"
        assert (oh["id"] >= 0).mean() > 0.05
    b.close()
