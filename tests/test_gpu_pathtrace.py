"""Path tracer and adjoint on the GPU against the oracle.

Forward: the seeded image equals the CPU rendering of the same sample
sequence (contract tolerance: RMSE <= 1e-4 per channel; the kernel uses only
IEEE +,-,*,/,sqrt in the oracle's order, so it is checked bit-exact too).
Adjoint: against the oracle's FP64 adjoint and central finite differences
(h = 1e-3) on sampled parameters.
"""
import numpy as np
import pytest
from bitcmp import same_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gi_small(gpu_ctx, oracle_mod):
    import torch
    from rtgpu import scenes
    from rtgpu.api import LBVH
    sc = scenes.gi_box(n_soup=20000, seed=3)
    depth = 16
    lb = LBVH(gpu_ctx, len(sc.tris), depth)
    dt = torch.from_numpy(sc.tris).cuda()
    lb.Build(dt)
    nodes, ids, _, _ = oracle_mod.lbvh_build(sc.tris, depth)
    return sc, lb, dt, nodes, ids, depth


def test_pathtrace_matches_cpu(gpu_ctx, oracle_mod, gi_small):
    import torch
    from rtgpu import scenes
    from rtgpu.api import RayTracer
    sc, lb, dt, nodes, ids, depth = gi_small
    cam = scenes.gi_camera(96, 80)
    alb = torch.from_numpy(sc.albedo).cuda()
    em = torch.from_numpy(sc.emission).cuda()
    img = RayTracer(gpu_ctx).pathtrace(lb, alb, em, cam, spp=3, bounces=4, seed=1234).cpu().numpy()
    gpu_ctx.check()
    ref = oracle_mod.pathtrace(nodes, depth, ids, sc.tris, sc.albedo, sc.emission, cam, 3, 4, 1234)
    rmse = np.sqrt(np.mean((img[:, :3].astype(np.float64) - ref[:, :3]) ** 2, axis=0))
    assert np.all(rmse <= 1e-4), rmse
    assert same_bits(img, ref)
    assert img[:, :3].mean() > 0.0


def test_adjoint_matches_fp64_and_fd(gpu_ctx, oracle_mod, gi_small):
    import torch
    from rtgpu import scenes
    from rtgpu.api import RayTracer
    from rtgpu.autograd import render
    sc, lb, dt, nodes, ids, depth = gi_small
    cam = scenes.gi_camera(48, 40)
    spp, bounces, seed = 2, 3, 99
    rt = RayTracer(gpu_ctx)
    mask = torch.from_numpy((sc.emission[:, 0] > 0).astype(np.float32)).cuda()
    rng = np.random.default_rng(5)
    target_alb = np.clip(sc.albedo + rng.uniform(-0.1, 0.1, sc.albedo.shape), 0, 1).astype(np.float32)
    le = torch.tensor([10.0, 10.0, 10.0], device="cuda")
    with torch.no_grad():
        target = render(torch.from_numpy(target_alb).cuda(), le, mask, rt, lb, cam, spp, bounces, seed)
    alb = torch.from_numpy(sc.albedo).cuda().requires_grad_(True)
    le_p = le.clone().requires_grad_(True)
    img = render(alb, le_p, mask, rt, lb, cam, spp, bounces, seed)
    loss = ((img[:, :3] - target[:, :3]) ** 2).mean()
    loss.backward()
    gpu_ctx.check()
    g_alb = alb.grad.cpu().numpy().astype(np.float64)
    g_le = le_p.grad.cpu().numpy().astype(np.float64)
    # FP64 CPU adjoint of the same loss
    d_img = np.zeros((cam.width * cam.height, 4), np.float32)
    d_img[:, :3] = (2.0 / (cam.width * cam.height * 3)) * (img.detach().cpu().numpy()[:, :3] - target.cpu().numpy()[:, :3])
    emission = sc.emission
    ref_alb, ref_le = oracle_mod.pathtrace_adjoint(nodes, depth, ids, sc.tris, sc.albedo, emission, cam, spp, bounces,
                                                   seed, d_img)
    scale = np.abs(ref_alb).max()
    assert scale > 0
    assert np.abs(g_alb - ref_alb).max() <= 1e-4 * scale
    assert np.allclose(g_le, ref_le, rtol=1e-4, atol=1e-4 * np.abs(ref_le).max())
    # central finite differences on the largest-gradient parameters (common random numbers)
    flat = np.argsort(-np.abs(ref_alb).ravel())[:8]
    h = 1e-3

    def loss_at(a):
        with torch.no_grad():
            im = render(torch.from_numpy(a).cuda(), le, mask, rt, lb, cam, spp, bounces, seed)
            return float(((im[:, :3].double() - target[:, :3].double()) ** 2).mean())

    for k in flat:
        a_p = sc.albedo.copy(); a_p.ravel()[k] += h
        a_m = sc.albedo.copy(); a_m.ravel()[k] -= h
        fd = (loss_at(a_p) - loss_at(a_m)) / (2 * h)
        assert abs(fd - ref_alb.ravel()[k]) <= 2e-2 * abs(ref_alb.ravel()[k]) + 1e-9, (k, fd, ref_alb.ravel()[k])


def test_progressive_accumulation_across_calls(gpu_ctx, oracle_mod, gi_small):
    """rt_pt_params.first_sample = n0 continues the progressive mean the image
    holds (the reference's frame counter, RayTracerCS.cpp:306, with the
    factors of ConstantBuffers.h:102-109): 2 spp from n0 = 0 then 2 spp from
    n0 = 2 equal one call of 4 spp bit for bit, and the oracle's
    continuation; n0 = 0 starts afresh (the reset on camera motion)."""
    import torch
    from rtgpu import scenes
    from rtgpu.api import RayTracer
    sc, lb, dt, nodes, ids, depth = gi_small
    cam = scenes.gi_camera(64, 48)
    alb = torch.from_numpy(sc.albedo).cuda()
    em = torch.from_numpy(sc.emission).cuda()
    rt = RayTracer(gpu_ctx)
    full = rt.pathtrace(lb, alb, em, cam, spp=4, bounces=3, seed=77).cpu().numpy()
    img = torch.full((cam.width * cam.height, 4), 123.0, device="cuda")  # not read at n0 = 0
    rt.pathtrace(lb, alb, em, cam, spp=2, bounces=3, seed=77, out=img)
    half = img.cpu().numpy()
    rt.pathtrace(lb, alb, em, cam, spp=2, bounces=3, seed=77, out=img, first_sample=2)
    gpu_ctx.check()
    assert same_bits(img.cpu().numpy(), full)
    o_half = oracle_mod.pathtrace(nodes, depth, ids, sc.tris, sc.albedo, sc.emission, cam, 2, 3, 77)
    assert same_bits(o_half, half)
    o_cont = oracle_mod.pathtrace(nodes, depth, ids, sc.tris, sc.albedo, sc.emission, cam, 2, 3, 77,
                                  first_sample=2, image=o_half)
    assert same_bits(o_cont, full)
    # frames of one sample each, as the reference renders (n0 = frame count)
    rt.pathtrace(lb, alb, em, cam, spp=1, bounces=3, seed=77, out=img)
    for n0 in (1, 2, 3):
        rt.pathtrace(lb, alb, em, cam, spp=1, bounces=3, seed=77, out=img, first_sample=n0)
    gpu_ctx.check()
    assert same_bits(img.cpu().numpy(), full)


def test_progressive_adjoint_differentiates_the_new_samples(gpu_ctx, oracle_mod, gi_small):
    """The adjoint of a call with n0 > 0 weights each new sample by its
    weight in the final mean; the FP64 oracle with the same n0 agrees."""
    import torch
    from rtgpu import scenes
    from rtgpu.api import RayTracer
    sc, lb, dt, nodes, ids, depth = gi_small
    cam = scenes.gi_camera(40, 32)
    rt = RayTracer(gpu_ctx)
    alb = torch.from_numpy(sc.albedo).cuda()
    em = torch.from_numpy(sc.emission).cuda()
    rng = np.random.default_rng(3)
    g = rng.normal(size=(cam.width * cam.height, 4)).astype(np.float32)
    g[:, 3] = 0.0
    d_alb, d_le = rt.pathtrace_adjoint(lb, alb, em, cam, 3, 2, 55, torch.from_numpy(g).cuda(), first_sample=2)
    gpu_ctx.check()
    ref_alb, ref_le = oracle_mod.pathtrace_adjoint(nodes, depth, ids, sc.tris, sc.albedo, sc.emission, cam, 3, 2, 55,
                                                   g, first_sample=2)
    scale = np.abs(ref_alb).max()
    assert scale > 0
    assert np.abs(d_alb.cpu().numpy().astype(np.float64) - ref_alb).max() <= 1e-4 * scale
