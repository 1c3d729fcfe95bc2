"""The per-frame rebuild + trace captured as a CUDA graph (rt_frame_capture)
replays to the same bits as the direct calls, frame after frame (the refit's
arrival epoch lives in device memory, so replays stay correct)."""
import numpy as np
import pytest
from bitcmp import same_bits

pytestmark = pytest.mark.gpu


def test_graph_frames_equal_direct_calls(gpu_ctx):
    import torch
    from rtgpu import scenes
    from rtgpu.api import LBVH, Frame, RayTracer, hits_to_numpy
    s = scenes.icosphere(freq=40)
    frames = [torch.from_numpy(s.frame(k)).cuda() for k in range(3)]
    cam = scenes.sphere_camera(320, 180)
    light = scenes.TORUS_LIGHT
    n = frames[0].shape[0]
    npx = cam.width * cam.height
    lb_g = LBVH(gpu_ctx, n, 16)
    prim = torch.empty((npx, 4), dtype=torch.int32, device="cuda")
    vis = torch.empty(npx, dtype=torch.uint8, device="cuda")
    mir = torch.empty((npx, 4), dtype=torch.int32, device="cuda")
    graphs = [Frame(gpu_ctx, lb_g, f, cam, light, prim, vis, mir) for f in frames]
    assert graphs[0].nodes >= 14
    rt = RayTracer(gpu_ctx)
    lb_d = LBVH(gpu_ctx, n, 16)
    for rep in range(2):
        for k, f in enumerate(frames):
            graphs[k].launch()
            gpu_ctx.check()
            gp, gv, gm = hits_to_numpy(prim), vis.cpu().numpy(), hits_to_numpy(mir)
            g_nodes, g_ids, g_keys = lb_g.download(True, True, True)
            lb_d.Build(f)
            dp, dl = rt.primary_leaves(lb_d, cam)
            dv, dm, _ = rt.shadow_mirror_from(lb_d, cam, light, dp, dl)
            gpu_ctx.check()
            d_nodes, d_ids, d_keys = lb_d.download(True, True, True)
            assert np.array_equal(g_keys, d_keys) and np.array_equal(g_ids, d_ids)
            assert same_bits(g_nodes, d_nodes), f"replay {rep} frame {k}: nodes differ"
            assert same_bits(gp, hits_to_numpy(dp))
            assert np.array_equal(gv, dv.cpu().numpy())
            assert same_bits(gm, hits_to_numpy(dm))
    for g in graphs:
        g.close()


def test_host_frame_graph(gpu_ctx):
    """rt_frame_capture_host: upload, rebuild, trace and read-back as one
    graph; each replay reads the soup's current contents and writes the same
    results as the device frame graph; pageable host buffers are refused."""
    import torch
    from rtgpu import scenes
    from rtgpu._lib import RtError
    from rtgpu.api import LBVH, Frame
    s = scenes.icosphere(freq=40)
    soups = [torch.from_numpy(s.frame(k)) for k in range(2)]
    cam = scenes.sphere_camera(320, 180)
    light = scenes.TORUS_LIGHT
    n, npx = soups[0].shape[0], cam.width * cam.height
    # device reference
    lb_d = LBVH(gpu_ctx, n, 16)
    dp = torch.empty((npx, 4), dtype=torch.int32, device="cuda")
    dv = torch.empty(npx, dtype=torch.uint8, device="cuda")
    dm = torch.empty((npx, 4), dtype=torch.int32, device="cuda")
    # host graph over one pinned soup buffer whose contents change per frame
    hs = torch.empty_like(soups[0]).pin_memory()
    hp = torch.empty((npx, 4), dtype=torch.int32).pin_memory()
    hv = torch.empty(npx, dtype=torch.uint8).pin_memory()
    hm = torch.empty((npx, 4), dtype=torch.int32).pin_memory()
    lb_h = LBVH(gpu_ctx, n, 16)
    fh = Frame(gpu_ctx, lb_h, hs, cam, light, hp, hv, hm, host=True)
    for k in range(2):
        hs.copy_(soups[k])
        fh.launch()
        gpu_ctx.sync()
        fd = Frame(gpu_ctx, lb_d, soups[k].cuda(), cam, light, dp, dv, dm)
        fd.launch()
        gpu_ctx.check()
        assert torch.equal(hp, dp.cpu()) and torch.equal(hv, dv.cpu()) and torch.equal(hm, dm.cpu())
        fd.close()
    fh.close()
    with pytest.raises(RtError):
        Frame(gpu_ctx, lb_h, soups[0].clone(), cam, light, hp, hv, hm, host=True)  # pageable soup


def test_frame_holds_its_structure(gpu_ctx):
    """A captured frame keeps its LBVH's buffers: a call that would grow them
    fails while the frame exists, destroying the LBVH first is deferred to
    the last frame destroy, and the frame still replays in between."""
    import torch
    from rtgpu import scenes
    from rtgpu._lib import RtError
    from rtgpu.api import LBVH, Frame, RayTracer
    s = scenes.icosphere(freq=30)
    tris = torch.from_numpy(s.frame(0)).cuda()
    cam = scenes.sphere_camera(160, 90)
    big = scenes.sphere_camera(320, 180)
    npx = cam.width * cam.height
    lb = LBVH(gpu_ctx, tris.shape[0], 14)
    prim = torch.empty((npx, 4), dtype=torch.int32, device="cuda")
    vis = torch.empty(npx, dtype=torch.uint8, device="cuda")
    mir = torch.empty((npx, 4), dtype=torch.int32, device="cuda")
    f = Frame(gpu_ctx, lb, tris, cam, scenes.TORUS_LIGHT, prim, vis, mir)
    f.launch()
    gpu_ctx.check()
    ref = (prim.clone(), vis.clone(), mir.clone())
    rt = RayTracer(gpu_ctx)
    hb = rt.primary(lb, big)
    with pytest.raises(RtError):
        rt.shadow_mirror(lb, big, scenes.TORUS_LIGHT, hb)  # would grow the shading lists
    lb.close()  # deferred: the frame still owns the buffers
    prim.zero_()
    f.launch()
    gpu_ctx.check()
    assert torch.equal(prim, ref[0]) and torch.equal(vis, ref[1]) and torch.equal(mir, ref[2])
    f.close()  # frees the LBVH


def test_pipe_frames_equal_device_frames(gpu_ctx):
    """rt_pipe_*: frames submitted back to back (two in flight, host result
    buffers alternating) read back the same bits as a device frame graph of
    each soup; a frame's results are complete once its ticket is waited on;
    pageable buffers, outputs the pipe was created without and unsubmitted
    tickets are refused."""
    import torch
    from rtgpu import scenes
    from rtgpu._lib import RtError
    from rtgpu.api import LBVH, Frame, Pipe
    s = scenes.icosphere(freq=40)
    soups = [torch.from_numpy(s.frame(k)).pin_memory() for k in range(3)]
    cam = scenes.sphere_camera(320, 180)
    light = scenes.TORUS_LIGHT
    n, npx = soups[0].shape[0], cam.width * cam.height
    ref = []
    lb_d = LBVH(gpu_ctx, n, 16)
    dp = torch.empty((npx, 4), dtype=torch.int32, device="cuda")
    dv = torch.empty(npx, dtype=torch.uint8, device="cuda")
    dm = torch.empty((npx, 4), dtype=torch.int32, device="cuda")
    for k in range(3):
        fd = Frame(gpu_ctx, lb_d, soups[k].cuda(), cam, light, dp, dv, dm)
        fd.launch()
        gpu_ctx.check()
        ref.append((dp.cpu(), dv.cpu(), dm.cpu()))
        fd.close()
    lb = LBVH(gpu_ctx, n, 16)
    pipe = Pipe(gpu_ctx, lb, n, cam, light)
    outs = [(torch.empty((npx, 4), dtype=torch.int32).pin_memory(), torch.empty(npx, dtype=torch.uint8).pin_memory(),
             torch.empty((npx, 4), dtype=torch.int32).pin_memory()) for _ in range(2)]
    order = [0, 1, 2, 2, 0, 1, 1]  # soup of each submitted frame
    for k, f in enumerate(order):
        if k >= 2:
            pipe.wait(k - 2)
            hp, hv, hm = outs[k % 2]
            r = ref[order[k - 2]]
            assert torch.equal(hp, r[0]) and torch.equal(hv, r[1]) and torch.equal(hm, r[2]), f"frame {k - 2}"
            for t in outs[k % 2]:
                t.fill_(0x55)
        assert pipe.submit(soups[f], *outs[k % 2]) == k
    for k in (len(order) - 2, len(order) - 1):
        pipe.wait(k)
        r = ref[order[k]]
        hp, hv, hm = outs[k % 2]
        assert torch.equal(hp, r[0]) and torch.equal(hv, r[1]) and torch.equal(hm, r[2]), f"frame {k}"
    gpu_ctx.check()
    with pytest.raises(RtError):
        pipe.wait(len(order))  # not submitted
    with pytest.raises(RtError):
        pipe.submit(soups[0].clone(), *outs[0])  # pageable soup
    pipe.close()
    prim_only = Pipe(gpu_ctx, lb, n, cam, light, vis=False, mirror=False)
    with pytest.raises(RtError):
        prim_only.submit(soups[0], *outs[0])  # visibility / mirror outputs the pipe does not have
    t = prim_only.submit(soups[1], outs[1][0])
    prim_only.wait(t)
    assert torch.equal(outs[1][0], ref[1][0])
    prim_only.close()
    gpu_ctx.check()
