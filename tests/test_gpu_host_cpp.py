"""The C++ drop-in stage classes (host/rt_stages.h: LBVHGpu, StructureConstruction,
RayTracerCS, FramePipeline) driven by host/rt_frame_demo, against the Python
binding of the same C ABI and the oracle."""
import json
import subprocess

import numpy as np
import pytest
from bitcmp import same_bits

pytestmark = pytest.mark.gpu


def test_cpp_stage_classes(gpu_ctx, oracle_mod, tmp_path):
    import torch
    from rtgpu import build, scenes
    from rtgpu._lib import HIT_DTYPE
    from rtgpu.api import LBVH, RayTracer, hits_to_numpy
    build.build_host()
    assert build.DEMO.exists()
    tris = scenes.torus(96, 48)
    cam = scenes.torus_camera(200, 120)
    light = scenes.TORUS_LIGHT
    depth = 16
    tris.tofile(tmp_path / "soup.f32")
    np.array([*cam.eye, *cam.right, *cam.up, *cam.fwd, cam.tan_half_fovy], np.float32).tofile(tmp_path / "cam.f32")
    out = tmp_path / "frame"
    r = subprocess.run([str(build.DEMO), str(tmp_path / "soup.f32"), str(len(tris)), str(tmp_path / "cam.f32"),
                        str(cam.width), str(cam.height), *map(str, light), str(depth), "3", str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    summary = json.loads(r.stdout.strip().splitlines()[-1])
    assert summary["name"] == "LBVH" and summary["elements"] == 1 << depth and summary["element_size"] == 32
    assert summary["world_bound_ok"] and summary["samples"] == 3
    prim = np.fromfile(str(out) + ".primary", HIT_DTYPE)
    vis = np.fromfile(str(out) + ".vis", np.uint8)
    mir = np.fromfile(str(out) + ".mirror", HIT_DTYPE)
    # the colour stage and progressive GI through RayTracerCS (RenderColor, RenderGI x 2)
    lbc = LBVH(gpu_ctx, len(tris), depth).Build(torch.from_numpy(tris).cuda())
    rtc = RayTracer(gpu_ctx)
    mats = np.array([[1.5, 0, 0, 0, 0.7, 0.4, 0.2, 1, 0.5, 0.5, 0.5, 1, 0.049, 0.6]], np.float32)
    acc, _ = rtc.whitted(lbc, cam, light, mats, bounces=1, shadows=True, env_mapping=-1, env_color=(0.2, 0.3, 0.4),
                         seed=7)
    assert same_bits(np.fromfile(str(out) + ".color", np.float32), acc.cpu().numpy().reshape(-1))
    albedo = torch.full((len(tris), 3), 0.6, dtype=torch.float32, device="cuda")
    emission = torch.zeros((len(tris), 3), dtype=torch.float32, device="cuda")
    emission[:64] = 2.0
    gi = rtc.pathtrace(lbc, albedo, emission, cam, 4, 2, 11)  # one call of 4 samples
    assert same_bits(np.fromfile(str(out) + ".gi", np.float32), gi.cpu().numpy().reshape(-1))
    # the same frames streamed from pinned host memory through FramePipeline (rt_pipe_*)
    assert same_bits(np.fromfile(str(out) + ".pipe.primary", HIT_DTYPE), prim)
    assert np.array_equal(np.fromfile(str(out) + ".pipe.vis", np.uint8), vis)
    assert same_bits(np.fromfile(str(out) + ".pipe.mirror", HIT_DTYPE), mir)
    # same frame through the Python binding
    lb = LBVH(gpu_ctx, len(tris), depth).Build(torch.from_numpy(tris).cuda())
    rt = RayTracer(gpu_ctx)
    hits, leaves = rt.primary_leaves(lb, cam)
    pv, pm, _ = rt.shadow_mirror_from(lb, cam, light, hits, leaves)
    assert same_bits(prim, hits_to_numpy(hits))
    assert np.array_equal(vis, pv.cpu().numpy())
    assert same_bits(mir, hits_to_numpy(pm))
    assert summary["primary_hits"] == int((prim["id"] >= 0).sum())
    # single-ray IntersectP through the AccelerationStructure interface
    f = np.float32
    t0 = tris[0]
    c = np.array([(f(t0[k] + t0[3 + k]) + t0[6 + k]) / f(3.0) for k in range(3)], f)
    eye = np.array(cam.eye, f)
    nodes, ids, _, _ = oracle_mod.lbvh_build(tris, depth)
    ray = oracle_mod.rays_array(eye, (c - eye)[None], 1e16, -1)
    oh = oracle_mod.trace(nodes, depth, ids, tris, ray)
    assert summary["single_ray_id"] == int(oh["id"][0])


def test_cpp_model_input(gpu_ctx, oracle_mod, tmp_path):
    """rt_frame_demo with a model file: Model (Model::LoadFile + Scale)
    feeds the same stage classes; the primary hits match the oracle traced
    over the reference loader's soup of that file."""
    from conftest import GOLDEN
    from rtgpu import build, scenes
    from rtgpu._lib import HIT_DTYPE
    build.build_host()
    soup = np.load(GOLDEN / "models" / "expected.npz")["torus_OBJ__soup"]
    cam = scenes.look_at((0.3, -1.2, 0.9), (0.0, 0.0, 0.0), width=160, height=120)
    np.array([*cam.eye, *cam.right, *cam.up, *cam.fwd, cam.tan_half_fovy], np.float32).tofile(tmp_path / "cam.f32")
    depth = 12
    r = subprocess.run([str(build.DEMO), str(GOLDEN / "models" / "torus.OBJ"), "0", str(tmp_path / "cam.f32"),
                        str(cam.width), str(cam.height), "1", "1", "1", str(depth), "1", str(tmp_path / "m")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    prim = np.fromfile(str(tmp_path / "m") + ".primary", HIT_DTYPE)
    nodes, ids, _, _ = oracle_mod.lbvh_build(soup, depth)
    oh = oracle_mod.trace(nodes, depth, ids, soup, oracle_mod.primary_rays(cam))
    assert (oh["id"] >= 0).sum() > 1000
    assert np.array_equal(prim["id"], oh["id"]) and same_bits(prim["t"], oh["t"])
