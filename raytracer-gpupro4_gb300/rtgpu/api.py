"""Python mirror of the reference's stage API over the C ABI.

  * ``LBVH``  -- the AccelerationStructure interface of the reference's LBVH
    (AccelerationStructures/AccelerationStructure.h:40-67, LBVH/LBVH.h:70-118):
    Build(), GetPtrToElements(), GetSizeOfElement(), GetNumberOfElements(),
    GetOrderedElementsIds(), WorldBound(), GetName().
  * ``StructureConstruction`` -- GPUBuildStructure(depth) of
    RayTracerCS/StructureConstruction.h:78-82.
  * ``RayTracer`` -- the per-frame stages of RayTracerCS::Render
    (RayTracerCS.cpp:241-311): primary rays, intersections, shadow and
    mirror rays, path-traced GI.

Every call goes through librtgb300.so (no CPU fallback).  PyTorch provides
device memory and the CUDA stream only.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L


def _dev_ptr(t: torch.Tensor) -> C.c_void_p:
    assert t.is_cuda and t.is_contiguous()
    return C.c_void_p(t.data_ptr())


def _host_ptr(a: np.ndarray) -> C.c_void_p:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


class Context:
    """rt_ctx bound to a CUDA device and torch's current stream on it."""

    def __init__(self, device: int = 0, stream: torch.cuda.Stream | None = None):
        self.device = device
        self.torch_device = torch.device("cuda", device)
        self.stream = stream if stream is not None else torch.cuda.current_stream(self.torch_device)
        h = C.c_void_p()
        L.check(L.lib().rt_ctx_create(device, C.c_void_p(self.stream.cuda_stream), C.byref(h)), None, "rt_ctx_create")
        self.h = h

    def close(self):
        if self.h:
            L.lib().rt_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self):
        """Synchronise and raise if a device-side error flag was set."""
        L.check(L.lib().rt_ctx_check(self.h), self.h, "rt_ctx_check")

    def sync(self):
        L.check(L.lib().rt_ctx_sync(self.h), self.h, "rt_ctx_sync")

    def set_tile_order(self, kinds: int):
        """Heavy-first tile order per trace kind (bit 0 primary, 1 shading, 2 generic rays)."""
        L.check(L.lib().rt_ctx_set_tile_order(self.h, int(kinds)), self.h, "rt_ctx_set_tile_order")

    DEFAULT_BUDGETS = (384, 768, 384)  # primary, shadow / mirror, generic rays

    def set_trace_budget(self, budget: int | None, kind: int | None = None):
        """Box + triangle tests a ray may spend in the per-lane traversal before
        it is handed to the warp-per-ray pass (0: never) for one trace kind
        (0 primary, 1 shadow / mirror, 2 generic rays) or all; None restores
        the defaults."""
        if budget is None:
            for k, b in enumerate(self.DEFAULT_BUDGETS):
                self.set_trace_budget(b, k)
            return
        if kind is None:
            L.check(L.lib().rt_ctx_set_trace_budget(self.h, int(budget)), self.h, "rt_ctx_set_trace_budget")
        else:
            L.check(L.lib().rt_ctx_set_trace_budget_kind(self.h, int(kind), int(budget)), self.h,
                    "rt_ctx_set_trace_budget_kind")

    DEFAULT_HEAVY_BLOCK = 2

    def set_heavy_block(self, kinds: int | None):
        """Trace kinds (bit 0 primary, 1 shadow / mirror, 2 generic rays) whose
        handed-over rays are traced a block per ray instead of a warp per
        ray; None restores the default."""
        k = self.DEFAULT_HEAVY_BLOCK if kinds is None else int(kinds)
        L.check(L.lib().rt_ctx_set_heavy_block(self.h, k), self.h, "rt_ctx_set_heavy_block")


class LBVH:
    """Device LBVH (heap layout, 1 << depth slots of 32 bytes)."""

    def __init__(self, ctx: Context, max_tris: int, depth: int = 20):
        self.ctx = ctx
        self.depth = depth
        h = C.c_void_p()
        L.check(L.lib().rt_lbvh_create(ctx.h, max_tris, depth, C.byref(h)), ctx.h, "rt_lbvh_create")
        self.h = h
        self._tris = None
        self.n = 0

    def close(self):
        if self.h:
            L.lib().rt_lbvh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # LBVH::Build (LBVH.cpp:488-632)
    def Build(self, tris, flags: int = 0) -> "LBVH":
        if isinstance(tris, torch.Tensor):
            t = tris.contiguous()
            assert t.dtype == torch.float32 and t.shape[-1] == 9
            self._tris = t  # the LBVH borrows the soup (as LBVH borrows Primitive**)
            L.check(L.lib().rt_lbvh_build(self.ctx.h, self.h, _dev_ptr(t), t.shape[0], flags), self.ctx.h,
                    "rt_lbvh_build")
            self.n = t.shape[0]
        else:
            a = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
            L.check(L.lib().rt_lbvh_build_host(self.ctx.h, self.h, _host_ptr(a), len(a), flags), self.ctx.h,
                    "rt_lbvh_build_host")
            self._tris = None
            self.n = len(a)
            self.ctx.sync()
        return self

    def Import(self, nodes: np.ndarray, ids: np.ndarray, tris: np.ndarray) -> "LBVH":
        """Uses a tree built elsewhere (RayTracerCS::SelectAccelerationStructure)."""
        nodes = np.ascontiguousarray(nodes).view(L.NODE_DTYPE)
        ids = np.ascontiguousarray(ids, np.uint32)
        tris = np.ascontiguousarray(tris, np.float32)
        assert len(nodes) == (1 << self.depth)
        L.check(L.lib().rt_lbvh_import_host(self.ctx.h, self.h, _host_ptr(nodes), _host_ptr(ids), _host_ptr(tris),
                                            len(tris)), self.ctx.h, "rt_lbvh_import_host")
        self.n = len(tris)
        self.ctx.sync()
        return self

    def view(self) -> L.LbvhView:
        v = L.LbvhView()
        L.check(L.lib().rt_lbvh_view_get(self.h, C.byref(v)), self.ctx.h, "rt_lbvh_view_get")
        return v

    def GetName(self) -> str:
        return "LBVH"

    def GetNumberOfElements(self) -> int:
        return 1 << self.depth

    def GetSizeOfElement(self) -> int:
        return 32

    def download(self, nodes=True, ids=True, keys=False):
        hn = np.zeros(1 << self.depth, L.NODE_DTYPE) if nodes else None
        hi = np.zeros(self.n, np.uint32) if ids else None
        hk = np.zeros(self.n, np.uint32) if keys else None
        L.check(L.lib().rt_lbvh_download(self.ctx.h, self.h, _host_ptr(hn) if nodes else None,
                                         _host_ptr(hi) if ids else None, _host_ptr(hk) if keys else None),
                self.ctx.h, "rt_lbvh_download")
        return hn, hi, hk

    def GetPtrToElements(self) -> np.ndarray:
        return self.download(True, False, False)[0]

    def GetOrderedElementsIds(self) -> np.ndarray:
        return self.download(False, True, False)[1]

    def keys(self) -> np.ndarray:
        return self.download(False, False, True)[2]

    def WorldBound(self) -> np.ndarray:
        out = (C.c_float * 6)()
        L.check(L.lib().rt_lbvh_world_bound(self.ctx.h, self.h, out), self.ctx.h, "rt_lbvh_world_bound")
        return np.array(out[:], np.float32)


class BVH:
    """The reference's SAH BVH on the device (rt_bvh): a flattened
    LinearBVHNode array (bvh.cpp:272-293, NODE_DTYPE layout) with its
    ordered primitive ids, imported from the reference's CPU build and traced
    as BVH_IntersectP (BVH.hlsl:124-217).  RayTracer's primary,
    shadow_mirror and rays accept it in place of an LBVH."""

    def __init__(self, ctx: Context, max_nodes: int, max_tris: int):
        self.ctx = ctx
        h = C.c_void_p()
        L.check(L.lib().rt_bvh_create(ctx.h, max_nodes, max_tris, C.byref(h)), ctx.h, "rt_bvh_create")
        self.h = h

    def close(self):
        if self.h:
            L.lib().rt_bvh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def Import(self, nodes: np.ndarray, ids: np.ndarray, tris: np.ndarray) -> "BVH":
        nodes = np.ascontiguousarray(nodes).view(L.NODE_DTYPE)
        ids = np.ascontiguousarray(ids, np.uint32)
        tris = np.ascontiguousarray(tris, np.float32)
        L.check(L.lib().rt_bvh_import_host(self.ctx.h, self.h, _host_ptr(nodes), len(nodes), _host_ptr(ids),
                                           _host_ptr(tris), len(tris)), self.ctx.h, "rt_bvh_import_host")
        return self


class StructureConstruction:
    """GPUBuildStructure(depth) over a device soup (StructureConstruction.cpp:86-131)."""

    def __init__(self, ctx: Context, max_tris: int, depth: int):
        self.lbvh = LBVH(ctx, max_tris, depth)

    def GPUBuildStructure(self, tris) -> LBVH:
        return self.lbvh.Build(tris)


class RadixSort:
    """The build's sort stage on its own (rt_radix_sort): a stable sort of
    (key, value) uint32 pairs by key, in place, in place of the reference's
    BitonicSort::GPUSort / RadixSort::Sort (BitonicSort.cpp:56-117,
    RadixSort.cpp:46-74).  The scratch is a device tensor kept between calls
    and grown when a larger n arrives."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self._scratch = None

    def scratch(self, n: int) -> torch.Tensor:
        need = int(L.lib().rt_radix_sort_scratch_bytes(n))
        if self._scratch is None or self._scratch.numel() * 4 < need:
            self._scratch = torch.empty((need + 3) // 4, dtype=torch.int32, device=self.ctx.torch_device)
        return self._scratch

    def Sort(self, keys: torch.Tensor, values: torch.Tensor) -> None:
        assert keys.dtype in (torch.int32, torch.uint32) and values.dtype in (torch.int32, torch.uint32)
        assert keys.numel() == values.numel()
        n = keys.numel()
        sc = self.scratch(n)
        L.check(L.lib().rt_radix_sort(self.ctx.h, _dev_ptr(keys), _dev_ptr(values), n, _dev_ptr(sc), sc.numel() * 4),
                self.ctx.h, "rt_radix_sort")

    def stall_test(self, keys: torch.Tensor, values: torch.Tensor, spin_limit: int) -> int:
        """Runs rt_radix_sort_stall_test; returns its status (the look-back
        timeout itself is reported by Context.check)."""
        n = keys.numel()
        sc = self.scratch(n)
        return L.lib().rt_radix_sort_stall_test(self.ctx.h, _dev_ptr(keys), _dev_ptr(values), n, _dev_ptr(sc),
                                                sc.numel() * 4, spin_limit)


def hits_to_numpy(t: torch.Tensor) -> np.ndarray:
    return t.cpu().numpy().view(L.HIT_DTYPE).reshape(-1)


class RayTracer:
    """Per-frame stages over an LBVH (RayTracerCS::Render)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def _alloc_hits(self, n: int) -> torch.Tensor:
        return torch.empty((n, 4), dtype=torch.int32, device=self.ctx.torch_device)

    def primary(self, lbvh: LBVH, cam: L.Camera, stats: bool = False, out: torch.Tensor | None = None):
        npx = cam.width * cam.height
        hits = out if out is not None else self._alloc_hits(npx)
        st = torch.empty((npx, 2), dtype=torch.int32, device=self.ctx.torch_device) if stats else None
        fn = L.lib().rt_bvh_trace_primary if isinstance(lbvh, BVH) else L.lib().rt_trace_primary
        L.check(fn(self.ctx.h, lbvh.h, C.byref(cam), _dev_ptr(hits), _dev_ptr(st) if stats else None), self.ctx.h,
                "rt_trace_primary")
        return (hits, st) if stats else hits

    def shadow_mirror(self, lbvh: LBVH, cam: L.Camera, light, primary: torch.Tensor, stats: bool = False,
                      vis: torch.Tensor | None = None, mirror: torch.Tensor | None = None,
                      with_mirror: bool = True):
        """Shadow rays (vis codes) and, unless with_mirror is False, mirror rays."""
        npx = cam.width * cam.height
        vis = vis if vis is not None else torch.empty(npx, dtype=torch.uint8, device=self.ctx.torch_device)
        if with_mirror:
            mirror = mirror if mirror is not None else self._alloc_hits(npx)
        else:
            mirror = None
        ss = torch.empty((npx, 2), dtype=torch.int32, device=self.ctx.torch_device) if stats else None
        ms = torch.empty((npx, 2), dtype=torch.int32, device=self.ctx.torch_device) if stats and with_mirror else None
        lf = (C.c_float * 3)(*light)
        fn = L.lib().rt_bvh_trace_shadow_mirror if isinstance(lbvh, BVH) else L.lib().rt_trace_shadow_mirror
        L.check(fn(self.ctx.h, lbvh.h, C.byref(cam), lf, _dev_ptr(primary), _dev_ptr(vis),
                   _dev_ptr(mirror) if mirror is not None else None, _dev_ptr(ss) if stats else None,
                   _dev_ptr(ms) if ms is not None else None), self.ctx.h, "rt_trace_shadow_mirror")
        return (vis, mirror, ss, ms) if stats else (vis, mirror)

    def primary_leaves(self, lbvh: LBVH, cam: L.Camera, stats: bool = False, out: torch.Tensor | None = None,
                       leaves: torch.Tensor | None = None):
        """Primary hits and the heap leaf of each hit (the reference's iRoot,
        rt_trace_primary_leaves).  Returns (hits, leaves[, stats])."""
        npx = cam.width * cam.height
        hits = out if out is not None else self._alloc_hits(npx)
        if leaves is None:
            leaves = torch.empty(npx, dtype=torch.int32, device=self.ctx.torch_device)
        st = torch.empty((npx, 2), dtype=torch.int32, device=self.ctx.torch_device) if stats else None
        L.check(L.lib().rt_trace_primary_leaves(self.ctx.h, lbvh.h, C.byref(cam), _dev_ptr(hits), _dev_ptr(leaves),
                                                _dev_ptr(st) if stats else None), self.ctx.h,
                "rt_trace_primary_leaves")
        return (hits, leaves, st) if stats else (hits, leaves)

    def shadow_mirror_from(self, lbvh: LBVH, cam: L.Camera, light, primary: torch.Tensor, leaves: torch.Tensor,
                           stats: bool = False, vis: torch.Tensor | None = None, mirror: torch.Tensor | None = None,
                           mirror_leaves: torch.Tensor | None = None, with_mirror: bool = True):
        """Shading rays started at the primary leaves (rt_trace_shadow_mirror_from).
        Returns (vis, mirror, mirror_leaves[, shadow_stats, mirror_stats]);
        with_mirror=False traces the shadow rays only (mirror outputs None)."""
        npx = cam.width * cam.height
        dev = self.ctx.torch_device
        vis = vis if vis is not None else torch.empty(npx, dtype=torch.uint8, device=dev)
        if with_mirror:
            mirror = mirror if mirror is not None else self._alloc_hits(npx)
            ml = mirror_leaves if mirror_leaves is not None else torch.empty(npx, dtype=torch.int32, device=dev)
        else:
            mirror = ml = None
        ss = torch.empty((npx, 2), dtype=torch.int32, device=dev) if stats else None
        ms = torch.empty((npx, 2), dtype=torch.int32, device=dev) if stats and with_mirror else None
        lf = (C.c_float * 3)(*light)
        opt = lambda t: _dev_ptr(t) if t is not None else None  # noqa: E731
        L.check(L.lib().rt_trace_shadow_mirror_from(self.ctx.h, lbvh.h, C.byref(cam), lf, _dev_ptr(primary),
                                                    _dev_ptr(leaves), _dev_ptr(vis), opt(mirror), opt(ml), opt(ss),
                                                    opt(ms)),
                self.ctx.h, "rt_trace_shadow_mirror_from")
        return (vis, mirror, ml, ss, ms) if stats else (vis, mirror, ml)

    def rays_from(self, lbvh: LBVH, rays: torch.Tensor, starts: torch.Tensor | None, any_hit: bool = False,
                  stats: bool = False):
        """rt_trace_rays_from: each ray's walk starts at heap node starts[i]
        (None: the root).  Returns (hits, leaves[, stats])."""
        n = rays.shape[0]
        hits = self._alloc_hits(n)
        leaves = torch.empty(n, dtype=torch.int32, device=self.ctx.torch_device)
        st = torch.empty((n, 2), dtype=torch.int32, device=self.ctx.torch_device) if stats else None
        L.check(L.lib().rt_trace_rays_from(self.ctx.h, lbvh.h, _dev_ptr(rays), n, int(any_hit),
                                           _dev_ptr(starts) if starts is not None else None, _dev_ptr(hits),
                                           _dev_ptr(leaves), _dev_ptr(st) if stats else None), self.ctx.h,
                "rt_trace_rays_from")
        return (hits, leaves, st) if stats else (hits, leaves)

    def whitted(self, lbvh: LBVH, cam: L.Camera, light, materials, material_ids: torch.Tensor | None = None,
                normals: torch.Tensor | None = None, bounces: int = 0, shadows: bool = True, phong: bool = False,
                gloss_mapping: bool = False, env_mapping: int = -1, env_color=(1.0, 1.0, 1.0), seed: int = 0,
                result: bool = True):
        """The colour stage with its bounce loop (rt_render_whitted).
        materials: (m, 14) float32 rows (ambient 4, diffuse 4, specular 4,
        shininess, alpha), host or device; material_ids: (n,) int32 device
        tensor; normals: (n, 9) float32 device tensor (Phong).  Returns
        (accum, result) as (w*h, 4) float32 device tensors (result None when
        result=False)."""
        dev = self.ctx.torch_device
        mats = torch.as_tensor(np.ascontiguousarray(materials, np.float32).reshape(-1, 14) if not isinstance(
            materials, torch.Tensor) else materials, device=dev).to(torch.float32).contiguous()
        npx = cam.width * cam.height
        acc = torch.empty((npx, 4), dtype=torch.float32, device=dev)
        res = torch.empty((npx, 4), dtype=torch.float32, device=dev) if result else None
        p = L.ShadeParams(bounces, int(shadows), int(phong), int(gloss_mapping), env_mapping,
                          (C.c_float * 3)(*env_color), seed)
        lf = (C.c_float * 3)(*light)
        L.check(L.lib().rt_render_whitted(self.ctx.h, lbvh.h, C.byref(cam), lf, C.byref(p),
                                          _dev_ptr(material_ids) if material_ids is not None else None,
                                          _dev_ptr(mats), mats.shape[0],
                                          _dev_ptr(normals) if normals is not None else None, _dev_ptr(acc),
                                          _dev_ptr(res) if res is not None else None), self.ctx.h,
                "rt_render_whitted")
        return acc, res

    def frame_shader_order(self, lbvh: LBVH, cam: L.Camera, light, stats: bool = False, with_mirror: bool = True):
        """rt_trace_frame_shader_order: primary, shadow and mirror rays in the
        reference shader's own walk order and tie rule.  Returns (primary, vis,
        mirror[, primary_stats, shadow_stats, mirror_stats]); mirror outputs are
        None with with_mirror=False."""
        npx = cam.width * cam.height
        dev = self.ctx.torch_device
        prim = self._alloc_hits(npx)
        vis = torch.empty(npx, dtype=torch.uint8, device=dev)
        mirror = self._alloc_hits(npx) if with_mirror else None
        st = [torch.zeros((npx, 2), dtype=torch.int32, device=dev) for _ in range(3)] if stats else [None] * 3
        if not with_mirror:
            st[2] = None
        lf = (C.c_float * 3)(*light)
        opt = lambda t: _dev_ptr(t) if t is not None else None  # noqa: E731
        L.check(L.lib().rt_trace_frame_shader_order(self.ctx.h, lbvh.h, C.byref(cam), lf, _dev_ptr(prim),
                                                    _dev_ptr(vis), opt(mirror), opt(st[0]), opt(st[1]), opt(st[2])),
                self.ctx.h, "rt_trace_frame_shader_order")
        return (prim, vis, mirror, *st) if stats else (prim, vis, mirror)

    def rays(self, lbvh: LBVH, rays: torch.Tensor, any_hit: bool = False, stats: bool = False):
        """rays: (n, 8) float32 device tensor laid out as rt_ray {o, exclude(int bits), d, tmax}."""
        n = rays.shape[0]
        hits = self._alloc_hits(n)
        st = torch.empty((n, 2), dtype=torch.int32, device=self.ctx.torch_device) if stats else None
        fn = L.lib().rt_bvh_trace_rays if isinstance(lbvh, BVH) else L.lib().rt_trace_rays
        L.check(fn(self.ctx.h, lbvh.h, _dev_ptr(rays), n, int(any_hit), _dev_ptr(hits),
                   _dev_ptr(st) if stats else None), self.ctx.h, "rt_trace_rays")
        return (hits, st) if stats else hits

    def render_frame_host(self, lbvh: LBVH, tris: np.ndarray, cam: L.Camera, light, primary: np.ndarray,
                          vis: np.ndarray, mirror: np.ndarray, wait: bool = True):
        """One frame from and to host buffers; wait=False queues it on the
        context stream (rt_render_frame_host_async; the buffers stay in use
        until Context.sync)."""
        lf = (C.c_float * 3)(*light)
        fn = L.lib().rt_render_frame_host if wait else L.lib().rt_render_frame_host_async
        L.check(fn(self.ctx.h, lbvh.h, _host_ptr(tris), len(tris), C.byref(cam), lf, _host_ptr(primary),
                   _host_ptr(vis), _host_ptr(mirror)), self.ctx.h, "rt_render_frame_host")

    def pathtrace(self, lbvh: LBVH, albedo: torch.Tensor, emission: torch.Tensor, cam: L.Camera, spp: int,
                  bounces: int, seed: int, sky=(1.0, 1.0, 1.0), out: torch.Tensor | None = None,
                  first_sample: int = 0) -> torch.Tensor:
        """Samples first_sample .. first_sample + spp - 1 of every pixel; with
        first_sample > 0, `out` holds the mean of the earlier samples and the
        new ones are blended into it (progressive accumulation)."""
        if first_sample > 0 and out is None:
            raise ValueError("first_sample > 0 continues an image: pass it as out")
        img = out if out is not None else torch.empty((cam.height * cam.width, 4), dtype=torch.float32,
                                                      device=self.ctx.torch_device)
        p = L.PtParams(spp, bounces, seed, (C.c_float * 3)(*sky), first_sample)
        L.check(L.lib().rt_pathtrace(self.ctx.h, lbvh.h, _dev_ptr(albedo), _dev_ptr(emission), C.byref(cam),
                                     C.byref(p), _dev_ptr(img)), self.ctx.h, "rt_pathtrace")
        return img

    def pathtrace_counted(self, lbvh: LBVH, albedo: torch.Tensor, emission: torch.Tensor, cam: L.Camera, spp: int,
                          bounces: int, seed: int, sky=(1.0, 1.0, 1.0)):
        """rt_pathtrace_counted: (image, {segments, box_tests, tri_tests, hits})."""
        img = torch.empty((cam.height * cam.width, 4), dtype=torch.float32, device=self.ctx.torch_device)
        cnt = torch.zeros(4, dtype=torch.int64, device=self.ctx.torch_device)
        p = L.PtParams(spp, bounces, seed, (C.c_float * 3)(*sky), 0)
        L.check(L.lib().rt_pathtrace_counted(self.ctx.h, lbvh.h, _dev_ptr(albedo), _dev_ptr(emission), C.byref(cam),
                                             C.byref(p), _dev_ptr(img), _dev_ptr(cnt)), self.ctx.h,
                "rt_pathtrace_counted")
        c = cnt.cpu().tolist()
        return img, {"segments": c[0], "box_tests": c[1], "tri_tests": c[2], "hits": c[3]}

    def pathtrace_adjoint(self, lbvh: LBVH, albedo: torch.Tensor, emission: torch.Tensor, cam: L.Camera, spp: int,
                          bounces: int, seed: int, d_image: torch.Tensor, sky=(1.0, 1.0, 1.0), first_sample: int = 0):
        d_alb = torch.zeros_like(albedo)
        d_le = torch.zeros(3, dtype=torch.float32, device=self.ctx.torch_device)
        p = L.PtParams(spp, bounces, seed, (C.c_float * 3)(*sky), first_sample)
        L.check(L.lib().rt_pathtrace_adjoint(self.ctx.h, lbvh.h, _dev_ptr(albedo), _dev_ptr(emission), C.byref(cam),
                                             C.byref(p), _dev_ptr(d_image.contiguous()), _dev_ptr(d_alb),
                                             _dev_ptr(d_le)), self.ctx.h, "rt_pathtrace_adjoint")
        return d_alb, d_le


class Frame:
    """One frame of the dynamic path (rebuild + primary + shadow + mirror)
    captured as a CUDA graph (rt_frame_capture); launch() replays it.  With
    host=True the tensors are pinned host tensors and the graph also holds
    the soup upload and the result read-back (rt_frame_capture_host)."""

    def __init__(self, ctx: Context, lbvh: LBVH, tris: torch.Tensor, cam: L.Camera, light, primary: torch.Tensor,
                 vis: torch.Tensor | None, mirror: torch.Tensor | None, flags: int = 0, host: bool = False):
        self.ctx = ctx
        self._keep = (tris, primary, vis, mirror)
        h = C.c_void_p()
        lf = (C.c_float * 3)(*light)
        fn = L.lib().rt_frame_capture_host if host else L.lib().rt_frame_capture

        def ptr(t):
            if t is None:
                return None
            assert t.is_contiguous() and t.is_cuda != host  # host buffers: rt_frame_capture_host checks pinning
            return C.c_void_p(t.data_ptr())

        L.check(fn(ctx.h, lbvh.h, ptr(tris), tris.shape[0], flags, C.byref(cam), lf, ptr(primary), ptr(vis),
                   ptr(mirror), C.byref(h)), ctx.h, "rt_frame_capture_host" if host else "rt_frame_capture")
        self.h = h
        lbvh.n = tris.shape[0]
        lbvh._tris = tris

    def launch(self):
        L.check(L.lib().rt_frame_launch(self.ctx.h, self.h), self.ctx.h, "rt_frame_launch")

    @property
    def nodes(self) -> int:
        return int(L.lib().rt_frame_node_count(self.h))

    def close(self):
        if self.h:
            L.lib().rt_frame_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Pipe:
    """Double-buffered host frames (rt_pipe_*): submit() queues the upload of
    a pinned host soup, the captured rebuild + trace and the read-back into
    pinned host tensors; frames' kernels run one after another on the
    context stream while their copies overlap them.  wait(ticket) returns
    once that frame's host results are complete."""

    def __init__(self, ctx: Context, lbvh: LBVH, n: int, cam: L.Camera, light, vis: bool = True,
                 mirror: bool = True, flags: int = 0):
        self.ctx = ctx
        self.lbvh = lbvh
        h = C.c_void_p()
        lf = (C.c_float * 3)(*light)
        L.check(L.lib().rt_pipe_create(ctx.h, lbvh.h, n, flags, C.byref(cam), lf, int(vis), int(mirror), C.byref(h)),
                ctx.h, "rt_pipe_create")
        self.h = h
        self._keep = {}
        lbvh.n = n

    def submit(self, tris: torch.Tensor, primary: torch.Tensor | None, vis: torch.Tensor | None = None,
               mirror: torch.Tensor | None = None) -> int:
        def ptr(t):
            if t is None:
                return None
            assert t.is_contiguous() and not t.is_cuda  # rt_pipe_submit checks that they are page-locked
            return C.c_void_p(t.data_ptr())

        ticket = C.c_uint64()
        L.check(L.lib().rt_pipe_submit(self.h, ptr(tris), ptr(primary), ptr(vis), ptr(mirror), C.byref(ticket)),
                self.ctx.h, "rt_pipe_submit")
        self._keep[ticket.value & 1] = (tris, primary, vis, mirror)
        return ticket.value

    def wait(self, ticket: int):
        L.check(L.lib().rt_pipe_wait(self.h, ticket), self.ctx.h, "rt_pipe_wait")

    def close(self):
        if self.h:
            L.lib().rt_pipe_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many scenes rebuilt and traced together (rt_batch_*): one pass of the
    build kernels over the concatenated soups, one persistent trace kernel
    over (scene, tile) work items.  Scene s's tree equals LBVH.Build of its
    triangles alone, with scene-local ids."""

    def __init__(self, ctx: Context, tri_counts, depth: int = 20):
        self.ctx = ctx
        self.counts = np.ascontiguousarray(tri_counts, np.uint32)
        self.offsets = np.concatenate([[0], np.cumsum(self.counts, dtype=np.int64)])
        self.depth = depth
        self.total = int(self.offsets[-1])
        h = C.c_void_p()
        L.check(L.lib().rt_batch_create(ctx.h, len(self.counts), _host_ptr(self.counts), depth, C.byref(h)), ctx.h,
                "rt_batch_create")
        self.h = h
        self._keep = ()
        self.width = self.height = 0

    @property
    def n_scenes(self) -> int:
        return len(self.counts)

    def close(self):
        if self.h:
            L.lib().rt_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build(self, tris: torch.Tensor, flags: int = 0) -> "Batch":
        t = tris.contiguous()
        assert t.dtype == torch.float32 and t.shape == (self.total, 9)
        self._keep = (t,)
        L.check(L.lib().rt_batch_build(self.ctx.h, self.h, _dev_ptr(t), flags), self.ctx.h, "rt_batch_build")
        return self

    def view(self, scene: int) -> L.LbvhView:
        v = L.LbvhView()
        L.check(L.lib().rt_batch_view_get(self.h, scene, C.byref(v)), self.ctx.h, "rt_batch_view_get")
        return v

    def download(self, scene: int):
        """(nodes, ids, keys) of one scene's tree, copied to the host."""
        n = int(self.counts[scene])
        nodes = np.zeros(1 << self.depth, L.NODE_DTYPE)
        ids = np.zeros(n, np.uint32)
        keys = np.zeros(n, np.uint32)
        L.check(L.lib().rt_batch_download(self.ctx.h, self.h, scene, _host_ptr(nodes), _host_ptr(ids),
                                          _host_ptr(keys)), self.ctx.h, "rt_batch_download")
        return nodes, ids, keys

    def set_views(self, cams, lights) -> "Batch":
        cams = list(cams)
        assert len(cams) == self.n_scenes
        arr = (L.Camera * len(cams))(*cams)
        lt = np.ascontiguousarray(np.asarray(lights, np.float32).reshape(self.n_scenes, 3))
        L.check(L.lib().rt_batch_set_views(self.ctx.h, self.h, C.cast(arr, C.c_void_p), _host_ptr(lt)), self.ctx.h,
                "rt_batch_set_views")
        self.width, self.height = cams[0].width, cams[0].height
        return self

    def alloc_outputs(self, shadow: bool = True):
        px = self.n_scenes * self.width * self.height
        hits = torch.empty((px, 4), dtype=torch.int32, device=self.ctx.torch_device)
        vis = torch.empty(px, dtype=torch.uint8, device=self.ctx.torch_device) if shadow else None
        return hits, vis

    def trace(self, hits: torch.Tensor, vis: torch.Tensor | None = None) -> None:
        L.check(L.lib().rt_batch_trace(self.ctx.h, self.h, _dev_ptr(hits), _dev_ptr(vis) if vis is not None else None),
                self.ctx.h, "rt_batch_trace")

    @property
    def tuning(self) -> dict:
        t = L.BatchTuning()
        L.check(L.lib().rt_batch_get_tuning(self.h, C.byref(t)), self.ctx.h, "rt_batch_get_tuning")
        return {"threads": t.threads, "blocks_per_sm": t.blocks_per_sm, "grab": t.grab, "order": t.order}

    @tuning.setter
    def tuning(self, cfg: dict) -> None:
        t = L.BatchTuning(int(cfg["threads"]), int(cfg.get("blocks_per_sm", 0)), int(cfg["grab"]), int(cfg["order"]))
        L.check(L.lib().rt_batch_set_tuning(self.ctx.h, self.h, C.byref(t)), self.ctx.h, "rt_batch_set_tuning")


class BatchFrame:
    """One batched frame (build + trace) captured as a CUDA graph."""

    def __init__(self, ctx: Context, batch: Batch, tris: torch.Tensor, hits: torch.Tensor,
                 vis: torch.Tensor | None, flags: int = 0):
        self.ctx = ctx
        t = tris.contiguous()
        self._keep = (t, hits, vis)
        h = C.c_void_p()
        L.check(L.lib().rt_batch_frame_capture(ctx.h, batch.h, _dev_ptr(t), flags, _dev_ptr(hits),
                                               _dev_ptr(vis) if vis is not None else None, C.byref(h)),
                ctx.h, "rt_batch_frame_capture")
        self.h = h
        batch._keep = (t,)

    def launch(self):
        L.check(L.lib().rt_frame_launch(self.ctx.h, self.h), self.ctx.h, "rt_frame_launch")

    @property
    def nodes(self) -> int:
        return int(L.lib().rt_frame_node_count(self.h))

    def close(self):
        if self.h:
            L.lib().rt_frame_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rays_tensor(o, d, tmax, exclude, device) -> torch.Tensor:
    """Packs rays into the rt_ray layout as an (n, 8) float32 tensor."""
    n = len(d)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = o
    r[:, 3] = np.asarray(exclude, np.int32).view(np.float32) if np.ndim(exclude) else np.int32(exclude).view(np.float32)
    r[:, 4:7] = d
    r[:, 7] = tmax
    return torch.from_numpy(r).to(device)
