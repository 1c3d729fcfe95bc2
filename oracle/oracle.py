"""Python binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Wraps
  * oracle/_build/liboracle.so: the C restatement in rt_oracle.c, and
  * oracle/_ref/libref.so: the reference's own CPU LBVH / BVH code
    (AccelerationStructures/LBVH/LBVH.cpp, BVH/bvh.cpp), built by
    ref/build_ref.sh where the reference checkout is present.
Only tests/, the smoke check and bench.py's CPU-baseline leg import this
module; the product path never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref.so"

NODE_DTYPE = np.dtype([("min", "<f4", (3,)), ("max", "<f4", (3,)), ("prim_count", "<i4"), ("prim_pos", "<i4")])
HIT_DTYPE = np.dtype([("id", "<i4"), ("u", "<f4"), ("v", "<f4"), ("t", "<f4")])
SENTINEL = -2147483647


class OrCamera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("right", C.c_float * 3), ("up", C.c_float * 3), ("fwd", C.c_float * 3),
                ("tan_half_fovy", C.c_float), ("width", C.c_uint32), ("height", C.c_uint32)]


class OrPtParams(C.Structure):
    _fields_ = [("spp", C.c_uint32), ("bounces", C.c_uint32), ("seed", C.c_uint64), ("sky", C.c_float * 3),
                ("first_sample", C.c_uint32), ("x0", C.c_uint32), ("y0", C.c_uint32), ("win_w", C.c_uint32),
                ("win_h", C.c_uint32)]


def _pt_params(spp, bounces, seed, sky, first_sample, window):
    x0, y0, w, h = window if window is not None else (0, 0, 0, 0)
    return OrPtParams(spp, bounces, seed, (C.c_float * 3)(*sky), first_sample, x0, y0, w, h)


class OrShadeParams(C.Structure):
    _fields_ = [("bounces", C.c_uint32), ("shadows", C.c_int32), ("phong", C.c_int32), ("gloss_mapping", C.c_int32),
                ("env_mapping", C.c_int32), ("env_color", C.c_float * 3), ("seed", C.c_uint32)]


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return ORACLE_LIB


def build_reference() -> Path | None:
    """Compiles the reference CPU code when its sources are present.  The
    recipe (ref/build_ref.sh) locates the checkout (RT_REFERENCE_DIR) and
    builds nothing where it is absent; None is returned then."""
    srcs = [HERE / "ref" / "ref_shim.cpp", HERE / "ref" / "build_ref.sh"]
    if REF_LIB.exists() and all(s.stat().st_mtime <= REF_LIB.stat().st_mtime for s in srcs):
        return REF_LIB
    subprocess.run(["bash", str(HERE / "ref" / "build_ref.sh")], check=True, capture_output=True)
    return REF_LIB if REF_LIB.exists() else None


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def to_or_camera(cam) -> OrCamera:
    o = OrCamera()
    for f in ("eye", "right", "up", "fwd"):
        src, dst = getattr(cam, f), getattr(o, f)
        for c in range(3):
            dst[c] = src[c]
    o.tan_half_fovy = cam.tan_half_fovy
    o.width = cam.width
    o.height = cam.height
    return o


_olib = None
_rlib = None


def olib() -> C.CDLL:
    global _olib
    if _olib is None:
        if not ORACLE_LIB.exists():
            build_oracle()
        L = C.CDLL(str(ORACLE_LIB))
        vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int
        L.or_scene_bounds.argtypes = [vp, u32, vp]
        L.or_morton.argtypes = [vp, u32, vp, vp]
        L.or_sort_pairs.argtypes = [vp, vp, u32]
        L.or_lbvh_emit.argtypes = [vp, vp, vp, u32, u32, vp, vp]
        L.or_lbvh_build.argtypes = [vp, u32, u32, vp, vp, vp, vp]
        L.or_trace.argtypes = [vp, u32, vp, vp, vp, u32, vp, vp, i32, i32]
        L.or_trace_from.argtypes = [vp, u32, vp, vp, vp, u32, vp, vp, vp, vp, i32, i32]
        L.or_trace_hlsl.argtypes = [vp, u32, vp, vp, vp, u32, vp, vp, vp, vp, i32]
        L.or_shadow_mirror_hlsl.argtypes = [vp, u32, vp, vp, C.POINTER(OrCamera), vp, vp, vp, vp, vp, vp, vp, i32]
        L.or_primary_rays.argtypes = [C.POINTER(OrCamera), vp]
        L.or_shadow_mirror.argtypes = [vp, u32, vp, vp, C.POINTER(OrCamera), vp, vp, vp, vp, vp, vp, i32]
        L.or_shadow_mirror_from.argtypes = [vp, u32, vp, vp, C.POINTER(OrCamera), vp, vp, vp, vp, vp, vp, vp, vp,
                                            i32]
        L.or_pathtrace.argtypes = [vp, u32, vp, vp, vp, vp, C.POINTER(OrCamera), C.POINTER(OrPtParams), vp, i32]
        L.or_pathtrace_adjoint.argtypes = [vp, u32, vp, vp, vp, vp, C.POINTER(OrCamera), C.POINTER(OrPtParams),
                                           vp, vp, vp, i32]
        L.or_render_whitted.argtypes = [vp, u32, vp, vp, vp, vp, vp, u32, C.POINTER(OrCamera), vp,
                                        C.POINTER(OrShadeParams), vp, vp, i32]
        L.or_whitted_rand.argtypes = [u32, u32, u32]
        L.or_whitted_rand.restype = C.c_float
        L.or_bvh_trace.argtypes = [vp, u32, vp, u32, vp, vp, u32, vp, vp, i32, i32]
        L.or_bvh_shadow_mirror.argtypes = [vp, u32, vp, u32, vp, C.POINTER(OrCamera), vp, vp, vp, vp, vp, vp, i32]
        L.or_pcg32_first.argtypes = [C.c_uint64, C.c_uint64, u32, vp]
        L.or_pcg32_first.restype = u32
        _olib = L
    return _olib


def nthreads_default() -> int:
    return max(1, os.cpu_count() or 1)


# --- build -----------------------------------------------------------------
def scene_bounds(tris: np.ndarray) -> np.ndarray:
    out = np.zeros(6, np.float32)
    olib().or_scene_bounds(_ptr(tris), len(tris), _ptr(out))
    return out


def morton(tris: np.ndarray, bounds: np.ndarray | None = None) -> np.ndarray:
    if bounds is None:
        bounds = scene_bounds(tris)
    keys = np.zeros(len(tris), np.uint32)
    olib().or_morton(_ptr(tris), len(tris), _ptr(np.ascontiguousarray(bounds, np.float32)), _ptr(keys))
    return keys


def sort_pairs(keys: np.ndarray, ids: np.ndarray | None = None):
    keys = np.array(keys, np.uint32, copy=True)
    ids = np.arange(len(keys), dtype=np.uint32) if ids is None else np.array(ids, np.uint32, copy=True)
    olib().or_sort_pairs(_ptr(keys), _ptr(ids), len(keys))
    return keys, ids


def lbvh_build(tris: np.ndarray, depth: int):
    """Returns (nodes, ids, keys, reached) of the restated LBVH::Build."""
    tris = np.ascontiguousarray(tris, np.float32)
    n = len(tris)
    nodes = np.zeros(1 << depth, NODE_DTYPE)
    ids = np.zeros(n, np.uint32)
    keys = np.zeros(n, np.uint32)
    reached = np.zeros(1 << depth, np.uint8)
    olib().or_lbvh_build(_ptr(tris), n, depth, _ptr(nodes), _ptr(ids), _ptr(keys), _ptr(reached))
    return nodes, ids, keys, reached.astype(bool)


# --- tracing ---------------------------------------------------------------
def rays_array(o, d, tmax, exclude) -> np.ndarray:
    n = len(d)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = o
    r[:, 3:6] = d
    r[:, 6] = tmax
    r[:, 7] = exclude
    return r


def trace(nodes, depth, ids, tris, rays, any_hit=False, nthreads=None, stats=False):
    rays = np.ascontiguousarray(rays, np.float32)
    n = len(rays)
    hits = np.zeros(n, HIT_DTYPE)
    st = np.zeros((n, 2), np.uint32) if stats else None
    olib().or_trace(_ptr(nodes), depth, _ptr(ids), _ptr(np.ascontiguousarray(tris, np.float32)), _ptr(rays), n,
                    _ptr(hits), _ptr(st) if stats else None, int(any_hit), nthreads or nthreads_default())
    return (hits, st) if stats else hits


def trace_from(nodes, depth, ids, tris, rays, starts=None, any_hit=False, nthreads=None, stats=False):
    """or_trace_from: the walk of each ray starts at heap node starts[i]
    (None: the root).  Returns (hits, leaves[, stats]); leaves[i] = the node
    whose triangles gave the closest hit (1 for a miss)."""
    rays = np.ascontiguousarray(rays, np.float32)
    n = len(rays)
    hits = np.zeros(n, HIT_DTYPE)
    leaves = np.zeros(n, np.uint32)
    st = np.zeros((n, 2), np.uint32) if stats else None
    sp = None if starts is None else np.ascontiguousarray(starts, np.uint32)
    olib().or_trace_from(_ptr(nodes), depth, _ptr(ids), _ptr(np.ascontiguousarray(tris, np.float32)), _ptr(rays), n,
                         _ptr(sp) if sp is not None else None, _ptr(hits), _ptr(leaves),
                         _ptr(st) if stats else None, int(any_hit), nthreads or nthreads_default())
    return (hits, leaves, st) if stats else (hits, leaves)


def trace_hlsl(nodes, depth, ids, tris, rays, starts=None, nthreads=None):
    """or_trace_hlsl: the reference's own LBVH_IntersectP walk.  Returns
    (hits, leaves, stats) with stats = {visited nodes, triangle tests}."""
    rays = np.ascontiguousarray(rays, np.float32)
    n = len(rays)
    hits = np.zeros(n, HIT_DTYPE)
    leaves = np.zeros(n, np.uint32)
    st = np.zeros((n, 2), np.uint32)
    sp = None if starts is None else np.ascontiguousarray(starts, np.uint32)
    olib().or_trace_hlsl(_ptr(nodes), depth, _ptr(ids), _ptr(np.ascontiguousarray(tris, np.float32)), _ptr(rays), n,
                         _ptr(sp) if sp is not None else None, _ptr(hits), _ptr(leaves), _ptr(st),
                         nthreads or nthreads_default())
    return hits, leaves, st


def frame_hlsl(nodes, depth, ids, tris, cam, light, nthreads=None):
    """A frame in the reference's own walk order (or_trace_hlsl +
    or_shadow_mirror_hlsl).  Returns (prim, vis, mirror, prim_stats,
    shadow_stats, mirror_stats)."""
    prim, leaves, pst = trace_hlsl(nodes, depth, ids, tris, primary_rays(cam), nthreads=nthreads)
    oc = to_or_camera(cam)
    npx = cam.width * cam.height
    vis = np.zeros(npx, np.uint8)
    mirror = np.zeros(npx, HIT_DTYPE)
    ss = np.zeros((npx, 2), np.uint32)
    ms = np.zeros((npx, 2), np.uint32)
    olib().or_shadow_mirror_hlsl(_ptr(nodes), depth, _ptr(ids), _ptr(np.ascontiguousarray(tris, np.float32)),
                                 C.byref(oc), _ptr(np.asarray(light, np.float32)), _ptr(prim), _ptr(leaves),
                                 _ptr(vis), _ptr(mirror), _ptr(ss), _ptr(ms), nthreads or nthreads_default())
    return prim, vis, mirror, pst, ss, ms


def primary_rays(cam) -> np.ndarray:
    oc = to_or_camera(cam)
    r = np.zeros((cam.width * cam.height, 8), np.float32)
    olib().or_primary_rays(C.byref(oc), _ptr(r))
    return r


def shadow_mirror(nodes, depth, ids, tris, cam, light, prim, nthreads=None, stats=False):
    oc = to_or_camera(cam)
    npx = cam.width * cam.height
    vis = np.zeros(npx, np.uint8)
    mirror = np.zeros(npx, HIT_DTYPE)
    ss = np.zeros((npx, 2), np.uint32) if stats else None
    ms = np.zeros((npx, 2), np.uint32) if stats else None
    olib().or_shadow_mirror(_ptr(nodes), depth, _ptr(ids), _ptr(np.ascontiguousarray(tris, np.float32)), C.byref(oc),
                            _ptr(np.asarray(light, np.float32)), _ptr(np.ascontiguousarray(prim)), _ptr(vis),
                            _ptr(mirror), _ptr(ss) if stats else None, _ptr(ms) if stats else None,
                            nthreads or nthreads_default())
    return (vis, mirror, ss, ms) if stats else (vis, mirror)


def shadow_mirror_from(nodes, depth, ids, tris, cam, light, prim, prim_leaves, nthreads=None, stats=False):
    """or_shadow_mirror_from: shading rays started at the primary hits'
    leaves.  Returns (vis, mirror, mirror_leaves[, shadow_stats, mirror_stats])."""
    oc = to_or_camera(cam)
    npx = cam.width * cam.height
    vis = np.zeros(npx, np.uint8)
    mirror = np.zeros(npx, HIT_DTYPE)
    ml = np.zeros(npx, np.uint32)
    ss = np.zeros((npx, 2), np.uint32) if stats else None
    ms = np.zeros((npx, 2), np.uint32) if stats else None
    pl = None if prim_leaves is None else np.ascontiguousarray(prim_leaves, np.uint32)
    olib().or_shadow_mirror_from(_ptr(nodes), depth, _ptr(ids), _ptr(np.ascontiguousarray(tris, np.float32)),
                                 C.byref(oc), _ptr(np.asarray(light, np.float32)), _ptr(np.ascontiguousarray(prim)),
                                 _ptr(pl) if pl is not None else None, _ptr(vis), _ptr(mirror), _ptr(ml),
                                 _ptr(ss) if stats else None, _ptr(ms) if stats else None,
                                 nthreads or nthreads_default())
    return (vis, mirror, ml, ss, ms) if stats else (vis, mirror, ml)


def render_whitted(nodes, depth, ids, tris, cam, light, materials, material_ids=None, normals=None, bounces=0,
                   shadows=True, phong=False, gloss_mapping=False, env_mapping=-1, env_color=(1.0, 1.0, 1.0), seed=0,
                   nthreads=None):
    """or_render_whitted: the colour stage and its bounce loop.  materials:
    (m, 14) float32 rows (ambient 4, diffuse 4, specular 4, shininess,
    alpha).  Returns (accum, result), each (w*h, 4) float32."""
    oc = to_or_camera(cam)
    sp = OrShadeParams(bounces, int(shadows), int(phong), int(gloss_mapping), env_mapping,
                       (C.c_float * 3)(*env_color), seed)
    mats = np.ascontiguousarray(materials, np.float32).reshape(-1, 14)
    mid = None if material_ids is None else np.ascontiguousarray(material_ids, np.int32)
    nrm = None if normals is None else np.ascontiguousarray(normals, np.float32)
    npx = cam.width * cam.height
    acc = np.zeros((npx, 4), np.float32)
    res = np.zeros((npx, 4), np.float32)
    olib().or_render_whitted(_ptr(nodes), depth, _ptr(ids), _ptr(np.ascontiguousarray(tris, np.float32)),
                             _ptr(nrm) if nrm is not None else None, _ptr(mid) if mid is not None else None,
                             _ptr(mats), len(mats), C.byref(oc), _ptr(np.asarray(light, np.float32)), C.byref(sp),
                             _ptr(acc), _ptr(res), nthreads or nthreads_default())
    return acc, res


def bvh_trace(nodes, ids, tris, rays, any_hit=False, nthreads=None, stats=False):
    """or_bvh_trace: BVH_IntersectP over a flattened SAH BVH (nodes in the
    LinearBVHNode = NODE_DTYPE layout, ids = ordered primitive ids)."""
    rays = np.ascontiguousarray(rays, np.float32)
    nodes = np.ascontiguousarray(nodes)
    ids = np.ascontiguousarray(ids, np.uint32)
    n = len(rays)
    hits = np.zeros(n, HIT_DTYPE)
    st = np.zeros((n, 2), np.uint32) if stats else None
    olib().or_bvh_trace(_ptr(nodes), len(nodes), _ptr(ids), len(ids), _ptr(np.ascontiguousarray(tris, np.float32)),
                        _ptr(rays), n, _ptr(hits), _ptr(st) if stats else None, int(any_hit),
                        nthreads or nthreads_default())
    return (hits, st) if stats else hits


def bvh_shadow_mirror(nodes, ids, tris, cam, light, prim, nthreads=None, stats=False):
    oc = to_or_camera(cam)
    npx = cam.width * cam.height
    nodes = np.ascontiguousarray(nodes)
    ids = np.ascontiguousarray(ids, np.uint32)
    vis = np.zeros(npx, np.uint8)
    mirror = np.zeros(npx, HIT_DTYPE)
    ss = np.zeros((npx, 2), np.uint32) if stats else None
    ms = np.zeros((npx, 2), np.uint32) if stats else None
    olib().or_bvh_shadow_mirror(_ptr(nodes), len(nodes), _ptr(ids), len(ids),
                                _ptr(np.ascontiguousarray(tris, np.float32)), C.byref(oc),
                                _ptr(np.asarray(light, np.float32)), _ptr(np.ascontiguousarray(prim)), _ptr(vis),
                                _ptr(mirror), _ptr(ss) if stats else None, _ptr(ms) if stats else None,
                                nthreads or nthreads_default())
    return (vis, mirror, ss, ms) if stats else (vis, mirror)


def pathtrace(nodes, depth, ids, tris, albedo, emission, cam, spp, bounces, seed, sky=(1.0, 1.0, 1.0), nthreads=None,
              first_sample=0, window=None, image=None):
    """CPU rendering of samples first_sample .. first_sample + spp - 1.
    window = (x0, y0, w, h) renders that crop of the cam.width x cam.height
    image (w*h x 4 floats, row-major); image (same shape) holds the mean of
    the first_sample earlier samples when first_sample > 0."""
    oc = to_or_camera(cam)
    p = _pt_params(spp, bounces, seed, sky, first_sample, window)
    npx = window[2] * window[3] if window is not None else cam.height * cam.width
    img = np.zeros((npx, 4), np.float32) if image is None else np.array(image, np.float32, copy=True).reshape(npx, 4)
    olib().or_pathtrace(_ptr(nodes), depth, _ptr(ids), _ptr(np.ascontiguousarray(tris, np.float32)),
                        _ptr(np.ascontiguousarray(albedo, np.float32)), _ptr(np.ascontiguousarray(emission, np.float32)),
                        C.byref(oc), C.byref(p), _ptr(img), nthreads or nthreads_default())
    return img


def pathtrace_adjoint(nodes, depth, ids, tris, albedo, emission, cam, spp, bounces, seed, d_image,
                      sky=(1.0, 1.0, 1.0), nthreads=None, first_sample=0, window=None):
    """FP64 adjoint; with window = (x0, y0, w, h), d_image holds that crop's
    w*h pixels and the pixels outside it contribute nothing."""
    oc = to_or_camera(cam)
    p = _pt_params(spp, bounces, seed, sky, first_sample, window)
    da = np.zeros((len(tris), 3), np.float64)
    de = np.zeros(3, np.float64)
    olib().or_pathtrace_adjoint(_ptr(nodes), depth, _ptr(ids), _ptr(np.ascontiguousarray(tris, np.float32)),
                                _ptr(np.ascontiguousarray(albedo, np.float32)),
                                _ptr(np.ascontiguousarray(emission, np.float32)), C.byref(oc), C.byref(p),
                                _ptr(np.ascontiguousarray(d_image, np.float32)), _ptr(da), _ptr(de),
                                nthreads or nthreads_default())
    return da, de


def pcg32_first(initstate: int, initseq: int, count: int) -> np.ndarray:
    out = np.zeros(count, np.uint32)
    olib().or_pcg32_first(initstate, initseq, count, _ptr(out))
    return out


# --- the reference's own CPU code ------------------------------------------
def ref_available() -> bool:
    return REF_LIB.exists()


def rlib() -> C.CDLL:
    global _rlib
    if _rlib is None:
        L = C.CDLL(str(REF_LIB))
        vp, i32 = C.c_void_p, C.c_int
        L.ref_lbvh_create.argtypes = [vp, i32, i32, i32, C.POINTER(C.c_double)]
        L.ref_lbvh_create.restype = vp
        L.ref_bvh_create.argtypes = [vp, i32, i32, i32, C.POINTER(C.c_double)]
        L.ref_bvh_create.restype = vp
        L.ref_destroy.argtypes = [vp]
        L.ref_num_elements.argtypes = [vp]
        L.ref_num_elements.restype = C.c_uint
        L.ref_element_size.argtypes = [vp]
        L.ref_element_size.restype = C.c_uint
        L.ref_copy_elements.argtypes = [vp, vp]
        L.ref_copy_ids.argtypes = [vp, vp]
        L.ref_world_bound.argtypes = [vp, vp]
        L.ref_intersect.argtypes = [vp, vp, C.c_long, vp, vp, vp, vp, i32]
        L.ref_obj_load.argtypes = [C.c_char_p]
        L.ref_obj_load.restype = i32
        L.ref_obj_fetch.argtypes = [vp, vp]
        L.ref_obj_material_count.restype = i32
        L.ref_txt_load.argtypes = [C.c_char_p]
        L.ref_txt_load.restype = i32
        L.ref_obj_fetch_materials.argtypes = [vp]
        _rlib = L
    return _rlib


class RefStructure:
    """The reference's LBVH (kind='lbvh') or SAH BVH (kind='bvh') over a soup."""

    def __init__(self, tris: np.ndarray, kind: str = "lbvh", depth: int = 20, max_prims: int = 1):
        self.tris = np.ascontiguousarray(tris, np.float32)
        self.n = len(tris)
        secs = C.c_double(0.0)
        L = rlib()
        if kind == "lbvh":
            self.h = L.ref_lbvh_create(_ptr(self.tris), self.n, depth, 1, C.byref(secs))
        else:
            self.h = L.ref_bvh_create(_ptr(self.tris), self.n, max_prims, 1, C.byref(secs))
        self.build_seconds = secs.value
        self.kind = kind

    def close(self):
        if self.h:
            rlib().ref_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def nodes(self) -> np.ndarray:
        L = rlib()
        n = L.ref_num_elements(self.h)
        esize = L.ref_element_size(self.h)
        assert esize == 32  # LBVHNode and LinearBVHNode: bounds, count, offset
        raw = np.zeros(n * esize, np.uint8)
        L.ref_copy_elements(self.h, _ptr(raw))
        return raw.view(NODE_DTYPE)

    def ids(self) -> np.ndarray:
        out = np.zeros(self.n, np.uint32)
        rlib().ref_copy_ids(self.h, _ptr(out))
        return out

    def world_bound(self) -> np.ndarray:
        out = np.zeros(6, np.float32)
        rlib().ref_world_bound(self.h, _ptr(out))
        return out

    def intersect(self, rays: np.ndarray, nthreads=None):
        rays = np.ascontiguousarray(rays, np.float32)
        n = len(rays)
        hid = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        u = np.zeros(n, np.float32)
        v = np.zeros(n, np.float32)
        rlib().ref_intersect(self.h, _ptr(rays), n, _ptr(hid), _ptr(t), _ptr(u), _ptr(v), nthreads or nthreads_default())
        return hid, t, u, v


def reachable_mask(nodes: np.ndarray) -> np.ndarray:
    """Heap slots reachable from the root of an LBVH node array (children of
    internal nodes only; unreached slots of the reference are uninitialised)."""
    m = np.zeros(len(nodes), bool)
    if len(nodes) < 2:
        return m
    m[1] = True
    leaf = (nodes["prim_count"] & 4) != 0
    lo = 2
    while lo < len(nodes):
        hi = min(2 * lo, len(nodes))
        par = np.arange(lo, hi) >> 1
        m[lo:hi] = m[par] & ~leaf[par]
        lo = hi
    return m


def ref_load_model(path):
    """(soup n x 9 float32, material id per triangle) of a model file: .obj
    through the reference's vendored loader + normalize(), .txt through a
    restatement of Model::LoadFile's .txt branch; both then through the
    reference's own Model::Scale (oracle/ref/ref_shim.cpp ref_obj_load,
    ref_txt_load)."""
    L = rlib()
    p = str(path)
    n = (L.ref_txt_load if ".txt" in p or ".TXT" in p else L.ref_obj_load)(p.encode())
    if n < 0:
        raise OSError(f"reference loader could not read {path}")
    soup = np.zeros((n, 9), np.float32)
    mat = np.zeros(n, np.int32)
    L.ref_obj_fetch(_ptr(soup), _ptr(mat))
    return soup, mat


def ref_obj_materials():
    """Materials of the file ref_load_model read last: (m, 14) float32 rows of
    ambient[4], diffuse[4], specular[4], shininess, alpha."""
    L = rlib()
    out = np.zeros((L.ref_obj_material_count(), 14), np.float32)
    L.ref_obj_fetch_materials(_ptr(out))
    return out
