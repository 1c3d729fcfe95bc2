"""Model files as triangle soups: ctypes binding of include/rt_model.h
(librthost.so), the headless form of the reference's Model::LoadFile +
Model::Scale (Common/Scenes/Model.cpp:107-113, 210-381, 647-709).

    m = load("scene.obj")     # .obj (with its .mtl) or the reference's .txt
    m.soup                    # (n, 9) float32: A.xyz B.xyz C.xyz, ready for
                              # RayTracer.build / rt_lbvh_build_host
    m.material_ids            # (n,) int32
    m.materials               # list of Material

The loader is native (C++); there is no Python fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import _lib
from .build import HOST_LIB, build_host

EXPORTED = ["rt_model_load", "rt_model_free", "rt_model_triangle_count", "rt_model_soup", "rt_model_material_ids",
            "rt_model_material_count", "rt_model_material"]


class _Material(C.Structure):
    _fields_ = [("ambient", C.c_float * 4), ("diffuse", C.c_float * 4), ("specular", C.c_float * 4),
                ("shininess", C.c_float), ("alpha", C.c_float)]


@dataclass(frozen=True)
class Material:
    ambient: tuple
    diffuse: tuple
    specular: tuple
    shininess: float  # Ns / 1000
    alpha: float      # d, or 1 - Tr

    def row(self) -> np.ndarray:
        """ambient, diffuse, specular, shininess, alpha as 14 float32."""
        return np.array([*self.ambient, *self.diffuse, *self.specular, self.shininess, self.alpha], np.float32)


@dataclass
class Model:
    soup: np.ndarray
    material_ids: np.ndarray
    materials: list

    @property
    def triangle_count(self) -> int:
        return len(self.soup)


_hl = None


def hostlib() -> C.CDLL:
    global _hl
    if _hl is None:
        if not HOST_LIB.exists():
            build_host()
        if not HOST_LIB.exists():
            raise OSError(f"{HOST_LIB} is missing: build it with rtgpu.build.build_all()")
        L = C.CDLL(str(HOST_LIB))
        vp, u32 = C.c_void_p, C.c_uint32
        sig = {
            "rt_model_load": (C.c_int, [C.c_char_p, C.POINTER(vp), C.c_char_p, C.c_size_t]),
            "rt_model_free": (None, [vp]),
            "rt_model_triangle_count": (u32, [vp]),
            "rt_model_soup": (C.POINTER(C.c_float), [vp]),
            "rt_model_material_ids": (C.POINTER(C.c_int32), [vp]),
            "rt_model_material_count": (u32, [vp]),
            "rt_model_material": (C.POINTER(_Material), [vp, u32]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _hl = L
    return _hl


def load(path) -> Model:
    """Loads a .obj or .txt model; raises ValueError with the loader's
    message when the file cannot be read."""
    L = hostlib()
    h = C.c_void_p()
    err = C.create_string_buffer(512)
    st = L.rt_model_load(str(path).encode(), C.byref(h), err, len(err))
    if st != _lib.RT_OK:
        raise ValueError(f"rt_model_load: {err.value.decode(errors='replace')}")
    try:
        n = L.rt_model_triangle_count(h)
        soup = np.ctypeslib.as_array(L.rt_model_soup(h), shape=(n * 9,)).reshape(n, 9).copy()
        ids = np.ctypeslib.as_array(L.rt_model_material_ids(h), shape=(n,)).copy()
        mats = []
        for i in range(L.rt_model_material_count(h)):
            m = L.rt_model_material(h, i).contents
            mats.append(Material(tuple(m.ambient), tuple(m.diffuse), tuple(m.specular), m.shininess, m.alpha))
    finally:
        L.rt_model_free(h)
    return Model(soup, ids, mats)

