"""Writes the model-file fixtures in tests/golden/models/ and their expected
triangle soups (tests/golden/models/expected.npz) from the reference's OWN loader:
Common/Scenes/Loaders/model_obj.cpp (ModelOBJ::import + normalize) and
Model::Scale from Common/Scenes/Model.cpp, compiled from the reference
checkout by oracle/ref/build_ref.sh (oracle.ref_load_model).  The .txt cases
go through a restatement of Model::LoadFile's .txt branch (positions only)
and the same compiled Model::Scale.

The model files are synthetic (seeded grids, tori and hand-written records
that exercise each rule of the loader).  Run from the repository root where
the reference checkout is present:
    python tests/golden/make_models.py
"""
from __future__ import annotations

import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))

import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent
MODELS = OUT / "models"


def grid_quads():
    """A perturbed 12 x 9 grid as quads, with a pentagon and a hexagon fan;
    every x is negative (the loader's bounds start its maximum at FLT_MIN)."""
    rng = np.random.Generator(np.random.PCG64(21))
    nx, ny = 12, 9
    lines = ["# grid of quads", "o grid"]
    for j in range(ny):
        for i in range(nx):
            x = -3.0 + 2.5 * i / (nx - 1) + rng.uniform(-0.02, 0.02)
            y = 1.0 * j / (ny - 1)
            z = 0.25 * math.sin(0.7 * i) * math.cos(0.9 * j) + rng.uniform(-0.01, 0.01)
            lines.append(f"v {x:.7f} {y:.7f} {z:.7f}")
    vid = lambda i, j: 1 + j * nx + i  # noqa: E731
    for j in range(ny - 1):
        for i in range(nx - 1):
            if (i, j) in ((3, 3), (4, 3), (6, 5), (7, 5), (8, 5)):
                continue
            lines.append(f"f {vid(i, j)} {vid(i + 1, j)} {vid(i + 1, j + 1)} {vid(i, j + 1)}")
    lines.append(f"f {vid(3, 3)} {vid(4, 3)} {vid(5, 3)} {vid(5, 4)} {vid(3, 4)}")
    lines.append(f"f {vid(6, 5)} {vid(7, 5)} {vid(9, 5)} {vid(9, 6)} {vid(7, 6)} {vid(6, 6)}")
    return "\n".join(lines) + "\n"


def forms_negative():
    """Every face form (v, v/vt, v//vn, v/vt/vn), relative (negative)
    indices, vt / vn / vp records, comments and group records, a face that
    names a vertex defined after it, and a 4-value v record."""
    L = ["# face forms", "mtllib missing.mtl", "g part1", "s 1"]
    pts = [(0.0, 0.0, 0.0), (1.0, 0.0, 0.1), (1.0, 1.0, 0.2), (0.0, 1.0, 0.3), (0.5, 1.5, -0.4),
           (2.0, 0.5, 0.25), (2.5, 1.25, -0.125), (1.75, 2.0, 0.5)]
    for p in pts[:4]:
        L.append("v %.6f %.6f %.6f" % p)
    L += ["vt 0 0", "vt 1 0", "vt 1 1", "vt 0 1", "vn 0 0 1", "vn 0 1 0", "vp 0.5 0.5"]
    L.append("f 1 2 3 4")
    L.append("f 1/1 2/2 3/3")
    L.append("f 1//1 3//1 4//2")
    L.append("f 2/2/1 3/3/1 4/4/2 1/1/2")
    L.append("f -3 -2 -1")          # relative: the loader maps -k to count - k - 1
    L.append("f -1/-1 -2/-2 -3/-3")
    L.append("f 2 3 7")             # vertex 7 is defined below: the loader sees zeros
    L.append("v %.6f %.6f %.6f 1.0" % pts[4])
    for p in pts[5:]:
        L.append("v %.6f %.6f %.6f" % p)
    L.append("usemtl nothing")
    L.append("f 5 6 7 8")
    L.append("f -2//1 -1//1 -3//2")
    return "\n".join(L) + "\n"


MATERIALS_MTL = """# three materials, one name twice
newmtl red
Ka 0.1 0.0 0.0
Kd 0.9 0.1 0.1 0.5
Ks 0.3 0.3
Ns 250
d 0.75
illum 2
map_Kd red.png
newmtl blue
Kd 0.1 0.2 0.9
Ni 1.45
Tr 0.25
Tf 1 1 1
illum 1
newmtl two words
Ka 0.5 0.5 0.5
Ns 1000
newmtl red
Kd 0.2 0.8 0.2
"""


def materials_obj():
    """usemtl before and after the mtllib record, an unknown name, a
    two-word name and a name defined twice in the MTL file."""
    rng = np.random.Generator(np.random.PCG64(22))
    L = ["usemtl blue"]
    v = rng.uniform(-1.0, 2.0, size=(40, 3))
    for p in v:
        L.append("v %.8f %.8f %.8f" % tuple(p))
    tri = lambda a: "f %d %d %d" % a  # noqa: E731
    L += [tri((1, 2, 3)), tri((4, 5, 6))]
    L.append("mtllib materials.mtl")
    L += [tri((7, 8, 9)), "usemtl red", tri((10, 11, 12)), "f 13 14 15 16", "usemtl nosuch", tri((17, 18, 19)),
          "usemtl two words", tri((20, 21, 22)), tri((23, 24, 25)), "usemtl blue", "f 26 27 28 29 30",
          "usemtl red", tri((31, 32, 33)), "usemtl words", tri((34, 35, 36)), tri((37, 38, 39))]
    return "\n".join(L) + "\n"


ONE_MTL = """newmtl only
Kd 0.3 0.6 0.9
"""


def one_material():
    L = ["mtllib one.mtl", "v 0 0 0", "v 1 0 0", "v 0 1 0", "v 0 0 1", "usemtl only", "f 1 2 3", "f 1 2 4",
         "f 1 3 4", "f 2 3 4"]
    return "\n".join(L) + "\n"


def torus(nu=40, nv=20, R=1.0, r=0.35):
    L = [f"# torus {nu}x{nv}"]
    for i in range(nu):
        a = 2 * math.pi * i / nu
        for j in range(nv):
            b = 2 * math.pi * j / nv
            x = (R + r * math.cos(b)) * math.cos(a)
            y = (R + r * math.cos(b)) * math.sin(a)
            z = r * math.sin(b) + 0.5
            L.append(f"v {x:.9g} {y:.9g} {z:.9g}")
    for i in range(nu):
        for j in range(nv):
            a = 1 + i * nv + j
            b = 1 + ((i + 1) % nu) * nv + j
            c = 1 + ((i + 1) % nu) * nv + (j + 1) % nv
            d = 1 + i * nv + (j + 1) % nv
            L.append(f"f {a} {b} {c} {d}")
    return "\n".join(L) + "\n"


def txt_model(nv, nt, seed, unused=0):
    """The reference's .txt format: counts, 8 floats per vertex, 3 indices
    per triangle; `unused` extra vertices no triangle names."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = rng.uniform(-2.0, 3.0, size=(nv + unused, 3)).astype(np.float32)
    nrm = rng.normal(size=(nv + unused, 3)).astype(np.float32)
    uv = rng.uniform(0, 1, size=(nv + unused, 2)).astype(np.float32)
    idx = rng.integers(0, nv, size=(nt, 3))
    L = [str(nv + unused), str(nt)]
    for p, n, t in zip(pos, nrm, uv):
        L.append(" ".join(f"{x:.7g}" for x in (*p, *n, *t)))
    for a in idx:
        L.append("%d %d %d" % tuple(a))
    return "\n".join(L) + "\n"


def files():
    return {
        "grid_quads.obj": grid_quads(),
        "forms_negative.obj": forms_negative(),
        "materials.obj": materials_obj(),
        "materials.mtl": MATERIALS_MTL,
        "one_material.obj": one_material(),
        "one.mtl": ONE_MTL,
        "torus.OBJ": torus(),
        "cloud.txt": txt_model(300, 500, seed=23),
        "unused_vertices.txt": txt_model(40, 60, seed=24, unused=7),
    }


MODEL_FILES = ["grid_quads.obj", "forms_negative.obj", "materials.obj", "one_material.obj", "torus.OBJ",
               "cloud.txt", "unused_vertices.txt"]


def main():
    O.build_oracle()
    if O.build_reference() is None:
        raise SystemExit("reference checkout not found; set RT_REFERENCE_DIR")
    MODELS.mkdir(exist_ok=True)
    for name, text in files().items():
        (MODELS / name).write_text(text)
    out = {}
    for name in MODEL_FILES:
        soup, mat = O.ref_load_model(MODELS / name)
        mats = O.ref_obj_materials()
        key = name.replace(".", "_")
        out[f"{key}__soup"] = soup
        out[f"{key}__material_ids"] = mat
        out[f"{key}__materials"] = mats
        print(f"{name}: triangles={len(soup)} materials={len(mats)} ids={np.unique(mat).tolist()}")
    np.savez_compressed(MODELS / "expected.npz", **out)


if __name__ == "__main__":
    main()
