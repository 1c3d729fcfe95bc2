"""Model ingestion (include/rt_model.h, librthost.so) against the reference's
own OBJ loader + Model::Scale: the golden soups in tests/golden/models/expected.npz
were made by oracle/_ref (tests/golden/make_models.py).  Bit-exact: every
soup coordinate, every material id and every material field.

CPU tests: the fixtures, error handling, the exported symbols, and seeded
random OBJ files against the live reference where oracle/_ref was built.
GPU test: a loaded model through the GPU LBVH build matches the oracle."""
import re
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

MODEL_FILES = ["grid_quads.obj", "forms_negative.obj", "materials.obj", "one_material.obj", "torus.OBJ",
               "cloud.txt", "unused_vertices.txt"]


@pytest.fixture(scope="module")
def model_mod():
    from rtgpu import build, model
    build.build_cuda()
    build.build_host()
    model.hostlib()
    return model


@pytest.fixture(scope="module")
def golden_models():
    return dict(np.load(GOLDEN / "models" / "expected.npz"))


def same_bits(a, b):
    a, b = np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def check_against(m, soup, ids, mats):
    assert same_bits(m.soup, soup), "triangle soup"
    assert np.array_equal(m.material_ids, ids), "material ids"
    assert same_bits(np.stack([x.row() for x in m.materials]), mats), "materials"


@pytest.mark.parametrize("name", MODEL_FILES)
def test_golden_models(model_mod, golden_models, name):
    key = name.replace(".", "_")
    m = model_mod.load(GOLDEN / "models" / name)
    check_against(m, golden_models[f"{key}__soup"], golden_models[f"{key}__material_ids"],
                  golden_models[f"{key}__materials"])
    assert m.triangle_count == len(m.soup) > 0
    # Model::Scale's result: every corner inside the 0.49 sphere (to rounding)
    r = np.sqrt((m.soup.reshape(-1, 3).astype(np.float64) ** 2).sum(1))
    assert r.max() <= 0.49 * (1 + 1e-6)


def test_materials_fixture_rules(golden_models):
    """What the reference loader does with the materials fixture: usemtl
    before mtllib still resolves, unknown names take material 0, and ids go
    through the name cache, so both materials named 'red' map to the last."""
    ids = golden_models["materials_obj__material_ids"]
    assert ids.tolist() == [1, 1, 1, 3, 3, 3, 3, 2, 2, 1, 1, 1, 3, 2, 2]
    mats = golden_models["materials_obj__materials"]
    assert mats[1, 8:12].tolist() == [0.0, 0.0, 0.0, 1.0]      # illum 1 clears specular
    assert mats[0, 8:12].tolist() == [np.float32(0.3)] * 2 + [0.0, 1.0]  # Ks with two values keeps the rest


def test_errors(model_mod, tmp_path):
    with pytest.raises(ValueError, match="cannot open"):
        model_mod.load(tmp_path / "missing.obj")
    (tmp_path / "a.ply").write_text("ply\n")
    with pytest.raises(ValueError, match="unknown model format"):
        model_mod.load(tmp_path / "a.ply")
    (tmp_path / "b.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 9\n")
    with pytest.raises(ValueError, match="names no vertex"):
        model_mod.load(tmp_path / "b.obj")
    (tmp_path / "c.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf -4 1 2\n")
    with pytest.raises(ValueError, match="names no vertex"):
        model_mod.load(tmp_path / "c.obj")
    (tmp_path / "d.obj").write_text("v 0 0 0\n# no faces\n")
    with pytest.raises(ValueError, match="no faces"):
        model_mod.load(tmp_path / "d.obj")
    (tmp_path / "e.txt").write_text("3 1\n0 0 0 0 0 1 0 0\n1 0 0 0 0 1 0 0\n0 1 0 0 0 1 0 0\n0 1 3\n")
    with pytest.raises(ValueError, match="out of range"):
        model_mod.load(tmp_path / "e.txt")


def test_host_library_exports_rt_model_h(model_mod):
    txt = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "rt_model.h").read_text(), flags=re.S)
    declared = sorted(set(re.findall(r"\b(rt_[a-z0-9_]+)\s*\(", txt)))
    L = model_mod.hostlib()
    assert [s for s in declared if not hasattr(L, s)] == []
    assert sorted(model_mod.EXPORTED) == declared


def random_obj(rng, nv, nf):
    """A seeded OBJ text mixing every face form, relative indices, polygons
    of 3..7 corners, vt / vn records and usemtl records."""
    L = []
    pts = rng.uniform(-5, 5, size=(nv, 3)) * rng.uniform(0.01, 3, size=3)
    for p in pts:
        L.append("v %.9g %.9g %.9g" % tuple(p))
    for _ in range(5):
        L.append("vt %.4f %.4f" % tuple(rng.uniform(0, 1, 2)))
        L.append("vn %.4f %.4f %.4f" % tuple(rng.normal(size=3)))
    for f in range(nf):
        if rng.random() < 0.1:
            L.append(f"usemtl m{rng.integers(0, 4)}")
        k = int(rng.integers(3, 8))
        corners = rng.choice(nv, size=k, replace=False) + 1
        form = int(rng.integers(0, 4))
        toks = []
        for c in corners:
            v = int(c) if rng.random() < 0.7 else int(c) - nv - 1  # relative: -k -> nv - k - 1
            if v < 0 and v + nv - 1 < 0:
                v = int(c)
            t, n = int(rng.integers(1, 6)), int(rng.integers(1, 6))
            toks.append([f"{v}", f"{v}/{t}", f"{v}//{n}", f"{v}/{t}/{n}"][form])
        L.append("f " + " ".join(toks))
    return "\n".join(L) + "\n"


@pytest.mark.parametrize("seed", range(12))
def test_random_obj_vs_live_reference(model_mod, oracle_mod, tmp_path, seed):
    oracle_mod.build_reference()
    if not oracle_mod.ref_available():
        pytest.skip("reference CPU code not built here")
    rng = np.random.Generator(np.random.PCG64(900 + seed))
    mtl = "".join(f"newmtl m{i}\nKd {0.2 * i:.2f} 0.5 0.5\nNs {100 * i}\n" for i in range(4))
    (tmp_path / "r.mtl").write_text(mtl)
    text = random_obj(rng, int(rng.integers(10, 400)), int(rng.integers(1, 300)))
    if seed % 2:
        text = "mtllib r.mtl\n" + text
    path = tmp_path / "r.obj"
    path.write_text(text)
    soup, ids = oracle_mod.ref_load_model(path)
    check_against(model_mod.load(path), soup, ids, oracle_mod.ref_obj_materials())


@pytest.mark.gpu
def test_loaded_model_gpu_build_matches_oracle(model_mod, gpu_ctx, oracle_mod):
    """A model file -> rt_model_load -> GPU LBVH build: the same tree as the
    oracle builds from the reference loader's soup."""
    import torch
    from rtgpu.api import LBVH
    g = dict(np.load(GOLDEN / "models" / "expected.npz"))
    for name, depth in (("torus.OBJ", 16), ("grid_quads.obj", 12), ("cloud.txt", 14)):
        m = model_mod.load(GOLDEN / "models" / name)
        assert same_bits(m.soup, g[name.replace(".", "_") + "__soup"])
        lb = LBVH(gpu_ctx, len(m.soup), depth)
        lb.Build(torch.from_numpy(m.soup).cuda(), 0)
        gpu_ctx.check()
        nodes, ids, keys = lb.download(True, True, True)
        onodes, oids, okeys, reached = oracle_mod.lbvh_build(m.soup, depth)
        assert np.array_equal(keys, okeys) and np.array_equal(ids, oids)
        idx = np.nonzero(reached)[0]
        assert np.array_equal(nodes[idx], onodes[idx])
