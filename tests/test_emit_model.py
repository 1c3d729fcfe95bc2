"""The scan-based emission algorithm used by the CUDA build, run as a host
model, reproduces the reference tree (via the oracle) node for node."""
import numpy as np
import pytest

import emit_model
from conftest import golden_cases, load_golden


def check(oracle_mod, tris, depth, tile=7):
    nodes, ids, keys, reached = oracle_mod.lbvh_build(tris, depth)
    got = emit_model.emit(keys, depth, tile=tile)
    idx = np.nonzero(reached)[0]
    assert sorted(got.keys()) == idx.tolist()
    for h in idx:
        assert got[h] == (int(nodes[h]["prim_count"]), int(nodes[h]["prim_pos"])), h


@pytest.mark.parametrize("case", golden_cases())
def test_model_golden(oracle_mod, case):
    g = load_golden(case)
    check(oracle_mod, g["tris"], int(g["depth"]))


@pytest.mark.parametrize("depth", [1, 2, 3, 5, 9, 13, 20])
@pytest.mark.parametrize("seed", [0, 1])
def test_model_random(oracle_mod, depth, seed):
    from rtgpu import scenes
    rng = np.random.default_rng(seed)
    tris = scenes.random_soup(int(rng.integers(200, 1500)), seed=100 + seed)
    # inject exact duplicates and near-duplicates (equal Morton codes)
    tris = np.concatenate([tris, tris[:50], tris[10:40] + np.float32(1e-7)])
    check(oracle_mod, np.ascontiguousarray(tris), depth, tile=int(rng.integers(1, 64)))


@pytest.mark.parametrize("n", [1, 2, 3, 4, 33])
def test_model_small(oracle_mod, n):
    from rtgpu import scenes
    tris = scenes.random_soup(n, seed=7)
    check(oracle_mod, tris, 12, tile=2)
    check(oracle_mod, np.ascontiguousarray(np.repeat(tris[:1], n, axis=0)), 12, tile=3)


@pytest.mark.parametrize("depth", [1, 3, 8, 14])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_model_batch(oracle_mod, depth, seed):
    """Separator records at scene boundaries: every scene of a concatenated
    batch gets the tree the oracle builds for it alone, whatever the tile
    size (so scans cross tiles that hold several scenes, or part of one)."""
    from rtgpu import scenes
    rng = np.random.default_rng(seed)
    sizes = [1, 2, 1] + [int(x) for x in rng.integers(1, 300, size=5)] + [1]
    rng.shuffle(sizes)
    keys_all, offsets, want = [], [0], []
    for s, n in enumerate(sizes):
        tris = scenes.random_soup(n, seed=500 + 10 * seed + s)
        if n > 20:  # equal codes inside a scene
            tris = np.ascontiguousarray(np.concatenate([tris, tris[:7]]))
        nodes, ids, keys, reached = oracle_mod.lbvh_build(tris, depth)
        keys_all.append(keys)
        offsets.append(offsets[-1] + len(keys))
        want.append((nodes, reached))
    got = emit_model.emit_batch(np.concatenate(keys_all), offsets, depth, tile=int(rng.integers(1, 40)))
    for s, (nodes, reached) in enumerate(want):
        idx = np.nonzero(reached)[0]
        assert sorted(got[s].keys()) == idx.tolist(), s
        for h in idx:
            assert got[s][h] == (int(nodes[h]["prim_count"]), int(nodes[h]["prim_pos"])), (s, h)
