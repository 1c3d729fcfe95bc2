"""GPU LBVH build parity (through the C ABI) against the oracle, which the
golden fixtures pin to the reference's own LBVH::Build.  Bit-exact: Morton
codes, the sorted permutation (cmpMorton order, LBVH.cpp:21-38), every
reachable node's PrimCount/PrimPos fields and boxes."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden
from bitcmp import assert_nodes_match_reference, same_bits

pytestmark = pytest.mark.gpu


def gpu_build(ctx, tris, depth, flags=0, device_input=True):
    import torch
    from rtgpu.api import LBVH
    lb = LBVH(ctx, max(1, len(tris)), depth)
    if device_input:
        lb.Build(torch.from_numpy(np.ascontiguousarray(tris)).cuda(), flags)
    else:
        lb.Build(np.ascontiguousarray(tris), flags)
    ctx.check()
    nodes, ids, keys = lb.download(True, True, True)
    return lb, nodes, ids, keys


def assert_same_tree(oracle_mod, tris, depth, nodes, ids, keys, all_slots=False):
    onodes, oids, okeys, reached = oracle_mod.lbvh_build(tris, depth)
    assert np.array_equal(keys, okeys), "Morton codes / sort"
    assert np.array_equal(ids, oids), "sorted permutation"
    idx = np.nonzero(reached)[0] if not all_slots else np.arange(1, len(onodes))
    a, b = nodes[idx], onodes[idx]
    bad = np.nonzero((a["prim_count"] != b["prim_count"]) | (a["prim_pos"] != b["prim_pos"]))[0]
    assert len(bad) == 0, f"{len(bad)} node field mismatches, first heap slot {idx[bad[0]]}"
    assert same_bits(a["min"], b["min"]) and same_bits(a["max"], b["max"]), "node boxes"


@pytest.mark.parametrize("case", golden_cases())
def test_build_golden_cases(gpu_ctx, oracle_mod, case):
    g = load_golden(case)
    depth = int(g["depth"])
    lb, nodes, ids, keys = gpu_build(gpu_ctx, g["tris"], depth)
    assert_same_tree(oracle_mod, g["tris"], depth, nodes, ids, keys)
    # and directly against the reference's own nodes: bit for bit, except the
    # sign of a zero bound where the reference's unstable partition lists a
    # leaf's triangles in another order (the signed_zero case)
    assert_nodes_match_reference(nodes, ids, g["nodes"], g["ids"], g["node_index"], case)
    wb = lb.WorldBound()
    assert np.array_equal(wb, g["world_bound"])
    if same_bits(nodes[1], g["nodes"][0]):
        assert same_bits(wb, g["world_bound"])


def test_build_torus_65536_depth20(gpu_ctx, oracle_mod):
    from rtgpu import scenes
    tris = scenes.torus()
    lb, nodes, ids, keys = gpu_build(gpu_ctx, tris, 20)
    assert_same_tree(oracle_mod, tris, 20, nodes, ids, keys)


def test_build_clear_unreached_matches_every_slot(gpu_ctx, oracle_mod):
    from rtgpu import scenes
    from rtgpu._lib import RT_BUILD_CLEAR_UNREACHED
    tris = scenes.random_soup(20000, seed=21)
    lb, nodes, ids, keys = gpu_build(gpu_ctx, tris, 16, flags=RT_BUILD_CLEAR_UNREACHED)
    assert_same_tree(oracle_mod, tris, 16, nodes, ids, keys, all_slots=True)


@pytest.mark.parametrize("n,depth", [(1_000_000, 20), (300_000, 22), (100_000, 10)])
def test_build_large(gpu_ctx, oracle_mod, n, depth):
    from rtgpu import scenes
    tris = scenes.random_soup(n, seed=n + depth)
    lb, nodes, ids, keys = gpu_build(gpu_ctx, tris, depth)
    assert_same_tree(oracle_mod, tris, depth, nodes, ids, keys)


# Radix-pass tile groups of the single-scene build (4,096 keys a tile, 32
# tiles a group): one group, a full group plus one ragged tile, and several
# groups whose last one is partial; codes, permutation and tree bit-exact.
@pytest.mark.parametrize("n", [32 * 4096 - 1, 32 * 4096 + 1, 65 * 4096 + 17, 97 * 4096])
def test_build_sort_tile_groups(gpu_ctx, oracle_mod, n):
    from rtgpu import scenes
    tris = scenes.random_soup(n, seed=n)
    lb, nodes, ids, keys = gpu_build(gpu_ctx, tris, 18)
    assert_same_tree(oracle_mod, tris, 18, nodes, ids, keys)


def test_build_host_input_and_rebuild(gpu_ctx, oracle_mod):
    """Host soup path, then rebuilds of the same object with other inputs
    (epoch-tagged refit words, reused scratch)."""
    import torch
    from rtgpu import scenes
    from rtgpu.api import LBVH
    lb = LBVH(gpu_ctx, 50000, 18)
    for seed, n in ((31, 50000), (32, 1234), (33, 49999), (31, 50000)):
        tris = scenes.random_soup(n, seed=seed)
        if seed % 2:
            lb.Build(tris)
        else:
            lb.Build(torch.from_numpy(tris).cuda())
        gpu_ctx.check()
        nodes, ids, keys = lb.download(True, True, True)
        assert_same_tree(oracle_mod, tris, 18, nodes, ids, keys)


def test_duplicates_and_flat(gpu_ctx, oracle_mod):
    from rtgpu import scenes
    base = scenes.random_soup(5000, seed=41)
    tris = np.ascontiguousarray(np.concatenate([base, base, base[:777], base[5:900] + np.float32(2e-7)]))
    for depth in (4, 12, 24):
        lb, nodes, ids, keys = gpu_build(gpu_ctx, tris, depth)
        assert_same_tree(oracle_mod, tris, depth, nodes, ids, keys)
    flat = scenes.random_soup(4000, seed=42)
    flat[:, 1::3] = np.float32(-0.25)
    lb, nodes, ids, keys = gpu_build(gpu_ctx, flat, 14)
    assert_same_tree(oracle_mod, flat, 14, nodes, ids, keys)


def test_errors(gpu_ctx):
    import torch
    from rtgpu import _lib as L
    from rtgpu.api import LBVH
    lb = LBVH(gpu_ctx, 100, 8)
    with pytest.raises(L.RtError) as e:
        lb.Build(np.zeros((101, 9), np.float32))
    assert e.value.status == L.RT_ERR_CAPACITY
    with pytest.raises(L.RtError) as e:
        lb.Build(np.zeros((0, 9), np.float32))
    assert e.value.status == L.RT_ERR_INVALID
    with pytest.raises(L.RtError) as e:
        LBVH(gpu_ctx, 10, 0)
    assert e.value.status == L.RT_ERR_INVALID
    bad = np.random.default_rng(0).random((50, 9)).astype(np.float32)
    bad[7, 4] = np.nan
    lb.Build(torch.from_numpy(bad).cuda())
    with pytest.raises(L.RtError) as e:
        gpu_ctx.check()
    assert e.value.status == L.RT_ERR_NONFINITE
    gpu_ctx.check()  # the flag was cleared


def test_context_setter_errors(gpu_ctx):
    """The context's tuning setters refuse out-of-range arguments and leave
    the previous setting in place."""
    from rtgpu import _lib as L
    for call in (lambda: gpu_ctx.set_trace_budget(10, kind=3), lambda: gpu_ctx.set_heavy_block(8)):
        with pytest.raises(L.RtError) as e:
            call()
        assert e.value.status == L.RT_ERR_INVALID
    assert L.lib().rt_ctx_set_tile_order(gpu_ctx.h, 8) == L.RT_ERR_INVALID
    gpu_ctx.set_heavy_block(None)
    gpu_ctx.set_trace_budget(None)
