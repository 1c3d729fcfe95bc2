"""The sort stage (rt_radix_sort) against known answers and a stable CPU
sort, and the bounded look-back wait made to run out.

The known-answer case is the reference's own sort check
(RayTracerCS/RadixSort.cpp:67-73): 512 x 512 elements holding the
reverse-order pattern (1023 - (i % 1024)) * 1024.  A stable ascending sort
of it has a closed form: position p holds (p // 256) * 1024, and the
elements with that key keep their input order, ids (1023 - p // 256) +
1024 * (p % 256).  Keys and values are compared bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sort(ctx, keys_np, vals_np=None):
    import torch
    from rtgpu.api import RadixSort
    n = len(keys_np)
    if vals_np is None:
        vals_np = np.arange(n, dtype=np.uint32)
    k = torch.from_numpy(keys_np.astype(np.uint32).view(np.int32)).cuda()
    v = torch.from_numpy(vals_np.astype(np.uint32).view(np.int32)).cuda()
    RadixSort(ctx).Sort(k, v)
    ctx.check()
    return k.cpu().numpy().view(np.uint32), v.cpu().numpy().view(np.uint32)


def test_reference_reverse_pattern_kat(gpu_ctx):
    n = 512 * 512
    i = np.arange(n, dtype=np.int64)
    keys = ((1023 - (i % 1024)) * 1024).astype(np.uint32)
    k, v = _sort(gpu_ctx, keys)
    p = np.arange(n, dtype=np.int64)
    assert np.array_equal(k, ((p // 256) * 1024).astype(np.uint32))
    assert np.array_equal(v, ((1023 - p // 256) + 1024 * (p % 256)).astype(np.uint32))


@pytest.mark.parametrize("n", [1, 2, 4095, 4096, 4097, 100_003, 32 * 4096 + 1, 33 * 4096, 2_099_520])
def test_random_keys_match_stable_cpu_sort(gpu_ctx, n):
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    keys[: n // 3] = keys[0]  # a long run of equal keys: stability shows
    vals = rng.permutation(n).astype(np.uint32)
    k, v = _sort(gpu_ctx, keys, vals)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order])
    assert np.array_equal(v, vals[order])


def test_extreme_keys_and_empty_input(gpu_ctx):
    from rtgpu import _lib as L
    keys = np.array([0xFFFFFFFF, 0, 0xFFFFFFFF, 1, 0x80000000, 0xFFFFFFFF, 0], np.uint32)
    k, v = _sort(gpu_ctx, keys)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order]) and np.array_equal(v, order.astype(np.uint32))
    # n = 0 sorts nothing and succeeds (no buffer is touched)
    assert L.lib().rt_radix_sort(gpu_ctx.h, None, None, 0, None, 0) == L.RT_OK


def test_scratch_too_small_is_rejected(gpu_ctx):
    import ctypes as C
    import torch
    from rtgpu import _lib as L
    n = 10_000
    k = torch.zeros(n, dtype=torch.int32, device="cuda")
    v = torch.zeros(n, dtype=torch.int32, device="cuda")
    need = L.lib().rt_radix_sort_scratch_bytes(n)
    sc = torch.empty(need // 4, dtype=torch.int32, device="cuda")
    st = L.lib().rt_radix_sort(gpu_ctx.h, C.c_void_p(k.data_ptr()), C.c_void_p(v.data_ptr()), n,
                               C.c_void_p(sc.data_ptr()), need - 4)
    assert st == L.RT_ERR_CAPACITY
    assert b"needed" in L.lib().rt_last_error(gpu_ctx.h)


def test_lookback_wait_runs_out_and_the_next_build_is_correct(gpu_ctx, oracle_mod):
    """The look-back of a radix pass waits for the digit counts of the
    earlier tiles of its group.  The stall hook never starts the first tile,
    so the waits of the other tiles of its group can never end: they must
    give up after the given number of polls, report RT_ERR_TIMEOUT through
    rt_ctx_check, leave the inputs untouched, and leave the context usable
    (a full build after it equals the oracle)."""
    import torch
    from rtgpu import _lib as L
    from rtgpu import scenes
    from rtgpu.api import LBVH, RadixSort
    n = 50_000
    rng = np.random.default_rng(7)
    keys = rng.integers(0, 1 << 30, n, dtype=np.int64).astype(np.uint32)
    k = torch.from_numpy(keys.view(np.int32)).cuda()
    v = torch.arange(n, dtype=torch.int32, device="cuda")
    rs = RadixSort(gpu_ctx)
    assert rs.stall_test(k, v, 300) == L.RT_OK
    with pytest.raises(L.RtError) as exc:
        gpu_ctx.check()
    assert exc.value.status == L.RT_ERR_TIMEOUT
    gpu_ctx.check()  # the flag was cleared by the check that reported it
    assert np.array_equal(k.cpu().numpy().view(np.uint32), keys)
    assert np.array_equal(v.cpu().numpy(), np.arange(n, dtype=np.int32))
    # a bad spin limit or a one-tile input is refused without a launch
    assert rs.stall_test(k[:4096], v[:4096], 300) == L.RT_ERR_INVALID
    assert rs.stall_test(k, v, 0) == L.RT_ERR_INVALID
    # the context and the sort still work
    tris = scenes.random_soup(30_000, seed=11)
    lb = LBVH(gpu_ctx, len(tris), 16).Build(torch.from_numpy(tris).cuda())
    gpu_ctx.check()
    nodes, ids, okeys = lb.download(True, True, True)
    onodes, oids, ookeys, reached = oracle_mod.lbvh_build(tris, 16)
    assert np.array_equal(okeys, ookeys) and np.array_equal(ids, oids)
    r = np.nonzero(reached)[0]
    assert np.array_equal(nodes[r].view(np.uint32), onodes[r].view(np.uint32))
    lb.close()
    k2, v2 = _sort(gpu_ctx, keys)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k2, keys[order]) and np.array_equal(v2, order.astype(np.uint32))
