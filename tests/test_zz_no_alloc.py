"""rt_lbvh_build_noalloc: the allocation-free rebuild, for callers that
cannot call cudaMalloc when they rebuild -- an engine whose own allocator
owns all device memory (a caching pool that has reserved the free memory,
or a budgeted heap that must account for every byte), or a real-time loop
that cannot absorb the device-wide synchronisation of an allocation.

Called through the C ABI on two different soups in a row; each result must
equal rt_lbvh_build's on the same soup bit for bit (the tolerance of every
build parity test), and a call must leave the device's free memory
unchanged.  The limits of the fixed scratch (262,144 triangles, depth 20)
are run too, and device-side errors reach rt_ctx_check.  The file is
collected last, so a failure here leaves every other test already run; it
passes alone and after the others alike."""
import ctypes as C

import numpy as np
import pytest

from bitcmp import same_bits

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr())


class Outputs:
    """Caller-owned output buffers of one rebuild."""

    def __init__(self, n, depth):
        import torch
        self.nodes = torch.zeros((1 << depth) * 8, dtype=torch.int32, device="cuda")
        self.ids = torch.zeros(n, dtype=torch.int32, device="cuda")
        self.keys = torch.zeros(n, dtype=torch.int32, device="cuda")
        self.sorted_tris = torch.zeros(n * 12, dtype=torch.float32, device="cuda")


def _noalloc_build(lib, ctx, tris_dev, depth, out, flags=0):
    import torch
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return lib.rt_lbvh_build_noalloc(ctx.h if ctx is not None else None, st, _ptr(tris_dev), tris_dev.shape[0], depth,
                                     flags, _ptr(out.nodes), _ptr(out.ids), _ptr(out.keys), _ptr(out.sorted_tris))


def _check_against_rt_lbvh_build(gpu_ctx, soup, tris, depth, out, what):
    from rtgpu import _lib as L
    from rtgpu.api import LBVH
    lb = LBVH(gpu_ctx, len(soup), depth)
    lb.Build(tris, L.RT_BUILD_CLEAR_UNREACHED)
    rn, ri, rk = lb.download(True, True, True)
    lb.close()
    assert same_bits(out.nodes.cpu().numpy().view(L.NODE_DTYPE), rn), f"{what}: nodes differ"
    assert np.array_equal(out.ids.cpu().numpy().view(np.uint32), ri), f"{what}: ids differ"
    assert np.array_equal(out.keys.cpu().numpy().view(np.uint32), rk), f"{what}: keys differ"
    # pre-gathered triangles: A.xyz,id | B.xyz,0 | C.xyz,0 in sorted order
    st = out.sorted_tris.cpu().numpy().reshape(-1, 12)
    exp = np.zeros_like(st)
    exp[:, 0:3] = soup[ri, 0:3]
    exp[:, 3] = ri.astype(np.int32).view(np.float32)
    exp[:, 4:7] = soup[ri, 3:6]
    exp[:, 8:11] = soup[ri, 6:9]
    assert same_bits(st, exp), f"{what}: sorted triangles differ"


def test_noalloc_build_matches_rt_lbvh_build_twice(gpu_ctx):
    import torch
    from rtgpu import _lib as L
    from rtgpu import scenes
    lib = L.lib()
    depth = 18
    soups = [scenes.random_soup(200_000, seed=901), scenes.torus(256, 120)]
    for k, soup in enumerate(soups):
        tris = torch.from_numpy(soup).cuda()
        out = Outputs(len(soup), depth)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        status = _noalloc_build(lib, gpu_ctx, tris, depth, out, L.RT_BUILD_CLEAR_UNREACHED)
        assert status == L.RT_OK, lib.rt_last_error(gpu_ctx.h)
        torch.cuda.synchronize()
        if k > 0:  # the first call on a device does the one-time set-up
            assert torch.cuda.mem_get_info()[0] == free_before, "the call allocated device memory"
        gpu_ctx.check()
        _check_against_rt_lbvh_build(gpu_ctx, soup, tris, depth, out, f"call {k}")


def test_noalloc_build_at_the_documented_limits(gpu_ctx):
    """262,144 triangles at depth 20: every scratch region at its full size."""
    import torch
    from rtgpu import _lib as L
    from rtgpu import scenes
    lib = L.lib()
    depth = L.RT_NOALLOC_MAX_DEPTH
    soup = scenes.random_soup(L.RT_NOALLOC_MAX_TRIS, seed=907)
    tris = torch.from_numpy(soup).cuda()
    out = Outputs(len(soup), depth)
    for call in range(2):
        assert _noalloc_build(lib, gpu_ctx, tris, depth, out, L.RT_BUILD_CLEAR_UNREACHED) == L.RT_OK
        gpu_ctx.check()
    _check_against_rt_lbvh_build(gpu_ctx, soup, tris, depth, out, "limits")


def test_noalloc_reports_a_nonfinite_soup_through_the_context(gpu_ctx):
    import torch
    from rtgpu import _lib as L
    from rtgpu import scenes
    lib = L.lib()
    soup = scenes.random_soup(5000, seed=911)
    soup[1234, 4] = np.nan
    tris = torch.from_numpy(soup).cuda()
    out = Outputs(len(soup), 14)
    assert _noalloc_build(lib, gpu_ctx, tris, 14, out) == L.RT_OK  # the launch itself succeeds
    with pytest.raises(L.RtError) as exc:
        gpu_ctx.check()
    assert exc.value.status == L.RT_ERR_NONFINITE
    gpu_ctx.check()  # reported once, then cleared
    # without a context the call still runs (its errors are not reported)
    good = torch.from_numpy(scenes.random_soup(5000, seed=912)).cuda()
    assert _noalloc_build(lib, None, good, 14, out) == L.RT_OK
    torch.cuda.synchronize()
    gpu_ctx.check()


def test_noalloc_rejects_sizes_beyond_the_fixed_scratch_and_other_flags(gpu_ctx):
    import torch
    from rtgpu import _lib as L
    lib = L.lib()
    big = torch.zeros((L.RT_NOALLOC_MAX_TRIS + 1, 9), dtype=torch.float32, device="cuda")
    assert _noalloc_build(lib, gpu_ctx, big, 12, Outputs(16, 12)) == L.RT_ERR_CAPACITY
    assert b"exceeds the fixed scratch" in lib.rt_last_error(gpu_ctx.h)
    small = torch.zeros((16, 9), dtype=torch.float32, device="cuda")
    assert _noalloc_build(lib, gpu_ctx, small, L.RT_NOALLOC_MAX_DEPTH + 1, Outputs(16, 1)) == L.RT_ERR_CAPACITY
    assert _noalloc_build(lib, gpu_ctx, small, 8, Outputs(16, 8), L.RT_BUILD_COMPACT) == L.RT_ERR_INVALID
    assert b"only RT_BUILD_CLEAR_UNREACHED" in lib.rt_last_error(gpu_ctx.h)
