"""rt_lbvh_build_noalloc: the allocation-free rebuild, for callers that may
not allocate device memory at rebuild time (a host capturing its frame into
a CUDA graph, an engine whose allocator owns all device memory, a real-time
loop that cannot absorb an allocation's implicit synchronisation).

Called through the C ABI on two different soups in a row; each result must
equal rt_lbvh_build's on the same soup bit for bit (the tolerance of every
build parity test), and a call must leave the device's free memory
unchanged.  The file is collected last, so a failure here leaves every other
test already run; it passes alone and after the others alike."""
import ctypes as C

import numpy as np
import pytest

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
    return lib.rt_lbvh_build_noalloc(ctx.h, st, _ptr(tris_dev), tris_dev.shape[0], depth, flags, _ptr(out.nodes),
                                     _ptr(out.ids), _ptr(out.keys), _ptr(out.sorted_tris))


def test_noalloc_build_matches_rt_lbvh_build_twice(gpu_ctx):
    import torch
    from rtgpu import _lib as L
    from rtgpu import scenes
    from rtgpu.api import LBVH
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
        lb = LBVH(gpu_ctx, len(soup), depth)
        lb.Build(tris, L.RT_BUILD_CLEAR_UNREACHED)
        rn, ri, rk = lb.download(True, True, True)
        lb.close()
        assert np.array_equal(out.nodes.cpu().numpy().view(L.NODE_DTYPE), rn), f"call {k}: nodes differ"
        assert np.array_equal(out.ids.cpu().numpy().view(np.uint32), ri), f"call {k}: ids differ"
        assert np.array_equal(out.keys.cpu().numpy().view(np.uint32), rk), f"call {k}: keys differ"
        # pre-gathered triangles: A.xyz,id | B.xyz,0 | C.xyz,0 in sorted order
        st = out.sorted_tris.cpu().numpy().reshape(-1, 12)
        exp = np.zeros_like(st)
        exp[:, 0:3] = soup[ri, 0:3]
        exp[:, 3] = ri.astype(np.int32).view(np.float32)
        exp[:, 4:7] = soup[ri, 3:6]
        exp[:, 8:11] = soup[ri, 6:9]
        assert np.array_equal(st.view(np.uint32), exp.view(np.uint32)), f"call {k}: sorted triangles differ"


def test_noalloc_rejects_sizes_beyond_the_fixed_scratch(gpu_ctx):
    import torch
    from rtgpu import _lib as L
    lib = L.lib()
    big = torch.zeros((L.RT_NOALLOC_MAX_TRIS + 1, 9), dtype=torch.float32, device="cuda")
    assert _noalloc_build(lib, gpu_ctx, big, 12, Outputs(16, 12)) == L.RT_ERR_CAPACITY
    assert b"exceeds the fixed scratch" in lib.rt_last_error(gpu_ctx.h)
    small = torch.zeros((16, 9), dtype=torch.float32, device="cuda")
    assert _noalloc_build(lib, gpu_ctx, small, L.RT_NOALLOC_MAX_DEPTH + 1, Outputs(16, 1)) == L.RT_ERR_CAPACITY
