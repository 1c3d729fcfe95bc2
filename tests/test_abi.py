"""The C ABI library loads and exports every entry point include/rt_api.h
declares (no compute call: this runs without a GPU)."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    txt = (ROOT / "include" / "rt_api.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(rt_[a-z0-9_]+)\s*\(", txt)))


def test_header_parses():
    syms = declared_symbols()
    assert "rt_lbvh_build" in syms and "rt_trace_primary" in syms and len(syms) >= 20


def test_library_exports_every_declared_symbol(rt_lib):
    missing = [s for s in declared_symbols() if not hasattr(rt_lib, s)]
    assert not missing, missing


def test_binding_covers_header(rt_lib):
    from rtgpu import _lib
    assert sorted(_lib.EXPORTED) == declared_symbols()


def test_status_strings_and_version(rt_lib):
    assert rt_lib.rt_api_version() == 1
    assert rt_lib.rt_status_string(0) == b"RT_OK"
    assert rt_lib.rt_status_string(4) == b"RT_ERR_TIMEOUT"


def test_layouts():
    from rtgpu import _lib
    assert _lib.NODE_DTYPE.itemsize == 32  # LBVHNode, LBVH.h:25-28
    assert _lib.HIT_DTYPE.itemsize == 16
    assert _lib.RAY_DTYPE.itemsize == 32


def test_null_handles_are_refused_without_touching_the_device(rt_lib):
    """Entry points given a null context or object return before any CUDA
    call: RT_ERR_INVALID, or RT_OK for the destroy calls (this runs without a
    GPU)."""
    import ctypes as C
    from rtgpu import _lib as L
    lib = L.lib()
    t = C.c_uint64()
    assert lib.rt_pipe_submit(None, None, None, None, None, C.byref(t)) == L.RT_ERR_INVALID
    assert lib.rt_pipe_wait(None, 0) == L.RT_ERR_INVALID
    assert lib.rt_pipe_create(None, None, 1, 0, None, None, 1, 1, None) == L.RT_ERR_INVALID
    assert lib.rt_frame_launch(None, None) == L.RT_ERR_INVALID
    assert lib.rt_lbvh_build(None, None, None, 1, 0) == L.RT_ERR_INVALID
    assert lib.rt_batch_build(None, None, None, 0) == L.RT_ERR_INVALID
    assert lib.rt_radix_sort(None, None, None, 1, None, 0) == L.RT_ERR_INVALID
    assert lib.rt_trace_primary(None, None, None, None, None) == L.RT_ERR_INVALID
    assert lib.rt_pathtrace(None, None, None, None, None, None, None) == L.RT_ERR_INVALID
    for destroy in ("rt_pipe_destroy", "rt_frame_destroy", "rt_lbvh_destroy", "rt_batch_destroy", "rt_ctx_destroy"):
        assert getattr(lib, destroy)(None) == L.RT_OK, destroy
