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
