"""Builds the native libraries in-tree.

* ``_build/librtgb300.so``: the CUDA kernels and the C ABI (``include/rt_api.h``),
  compiled by nvcc for sm_103a only.
* ``host/_build/librthost.so`` and ``host/_build/rt_frame_demo``: the C++
  stage classes that mirror the reference's AccelerationStructure /
  StructureConstruction / RayTracerCS interface on top of the C ABI, and the
  model loader (``include/rt_model.h``).

Translation units are compiled in parallel processes and linked once; a
library is rebuilt only when one of its sources is newer than it.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # raytracer-gpupro4_gb300/
REPO_ROOT = PKG_ROOT.parent
CSRC = PKG_ROOT / "csrc"
HOST = PKG_ROOT / "host"
BUILD = PKG_ROOT / "_build"
HOST_BUILD = HOST / "_build"
INCLUDE = REPO_ROOT / "include"
LIB = BUILD / "librtgb300.so"
HOST_LIB = HOST_BUILD / "librthost.so"
DEMO = HOST_BUILD / "rt_frame_demo"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librtgb300.so")


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def _newer(srcs, out: Path) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(s).stat().st_mtime > t for s in srcs)


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r


def cuda_sources():
    return sorted(CSRC.glob("*.cu"))


def build_cuda(force: bool = False, verbose: bool = False) -> Path:
    srcs = cuda_sources()
    deps = srcs + sorted(CSRC.glob("*.cuh")) + [INCLUDE / "rt_api.h"]
    if not force and not _newer(deps, LIB):
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    objs = []

    def compile_one(src: Path):
        obj = BUILD / (src.stem + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = _run(cmd)
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        for obj, log in ex.map(compile_one, srcs):
            objs.append(obj)
            if verbose and log:
                print(log)
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


def build_host(force: bool = False) -> Path | None:
    """C++ drop-in stage classes (optional: skipped if the sources are absent)."""
    srcs = sorted(HOST.glob("*.cpp"))
    if not srcs:
        return None
    lib_srcs = [s for s in srcs if s.name != "rt_frame_demo.cpp"]
    hdrs = sorted(HOST.glob("*.h"))
    cxx = os.environ.get("CXX", "g++")
    cuda = _cuda_home()
    inc = ["-I", str(INCLUDE), "-I", str(HOST), "-I", str(cuda / "include")]
    cudart = ["-L", str(cuda / "lib64"), "-lcudart", f"-Wl,-rpath,{cuda / 'lib64'}"]
    HOST_BUILD.mkdir(parents=True, exist_ok=True)
    if force or _newer(lib_srcs + hdrs + [INCLUDE / "rt_api.h", INCLUDE / "rt_model.h", LIB], HOST_LIB):
        tmp = HOST_LIB.with_suffix(".so.tmp")
        _run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", *inc, *map(str, lib_srcs), "-o", str(tmp),
              "-L", str(BUILD), "-lrtgb300", f"-Wl,-rpath,{BUILD}", *cudart])
        os.replace(tmp, HOST_LIB)
    demo_src = HOST / "rt_frame_demo.cpp"
    if demo_src.exists() and (force or _newer([demo_src, HOST_LIB] + hdrs, DEMO)):
        _run([cxx, "-O2", "-std=c++17", *inc, str(demo_src), "-o", str(DEMO),
              "-L", str(HOST_BUILD), "-lrthost", "-L", str(BUILD), "-lrtgb300",
              f"-Wl,-rpath,{HOST_BUILD}", f"-Wl,-rpath,{BUILD}", *cudart])
    return HOST_LIB


def build_all(force: bool = False, verbose: bool = False) -> Path:
    lib = build_cuda(force=force, verbose=verbose)
    build_host(force=force)
    return lib
