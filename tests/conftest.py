"""Test configuration: the `gpu` marker and import paths.

CPU tests (-m "not gpu") cover the oracle against the golden fixtures made
by the reference's own code, the emission algorithm's host model, the scene
generators and the C ABI library's exported symbols.  GPU tests (-m gpu)
are the parity tests proper; they call the CUDA kernels through the C ABI
and compare with the oracle.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT / "raytracer-gpupro4_gb300", ROOT / "oracle", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle as O
    O.build_oracle()
    return O


@pytest.fixture(scope="session")
def rt_lib():
    from rtgpu import build, _lib
    build.build_cuda()
    return _lib.lib()


@pytest.fixture(scope="session")
def gpu_ctx(rt_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from rtgpu.api import Context
    ctx = Context(0)
    yield ctx
    ctx.close()


def golden_cases():
    return sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load_golden(name):
    import numpy as np
    return dict(np.load(GOLDEN / f"{name}.npz"))


def camera_from_array(a):
    from rtgpu._lib import Camera
    cam = Camera()
    for k, f in enumerate(("eye", "right", "up", "fwd")):
        arr = getattr(cam, f)
        for c in range(3):
            arr[c] = float(a[3 * k + c])
    cam.tan_half_fovy = float(a[12])
    cam.width = int(a[13])
    cam.height = int(a[14])
    return cam
