import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (str(ROOT), str(ROOT / "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libmgpu.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.load()
    return pyoracle


@pytest.fixture(scope="session")
def hostcheck():
    import ctypes as C
    from native import build as hb
    lib = C.CDLL(str(hb.build()))
    vp = C.c_void_p
    lib.hc_trace.argtypes = [vp, vp, C.c_int64, vp, C.c_int64, vp, vp, vp, C.c_uint32, C.c_int]
    lib.hc_trace.restype = C.c_int
    lib.hc_bsdf_sample.argtypes = [vp, vp, vp, C.c_int, vp, vp, vp]
    lib.hc_bsdf_sample.restype = C.c_int
    lib.hc_bsdf_eval.argtypes = [vp, vp, vp, vp, vp]
    lib.hc_uniforms.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32, vp]
    lib.hc_offset.argtypes = [vp, vp, vp]
    lib.hc_light_point.argtypes = [vp, vp, vp, vp, vp, vp]
    lib.hc_camera_ray.argtypes = [vp, C.c_float, C.c_float, C.c_float, C.c_float, vp]
    return lib


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    from milton_gb300 import _native
    _native.load()
    return torch
