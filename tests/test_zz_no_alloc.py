"""The allocation-free render entry point (mgpu_render_noalloc) against mgpu_render.

Hosts that forbid device allocation while rendering call mgpu_render_noalloc, which works in a
fixed device array inside libmgpu.so instead of a cudaMalloc'd workspace.  Its images must be
the ones mgpu_render makes.  The film is deterministic and independent of wave size, so the
comparison is exact (tolerance zero); it runs twice in a row because the fixed array keeps the
previous call's contents and each call must clear what has to start at zero.

This file is collected last so that a failure here cannot hide other tests' results; it also
passes when run alone in a fresh process.  One test runs in a child process of its own, so
that the entry point is exercised with no mgpu_render before it in that process, and checks
with cudaMemGetInfo that a call takes no device memory.
"""
import ctypes as C
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _render(pt, lib, ds, settings, noalloc):
    film = pt.Film(settings.width, settings.height)
    p = settings.to_c(ds.scene.camera)
    fn = lib.mgpu_render_noalloc if noalloc else lib.mgpu_render
    rc = fn(ds.handle, C.byref(p), film.handle, None)
    assert rc == 0, lib.mgpu_last_error()
    raw = film.raw()
    film.close()
    return raw


@pytest.mark.parametrize("scene_kind", ["plain", "spheres"])
def test_noalloc_matches_render_twice(cuda, scene_kind):
    from milton_gb300 import _native
    from milton_gb300 import pathtracer as pt
    from milton_gb300 import scenegen
    lib = _native.load()
    if scene_kind == "plain":
        s = scenegen.plain(0)
        settings = pt.RenderSettings(96, 80, 16, max_depth=5, rr_start_depth=3, seed=21)
    else:
        s = scenegen.random_scene(13, 20000)
        settings = pt.RenderSettings(120, 96, 8, max_depth=8, rr_start_depth=3, seed=22)
    ds = pt.DeviceScene(s, pt.Accel(s))
    want = _render(pt, lib, ds, settings, noalloc=False)
    for _ in range(2):  # twice in a row: the fixed scratch keeps the previous call's contents
        got = _render(pt, lib, ds, settings, noalloc=True)
        assert np.array_equal(got, want)
    # unlimited depth (Milton's default estimator) goes through the live-count read-back path
    ref = pt.RenderSettings(64, 64, 4, max_depth=0, rr_start_depth=2, seed=23)
    want = _render(pt, lib, ds, ref, noalloc=False)
    assert np.array_equal(_render(pt, lib, ds, ref, noalloc=True), want)


def test_noalloc_rejects_oversized_requests(cuda):
    from milton_gb300 import _native
    from milton_gb300 import pathtracer as pt
    from milton_gb300 import scenegen
    lib = _native.load()
    s = scenegen.plain(0)
    ds = pt.DeviceScene(s, pt.Accel(s))
    film = pt.Film(64, 64)
    # a wave of 2^20 paths does not fit the 32 MiB fixed scratch: rejected, film untouched
    p = pt.RenderSettings(64, 64, 16, max_depth=5, rr_start_depth=3, wave_paths=1 << 20).to_c(s.camera)
    rc = lib.mgpu_render_noalloc(ds.handle, C.byref(p), film.handle, None)
    assert rc == -1
    assert b"exceeds the fixed scratch" in lib.mgpu_last_error()
    assert not film.raw().any()


_CHILD = textwrap.dedent("""
    import ctypes as C
    import numpy as np
    import torch
    from milton_gb300 import _native
    from milton_gb300 import pathtracer as pt
    from milton_gb300 import scenegen
    torch.cuda.set_device(0)
    lib = _native.load()
    s = scenegen.plain(0)
    ds = pt.DeviceScene(s, pt.Accel(s))
    films = [pt.Film(160, 120) for _ in range(3)]
    st = pt.RenderSettings(160, 120, 16, max_depth=5, rr_start_depth=3, seed=31)
    p = st.to_c(s.camera)
    torch.cuda.synchronize()
    # the first render call of this process is the allocation-free one; under lazy module
    # loading it is the call that loads the rendering module (and with it the fixed array)
    assert lib.mgpu_render_noalloc(ds.handle, C.byref(p), films[0].handle, None) == 0, lib.mgpu_last_error()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    assert lib.mgpu_render_noalloc(ds.handle, C.byref(p), films[1].handle, None) == 0, lib.mgpu_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, ("device memory taken by an allocation-free call", free0 - free1)
    assert lib.mgpu_render(ds.handle, C.byref(p), films[2].handle, None) == 0, lib.mgpu_last_error()
    a, b, c = (f.raw() for f in films)
    assert np.array_equal(a, c) and np.array_equal(b, c)
    print("ok", free0 - free1)
""")


def test_noalloc_first_call_in_a_fresh_process_takes_no_device_memory(cuda):
    root = Path(__file__).resolve().parent.parent
    r = subprocess.run([sys.executable, "-c", _CHILD], cwd=root, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok 0")
