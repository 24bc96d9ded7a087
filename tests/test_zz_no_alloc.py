"""The allocation-free render entry point (mgpu_render_noalloc) against mgpu_render.

Hosts that forbid device allocation while rendering call mgpu_render_noalloc, which works in a
fixed device array inside libmgpu.so instead of a cudaMalloc'd workspace.  Its images must be
the ones mgpu_render makes.  The film is deterministic and independent of wave size, so the
comparison is exact (tolerance zero); it runs twice in a row because the fixed array keeps the
previous call's contents and each call must clear what has to start at zero.

This file is collected last so that a failure here cannot hide other tests' results; it also
passes when run alone in a fresh process.
"""
import ctypes as C

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
