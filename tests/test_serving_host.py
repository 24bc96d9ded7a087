"""Render-service host logic without a GPU: scene library, background kd-tree builds, job
queue, argument checks, and the film error estimate's host model."""
import numpy as np
import pytest

from milton_gb300 import scenegen
from milton_gb300.parallel import kahan_film
from milton_gb300.pathtracer import RenderSettings, rmse_estimate


def test_rmse_estimate_matches_direct_variance():
    rng = np.random.default_rng(3)
    h, w, n = 6, 5, 12
    paths = rng.gamma(0.7, 0.4, (h, w, n, 3)).astype(np.float32)
    raw = kahan_film(paths)
    lum = paths.astype(np.float64).mean(-1)
    var = lum.var(axis=2, ddof=1)
    want = np.sqrt(np.mean(var / n))
    assert rmse_estimate(raw) == pytest.approx(want, rel=1e-5)
    # one sample per pixel: no variance estimate
    assert rmse_estimate(kahan_film(paths[:, :, :1])) == float("inf")


def test_server_queue_and_builds_without_gpu():
    from milton_gb300 import _native as N
    from milton_gb300.serving import Server, ServerSettings
    with Server(ServerSettings(build_threads=2)) as srv:
        a = srv.add_scene(scenegen.plain(0))
        b = srv.add_scene(scenegen.random_scene(4, 5000))
        srv.prefetch(a)
        srv.prefetch(b)
        srv.wait_builds()
        st = srv.stats()
        assert st["builds"] == 2 and st["building"] == 0 and st["resident_scenes"] == 0
        s = scenegen.plain(0)
        rs = RenderSettings(16, 16, 4, max_depth=5, rr_start_depth=3)
        j0 = srv.submit(a, rs, s.camera, 16, 0.0, arrival=1e9)  # arrives far in the future
        j1 = srv.submit(b, rs, s.camera, 4, 0.05, arrival=5e8)
        info = srv.job(j0)
        assert info["state"] == "queued" and info["spp_done"] == 0 and np.isnan(info["t_admit"])
        assert srv.stats()["queued"] == 2
        # bad requests are refused before they queue
        with pytest.raises(N.MgpuError, match="unknown scene"):
            srv.submit(7, rs, s.camera, 4)
        with pytest.raises(N.MgpuError, match="bad parameters"):
            srv.submit(a, rs, s.camera, 0)
        with pytest.raises(N.MgpuError, match="bad parameters"):
            srv.submit(a, RenderSettings(0, 16, 4), s.camera, 4)
        with pytest.raises(N.MgpuError, match="no film"):
            srv.read(j1)
        # releasing a queued job cancels it
        srv.release(j1)
        assert srv.job(j1)["state"] == "failed"
        st = srv.stats()
        assert st["queued"] == 1 and st["failed"] == 1 and st["resident_bytes"] == 0


def test_server_rejects_bad_arguments():
    import ctypes as C
    from milton_gb300 import _native as N
    lib = N.load()
    p = N.ServerParams()
    p.tick_paths = -1
    out = C.c_void_p()
    assert lib.mgpu_server_create(C.byref(p), C.byref(out)) == -1
    assert lib.mgpu_server_step(None, None, None) == -1
    assert lib.mgpu_film_error(None, 1, None, None) == -1
    assert lib.mgpu_film_error(None, 0, None, None) == 0
