"""Render service on the GPU (mgpu_server_*): each job's image is the same alone and in the mix,
equals a plain render with the same number of samples, admission respects the memory budget,
and the film error estimate agrees with its host model and with the measured error."""
import numpy as np
import pytest

from milton_gb300 import pathtracer as pt
from milton_gb300 import scenegen
from milton_gb300.serving import Server, ServerSettings, replay, latency_summary

pytestmark = pytest.mark.gpu


def _scenes():
    return [scenegen.plain(0), scenegen.random_scene(21, 4000), scenegen.random_scene(22, 20000)]


# (scene, side, spp stratification, max_spp, target_rmse)
JOBS = [(0, 48, 4, 64, 0.0), (1, 40, 4, 32, 0.05), (2, 64, 1, 16, 0.0), (0, 24, 16, 256, 0.02),
        (1, 56, 4, 8, 0.0), (2, 32, 4, 128, 0.04), (0, 8, 1, 1, 0.0)]


def _settings(k, side, spp):
    return pt.RenderSettings(side, side, spp, max_depth=6, rr_start_depth=3, seed=100 + k)


def _run(scenes, jobs, settings=None, keys=None):
    """Serves jobs (scene, side, spp, max_spp, target); keys[i] seeds job i (default i)."""
    keys = list(range(len(jobs))) if keys is None else keys
    with Server(settings or ServerSettings(tick_paths=20000)) as srv:
        ids = [srv.add_scene(s) for s in scenes]
        jids = []
        for k, (si, side, spp, mx, tgt) in zip(keys, jobs):
            jids.append(srv.submit(ids[si], _settings(k, side, spp), scenes[si].camera, mx, tgt))
        peak = 0
        res = {}
        for _ in range(100000):  # a stalled server fails the test instead of hanging it
            left = srv.step()
            peak = max(peak, srv.stats()["resident_bytes"])
            # a finished job's film stays resident (and counted) until the client releases it
            for j in jids:
                if j not in res:
                    info = srv.job(j)
                    if info["state"] in ("done", "failed"):
                        res[j] = (info, srv.read(j) if info["state"] == "done" else None)
                        srv.release(j)
            if left == 0:
                break
        else:
            raise AssertionError(f"server did not finish: {srv.stats()}")
        return [res[j] for j in jids], srv.stats(), peak


@pytest.mark.parametrize("policy", ["fair", "oldest", "rotate"])
def test_same_image_alone_and_in_the_mix(cuda, policy):
    scenes = _scenes()
    mix, st, _ = _run(scenes, JOBS, ServerSettings(tick_paths=20000, policy=policy))
    assert st["finished"] == len(JOBS) and st["failed"] == 0
    assert st["ticks"] > 3  # the small tick budget spreads the jobs over many shared ticks
    stopped_early = 0
    for k, job in enumerate(JOBS):
        info_m, img_m = mix[k]
        (info_a, img_a), = _run(scenes, [job], keys=[k])[0]
        assert info_m["state"] == info_a["state"] == "done"
        assert info_m["spp_done"] == info_a["spp_done"]
        assert info_m["rmse"] == info_a["rmse"]
        assert np.array_equal(img_m, img_a), f"job {k}: image differs alone and in the mix"
        stopped_early += info_m["spp_done"] < job[3]
        if info_m["reached_target"]:
            assert info_m["rmse"] <= job[4]
        else:
            assert info_m["spp_done"] == job[3]
    assert stopped_early >= 1  # some error target was met before the cap


def test_jobs_admitted_while_others_render_match_alone(cuda):
    """Continuous batching: jobs are submitted between ticks while earlier jobs are on the GPU
    (active, part of their samples done); each still finishes with the image and sample count it
    gets alone."""
    scenes = _scenes()
    # (ticks to run before submitting the next group, jobs of the group)
    schedule = [(0, [0, 1]), (2, [2, 3]), (1, [4]), (3, [5, 6])]
    with Server(ServerSettings(tick_paths=20000, policy="rotate")) as srv:
        ids = [srv.add_scene(s) for s in scenes]
        jids = {}
        res = {}
        overlapped = 0

        def harvest():
            for k, j in jids.items():
                if k not in res:
                    info = srv.job(j)
                    if info["state"] in ("done", "failed"):
                        res[k] = (info, srv.read(j) if info["state"] == "done" else None)
                        srv.release(j)

        for ticks, group in schedule:
            for _ in range(ticks):
                srv.step()
                harvest()
            # the jobs already on the GPU with part of their samples rendered
            mid = [k for k, j in jids.items() if k not in res and srv.job(j)["state"] == "active"
                   and 0 < srv.job(j)["spp_done"] < JOBS[k][3]]
            overlapped += bool(mid) and bool(jids)
            for k in group:
                si, side, spp, mx, tgt = JOBS[k]
                jids[k] = srv.submit(ids[si], _settings(k, side, spp), scenes[si].camera, mx, tgt)
        for _ in range(100000):
            left = srv.step()
            harvest()
            if left == 0:
                break
        harvest()
    assert overlapped >= 2, "later groups must arrive while earlier jobs are mid-render"
    assert sorted(res) == list(range(len(JOBS)))
    for k, job in enumerate(JOBS):
        info_m, img_m = res[k]
        (info_a, img_a), = _run(scenes, [job], keys=[k])[0]
        assert info_m["state"] == info_a["state"] == "done"
        assert info_m["spp_done"] == info_a["spp_done"]
        assert np.array_equal(img_m, img_a), f"job {k}: image differs alone and admitted mid-stream"


def test_served_image_equals_plain_render(cuda):
    scenes = _scenes()
    mix, _, _ = _run(scenes, JOBS)
    for k, (si, side, spp, mx, tgt) in enumerate(JOBS):
        info, img = mix[k]
        acc = pt.Accel(scenes[si])
        ds = pt.DeviceScene(scenes[si], acc)
        f = pt.Film(side, side)
        st = _settings(k, side, spp)
        st.sample_count = info["spp_done"]
        pt.render(ds, st, f)
        assert np.array_equal(f.mean(), img)
        if info["spp_done"] > 1:
            assert pt.film_error([f])[0] == info["rmse"]


def test_admission_respects_the_memory_budget(cuda):
    scenes = _scenes()
    # room for the largest scene plus one film of the largest job, not for two scenes
    sizes = []
    for s in scenes:
        acc = pt.Accel(s)
        sizes.append(pt.DeviceScene(s, acc).nbytes)
    budget = max(sizes) + 64 * 64 * 32 + 1024
    assert budget < sorted(sizes)[-1] + sorted(sizes)[-2] + 24 * 24 * 32
    solo, _, _ = _run(scenes, JOBS)
    tight, st, peak = _run(scenes, JOBS, ServerSettings(hbm_budget=budget, tick_paths=20000))
    assert st["finished"] == len(JOBS)
    assert st["peak_resident_bytes"] <= budget and peak <= budget
    assert st["evictions"] >= 1 and st["uploads"] >= len(scenes)
    for (ia, a), (ib, b) in zip(solo, tight):
        assert ia["spp_done"] == ib["spp_done"] and np.array_equal(a, b)
    # a job that can never fit fails instead of blocking the queue
    with Server(ServerSettings(hbm_budget=1000)) as srv:
        sid = srv.add_scene(scenes[0])
        j = srv.submit(sid, _settings(0, 32, 1), scenes[0].camera, 1)
        for _ in range(100000):
            if srv.step() == 0:
                break
        assert srv.job(j)["state"] == "failed"


def test_film_error_matches_host_model_and_measured_error(cuda):
    s = scenegen.plain(0)
    acc = pt.Accel(s)
    ds = pt.DeviceScene(s, acc)
    W = H = 32
    films = []
    for n in (4, 16, 64):
        f = pt.Film(W, H)
        pt.render(ds, pt.RenderSettings(W, H, n, max_depth=5, rr_start_depth=3, seed=1), f)
        films.append(f)
    dev = pt.film_error(films)
    for f, e in zip(films, dev):
        assert e == pytest.approx(pt.rmse_estimate(f.raw()), rel=1e-9)
    assert dev[0] > dev[1] > dev[2]
    # the estimate falls as 1 / sqrt(n) ...
    assert 0.35 < dev[1] / dev[0] < 0.65 and 0.35 < dev[2] / dev[1] < 0.65
    # ... and bounds the measured luminance RMSE against a converged image of independent
    # samples (other seed): the sample variance counts the spread between a pixel's sub-pixel
    # strata, which the stratified mean does not suffer, so the estimate errs on the safe side
    ref = pt.Film(W, H)
    pt.render(ds, pt.RenderSettings(W, H, 4096, max_depth=5, rr_start_depth=3, seed=77), ref)
    lum_ref = ref.mean().mean(-1)
    for f, e in zip(films, dev):
        measured = np.sqrt(np.mean((f.mean().mean(-1) - lum_ref) ** 2))
        print(f"rmse estimate {e:.4f}, measured {measured:.4f}")
        assert 0.2 * e < measured < 1.2 * e, (measured, e)


def test_replay_reports_latency(cuda):
    scenes = _scenes()
    reqs = [dict(id=k, arrival=0.01 * k, job=j) for k, j in enumerate(JOBS)]
    with Server(ServerSettings(tick_paths=50000)) as srv:
        ids = [srv.add_scene(s) for s in scenes]
        for i in ids:
            srv.prefetch(i)
        srv.wait_builds()
        seen = []

        def make(r):
            si, side, spp, mx, tgt = r["job"]
            return ids[si], _settings(r["id"], side, spp), scenes[si].camera, mx, tgt

        infos, _ = replay(srv, reqs, make, on_done=lambda r, j, i: seen.append(srv.read(j).shape))
        lat = latency_summary(infos)
        assert lat["jobs"] == len(JOBS) and lat["failed"] == 0
        assert 0 < lat["p50_s"] <= lat["p99_s"] <= lat["max_s"]
        assert len(seen) == len(JOBS)
        for v in infos.values():
            assert v["t_arrival"] <= v["t_admit"] <= v["t_done"]
        assert srv.stats()["film_bytes"] == 0  # every film released


def test_served_textured_and_sphere_scenes_equal_plain_renders(cuda):
    # the service owns copies of image maps, uvs, backgrounds and spheres: served images of such
    # scenes equal their plain renders with the same sample counts
    from milton_gb300.scene import SceneBuilder, dielectric
    tex = scenegen.textured(9)
    tex.background_le = np.array([0.1, 0.2, 0.3], np.float32)
    b = SceneBuilder()
    s0 = scenegen.plain(9)
    for name, first, count in s0.shapes:
        b.add(name, s0.tri_v[first:first + count], s0.tri_n[first:first + count],
              b.material(s0.materials[s0.tri_mat[first]]),
              light=int(s0.tri_light[first]) if s0.tri_light[first] >= 0 else -1)
    for rec, ext in zip(s0.lights, s0.light_ext):
        b.add_light(rec, ext)
    b.add_sphere((0.1, 0.4, 0.2), 0.3, b.material(dielectric([1.4, 1.5, 1.7])))
    sph = b.build(s0.camera)
    scenes = [tex, sph]
    jobs = [(0, 32, 4, 16, 0.0), (1, 40, 4, 16, 0.0), (0, 24, 1, 4, 0.0)]
    served, _, _ = _run(scenes, jobs)
    for k, ((si, side, spp, mx, _), (info, img)) in enumerate(zip(jobs, served)):
        st = _settings(k, side, spp)
        st.sample_count = info["spp_done"]
        f = pt.Film(side, side)
        pt.render(pt.DeviceScene(scenes[si], pt.Accel(scenes[si])), st, f)
        assert info["spp_done"] == mx and np.array_equal(f.mean(), img)
