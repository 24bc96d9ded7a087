"""Continuous-batching render service (include/mgpu_server.h) and a request-replay driver.

The server (libmgpu.so, C++) keeps a library of scenes and a queue of render jobs on one device:
it admits jobs in arrival order against a device-memory budget, keeps kd-trees, films and the
shared wave workspace resident, renders every active job's next sample passes together in one
batch per tick, and finishes a job at the first checkpoint (its sample counts spp, 2 spp, 4 spp,
... up to max_spp) where the film's error estimate is at most the job's target.  A job's image
is bit-for-bit the one it gets alone.

No counterpart in the reference (Milton renders one scene per process); the progressive
refinement it schedules is Milton's own: further super-sample passes over the same film
(mlt/src/milton/renderers/generators/SuperSampleGenerator.cpp:54-92).
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .pathtracer import KdSettings, RenderSettings, _desc, _stream_handle
from .scene import Scene

JOB_STATES = {0: "queued", 1: "active", 2: "done", 3: "failed"}


@dataclass
class ServerSettings:
    hbm_budget: int = 120_000_000_000
    tick_paths: int = 1 << 26
    max_active: int = 256
    wave_paths: int = 0
    use_graph: int = 0
    build_threads: int = 2
    kd: KdSettings = field(default_factory=KdSettings)
    policy: str = "rotate"  # "rotate" (default), "fair" or "oldest" (include/mgpu_server.h)

    def to_c(self) -> N.ServerParams:
        p = N.ServerParams()
        p.hbm_budget, p.tick_paths, p.max_active = self.hbm_budget, self.tick_paths, self.max_active
        p.wave_paths, p.use_graph, p.build_threads = self.wave_paths, self.use_graph, self.build_threads
        p.kd = self.kd.to_c()
        policies = {"fair": 0, "oldest": 1, "rotate": 2}
        if self.policy not in policies:
            raise ValueError(f"unknown serving policy {self.policy!r}")
        p.policy = policies[self.policy]
        return p


class Server:
    """mgpu_server_*: one render service on the current CUDA device."""

    def __init__(self, settings: ServerSettings | None = None):
        self._lib = N.load()
        self.handle = C.c_void_p()
        self.settings = settings or ServerSettings()
        N.check(self._lib.mgpu_server_create(C.byref(self.settings.to_c()), C.byref(self.handle)))
        self._shapes = {}

    def clock(self) -> float:
        return float(self._lib.mgpu_server_clock(self.handle))

    def add_scene(self, scene: Scene) -> int:
        d = _desc(scene)
        sid = C.c_int32()
        N.check(self._lib.mgpu_server_add_scene(self.handle, C.byref(d), C.byref(sid)))
        return sid.value

    def prefetch(self, scene_id: int) -> None:
        N.check(self._lib.mgpu_server_prefetch(self.handle, scene_id))

    def wait_builds(self, timeout: float = 600.0) -> None:
        """Blocks until no kd-tree build is running (a warm service)."""
        t_end = time.monotonic() + timeout
        while self.stats()["building"] > 0:
            if time.monotonic() > t_end:
                raise TimeoutError("kd-tree builds still running")
            time.sleep(0.01)

    def submit(self, scene_id: int, settings: RenderSettings, camera: np.ndarray, max_spp: int,
               target_rmse: float = 0.0, arrival: float = -1.0) -> int:
        p = settings.to_c(camera)
        jid = C.c_int64()
        N.check(self._lib.mgpu_server_submit(self.handle, scene_id, C.byref(p), int(max_spp), float(target_rmse),
                                             float(arrival), C.byref(jid)))
        self._shapes[jid.value] = (settings.height, settings.width)
        return jid.value

    def step(self, stream=None) -> int:
        """One tick; returns the number of jobs still queued or active."""
        n = C.c_int32()
        N.check(self._lib.mgpu_server_step(self.handle, _stream_handle(stream), C.byref(n)))
        return n.value

    def job(self, job_id: int) -> dict:
        i = N.ServerJobInfo()
        N.check(self._lib.mgpu_server_job(self.handle, job_id, C.byref(i)))
        d = {f: getattr(i, f) for f, _ in N.ServerJobInfo._fields_}
        d["state"] = JOB_STATES.get(d["state"], d["state"])
        return d

    def read(self, job_id: int, stream=None) -> np.ndarray:
        h, w = self._shapes[job_id]
        out = np.zeros((h, w, 3), np.float64)
        N.check(self._lib.mgpu_server_read(self.handle, job_id, N.ptr(out), _stream_handle(stream)))
        return out

    def release(self, job_id: int) -> None:
        N.check(self._lib.mgpu_server_release(self.handle, job_id))

    def stats(self) -> dict:
        s = N.ServerStats()
        N.check(self._lib.mgpu_server_stats_get(self.handle, C.byref(s)))
        return {f: getattr(s, f) for f, _ in N.ServerStats._fields_}

    def close(self):
        if self.handle:
            self._lib.mgpu_server_destroy(self.handle)
            self.handle = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def replay(server: Server, requests: list[dict], make_job, stream=None, on_done=None, release: bool = True,
           stall_timeout: float = 300.0):
    """Replays a request stream against the server in real time.

    Each request is submitted when the server clock passes its arrival time (seconds after the
    replay starts, request["arrival"]) and carries that arrival time, so queueing before
    submission counts toward its latency.  make_job(request) -> (scene_id, RenderSettings,
    camera, max_spp, target_rmse).  on_done(request, job_id, info) is called once per finished
    job before its film is released.  Raises TimeoutError when no job finishes and no tick
    renders for stall_timeout seconds.  Returns ({request id: job info}, replay start time)."""
    order = sorted(requests, key=lambda r: r["arrival"])
    t0 = server.clock()
    i = 0
    live = {}
    infos = {}
    last_progress = time.monotonic()
    while True:
        if time.monotonic() - last_progress > stall_timeout:
            raise TimeoutError(f"render service made no progress for {stall_timeout} s: {server.stats()}")
        now = server.clock()
        while i < len(order) and t0 + order[i]["arrival"] <= now:
            r = order[i]
            sid, st, cam, max_spp, target = make_job(r)
            live[server.submit(sid, st, cam, max_spp, target, arrival=t0 + r["arrival"])] = r
            i += 1
        ticks = server.stats()["ticks"]
        unfinished = server.step(stream)
        if server.stats()["ticks"] != ticks or not live:
            last_progress = time.monotonic()
        for jid in list(live):
            info = server.job(jid)
            if info["state"] in ("done", "failed"):
                r = live.pop(jid)
                if on_done is not None:
                    on_done(r, jid, info)
                if release:
                    server.release(jid)
                infos[r["id"]] = info
        if i == len(order) and not live:
            break
        if unfinished == 0 and i < len(order):
            time.sleep(max(0.0, t0 + order[i]["arrival"] - server.clock()))
        elif server.stats()["ticks"] == ticks:
            time.sleep(0.001)  # nothing rendered (jobs waiting on kd-tree builds)
    return infos, t0


def latency_summary(infos: dict) -> dict:
    """p50 / p99 / max time-to-target (arrival to finish) and queueing (arrival to admission)."""
    done = [v for v in infos.values() if v["state"] == "done"]
    if not done:
        return {"jobs": 0}
    lat = np.array([v["t_done"] - v["t_arrival"] for v in done])
    wait = np.array([v["t_admit"] - v["t_arrival"] for v in done])
    return {"jobs": len(done), "failed": len(infos) - len(done),
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "max_s": float(lat.max()), "mean_s": float(lat.mean()),
            "admit_wait_p50_s": float(np.percentile(wait, 50)), "admit_wait_p99_s": float(np.percentile(wait, 99)),
            "reached_target": int(sum(v["reached_target"] for v in done))}
