"""Seeded multi-scene workloads: the batched configuration and the serving request stream.

* batched: 64 independent scenes of uneven size (triangle count log-uniform in [1k, 500k],
  spheres and boxes on a ground quad), resolutions log-uniform in [128, 1024] per side (multiples
  of 8), 16 spp each, max depth 8, RR from depth 3.
* serving: Poisson arrivals (seeded exponential gaps) at a given rate; each request picks a scene
  (10k-2M triangles), a resolution from {256, 512, 1024, 2048} and a target spp from
  {1, 16, 64, 256} uniformly, and views its scene from its own camera (the scene's camera
  turned about the vertical axis by a seeded angle).
"""
from __future__ import annotations

import numpy as np

from . import scenegen


def batched_specs(seed: int = 0, n: int = 64, tri_lo: int = 1000, tri_hi: int = 500_000, res_lo: int = 128,
                  res_hi: int = 1024, spp: int = 16):
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(n):
        tris = int(np.exp(rng.uniform(np.log(tri_lo), np.log(tri_hi))))
        side = int(np.exp(rng.uniform(np.log(res_lo), np.log(res_hi)))) // 8 * 8
        specs.append(dict(scene_seed=int(rng.integers(1 << 30)), tris=tris, width=side, height=side, spp=spp))
    return specs


def build_scene(spec):
    return scenegen.random_scene(spec["scene_seed"], spec["tris"])


def serving_requests(seed: int = 0, n: int = 64, rate: float = 200.0, tri_lo: int = 10_000, tri_hi: int = 2_000_000,
                     sides=(256, 512, 1024, 2048), spps=(1, 16, 64, 256), n_scenes: int = 8):
    """Returns (scene specs, requests); requests reference scenes by index (scenes are
    shared between requests, as a render service keeps a library of resident scenes)."""
    rng = np.random.default_rng(seed)
    scenes = [dict(scene_seed=int(rng.integers(1 << 30)),
                   tris=int(np.exp(rng.uniform(np.log(tri_lo), np.log(tri_hi))))) for _ in range(n_scenes)]
    t = 0.0
    reqs = []
    for k in range(n):
        t += rng.exponential(1.0 / rate)
        side = int(rng.choice(sides))
        reqs.append(dict(id=k, arrival=t, scene=int(rng.integers(n_scenes)), width=side, height=side,
                         spp=int(rng.choice(spps)), seed=int(rng.integers(1 << 30))))
    return scenes, reqs


def request_camera(camera, seed: int, max_turn: float = 0.6) -> np.ndarray:
    """The scene camera turned about the y axis through the origin by a seeded angle in
    [-max_turn, max_turn] radians (a per-request view of a shared scene)."""
    a = np.random.default_rng(seed).uniform(-max_turn, max_turn)
    c, s = np.cos(a), np.sin(a)
    R = np.array([[c, 0.0, s], [0.0, 1.0, 0.0], [-s, 0.0, c]])
    out = np.array(camera, np.float32).copy()
    out[0:3] = R @ np.asarray(camera[0:3], np.float64)
    look = R @ np.asarray(camera[3:6], np.float64)
    out[3:6] = look / np.linalg.norm(look)
    return out
