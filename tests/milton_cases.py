"""Ray batches on which the GPU kernels and the oracle are compared with Milton's own
intersection code (the fixture tests/golden/milton_hits.npz, written by
tests/golden/make_milton_hits.py from the reference's kdTreeAccel / Mesh / MeshTriangle /
Triangle compiled unmodified).

Cases:
  plain_culled  the plain box (34 triangles + the light quad), every triangle a standalone,
                back-face culled Milton `Triangle` shape (Triangle.cpp:245-272)
  mid           the mid configuration's 1,000,010 triangles: 400 sphere Meshes, the ground and
                4 light quads as two-sided Meshes (MeshTriangle.cpp:92-168) under Milton's
                two-level kd-trees (one per Mesh and one over the shapes)

Each case has closest-hit rays (camera rays and rays from random points in all directions) and
any-hit segments (the same kind of rays with a random tMax).
"""
from __future__ import annotations

import hashlib

import numpy as np

from milton_gb300 import scenegen
from raygen import camera_rays, sphere_rays

CASES = ("plain_culled", "mid")
N_CLOSEST = 1 << 14  # per kind (camera, sphere)
N_ANY = 1 << 14


def scene(case: str):
    if case == "plain_culled":
        s = scenegen.plain(0)
        s.tri_flags = np.ones_like(s.tri_flags)
        s.shapes = [(f"triangle{i}", i, 1) for i in range(s.ntri)]
        return s
    if case == "mid":
        return scenegen.mid(0)
    raise KeyError(case)


def _bounds(case: str, s):
    if case == "plain_culled":
        return np.array((-1.0, 0.0, -1.0)), np.array((1.0, 2.0, 1.0)), 3.0
    lo = s.tri_v.reshape(-1, 3).min(0).astype(np.float64)
    hi = s.tri_v.reshape(-1, 3).max(0).astype(np.float64)
    hi[1] = 3.0  # origins among the spheres, below the lights
    return lo, hi, 12.0


def closest_rays(case: str, s) -> np.ndarray:
    lo, hi, _ = _bounds(case, s)
    return np.concatenate([camera_rays(s.camera, N_CLOSEST, 11), sphere_rays(lo, hi, N_CLOSEST, 12)])


def any_rays(case: str, s) -> np.ndarray:
    lo, hi, reach = _bounds(case, s)
    r = sphere_rays(lo, hi, N_ANY, 13)
    r[:, 7] = np.random.default_rng(14).uniform(0.0, reach, N_ANY).astype(np.float32)
    return r


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]
