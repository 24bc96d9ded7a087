"""Milton's own ray queries, as a test oracle (test infrastructure only).

`closest` / `any_hit` run oracle/_ref/milton_ref -- the reference's kdTreeAccel, Mesh,
MeshTriangle and Triangle compiled from its unmodified sources (oracle/milton_ref/build.py) --
over a flattened scene in ShapeSet order: every shape of `scene.shapes` becomes a Milton Mesh
with an identity transform (two-sided MeshTriangles) or, when its triangles are flagged culled,
standalone Milton Triangles.  Vertices and normals are the scene's float32 values widened to
double, as a scene file's numbers are read (real_t = double).  Rays are given in double.
Available only where the reference tree is (MILTON_REFERENCE); tests skip otherwise.
"""
from __future__ import annotations

import subprocess
import tempfile
from pathlib import Path

import numpy as np

from . import build as _build

TRI_CULLED = 1


def available() -> bool:
    return _build.available()


def executable() -> Path:
    exe = _build.build()
    if exe is None:
        raise RuntimeError("the reference tree is not present: Milton's own kd-tree cannot be built here")
    return exe


def write_scene(scene, path: Path, min_prims: int = 3, max_depth: int = 24, cost_traversal: float = 1.0,
                empty_bias: float = 0.9) -> None:
    """The scene file of driver.cpp: kd parameters (Milton's defaults, kdTreeAccel.h:97-104), then
    every shape of scene.shapes with its vertices and normals."""
    if len(getattr(scene, "spheres", [])):
        raise ValueError("analytic spheres are not part of this oracle")
    shapes = scene.shapes or [("all", 0, scene.ntri)]
    with open(path, "wb") as f:
        f.write(b"MRSC")
        np.array([1, len(shapes), min_prims, max_depth], np.uint32).tofile(f)
        np.array([cost_traversal, empty_bias], np.float64).tofile(f)
        for _, first, count in shapes:
            flags = scene.tri_flags[first:first + count]
            culled = bool(np.all(flags & TRI_CULLED))
            if not culled and np.any(flags & TRI_CULLED):
                raise ValueError("a shape mixes culled and two-sided triangles")
            np.array([1 if culled else 0, count], np.uint32).tofile(f)
            np.array([first], np.uint64).tofile(f)
            np.ascontiguousarray(scene.tri_v[first:first + count], np.float64).tofile(f)
            np.ascontiguousarray(scene.tri_n[first:first + count], np.float64).tofile(f)


def _run(mode: str, scene, org: np.ndarray, dirs: np.ndarray, tmax: np.ndarray | None, out_itemsize: int):
    org = np.asarray(org, np.float64).reshape(-1, 3)
    dirs = np.asarray(dirs, np.float64).reshape(-1, 3)
    n = org.shape[0]
    rec = np.zeros((n, 7), np.float64)
    rec[:, 0:3] = org
    rec[:, 3:6] = dirs
    rec[:, 6] = np.inf if tmax is None else np.asarray(tmax, np.float64).reshape(-1)
    exe = executable()
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        write_scene(scene, td / "scene.bin")
        with open(td / "rays.bin", "wb") as f:
            f.write(b"MRRY")
            np.array([1], np.uint32).tofile(f)
            np.array([n], np.uint64).tofile(f)
            rec.tofile(f)
        r = subprocess.run([str(exe), mode, str(td / "scene.bin"), str(td / "rays.bin"), str(td / "out.bin")],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"milton_ref {mode} failed: {r.stderr.strip()}")
        raw = np.fromfile(td / "out.bin", np.uint8)
    if raw.size != n * out_itemsize:
        raise RuntimeError("milton_ref wrote a short result")
    return raw


def closest(scene, org, dirs, naive: bool = False) -> tuple[np.ndarray, np.ndarray]:
    """Scene::getIntersection per ray: (t as float64, global primitive id as int64; inf / -1 on
    a miss).  naive: Milton's NaiveSpatialAccel instead of its kd-trees."""
    raw = _run("closest_naive" if naive else "closest", scene, org, dirs, None, 16)
    rec = raw.view(np.uint8).reshape(-1, 16)
    t = rec[:, :8].copy().view(np.float64).reshape(-1)
    pid = rec[:, 8:].copy().view(np.int64).reshape(-1)
    return t, pid


def any_hit(scene, org, dirs, tmax, naive: bool = False) -> np.ndarray:
    """Scene::intersects(ray, tMax) per ray (Milton's any-hit window (EPSILON, tMax - 2 EPSILON))."""
    raw = _run("any_naive" if naive else "any", scene, org, dirs, tmax, 1)
    return raw.astype(bool)
