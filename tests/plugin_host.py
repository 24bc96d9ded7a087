"""Runs Milton's renderer plugin (milton_gb300/lib/libmgpu_milton.so) under the stand-in Milton
host tests/_build/milton_host (tests/native/milton_host.cpp): the host loads it the way Milton's
scene loader does and calls init() and render() through milton::Renderer*."""
from __future__ import annotations

import subprocess
import tempfile
from pathlib import Path

import numpy as np


def host_path() -> Path:
    from native import build as nb
    return nb.build_host()


def write_scene(scene, width: int, height: int, path: Path) -> None:
    """The stand-in host's scene file (milton_host.cpp): the flattened scene, camera and film size."""
    nl = len(scene.lights)
    ext = scene.light_ext if len(scene.light_ext) else np.zeros((nl, 16), np.float32)
    cam = np.zeros(16, np.float32)
    c = np.asarray(scene.camera, np.float32).reshape(-1)
    cam[:c.shape[0]] = c
    with open(path, "wb") as f:
        f.write(b"MHSC")
        np.array([scene.ntri], np.int64).tofile(f)
        np.array([len(scene.materials), nl], np.int32).tofile(f)
        cam.tofile(f)
        np.array([width, height], np.int32).tofile(f)
        for a, dt in ((scene.tri_v, np.float32), (scene.tri_n, np.float32), (scene.tri_mat, np.int32),
                      (scene.tri_light, np.int32), (scene.tri_flags, np.uint32), (scene.materials, np.float32),
                      (scene.lights, np.float32), (ext, np.float32)):
            np.ascontiguousarray(a, dt).tofile(f)


def run(plugin: Path, scene, width: int, height: int, props: dict) -> tuple[np.ndarray, np.ndarray, str]:
    """(per-pixel output values (h, w, 3), samples per pixel (h, w), stderr) of one render."""
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        write_scene(scene, width, height, td / "scene.bin")
        kv = [f"{k}={str(v).lower() if isinstance(v, bool) else v}" for k, v in props.items()]
        r = subprocess.run([str(host_path()), str(plugin), str(td / "scene.bin"), str(td / "out.bin"), *kv],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"milton_host failed ({r.returncode}): {r.stderr.strip()}")
        raw = np.fromfile(td / "out.bin", np.uint8)
    n = width * height
    vals = raw[:24 * n].view(np.float64).reshape(height, width, 3)
    cnt = raw[24 * n:].view(np.uint64).reshape(height, width)
    return vals, cnt, r.stderr
