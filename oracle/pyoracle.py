"""ctypes wrapper of the oracle (oracle.c) -- TEST INFRASTRUCTURE.

Loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm.
The product package never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import build as _build

_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build()
    lib = C.CDLL(str(path))
    vp, i64, u32, u64 = C.c_void_p, C.c_int64, C.c_uint32, C.c_uint64
    lib.orc_kd_build.restype = vp
    lib.orc_kd_build.argtypes = [vp, i64, C.c_uint, C.c_uint, C.c_double, C.c_double]
    lib.orc_kd_free.argtypes = [vp]
    lib.orc_kd_from_serial.restype = vp
    lib.orc_kd_from_serial.argtypes = [vp, i64, vp, vp, vp, vp, i64, i64]
    lib.orc_kd_stats.argtypes = [vp, vp]
    lib.orc_kd_bounds.argtypes = [vp, vp]
    lib.orc_kd_serialize.restype = i64
    lib.orc_kd_serialize.argtypes = [vp, vp, vp, vp, vp, C.POINTER(i64)]
    lib.orc_trace_closest.argtypes = [vp, i64, vp, vp, vp, i64, vp, vp, vp, vp]
    lib.orc_trace_any.argtypes = [vp, i64, vp, vp, vp, i64, vp, vp]
    lib.orc_render.restype = C.c_int
    lib.orc_render.argtypes = [i64, vp, vp, vp, vp, vp, C.c_int, vp, C.c_int, vp, vp, vp, C.c_int, vp, vp, vp,
                               C.c_int, vp, vp, vp, vp, vp, vp, u64, u32, vp, vp, vp]
    lib.orc_sphere_closest.restype = C.c_double
    lib.orc_sphere_closest.argtypes = [vp, vp, vp]
    lib.orc_background.argtypes = [vp, vp, vp, vp, vp]
    lib.orc_texture_lookup.argtypes = [vp, vp, C.c_double, C.c_double, vp, vp]
    lib.orc_philox4x32_10.argtypes = [vp, vp, vp]
    lib.orc_camera_dir.argtypes = [vp, C.c_double, C.c_double, vp]
    lib.orc_camera_ray.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double, vp, vp]
    lib.orc_bsdf_sample.restype = C.c_int
    lib.orc_bsdf_sample.argtypes = [vp, vp, vp, C.c_int, vp, vp, vp]
    lib.orc_bsdf_eval.argtypes = [vp, vp, vp, vp, vp]
    lib.orc_uniforms.argtypes = [u64, u32, u64, u32, u32, vp]
    _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data


class Tree:
    """The reference's kd-tree, restated (kdTreeAccel.cpp:403-877)."""

    def __init__(self, tri_v: np.ndarray, min_prims=3, max_depth=24, cost_traversal=1.0, empty_bias=0.9):
        self._lib = load()
        self.v = np.ascontiguousarray(tri_v, np.float32).reshape(-1, 9)
        self.ntri = self.v.shape[0]
        self.h = self._lib.orc_kd_build(_p(self.v), self.ntri, min_prims, max_depth, cost_traversal, empty_bias)

    @classmethod
    def from_serial(cls, tri_v: np.ndarray, kind, split, count, prims) -> "Tree":
        """The tree given by a depth-first serialisation (orc_kd_serialize's layout, which the
        product's Accel.serialize also gives): for scenes whose restated build takes too long."""
        self = cls.__new__(cls)
        self._lib = load()
        self.v = np.ascontiguousarray(tri_v, np.float32).reshape(-1, 9)
        self.ntri = self.v.shape[0]
        self._ser = [np.ascontiguousarray(kind, np.int32), np.ascontiguousarray(split, np.float32),
                     np.ascontiguousarray(count, np.int32), np.ascontiguousarray(prims, np.int32)]
        k, sp, c, pr = self._ser
        self.h = self._lib.orc_kd_from_serial(_p(self.v), self.ntri, _p(k), _p(sp), _p(c), _p(pr), len(k), len(pr))
        if not self.h:
            raise ValueError("malformed tree serialisation")
        return self

    def stats(self) -> dict:
        out = np.zeros(8, np.uint64)
        self._lib.orc_kd_stats(self.h, _p(out))
        keys = ("no_internal", "no_leaves", "min_depth", "max_depth", "sum_depth", "min_prims", "max_prims",
                "sum_prims")
        return {k: int(v) for k, v in zip(keys, out)}

    def bounds(self) -> np.ndarray:
        out = np.zeros(6, np.float64)
        self._lib.orc_kd_bounds(self.h, _p(out))
        return out

    def serialize(self):
        npr = C.c_int64()
        n = self._lib.orc_kd_serialize(self.h, None, None, None, None, C.byref(npr))
        kind = np.zeros(n, np.int32)
        split = np.zeros(n, np.float32)
        count = np.zeros(n, np.int32)
        prims = np.zeros(max(npr.value, 1), np.int32)
        self._lib.orc_kd_serialize(self.h, _p(kind), _p(split), _p(count), _p(prims), C.byref(npr))
        return kind, split, count, prims[:npr.value]

    def __del__(self):
        try:
            if self.h:
                self._lib.orc_kd_free(self.h)
                self.h = None
        except Exception:
            pass


def trace_closest(tree: Tree | None, tri_v, tri_flags, rays: np.ndarray, with_counts=False):
    """Closest hit per ray (rays: (n, 8) float32).  tree None = brute force, which also
    returns the second-nearest t.  Returns t (inf on miss), prim (-1), t2, counters."""
    lib = load()
    v = np.ascontiguousarray(tri_v, np.float32).reshape(-1, 9)
    fl = None if tri_flags is None else np.ascontiguousarray(tri_flags, np.uint32)
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    n = rays.shape[0]
    t = np.zeros(n, np.float64)
    prim = np.zeros(n, np.int64)
    t2 = np.zeros(n, np.float64)
    cnt = np.zeros(3, np.uint64)
    lib.orc_trace_closest(tree.h if tree else None, v.shape[0], _p(v), _p(fl), _p(rays), n, _p(t), _p(prim), _p(t2),
                          _p(cnt) if with_counts else None)
    return t, prim, t2, cnt


def trace_any(tree: Tree | None, tri_v, tri_flags, rays: np.ndarray):
    lib = load()
    v = np.ascontiguousarray(tri_v, np.float32).reshape(-1, 9)
    fl = None if tri_flags is None else np.ascontiguousarray(tri_flags, np.uint32)
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    occ = np.zeros(rays.shape[0], np.uint8)
    lib.orc_trace_any(tree.h if tree else None, v.shape[0], _p(v), _p(fl), _p(rays), rays.shape[0], _p(occ), None)
    return occ


def render(scene, tree: Tree, width, height, spp, sample_begin=0, sample_count=None, nds=1, max_depth=0,
           rr_start=2, efficient_direct=1, seed=0, stream=0, rows=None, threads=None, per_path=False):
    """FP64 PathTracer restatement.  Returns (mean image (h, w, 3) over the rendered rows,
    per-path radiance or None, stats dict)."""
    lib = load()
    sample_count = spp - sample_begin if sample_count is None else sample_count
    r0, r1 = (0, height) if rows is None else rows
    threads = threads or os.cpu_count() or 1
    ip = np.array([width, height, spp, nds, max_depth, rr_start, efficient_direct, sample_begin, sample_count, r0, r1,
                   threads], np.int32)
    film = np.zeros((height, width, 3), np.float64)
    # per-path radiance of the rendered rows only: ((y - r0) * width + x) * sample_count + s
    paths = np.zeros(((r1 - r0) * width * sample_count, 3), np.float64) if per_path else None
    st = np.zeros(4, np.uint64)
    lights = scene.lights if len(scene.lights) else np.zeros((1, 16), np.float32)
    cam = np.zeros(16, np.float32)
    cam[:np.asarray(scene.camera).reshape(-1).shape[0]] = np.asarray(scene.camera, np.float32).reshape(-1)
    ext = getattr(scene, "light_ext", None)
    ext = np.ascontiguousarray(ext, np.float32) if ext is not None and len(ext) else None
    uv = getattr(scene, "tri_uv", None)
    uv = None if uv is None else np.ascontiguousarray(uv, np.float32)
    textures = list(getattr(scene, "textures", []))
    tparams, trgb = texture_params(textures)
    sph = np.ascontiguousarray(getattr(scene, "spheres", np.zeros((0, 8))), np.float32).reshape(-1, 8)
    sph_mat = np.ascontiguousarray(getattr(scene, "sphere_mat", np.zeros(0)), np.int32)
    sph_light = getattr(scene, "sphere_light", None)
    sph_light = None if sph_light is None else np.ascontiguousarray(sph_light, np.int32)
    bg = np.zeros(4, np.float32)
    bg[0] = getattr(scene, "background_tex", 0)
    bg[1:4] = getattr(scene, "background_le", (0.0, 0.0, 0.0))
    lib.orc_render(scene.ntri, _p(scene.tri_v), _p(scene.tri_n), _p(scene.tri_mat), _p(scene.tri_light),
                   _p(scene.tri_flags), len(scene.materials), _p(scene.materials), len(scene.lights), _p(lights),
                   _p(ext), _p(uv), len(textures), _p(tparams), C.cast(trgb, C.c_void_p), _p(bg), len(sph), _p(sph),
                   _p(sph_mat), _p(sph_light), tree.h, _p(cam), _p(ip), seed, stream, _p(film), _p(paths), _p(st))
    mean = film[r0:r1] / max(sample_count, 1)
    if per_path:
        paths = paths.reshape(r1 - r0, width, sample_count, 3)
    stats = dict(extension_rays=int(st[0]), shadow_rays=int(st[1]), zero_pdf=int(st[2]), truncated=int(st[3]))
    return mean, paths, stats


def texture_params(textures):
    """(12 floats per texture, array of rgb pointers) for orc_render: width, height, kind,
    filter, support, p1, p2, repeat u, repeat v, bump intensity."""
    params = np.zeros((max(1, len(textures)), 12), np.float32)
    ptrs = (C.c_void_p * max(1, len(textures)))()
    for i, t in enumerate(textures):
        h, w, _ = t.rgb.shape
        f, support, p1, p2 = t.filter_params()
        params[i, :10] = (w, h, t.kind, f, support, p1, p2, t.repeat_u, t.repeat_v, t.bump_intensity)
        ptrs[i] = t.rgb.ctypes.data
    return params, ptrs


def texture_lookup(tex, u, v, normal=None) -> np.ndarray:
    """One oracle lookup of a Texture at (u, v): filtered rgb (colour maps) or (gx, gy, bumped
    normal xyz) (bump maps)."""
    lib = load()
    params, _ = texture_params([tex])
    rgb = np.ascontiguousarray(tex.rgb, np.float32)
    out = np.zeros(5, np.float64)
    n = None if normal is None else np.ascontiguousarray(normal, np.float64)
    lib.orc_texture_lookup(_p(params), rgb.ctypes.data, float(u), float(v), _p(n), _p(out))
    return out[:3] if tex.kind == 0 else out


def background(direction, tex=None, le=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Background radiance of a ray with this direction: the environment map tex, or the
    constant le."""
    lib = load()
    out = np.zeros(3, np.float64)
    d = np.ascontiguousarray(direction, np.float64)
    if tex is None:
        le = np.ascontiguousarray(le, np.float64)
        lib.orc_background(None, None, _p(le), _p(d), _p(out))
    else:
        params, _ = texture_params([tex])
        rgb = np.ascontiguousarray(tex.rgb, np.float32)
        lib.orc_background(_p(params), rgb.ctypes.data, None, _p(d), _p(out))
    return out


def sphere_closest(sphere8, o, d) -> float:
    """Milton's Sphere::getIntersection for one sphere record (center, radius, quaternion)."""
    sp = np.ascontiguousarray(sphere8, np.float32)
    o = np.ascontiguousarray(o, np.float64)
    d = np.ascontiguousarray(d, np.float64)
    return float(load().orc_sphere_closest(_p(sp), _p(o), _p(d)))


def philox(ctr, key) -> np.ndarray:
    lib = load()
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib.orc_philox4x32_10(_p(c), _p(k), _p(out))
    return out


def uniforms(seed, stream, path, depth, block) -> np.ndarray:
    out = np.zeros(4, np.float64)
    load().orc_uniforms(seed, stream, path, depth, block, _p(out))
    return out


def camera_ray(camera, x, y, u1, u2):
    """Thin-lens camera ray (origin, direction) through film point (x, y), lens lanes u1, u2."""
    cam = np.zeros(16, np.float32)
    c = np.asarray(camera, np.float32).reshape(-1)
    cam[:c.shape[0]] = c
    o = np.zeros(3, np.float64)
    d = np.zeros(3, np.float64)
    load().orc_camera_ray(_p(cam), x, y, u1, u2, _p(o), _p(d))
    return o, d


def camera_dir(camera, x, y) -> np.ndarray:
    """Pinhole direction through film point (x, y) (the thin lens, if any, is not applied)."""
    out = np.zeros(3, np.float64)
    cam = np.zeros(16, np.float32)
    c = np.asarray(camera, np.float32).reshape(-1)
    cam[:c.shape[0]] = c
    load().orc_camera_dir(_p(cam), x, y, _p(out))
    return out


def bsdf_sample(mat16, ns, wi, ior_index, u):
    lib = load()
    m = np.ascontiguousarray(mat16, np.float32)
    ns = np.ascontiguousarray(ns, np.float64)
    wi = np.ascontiguousarray(wi, np.float64)
    u = np.ascontiguousarray(u, np.float64)
    wo = np.zeros(3, np.float64)
    fs = np.zeros(3, np.float64)
    ev = lib.orc_bsdf_sample(_p(m), _p(ns), _p(wi), int(ior_index), _p(u), _p(wo), _p(fs))
    return ev, wo, fs


def bsdf_eval(mat16, ns, wi, wo):
    lib = load()
    m = np.ascontiguousarray(mat16, np.float32)
    arrs = [np.ascontiguousarray(a, np.float64) for a in (ns, wi, wo)]
    f = np.zeros(3, np.float64)
    lib.orc_bsdf_eval(_p(m), _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), _p(f))
    return f
