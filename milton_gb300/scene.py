"""Host-side scene: the world-space triangle soup Milton's ShapeSet flattens to.

A `Scene` holds exactly what crosses the C ABI (``mgpu_scene_desc``):

* ``tri_v``     (T, 3, 3) float32  world-space vertices v0, v1, v2
* ``tri_n``     (T, 3, 3) float32  per-vertex shading normals (unit)
* ``tri_mat``   (T,)      int32    material index
* ``tri_light`` (T,)      int32    light index, -1 if the triangle is not an emitter
* ``tri_flags`` (T,)      uint32   bit 0: back-face culled (Milton ``Triangle``,
                                   mlt/src/milton/shapes/Triangle.cpp:245-272); else two-sided
                                   (``MeshTriangle``, MeshTriangle.cpp:142-167)
* ``materials`` (M, 16)   float32  type, kd[3], ks[3], n, ior, transparency, 0...
* ``lights``    (L, 16)   float32  center[3], ex[3], ez[3], normal[3], area, Le[3]
* ``camera``    (11,)     float32  eye[3], look[3], up[3], heightAngle (deg), aspectRatio

Materials use Milton's keys and defaults (Material.cpp:67-92, DiffuseBSDF.cpp:44-46,
ModifiedPhongBSDF.cpp:48-81, DielectricBSDF.cpp:48-53): diffuse ``kd`` (0.5), Phong ``kd``/
``ks``/``n``, dielectric ``ior`` (AIR = 1.0003), ``transparency`` (1) and ``ks`` (1).
A quad light is a Milton ``plane`` under a transform with an ``oriented`` emitter of
``power``; its radiance is power / (area * pi) (Emitter.cpp:34-50,
OrientedEmitter.cpp:17-23).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

MAT_DIFFUSE = 0
MAT_PHONG = 1
MAT_DIELECTRIC = 2
TRI_CULLED = 1
AIR_IOR = 1.0003


def diffuse(kd) -> np.ndarray:
    m = np.zeros(16, np.float32)
    m[0] = MAT_DIFFUSE
    m[1:4] = np.broadcast_to(np.asarray(kd, np.float32), 3)
    m[4:7] = 0.0
    m[7] = 1.0
    m[8] = AIR_IOR
    m[9] = 1.0
    return m


def phong(kd, ks, n) -> np.ndarray:
    kd = np.broadcast_to(np.asarray(kd, np.float32), 3)
    ks = np.broadcast_to(np.asarray(ks, np.float32), 3)
    if np.any(kd + ks > 1.0 + 1e-6):
        raise ValueError("modified Phong requires kd + ks <= 1 per channel (ModifiedPhongBSDF.cpp:75)")
    m = np.zeros(16, np.float32)
    m[0] = MAT_PHONG
    m[1:4] = kd
    m[4:7] = ks
    m[7] = n
    m[8] = AIR_IOR
    m[9] = 1.0
    return m


def dielectric(ior=1.5, transparency=1.0, ks=1.0) -> np.ndarray:
    m = np.zeros(16, np.float32)
    m[0] = MAT_DIELECTRIC
    m[4:7] = np.broadcast_to(np.asarray(ks, np.float32), 3)
    m[7] = 1.0
    m[8] = ior
    m[9] = transparency
    return m


def quad_light(center, ex, ez, radiance) -> np.ndarray:
    """Record for a parallelogram light p(u, v) = center + (u - .5) ex + (v - .5) ez.

    The emitting side is normalize(ez x ex), the transformed +y of Milton's unit plane
    (Plane.cpp:61-65, 91-93)."""
    center, ex, ez = (np.asarray(a, np.float64) for a in (center, ex, ez))
    nrm = np.cross(ez, ex)
    area = float(np.linalg.norm(nrm))
    rec = np.zeros(16, np.float32)
    rec[0:3] = center
    rec[3:6] = ex
    rec[6:9] = ez
    rec[9:12] = nrm / area
    rec[12] = area
    rec[13:16] = np.broadcast_to(np.asarray(radiance, np.float64), 3)
    return rec


def light_power(radiance, area) -> float:
    """Milton ``power`` for a given radiance: L * pi * area."""
    return float(radiance) * np.pi * float(area)


def camera(eye, focus=None, look=None, up=(0, 1, 0), height_angle=45.0, aspect=1.0) -> np.ndarray:
    """ThinLensCamera keys: eye, focus or look, up, heightAngle, aspectRatio."""
    eye = np.asarray(eye, np.float64)
    if look is None:
        look = np.asarray(focus if focus is not None else (0, 0, 0), np.float64) - eye
    look = np.asarray(look, np.float64)
    look = look / np.linalg.norm(look)
    c = np.zeros(11, np.float32)
    c[0:3] = eye
    c[3:6] = look
    c[6:9] = up
    c[9] = height_angle
    c[10] = aspect
    return c


@dataclass
class Scene:
    tri_v: np.ndarray
    tri_n: np.ndarray
    tri_mat: np.ndarray
    tri_light: np.ndarray
    tri_flags: np.ndarray
    materials: np.ndarray
    lights: np.ndarray
    camera: np.ndarray
    name: str = "scene"
    shapes: list = field(default_factory=list)  # (name, first triangle, count) in ShapeSet order

    def __post_init__(self):
        self.tri_v = np.ascontiguousarray(self.tri_v, np.float32).reshape(-1, 3, 3)
        self.tri_n = np.ascontiguousarray(self.tri_n, np.float32).reshape(-1, 3, 3)
        self.tri_mat = np.ascontiguousarray(self.tri_mat, np.int32).reshape(-1)
        self.tri_light = np.ascontiguousarray(self.tri_light, np.int32).reshape(-1)
        self.tri_flags = np.ascontiguousarray(self.tri_flags, np.uint32).reshape(-1)
        self.materials = np.ascontiguousarray(self.materials, np.float32).reshape(-1, 16)
        self.lights = np.ascontiguousarray(self.lights, np.float32).reshape(-1, 16)
        self.camera = np.ascontiguousarray(self.camera, np.float32).reshape(11)
        T = self.tri_v.shape[0]
        for name, arr in (("tri_n", self.tri_n), ("tri_mat", self.tri_mat), ("tri_light", self.tri_light),
                          ("tri_flags", self.tri_flags)):
            if arr.shape[0] != T:
                raise ValueError(f"{name} has {arr.shape[0]} rows, expected {T}")
        if T and (self.tri_mat.min() < 0 or self.tri_mat.max() >= len(self.materials)):
            raise ValueError("material index out of range")
        if T and (self.tri_light.min() < -1 or self.tri_light.max() >= len(self.lights)):
            raise ValueError("light index out of range")

    @property
    def ntri(self) -> int:
        return int(self.tri_v.shape[0])

    def nbytes(self) -> int:
        return sum(a.nbytes for a in (self.tri_v, self.tri_n, self.tri_mat, self.tri_light, self.tri_flags,
                                      self.materials, self.lights))


class SceneBuilder:
    """Accumulates shapes in ShapeSet order; global prim id = shape offset + local index."""

    def __init__(self):
        self.v, self.n, self.mat, self.light, self.flags = [], [], [], [], []
        self.materials: list[np.ndarray] = []
        self.lights: list[np.ndarray] = []
        self.shapes: list[tuple[str, int, int]] = []
        self._ntri = 0

    def material(self, rec: np.ndarray) -> int:
        self.materials.append(np.asarray(rec, np.float32))
        return len(self.materials) - 1

    def add(self, name: str, v: np.ndarray, n: np.ndarray | None, mat: int, light: int = -1, culled: bool = False):
        v = np.asarray(v, np.float32).reshape(-1, 3, 3)
        if n is None:
            fn = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
            fn = fn / np.linalg.norm(fn, axis=1, keepdims=True)
            n = np.repeat(fn[:, None, :], 3, axis=1)
        n = np.asarray(n, np.float32).reshape(-1, 3, 3)
        k = v.shape[0]
        self.v.append(v)
        self.n.append(n)
        self.mat.append(np.full(k, mat, np.int32))
        self.light.append(np.full(k, light, np.int32))
        self.flags.append(np.full(k, TRI_CULLED if culled else 0, np.uint32))
        self.shapes.append((name, self._ntri, k))
        self._ntri += k

    def add_quad_light(self, name: str, center, ex, ez, radiance, mat: int) -> int:
        """A quad emitter: light record plus its two (two-sided) triangles."""
        rec = quad_light(center, ex, ez, radiance)
        self.lights.append(rec)
        li = len(self.lights) - 1
        c = np.asarray(center, np.float32)
        ex = np.asarray(ex, np.float32)
        ez = np.asarray(ez, np.float32)
        p00 = c - 0.5 * ex - 0.5 * ez
        p10 = c + 0.5 * ex - 0.5 * ez
        p11 = c + 0.5 * ex + 0.5 * ez
        p01 = c - 0.5 * ex + 0.5 * ez
        nrm = rec[9:12]
        tris = np.array([[p00, p01, p11], [p00, p11, p10]], np.float32)
        # orient so that (v1 - v0) x (v2 - v0) faces the emitting side
        fn = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
        for i in range(2):
            if np.dot(fn[i], nrm) < 0:
                tris[i] = tris[i][[0, 2, 1]]
        self.add(name, tris, np.broadcast_to(nrm, (2, 3, 3)), mat, light=li)
        return li

    def build(self, camera: np.ndarray, name: str = "scene") -> Scene:
        cat = lambda xs, shape, dt: np.concatenate(xs) if xs else np.zeros(shape, dt)  # noqa: E731
        return Scene(
            tri_v=cat(self.v, (0, 3, 3), np.float32), tri_n=cat(self.n, (0, 3, 3), np.float32),
            tri_mat=cat(self.mat, (0,), np.int32), tri_light=cat(self.light, (0,), np.int32),
            tri_flags=cat(self.flags, (0,), np.uint32),
            materials=np.stack(self.materials) if self.materials else np.zeros((0, 16), np.float32),
            lights=np.stack(self.lights) if self.lights else np.zeros((0, 16), np.float32),
            camera=camera, name=name, shapes=list(self.shapes))
