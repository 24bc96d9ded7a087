"""Host-side scene: the world-space triangle soup Milton's ShapeSet flattens to.

A `Scene` holds exactly what crosses the C ABI (``mgpu_scene_desc``):

* ``tri_v``     (T, 3, 3) float32  world-space vertices v0, v1, v2
* ``tri_n``     (T, 3, 3) float32  per-vertex shading normals (unit)
* ``tri_mat``   (T,)      int32    material index
* ``tri_light`` (T,)      int32    light index, -1 if the triangle is not an emitter
* ``tri_flags`` (T,)      uint32   bit 0: back-face culled (Milton ``Triangle``,
                                   mlt/src/milton/shapes/Triangle.cpp:245-272); else two-sided
                                   (``MeshTriangle``, MeshTriangle.cpp:142-167)
* ``materials`` (M, 16)   float32  type, kd[3], ks[3], n, ior, transparency, texture slots [10..13],
                                   per-channel IOR [14], [15] (0, 0 = [8] for every channel)
* ``lights``    (L, 16)   float32  center[3], ex[3], ez[3], normal[3], area, Le[3]
* ``light_ext`` (L, 16)   float32  type (0 plane, 1 Triangle, 2 Mesh) and its parameters
                                   (include/mgpu.h); all zeros = planes
* ``camera``    (16,)     float32  eye[3], look[3], up[3], heightAngle (deg), aspectRatio, aperture (m),
                                   focal length, focal distance, 0, 0 (aperture 0 = pinhole)
* ``tri_uv``    (T, 3, 2) float32  per-vertex uvs, or None (every uv is (0, 0))
* ``textures``  list of `Texture`: image maps named by the material texture slots
                                   [10] kd, [11] ks, [12] transparency, [13] bump (1 + index)
* ``spheres``   (S, 8)    float32  analytic spheres beside the soup: center[3], radius, world-to-object
                                   rotation quaternion (x, y, z, w); primitive ids ntri + index
* ``sphere_mat`` (S,)     int32    their material indices
* ``sphere_light`` (S,)   int32    their light indices (-1 = not an emitter)
* ``background_tex`` int           1 + index of the environment map (latitude-longitude), or 0
* ``background_le``  (3,) float32  constant background radiance when background_tex is 0

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
    """ior: one value, or three (per colour channel: a path refracts with its channel's, which
    disperses light as Milton's spectral IOR does)."""
    m = np.zeros(16, np.float32)
    m[0] = MAT_DIELECTRIC
    m[4:7] = np.broadcast_to(np.asarray(ks, np.float32), 3)
    m[7] = 1.0
    set_ior(m, ior)
    m[9] = transparency
    return m


def set_ior(rec: np.ndarray, ior) -> None:
    """Material record IOR: [8] for every channel, or [8], [14], [15] per channel."""
    a = np.broadcast_to(np.asarray(ior, np.float32), 3)
    rec[8] = a[0]
    rec[14], rec[15] = (0.0, 0.0) if a[0] == a[1] == a[2] else (a[1], a[2])


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


def camera(eye, focus=None, look=None, up=(0, 1, 0), height_angle=45.0, aspect=1.0, aperture=0.0,
           focal_length=0.0, focal_distance=1.0) -> np.ndarray:
    """ThinLensCamera keys: eye, focus or look, up, heightAngle, aspectRatio; aperture in metres
    (0 = pinhole), focal length (fstop x aperture) and focal distance for the thin lens."""
    eye = np.asarray(eye, np.float64)
    if look is None:
        look = np.asarray(focus if focus is not None else (0, 0, 0), np.float64) - eye
    look = np.asarray(look, np.float64)
    look = look / np.linalg.norm(look)
    c = np.zeros(16, np.float32)
    c[0:3] = eye
    c[3:6] = look
    c[6:9] = up
    c[9] = height_angle
    c[10] = aspect
    c[11], c[12], c[13] = aperture, focal_length, focal_distance
    return c


TEX_COLOR = 0
TEX_BUMP = 1
FILTERS = {"box": 1, "triangle": 2, "gaussian": 3, "mitchell": 4, "lanczosSinc": 5}


def quat_from_matrix(R) -> np.ndarray:
    """Unit quaternion (x, y, z, w) of a 3 x 3 rotation matrix (Shepperd's method)."""
    R = np.asarray(R, np.float64)
    tr = np.trace(R)
    if tr > 0:
        s = 2.0 * np.sqrt(tr + 1.0)
        q = [(R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s, 0.25 * s]
    else:
        i = int(np.argmax(np.diag(R)))
        j, k = (i + 1) % 3, (i + 2) % 3
        s = 2.0 * np.sqrt(1.0 + R[i, i] - R[j, j] - R[k, k])
        q = [0.0, 0.0, 0.0, (R[k, j] - R[j, k]) / s]
        q[i] = 0.25 * s
        q[j] = (R[j, i] + R[i, j]) / s
        q[k] = (R[k, i] + R[i, k]) / s
    q = np.asarray(q)
    return (q / np.linalg.norm(q)).astype(np.float32)


@dataclass
class Texture:
    """A material's image map (include/mgpu.h, mgpu_texture): rgb (H, W, 3) linear values, row 0
    the top row.  Colour maps are filtered per texel with the material's filter (kind, support,
    params as for the film); bump maps keep luminance differences."""
    rgb: np.ndarray
    kind: int = TEX_COLOR
    filter: tuple = ("triangle", 2.0, {})
    repeat_u: float = 1.0
    repeat_v: float = 1.0
    bump_intensity: float = 5.0

    def __post_init__(self):
        self.rgb = np.ascontiguousarray(self.rgb, np.float32)
        if self.rgb.ndim != 3 or self.rgb.shape[2] != 3 or self.rgb.shape[0] < 1 or self.rgb.shape[1] < 1:
            raise ValueError("texture rgb must be (H, W, 3)")
        if self.filter[0] not in FILTERS:
            raise ValueError(f"unknown texture filter {self.filter[0]!r}")

    def filter_params(self) -> tuple[int, float, float, float]:
        kind, support, params = self.filter
        p1 = {"gaussian": params.get("sigma", 1.0), "mitchell": params.get("B", 1.0 / 3.0),
              "lanczosSinc": params.get("tau", 3.0)}.get(kind, 0.0)
        p2 = params.get("C", 1.0 / 3.0) if kind == "mitchell" else 0.0
        return FILTERS[kind], float(support), float(p1), float(p2)


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
    light_ext: np.ndarray | None = None
    tri_uv: np.ndarray | None = None
    textures: list = field(default_factory=list)
    background_tex: int = 0
    background_le: np.ndarray = field(default_factory=lambda: np.zeros(3, np.float32))
    spheres: np.ndarray = field(default_factory=lambda: np.zeros((0, 8), np.float32))
    sphere_mat: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    sphere_light: np.ndarray | None = None

    def __post_init__(self):
        self.tri_v = np.ascontiguousarray(self.tri_v, np.float32).reshape(-1, 3, 3)
        self.tri_n = np.ascontiguousarray(self.tri_n, np.float32).reshape(-1, 3, 3)
        self.tri_mat = np.ascontiguousarray(self.tri_mat, np.int32).reshape(-1)
        self.tri_light = np.ascontiguousarray(self.tri_light, np.int32).reshape(-1)
        self.tri_flags = np.ascontiguousarray(self.tri_flags, np.uint32).reshape(-1)
        self.materials = np.ascontiguousarray(self.materials, np.float32).reshape(-1, 16)
        self.lights = np.ascontiguousarray(self.lights, np.float32).reshape(-1, 16)
        if self.light_ext is None:
            self.light_ext = np.zeros((len(self.lights), 16), np.float32)
        self.light_ext = np.ascontiguousarray(self.light_ext, np.float32).reshape(-1, 16)
        if len(self.light_ext) != len(self.lights):
            raise ValueError("light_ext needs one row per light")
        cam = np.ascontiguousarray(self.camera, np.float32).reshape(-1)
        if cam.shape[0] not in (11, 16):
            raise ValueError("camera needs 11 (pinhole) or 16 (thin lens) floats")
        self.camera = np.zeros(16, np.float32)
        self.camera[:cam.shape[0]] = cam
        T = self.tri_v.shape[0]
        for name, arr in (("tri_n", self.tri_n), ("tri_mat", self.tri_mat), ("tri_light", self.tri_light),
                          ("tri_flags", self.tri_flags)):
            if arr.shape[0] != T:
                raise ValueError(f"{name} has {arr.shape[0]} rows, expected {T}")
        if T and (self.tri_mat.min() < 0 or self.tri_mat.max() >= len(self.materials)):
            raise ValueError("material index out of range")
        if T and (self.tri_light.min() < -1 or self.tri_light.max() >= len(self.lights)):
            raise ValueError("light index out of range")
        if self.tri_uv is not None:
            self.tri_uv = np.ascontiguousarray(self.tri_uv, np.float32).reshape(-1, 3, 2)
            if self.tri_uv.shape[0] != T:
                raise ValueError(f"tri_uv has {self.tri_uv.shape[0]} rows, expected {T}")
        self.background_le = np.ascontiguousarray(np.broadcast_to(np.asarray(self.background_le, np.float32), 3))
        self.spheres = np.ascontiguousarray(self.spheres, np.float32).reshape(-1, 8)
        self.sphere_mat = np.ascontiguousarray(self.sphere_mat, np.int32).reshape(-1)
        if len(self.sphere_mat) != len(self.spheres):
            raise ValueError("sphere_mat needs one entry per sphere")
        if self.sphere_light is None:
            self.sphere_light = np.full(len(self.spheres), -1, np.int32)
        self.sphere_light = np.ascontiguousarray(self.sphere_light, np.int32).reshape(-1)
        if len(self.sphere_light) != len(self.spheres):
            raise ValueError("sphere_light needs one entry per sphere")
        if len(self.spheres) and (self.sphere_mat.min() < 0 or self.sphere_mat.max() >= len(self.materials)):
            raise ValueError("sphere material index out of range")
        if not 0 <= self.background_tex <= len(self.textures):
            raise ValueError("background texture out of range")
        slots = self.materials[:, 10:14] if len(self.materials) else np.zeros((0, 4), np.float32)
        if np.any(slots < 0) or np.any(slots > len(self.textures)) or np.any(slots != np.floor(slots)):
            raise ValueError("material texture slot out of range")

    @property
    def ntri(self) -> int:
        return int(self.tri_v.shape[0])

    def nbytes(self) -> int:
        extra = (0 if self.tri_uv is None else self.tri_uv.nbytes) + sum(t.rgb.nbytes for t in self.textures) + \
            self.spheres.nbytes + self.sphere_mat.nbytes
        return extra + sum(a.nbytes for a in (self.tri_v, self.tri_n, self.tri_mat, self.tri_light, self.tri_flags,
                                              self.materials, self.lights, self.light_ext))


class SceneBuilder:
    """Accumulates shapes in ShapeSet order; global prim id = shape offset + local index."""

    def __init__(self):
        self.v, self.n, self.mat, self.light, self.flags = [], [], [], [], []
        self.uv: list[np.ndarray | None] = []
        self.textures: list[Texture] = []
        self.bg_tex = 0
        self.bg_le = np.zeros(3, np.float32)
        self.spheres: list[np.ndarray] = []
        self.sphere_mat: list[int] = []
        self.sphere_light: list[int] = []
        self.materials: list[np.ndarray] = []
        self.lights: list[np.ndarray] = []
        self.light_ext: list[np.ndarray] = []
        self.shapes: list[tuple[str, int, int]] = []
        self._ntri = 0

    def material(self, rec: np.ndarray) -> int:
        self.materials.append(np.asarray(rec, np.float32))
        return len(self.materials) - 1

    def add_sphere(self, center, radius: float, mat: int, rotation=None, radiance=None, omni: bool = False) -> int:
        """An analytic sphere (Milton's Sphere: its centre, radius and object frame, given by the
        3 x 3 rotation from object to world, identity by default).  radiance: an emitting sphere
        of that Le (a light of type 4, area pi).  Returns its index among the spheres (its
        primitive id is the triangle count plus this index)."""
        R = np.eye(3) if rotation is None else np.asarray(rotation, np.float64)
        rec = np.zeros(8, np.float32)
        rec[0:3] = center
        rec[3] = radius
        rec[4:8] = quat_from_matrix(R.T)
        li = -1
        if radiance is not None:
            lrec = np.zeros(16, np.float32)
            lrec[0:3] = center
            lrec[9:12] = (0.0, 0.0, 1.0)
            lrec[12] = np.pi  # Sphere::_getSurfaceArea: the object-space area
            lrec[13:16] = np.broadcast_to(np.asarray(radiance, np.float64), 3)
            ext = np.zeros(16, np.float32)
            ext[0] = 4
            ext[1:5] = quat_from_matrix(R)
            ext[5] = radius
            ext[15] = 1.0 if omni else 0.0
            li = self.add_light(lrec, ext)
        self.spheres.append(rec)
        self.sphere_mat.append(int(mat))
        self.sphere_light.append(li)
        return len(self.spheres) - 1

    def background(self, tex: int = 0, le=(0.0, 0.0, 0.0)) -> None:
        """The scene's background: an environment map (tex = a value from texture()) or the
        constant radiance le."""
        self.bg_tex = int(tex)
        self.bg_le = np.broadcast_to(np.asarray(le, np.float32), 3).copy()

    def texture(self, tex: Texture) -> int:
        """Appends an image map; returns the value for a material texture slot (1 + index)."""
        self.textures.append(tex)
        return len(self.textures)

    def add(self, name: str, v: np.ndarray, n: np.ndarray | None, mat: int, light: int = -1, culled: bool = False,
            uv: np.ndarray | None = None):
        v = np.asarray(v, np.float32).reshape(-1, 3, 3)
        self.uv.append(None if uv is None else np.asarray(uv, np.float32).reshape(v.shape[0], 3, 2))
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
        li = self.add_light(rec)
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

    def add_light(self, rec: np.ndarray, ext: np.ndarray | None = None) -> int:
        """Appends a light record (and its extension, default: a plane); returns its index."""
        self.lights.append(np.asarray(rec, np.float32))
        self.light_ext.append(np.zeros(16, np.float32) if ext is None else np.asarray(ext, np.float32))
        return len(self.lights) - 1

    def add_triangle_light(self, name: str, v_world, obj_area: float, uvs, normal, radiance, mat: int,
                           culled: bool = True) -> int:
        """An emitting Milton `Triangle` (v1, v2, v3 in world space): one culled triangle and its
        light record (type 1, uv frame from its three uvs; area = its object-space area)."""
        v = np.asarray(v_world, np.float64).reshape(3, 3)
        uv = np.asarray(uvs, np.float64).reshape(3, 2)
        a, b = uv[1] - uv[0], uv[2] - uv[0]
        cross = abs(a[0] * b[1] - a[1] * b[0])
        if cross == 0:
            raise ValueError("degenerate triangle uv frame")
        rec = np.zeros(16, np.float32)
        rec[0:3], rec[3:6], rec[6:9] = v[0], v[1] - v[0], v[2] - v[0]
        rec[9:12] = np.asarray(normal, np.float64) / np.linalg.norm(normal)
        rec[12] = obj_area
        rec[13:16] = np.broadcast_to(np.asarray(radiance, np.float64), 3)
        ext = np.zeros(16, np.float32)
        ext[0] = 1
        ext[1:3], ext[3:5], ext[5:7], ext[7] = uv[0], a, b, 1.0 / cross
        li = self.add_light(rec, ext)
        self.add(name, v[None], np.broadcast_to(rec[9:12], (1, 3, 3)), mat, light=li, culled=culled)
        return li

    def add_mesh_light(self, name: str, v_world, n_world, radiance, mat: int, uv=None) -> int:
        """An emitting Milton `Mesh`: its two-sided triangles and one light record (type 2) over
        their run in the soup, area = the world-space area (Mesh::_getSurfaceArea)."""
        v = np.asarray(v_world, np.float64).reshape(-1, 3, 3)
        area = 0.5 * float(np.linalg.norm(np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]), axis=1).sum())
        rec = np.zeros(16, np.float32)
        rec[9:12] = (0.0, 1.0, 0.0)  # unused: a mesh light's normal is taken per sample
        rec[12] = area
        rec[13:16] = np.broadcast_to(np.asarray(radiance, np.float64), 3)
        ext = np.zeros(16, np.float32)
        ext[0] = 2
        ext.view(np.uint32)[8] = self._ntri
        ext.view(np.uint32)[9] = v.shape[0]
        li = self.add_light(rec, ext)
        self.add(name, v, n_world, mat, light=li, uv=uv)
        return li

    def build(self, camera: np.ndarray, name: str = "scene") -> Scene:
        cat = lambda xs, shape, dt: np.concatenate(xs) if xs else np.zeros(shape, dt)  # noqa: E731
        tri_uv = None
        if any(u is not None for u in self.uv):
            tri_uv = np.concatenate([np.zeros((v.shape[0], 3, 2), np.float32) if u is None else u
                                     for u, v in zip(self.uv, self.v)])
        return Scene(
            tri_uv=tri_uv, textures=list(self.textures), background_tex=self.bg_tex, background_le=self.bg_le,
            spheres=np.stack(self.spheres) if self.spheres else np.zeros((0, 8), np.float32),
            sphere_mat=np.asarray(self.sphere_mat, np.int32), sphere_light=np.asarray(self.sphere_light, np.int32),
            tri_v=cat(self.v, (0, 3, 3), np.float32), tri_n=cat(self.n, (0, 3, 3), np.float32),
            tri_mat=cat(self.mat, (0,), np.int32), tri_light=cat(self.light, (0,), np.int32),
            tri_flags=cat(self.flags, (0,), np.uint32),
            materials=np.stack(self.materials) if self.materials else np.zeros((0, 16), np.float32),
            lights=np.stack(self.lights) if self.lights else np.zeros((0, 16), np.float32),
            camera=camera, name=name, shapes=list(self.shapes),
            light_ext=np.stack(self.light_ext) if self.light_ext else np.zeros((0, 16), np.float32))
