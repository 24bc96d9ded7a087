"""Python host mirroring Milton's PathTracer / PointSampleRenderer interface over libmgpu.

Milton drives a renderer through a PropertyMap of string keys (mlt/src/milton/utils/PropertyMap.h),
``init()`` (Renderer.cpp:28-53) and a synchronous ``render()``; output is a per-pixel mean of
radiance samples (RenderOutput.cpp:72-101).  ``PathTracer`` here takes the same keys
(noSuperSamples, noDirectSamples, efficientDirect, kdMinPrimitives, kdMaxDepth,
kdCostTraversal, kdEmptyBias) plus maxDepth / rrStartDepth (defaults: no cap and 2, Milton's
behaviour, PathTracer.cpp:88-92), seed and wavePaths.

All rendering runs in libmgpu.so on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .scene import Scene


def _stream_handle(stream) -> int | None:
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available():
                return torch.cuda.current_stream().cuda_stream
        except Exception:  # torch absent: legacy default stream
            return None
        return None
    if isinstance(stream, int):
        return stream
    return getattr(stream, "cuda_stream", None)


def _desc(scene: Scene) -> N.SceneDesc:
    d = N.SceneDesc()
    d.ntri = scene.ntri
    d.tri_v = N.ptr(scene.tri_v)
    d.tri_n = N.ptr(scene.tri_n)
    d.tri_mat = N.ptr(scene.tri_mat)
    d.tri_light = N.ptr(scene.tri_light)
    d.tri_flags = N.ptr(scene.tri_flags)
    d.nmat = len(scene.materials)
    d.materials = N.ptr(scene.materials)
    d.nlight = len(scene.lights)
    lights = scene.lights if len(scene.lights) else np.zeros((1, 16), np.float32)
    d.lights = N.ptr(lights)
    d.light_ext = N.ptr(scene.light_ext) if len(scene.lights) else None
    d.tri_uv = None if scene.tri_uv is None else N.ptr(scene.tri_uv)
    d.ntex = len(scene.textures)
    texs = (N.Texture * max(1, len(scene.textures)))()
    for i, t in enumerate(scene.textures):
        h, w, _ = t.rgb.shape
        f, support, p1, p2 = t.filter_params()
        texs[i] = N.Texture(w, h, N.ptr(t.rgb), t.kind, f, support, p1, p2, t.repeat_u, t.repeat_v,
                            t.bump_intensity)
    d.textures = texs
    d.nsphere = len(scene.spheres)
    d.spheres = N.ptr(scene.spheres) if len(scene.spheres) else None
    d.sphere_mat = N.ptr(scene.sphere_mat) if len(scene.spheres) else None
    d.sphere_light = N.ptr(scene.sphere_light) if len(scene.spheres) else None
    d.background_tex = int(scene.background_tex)
    for k in range(3):
        d.background_le[k] = float(scene.background_le[k])
    d._keep = (scene, lights, texs)  # keep buffers alive while the struct is used
    return d


@dataclass
class KdSettings:
    """kdTreeAccel build parameters: Milton's defaults (kdTreeAccel.h:97-104) except the traversal
    cost, MGPU_KD_COST_TRAVERSAL = 3 (include/mgpu.h: a node step costs the GPU's traversal
    kernels about three triangle tests); ``KdSettings.milton()`` is Milton's set exactly."""
    min_prims: int = 3
    max_depth: int = 24
    cost_traversal: float = 3.0
    empty_bias: float = 0.9
    threads: int = 0

    @classmethod
    def milton(cls, **kw) -> "KdSettings":
        return cls(**{"cost_traversal": 1.0, **kw})

    def to_c(self) -> N.KdParams:
        return N.KdParams(self.min_prims, self.max_depth, self.cost_traversal, self.empty_bias, self.threads)


class Accel:
    """Host SAH kd-tree over a scene's triangle soup (mgpu_accel_*)."""

    def __init__(self, scene: Scene, kd: KdSettings | None = None):
        self._lib = N.load()
        self.handle = C.c_void_p()
        d = _desc(scene)
        N.check(self._lib.mgpu_accel_build(C.byref(d), C.byref((kd or KdSettings()).to_c()), C.byref(self.handle)))
        self.ntri = scene.ntri

    def stats(self) -> dict:
        s = N.KdStats()
        N.check(self._lib.mgpu_accel_stats(self.handle, C.byref(s)))
        return {f: getattr(s, f) for f, _ in N.KdStats._fields_}

    def serialize(self):
        nn, npr = C.c_int64(), C.c_int64()
        N.check(self._lib.mgpu_accel_serialize(self.handle, None, None, None, None, C.byref(nn), C.byref(npr)))
        kind = np.zeros(nn.value, np.int32)
        split = np.zeros(nn.value, np.float32)
        count = np.zeros(nn.value, np.int32)
        prims = np.zeros(max(npr.value, 1), np.int32)
        N.check(self._lib.mgpu_accel_serialize(self.handle, N.ptr(kind), N.ptr(split), N.ptr(count), N.ptr(prims),
                                               C.byref(nn), C.byref(npr)))
        return kind, split, count, prims[:npr.value]

    def close(self):
        if self.handle:
            self._lib.mgpu_accel_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceScene:
    """Scene resident on the current CUDA device (mgpu_scene_create)."""

    def __init__(self, scene: Scene, accel: Accel, stream=None):
        self._lib = N.load()
        self.handle = C.c_void_p()
        d = _desc(scene)
        N.check(self._lib.mgpu_scene_create(C.byref(d), accel.handle, _stream_handle(stream), C.byref(self.handle)))
        self.scene = scene

    def set_top_pairs(self, n: int) -> None:
        N.check(self._lib.mgpu_scene_set_top_pairs(self.handle, n))

    @property
    def nbytes(self) -> int:
        v = C.c_uint64()
        N.check(self._lib.mgpu_scene_bytes(self.handle, C.byref(v)))
        return v.value

    def texels(self, tex: int, stream=None) -> np.ndarray:
        """Texture tex as the device holds it: (H, W, 4) float32 (filtered rgb, or bump gx, gy)."""
        h, w, _ = self.scene.textures[tex].rgb.shape
        out = np.zeros((h, w, 4), np.float32)
        N.check(self._lib.mgpu_scene_read_texels(self.handle, tex, N.ptr(out), _stream_handle(stream)))
        return out

    def close(self):
        if self.handle:
            self._lib.mgpu_scene_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Film:
    """Compensated FP32 film (per pixel: rgb sum + count, rgb Kahan compensation + sum of
    squared per-sample luminance)."""

    def __init__(self, width: int, height: int, stream=None):
        self._lib = N.load()
        self.width, self.height = width, height
        self.handle = C.c_void_p()
        N.check(self._lib.mgpu_film_create(width, height, _stream_handle(stream), C.byref(self.handle)))

    def clear(self, stream=None):
        N.check(self._lib.mgpu_film_clear(self.handle, _stream_handle(stream)))

    filter = ("none", 0.0, {})

    def mean(self, stream=None) -> np.ndarray:
        out = np.zeros((self.height, self.width, 3), np.float64)
        N.check(self._lib.mgpu_film_read(self.handle, N.ptr(out), _stream_handle(stream)))
        return out

    def raw(self, stream=None) -> np.ndarray:
        out = np.zeros((2, self.height, self.width, 4), np.float32)
        N.check(self._lib.mgpu_film_read_raw(self.handle, N.ptr(out), _stream_handle(stream)))
        return out

    def set_filter(self, kind: str = "none", support: float = 2.0, stream=None, **params) -> None:
        """Reconstruction filter of the film's output (mgpu_film_set_filter): "none", "box",
        "triangle", "gaussian" (sigma), "mitchell" (B, C), "lanczosSinc" (tau), with Milton's
        defaults (M/filters/KernelFilter.cpp:18-40)."""
        kinds = {"none": 0, "box": 1, "triangle": 2, "gaussian": 3, "mitchell": 4, "lanczosSinc": 5}
        if kind not in kinds:
            raise ValueError(f"unknown filter {kind!r}")
        p1, p2 = 0.0, 0.0
        if kind == "gaussian":
            p1 = params.get("sigma", 1.0)
        elif kind == "mitchell":
            p1, p2 = params.get("B", 1.0 / 3.0), params.get("C", 1.0 / 3.0)
        elif kind == "lanczosSinc":
            p1 = params.get("tau", 3.0)
        N.check(self._lib.mgpu_film_set_filter(self.handle, kinds[kind], float(support), float(p1), float(p2),
                                               _stream_handle(stream)))
        self.filter = (kind, float(support), dict(params))

    def tonemap(self, stream=None) -> np.ndarray:
        """mgpu_film_tonemap: Milton's Reinhard tone map of the per-pixel means, (H, W, 4) uint8."""
        out = np.zeros((self.height, self.width, 4), np.uint8)
        N.check(self._lib.mgpu_film_tonemap(self.handle, N.ptr(out), _stream_handle(stream)))
        return out

    def rmse_estimate(self, stream=None) -> float:
        """Estimated RMSE of the per-pixel mean luminance: sqrt(mean over pixels of the sample
        variance / n), from the film's second moment."""
        return rmse_estimate(self.raw(stream))

    def close(self):
        if self.handle:
            self._lib.mgpu_film_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rmse_estimate(raw: np.ndarray) -> float:
    """sqrt(mean_pixels(var / n)) of the per-pixel mean luminance, from a raw film."""
    s, c = raw[0].astype(np.float64), raw[1].astype(np.float64)
    n = s[..., 3]
    ok = n > 1
    if not ok.any():
        return float("inf")
    mean = ((s[..., :3] - c[..., :3]).sum(-1) / 3.0)[ok] / n[ok]
    m2 = c[..., 3][ok] / n[ok]
    var = np.maximum(m2 - mean * mean, 0.0) * n[ok] / (n[ok] - 1)
    return float(np.sqrt(np.mean(var / n[ok])))


def film_error(films, stream=None) -> np.ndarray:
    """mgpu_film_error: the device-side rmse_estimate of several films in one pass."""
    films = list(films)
    arr = (C.c_void_p * max(1, len(films)))(*[f.handle.value for f in films])
    out = np.zeros(max(1, len(films)), np.float64)
    N.check(N.load().mgpu_film_error(arr, len(films), N.ptr(out), _stream_handle(stream)))
    return out[:len(films)]


def resolve_autofocus(camera: np.ndarray, dscene: "DeviceScene", stream=None) -> np.ndarray:
    """ThinLensCamera's autofocus (ThinLensCamera.cpp:97-121).  A camera whose focal distance
    is negative asks for it: the ray through focal point (camera[14], camera[15]) -- taken, as
    in the reference, at (p - 0.5) in film coordinates, half the offset a pixel ray uses -- is
    traced on the device, and its hit distance becomes the focal distance; on a miss the
    fallback |camera[13]| (the focalDistance key, default 1) is kept.  Returns the camera."""
    cam = np.array(camera, np.float32).reshape(-1)
    if cam.shape[0] < 16 or not (cam[11] > 0 and cam[13] < 0):
        return cam
    eye, look, up = (cam[0:3].astype(np.float64), cam[3:6].astype(np.float64), cam[6:9].astype(np.float64))
    n = -look
    u = np.cross(up, n)
    n /= np.linalg.norm(n)
    u /= np.linalg.norm(u)
    v = np.cross(n, u)
    th = np.tan(np.radians(float(cam[9])) / 2)
    tw = float(cam[10]) * th
    fx = np.clip(cam[14], 0, 1) - 0.5
    fy = 0.5 - np.clip(cam[15], 0, 1)
    d = u * (tw * fx) + v * (th * fy) - n
    d /= np.linalg.norm(d)
    import torch
    rays = torch.tensor([[*eye, 0.0, *d, float("inf")]], dtype=torch.float32, device="cuda")
    hits = trace_closest(dscene, rays, stream=stream)
    torch.cuda.synchronize()
    t = float(hits[0, 0].item())
    cam[13] = t if np.isfinite(t) and t > 0 else -cam[13]
    cam[14] = cam[15] = 0.0
    return cam


@dataclass
class RenderSettings:
    width: int
    height: int
    spp: int
    sample_begin: int = 0
    sample_count: int | None = None
    no_direct_samples: int = 1
    max_depth: int = 0
    rr_start_depth: int = 2
    efficient_direct: int = 1
    wave_paths: int = 0
    seed: int = 0
    stream_id: int = 0

    def to_c(self, camera: np.ndarray) -> N.RenderParams:
        p = N.RenderParams()
        p.width, p.height, p.spp = self.width, self.height, self.spp
        p.sample_begin = self.sample_begin
        p.sample_count = self.spp - self.sample_begin if self.sample_count is None else self.sample_count
        p.no_direct_samples = self.no_direct_samples
        p.max_depth, p.rr_start_depth = self.max_depth, self.rr_start_depth
        p.efficient_direct, p.wave_paths = self.efficient_direct, self.wave_paths
        p.seed, p.stream_id = self.seed, self.stream_id
        cam = np.asarray(camera, np.float32).reshape(-1)
        for i in range(16):
            p.camera[i] = float(cam[i]) if i < cam.shape[0] else 0.0
        return p


def render(dscene: DeviceScene, settings: RenderSettings, film: Film, camera: np.ndarray | None = None,
           stream=None, path_out=None) -> None:
    """mgpu_render: add sample passes to the film (stream-ordered)."""
    lib = N.load()
    p = settings.to_c(dscene.scene.camera if camera is None else camera)
    if path_out is None:
        N.check(lib.mgpu_render(dscene.handle, C.byref(p), film.handle, _stream_handle(stream)))
    else:
        N.check(lib.mgpu_render_paths(dscene.handle, C.byref(p), film.handle, path_out.data_ptr(),
                                      _stream_handle(stream)))


def render_noalloc(dscene: DeviceScene, settings: RenderSettings, film: Film, camera: np.ndarray | None = None,
                   stream=None) -> None:
    """mgpu_render_noalloc: like render(), but over the library's fixed 32 MiB device scratch
    instead of allocating a workspace (for hosts that forbid device allocation while rendering;
    calls must not overlap on the GPU)."""
    lib = N.load()
    p = settings.to_c(dscene.scene.camera if camera is None else camera)
    N.check(lib.mgpu_render_noalloc(dscene.handle, C.byref(p), film.handle, _stream_handle(stream)))


def render_counted(dscene: DeviceScene, settings: RenderSettings, film: Film, stream=None) -> dict:
    """Render with traversal counters (slower; measurement only)."""
    lib = N.load()
    p = settings.to_c(dscene.scene.camera)
    out = np.zeros(8, np.uint64)
    N.check(lib.mgpu_render_counted(dscene.handle, C.byref(p), film.handle, N.ptr(out), _stream_handle(stream)))
    keys = ("ext_nodes", "ext_refs", "ext_tris", "ext_rays", "sh_nodes", "sh_refs", "sh_tris", "sh_rays")
    return {k: int(v) for k, v in zip(keys, out)}


KERNELS = ("generate", "extend", "shade", "shadow", "accumulate", "binning")


def profile_enable(enable: bool = True) -> None:
    N.check(N.load().mgpu_profile_enable(1 if enable else 0))


def tune(key: str, value: int) -> None:
    """Process-wide tuning knob (persistent, bin_shadow, bin_extension); results are unchanged."""
    N.check(N.load().mgpu_tune_set(key.encode(), int(value)))


def tune_get(key: str) -> int:
    v = C.c_int64()
    N.check(N.load().mgpu_tune_get(key.encode(), C.byref(v)))
    return int(v.value)


def profile_read() -> dict:
    ms = np.zeros(6, np.float64)
    n = np.zeros(6, np.uint64)
    N.check(N.load().mgpu_profile_read(N.ptr(ms), N.ptr(n)))
    return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(KERNELS)}


def wave_queues(max_bounces: int = 16) -> tuple[np.ndarray, np.ndarray]:
    """Per-bounce extension and shadow queue sizes of the last wave rendered on this thread."""
    ext = np.zeros(max_bounces, np.uint32)
    sh = np.zeros(max_bounces, np.uint32)
    N.check(N.load().mgpu_render_wave_queues(N.ptr(ext), N.ptr(sh), max_bounces))
    return ext, sh


class Batch:
    """Render requests of different scenes / resolutions / sample counts sharing waves
    (mgpu_batch_*); each film receives exactly the image render() would give it."""

    def __init__(self, wave_paths: int = 0, use_graph: bool = True):
        self._lib = N.load()
        self.handle = C.c_void_p()
        N.check(self._lib.mgpu_batch_create(C.byref(self.handle)))
        N.check(self._lib.mgpu_batch_set(self.handle, wave_paths, 1 if use_graph else 0))
        self._keep = []

    def add(self, dscene: DeviceScene, settings: RenderSettings, film: Film, camera: np.ndarray | None = None):
        p = settings.to_c(dscene.scene.camera if camera is None else camera)
        N.check(self._lib.mgpu_batch_add(self.handle, dscene.handle, C.byref(p), film.handle))
        self._keep.append((dscene, film))

    def render(self, stream=None):
        N.check(self._lib.mgpu_batch_render(self.handle, _stream_handle(stream)))

    def clear(self):
        N.check(self._lib.mgpu_batch_clear(self.handle))
        self._keep = []

    def close(self):
        if self.handle:
            self._lib.mgpu_batch_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def measure_read_bandwidth(nbytes: int, reps: int, stream=None) -> float:
    """GB/s of reading a device buffer of nbytes reps times in one launch (L2-only loads):
    an L2-resident buffer measures the L2's read bandwidth, a larger one the HBM's."""
    out = C.c_double()
    N.check(N.load().mgpu_measure_read_bandwidth(int(nbytes), int(reps), C.byref(out), _stream_handle(stream)))
    return out.value


def render_stats() -> dict:
    s = N.RenderStats()
    N.check(N.load().mgpu_render_stats_get(C.byref(s)))
    return {f: getattr(s, f) for f, _ in N.RenderStats._fields_}


def launch_count() -> int:
    return int(N.load().mgpu_launch_count())


def trace_closest(dscene: DeviceScene, rays, stream=None, counts=None):
    """rays: CUDA float32 tensor (n, 8) -> hits (n, 4): t, prim (int bits), b1, b2."""
    import torch
    n = rays.shape[0]
    hits = torch.empty((n, 4), dtype=torch.float32, device=rays.device)
    lib = N.load()
    if counts is None:
        N.check(lib.mgpu_trace_closest(dscene.handle, rays.data_ptr(), hits.data_ptr(), n, _stream_handle(stream)))
    else:
        N.check(lib.mgpu_trace_closest_counted(dscene.handle, rays.data_ptr(), hits.data_ptr(), counts.data_ptr(), n,
                                               _stream_handle(stream)))
    return hits


def trace_any(dscene: DeviceScene, rays, stream=None):
    import torch
    n = rays.shape[0]
    occ = torch.empty((n,), dtype=torch.uint8, device=rays.device)
    N.check(N.load().mgpu_trace_any(dscene.handle, rays.data_ptr(), occ.data_ptr(), n, _stream_handle(stream)))
    return occ


@dataclass
class PathTracer:
    """Milton ``PathTracer`` with its PropertyMap keys; ``init`` builds the kd-tree and makes
    the scene resident, ``render`` runs every super-sample pass on the GPU."""
    props: dict = field(default_factory=dict)
    scene: Scene | None = None
    width: int = 0
    height: int = 0

    # reconstruction filter of the output (kind, support, params), e.g. from a scene file's
    # "output" block; None = per-pixel mean
    output_filter: tuple | None = None

    def __post_init__(self):
        self._accel = None
        self._dscene = None
        self._film = None
        self._camera = None

    # PropertyMap::getValue(key, default)
    def get(self, key, default):
        return self.props.get(key, default)

    def set_scene(self, scene: Scene):
        self.scene = scene

    def set_output(self, width: int, height: int):
        self.width, self.height = width, height

    def kd_settings(self) -> KdSettings:
        return KdSettings(int(self.get("kdMinPrimitives", 3)), int(self.get("kdMaxDepth", 24)),
                          float(self.get("kdCostTraversal", KdSettings.cost_traversal)),
                          float(self.get("kdEmptyBias", 0.9)),
                          int(self.get("kdNoThreads", 0)))

    def settings(self) -> RenderSettings:
        return RenderSettings(
            width=self.width, height=self.height, spp=int(self.get("noSuperSamples", 4)),
            no_direct_samples=int(self.get("noDirectSamples", 1)), max_depth=int(self.get("maxDepth", 0)),
            rr_start_depth=int(self.get("rrStartDepth", 2)), efficient_direct=int(bool(self.get("efficientDirect", True))),
            wave_paths=int(self.get("wavePaths", 0)), seed=int(self.get("seed", 0)))

    def init(self):
        if self.scene is None:
            raise ValueError("PathTracer.init: no scene set")
        if self.width <= 0 or self.height <= 0:
            raise ValueError("PathTracer.init: no output set")
        self._accel = Accel(self.scene, self.kd_settings())
        self._dscene = DeviceScene(self.scene, self._accel)
        self._film = Film(self.width, self.height)
        if self.output_filter is not None:
            kind, support, params = self.output_filter
            self._film.set_filter(kind, support, **params)
        self._camera = resolve_autofocus(self.scene.camera, self._dscene)

    def render(self, stream=None):
        if self._dscene is None:
            raise RuntimeError("PathTracer.render: init() has not been called")
        self._film.clear(stream)
        render(self._dscene, self.settings(), self._film, camera=self._camera, stream=stream)

    def output(self) -> np.ndarray:
        return self._film.mean()

    def write_png(self, path: str) -> None:
        """The output through Milton's Reinhard tone map (on the device), as an 8-bit PNG."""
        from .imageio import write_png
        write_png(path, self._film.tonemap())

    @property
    def accel(self) -> Accel:
        return self._accel

    @property
    def device_scene(self) -> DeviceScene:
        return self._dscene

    @property
    def film(self) -> Film:
        return self._film
