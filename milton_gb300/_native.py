"""ctypes binding of libmgpu.so (include/mgpu.h, include/mgpu_server.h, include/mgpu_renderer.h).

There is no fallback: if the in-tree library is missing, importing this module raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libmgpu.so"

MGPU_OK = 0
ERRORS = {-1: "MGPU_E_INVALID", -2: "MGPU_E_CUDA", -3: "MGPU_E_NOMEM", -4: "MGPU_E_BUDGET", -5: "MGPU_E_STATE",
          -6: "MGPU_E_DEVICE"}


class MgpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class KdParams(C.Structure):
    _fields_ = [("min_prims", C.c_uint32), ("max_depth", C.c_uint32), ("cost_traversal", C.c_double),
                ("empty_bias", C.c_double), ("threads", C.c_uint32)]


class KdStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("no_internal", "no_leaves", "min_depth", "max_depth", "sum_depth",
                                          "min_prims", "max_prims", "sum_prims", "node_pairs", "refs",
                                          "bytes_nodes", "bytes_refs")] + [("build_seconds", C.c_double)]


class Texture(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("rgb", C.c_void_p), ("kind", C.c_int32),
                ("filter", C.c_int32), ("support", C.c_float), ("p1", C.c_float), ("p2", C.c_float),
                ("repeat_u", C.c_float), ("repeat_v", C.c_float), ("bump_intensity", C.c_float)]


class SceneDesc(C.Structure):
    _fields_ = [("ntri", C.c_int64), ("tri_v", C.c_void_p), ("tri_n", C.c_void_p), ("tri_mat", C.c_void_p),
                ("tri_light", C.c_void_p), ("tri_flags", C.c_void_p), ("nmat", C.c_int32),
                ("materials", C.c_void_p), ("nlight", C.c_int32), ("lights", C.c_void_p),
                ("light_ext", C.c_void_p), ("tri_uv", C.c_void_p), ("ntex", C.c_int32),
                ("textures", C.POINTER(Texture)), ("background_tex", C.c_int32), ("background_le", C.c_float * 3),
                ("nsphere", C.c_int32), ("spheres", C.c_void_p), ("sphere_mat", C.c_void_p),
                ("sphere_light", C.c_void_p)]


class RenderParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("sample_begin", C.c_int32),
                ("sample_count", C.c_int32), ("no_direct_samples", C.c_int32), ("max_depth", C.c_int32),
                ("rr_start_depth", C.c_int32), ("efficient_direct", C.c_int32), ("wave_paths", C.c_int32),
                ("seed", C.c_uint64), ("stream_id", C.c_uint32), ("camera", C.c_float * 16)]


class ServerParams(C.Structure):
    _fields_ = [("hbm_budget", C.c_uint64), ("tick_paths", C.c_int64), ("max_active", C.c_int32),
                ("wave_paths", C.c_int32), ("use_graph", C.c_int32), ("build_threads", C.c_int32),
                ("kd", KdParams), ("policy", C.c_int32)]


class ServerJobInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("scene", C.c_int32), ("spp_done", C.c_int32), ("reached_target", C.c_int32),
                ("rmse", C.c_double), ("t_arrival", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double),
                ("paths", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = ([(n, C.c_uint64) for n in ("resident_bytes", "peak_resident_bytes", "scene_bytes", "film_bytes",
                                           "paths", "ticks", "admitted", "finished", "failed", "evictions",
                                           "uploads", "builds")]
                + [(n, C.c_int32) for n in ("queued", "active", "resident_scenes", "building")]
                + [("render_seconds", C.c_double)])


class RenderStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("paths", "extension_rays", "shadow_rays", "truncated_paths", "bounces",
                                          "kernel_launches")]


# (name, restype, argtypes) for every exported entry point; the ABI test checks this list
# against include/*.h.
SIGNATURES = [
    ("mgpu_last_error", C.c_char_p, []),
    ("mgpu_version", C.c_int, []),
    ("mgpu_accel_build", C.c_int, [C.POINTER(SceneDesc), C.POINTER(KdParams), C.POINTER(C.c_void_p)]),
    ("mgpu_accel_stats", C.c_int, [C.c_void_p, C.POINTER(KdStats)]),
    ("mgpu_accel_serialize", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("mgpu_accel_destroy", C.c_int, [C.c_void_p]),
    ("mgpu_scene_create", C.c_int, [C.POINTER(SceneDesc), C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    ("mgpu_scene_destroy", C.c_int, [C.c_void_p]),
    ("mgpu_scene_bytes", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    ("mgpu_scene_set_top_pairs", C.c_int, [C.c_void_p, C.c_uint32]),
    ("mgpu_accel_device_bytes", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_uint64)]),
    ("mgpu_scene_device_bytes", C.c_int, [C.POINTER(SceneDesc), C.c_void_p, C.POINTER(C.c_uint64)]),
    ("mgpu_scene_read_texels", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    ("mgpu_trace_closest", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    ("mgpu_trace_any", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    ("mgpu_trace_closest_counted", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                             C.c_void_p]),
    ("mgpu_film_create", C.c_int, [C.c_int32, C.c_int32, C.c_void_p, C.POINTER(C.c_void_p)]),
    ("mgpu_film_clear", C.c_int, [C.c_void_p, C.c_void_p]),
    ("mgpu_film_destroy", C.c_int, [C.c_void_p]),
    ("mgpu_film_read", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("mgpu_film_read_raw", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("mgpu_film_error", C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.c_void_p, C.c_void_p]),
    ("mgpu_film_tonemap", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("mgpu_film_set_filter", C.c_int, [C.c_void_p, C.c_int32, C.c_float, C.c_float, C.c_float, C.c_void_p]),
    ("mgpu_render", C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.c_void_p, C.c_void_p]),
    ("mgpu_render_noalloc", C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.c_void_p, C.c_void_p]),
    ("mgpu_batch_create", C.c_int, [C.POINTER(C.c_void_p)]),
    ("mgpu_batch_add", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(RenderParams), C.c_void_p]),
    ("mgpu_batch_set", C.c_int, [C.c_void_p, C.c_int64, C.c_int32]),
    ("mgpu_batch_render", C.c_int, [C.c_void_p, C.c_void_p]),
    ("mgpu_batch_clear", C.c_int, [C.c_void_p]),
    ("mgpu_batch_destroy", C.c_int, [C.c_void_p]),
    ("mgpu_render_paths", C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.c_void_p, C.c_void_p, C.c_void_p]),
    ("mgpu_render_stats_get", C.c_int, [C.POINTER(RenderStats)]),
    ("mgpu_render_wave_queues", C.c_int, [C.c_void_p, C.c_void_p, C.c_int32]),
    ("mgpu_render_counted", C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.c_void_p, C.c_void_p, C.c_void_p]),
    ("mgpu_profile_enable", C.c_int, [C.c_int]),
    ("mgpu_profile_read", C.c_int, [C.c_void_p, C.c_void_p]),
    ("mgpu_tune_set", C.c_int, [C.c_char_p, C.c_int64]),
    ("mgpu_tune_get", C.c_int, [C.c_char_p, C.POINTER(C.c_int64)]),
    ("mgpu_launch_count", C.c_uint64, []),
    ("mgpu_server_create", C.c_int, [C.POINTER(ServerParams), C.POINTER(C.c_void_p)]),
    ("mgpu_server_destroy", C.c_int, [C.c_void_p]),
    ("mgpu_server_clock", C.c_double, [C.c_void_p]),
    ("mgpu_server_add_scene", C.c_int, [C.c_void_p, C.POINTER(SceneDesc), C.POINTER(C.c_int32)]),
    ("mgpu_server_prefetch", C.c_int, [C.c_void_p, C.c_int32]),
    ("mgpu_server_submit", C.c_int, [C.c_void_p, C.c_int32, C.POINTER(RenderParams), C.c_int32, C.c_double,
                                     C.c_double, C.POINTER(C.c_int64)]),
    ("mgpu_server_step", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int32)]),
    ("mgpu_server_job", C.c_int, [C.c_void_p, C.c_int64, C.POINTER(ServerJobInfo)]),
    ("mgpu_server_read", C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    ("mgpu_server_release", C.c_int, [C.c_void_p, C.c_int64]),
    ("mgpu_server_stats_get", C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    ("mgpu_measure_read_bandwidth", C.c_int, [C.c_uint64, C.c_int32, C.POINTER(C.c_double), C.c_void_p]),
    ("mgpu_renderer_create", C.c_int, [C.POINTER(C.c_void_p)]),
    ("mgpu_renderer_destroy", C.c_int, [C.c_void_p]),
    ("mgpu_renderer_set_value", C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p]),
    ("mgpu_renderer_get_value", C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_size_t]),
    ("mgpu_renderer_set_scene", C.c_int, [C.c_void_p, C.POINTER(SceneDesc)]),
    ("mgpu_renderer_set_camera", C.c_int, [C.c_void_p, C.c_void_p]),
    ("mgpu_renderer_set_lens", C.c_int, [C.c_void_p, C.c_float, C.c_float, C.c_float]),
    ("mgpu_renderer_set_output", C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    ("mgpu_renderer_init", C.c_int, [C.c_void_p]),
    ("mgpu_renderer_render", C.c_int, [C.c_void_p]),
    ("mgpu_renderer_get_output", C.c_int, [C.c_void_p, C.c_void_p]),
]

_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
                          "(there is no CPU fallback for the GPU path)")
    lib = C.CDLL(str(LIB_PATH))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != MGPU_OK:
        msg = load().mgpu_last_error()
        raise MgpuError(rc, msg.decode() if msg else "")


def ptr(a) -> int:
    """Address of a numpy array's data (or None)."""
    if a is None:
        return None
    return a.ctypes.data
