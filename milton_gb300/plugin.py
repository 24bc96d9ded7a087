"""Milton's `"renderer": {"type": "dynamic", "path": ...}` plugin loading, for hosts that speak
the C interface (MiltonJSONSceneLoader::_parse_dynamic_plugin,
mlt/src/milton/loaders/MiltonJSONSceneLoader.cpp:1770-1813): dlopen, resolve plugin_type and
plugin_new, check the type, instantiate; the same error cases raise PluginError."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .pathtracer import _desc
from .scene import Scene

MILTON_PLUGIN_TYPE_RENDERER = 0


class PluginError(RuntimeError):
    pass


class DynamicRenderer:
    """The renderer object behind plugin_new(), driven through mgpu_renderer_*."""

    def __init__(self, lib: C.CDLL, handle: int):
        self.lib, self.handle = lib, handle
        self.width = self.height = 0

    def __setitem__(self, key: str, value) -> None:
        if isinstance(value, bool):
            value = "true" if value else "false"
        N.check(self.lib.mgpu_renderer_set_value(self.handle, key.encode(), str(value).encode()))

    def set_scene(self, scene: Scene) -> None:
        d = _desc(scene)
        N.check(self.lib.mgpu_renderer_set_scene(self.handle, C.byref(d)))
        cam = np.ascontiguousarray(scene.camera, np.float32)
        N.check(self.lib.mgpu_renderer_set_camera(self.handle, cam.ctypes.data))
        N.check(self.lib.mgpu_renderer_set_lens(self.handle, float(cam[11]), float(cam[12]), float(cam[13])))

    def set_output(self, width: int, height: int) -> None:
        self.width, self.height = width, height
        N.check(self.lib.mgpu_renderer_set_output(self.handle, width, height))

    def init(self) -> None:
        N.check(self.lib.mgpu_renderer_init(self.handle))

    def render(self) -> None:
        N.check(self.lib.mgpu_renderer_render(self.handle))

    def output(self) -> np.ndarray:
        out = np.zeros((self.height, self.width, 3), np.float64)
        N.check(self.lib.mgpu_renderer_get_output(self.handle, out.ctypes.data))
        return out

    def close(self) -> None:
        if self.handle:
            self.lib.plugin_delete(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def load_dynamic_renderer(path: str) -> DynamicRenderer:
    try:
        lib = C.CDLL(path, mode=C.RTLD_LOCAL)
    except OSError as e:
        raise PluginError(f"{path}: plugin failed to load: {e}") from None
    for sym in ("plugin_type", "plugin_new"):
        if not hasattr(lib, sym):
            raise PluginError(f"{path}: invalid plugin; could not find {sym} symbol")
    lib.plugin_type.restype = C.c_int
    lib.plugin_new.restype = C.c_void_p
    kind = lib.plugin_type()
    if kind != MILTON_PLUGIN_TYPE_RENDERER:
        raise PluginError(f"{path}: dynamic plugin expected type '{MILTON_PLUGIN_TYPE_RENDERER}' but found type '{kind}'")
    # the entry points behind the handle are libmgpu's; bind them with the shared signatures
    for name, res, args in N.SIGNATURES:
        if hasattr(lib, name):
            fn = getattr(lib, name)
            fn.restype, fn.argtypes = res, args
    handle = lib.plugin_new()
    if not handle:
        raise PluginError(f"{path}: invalid plugin; plugin_new returned NULL")
    return DynamicRenderer(lib, handle)
