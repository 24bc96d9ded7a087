"""The GPU PathTracer as a renderer object for Python hosts (include/mgpu_renderer.h): Milton's
PropertyMap keys, setScene / setCamera / setOutput, Renderer::init, Renderer::render and the
finalized output (mlt/src/milton/renderers/Renderer.h:52-62, PointSampleRenderer.h:61-95).

Milton itself loads the C++ plugin milton_gb300/lib/libmgpu_milton.so (`PLUGIN_PATH`), a
milton::PointSampleRenderer built from milton_gb300/milton_plugin/gpu_path_tracer.cpp."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _native as N
from .pathtracer import _desc
from .scene import Scene

PLUGIN_PATH = Path(__file__).resolve().parent / "lib" / "libmgpu_milton.so"


class RendererObject:
    """One mgpu_renderer: a GPU PathTracer driven through mgpu_renderer_*."""

    def __init__(self):
        self.lib = N.load()
        h = C.c_void_p()
        N.check(self.lib.mgpu_renderer_create(C.byref(h)))
        self.handle = h.value
        self.width = self.height = 0

    def __setitem__(self, key: str, value) -> None:
        if isinstance(value, bool):
            value = "true" if value else "false"
        N.check(self.lib.mgpu_renderer_set_value(self.handle, key.encode(), str(value).encode()))

    def __getitem__(self, key: str) -> str:
        buf = C.create_string_buffer(256)
        N.check(self.lib.mgpu_renderer_get_value(self.handle, key.encode(), buf, 256))
        return buf.value.decode()

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
            self.lib.mgpu_renderer_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
