"""The C-ABI library loads and exports every entry point include/*.h declares (no GPU calls)."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
DECL = re.compile(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b((?:mgpu|plugin)_\w+)\s*\(", re.M)


def declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in DECL.finditer(text):
            if "typedef" not in text[max(0, m.start() - 40):m.start()]:
                names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_boundary():
    names = declared()
    for must in ("mgpu_accel_build", "mgpu_scene_create", "mgpu_trace_closest", "mgpu_trace_any", "mgpu_render",
                 "mgpu_film_read", "mgpu_last_error", "plugin_type", "plugin_new", "plugin_delete"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from milton_gb300 import _native
    lib = _native.load()
    bound = {n for n, _, _ in _native.SIGNATURES}
    for name in declared():
        assert hasattr(lib, name), f"{name} not exported"
        assert name in bound, f"{name} has no ctypes signature"


def test_plugin_abi_and_errors_without_gpu():
    from milton_gb300 import _native
    lib = _native.load()
    assert lib.plugin_type() == 0  # MILTON_PLUGIN_TYPE_RENDERER
    r = lib.plugin_new()
    assert r
    # PropertyMap round trip and Renderer::init preconditions (host-only paths)
    assert lib.mgpu_renderer_set_value(r, b"noSuperSamples", b"16") == 0
    buf = C.create_string_buffer(32)
    assert lib.mgpu_renderer_get_value(r, b"noSuperSamples", buf, 32) == 0 and buf.value == b"16"
    assert lib.mgpu_renderer_init(r) == -1
    assert b"no scene" in lib.mgpu_last_error()
    assert lib.mgpu_renderer_render(r) == -1
    lib.plugin_delete(r)
    # argument validation happens before any device work
    assert lib.mgpu_accel_build(None, None, None) == -1
    assert lib.mgpu_trace_closest(None, None, None, 1, None) == -1
    assert lib.mgpu_render(None, None, None, None) == -1
    assert lib.mgpu_version() == 1


def test_dynamic_loader_mirrors_milton(tmp_path):
    from milton_gb300.plugin import load_dynamic_renderer, PluginError
    r = load_dynamic_renderer(str(ROOT / "milton_gb300" / "lib" / "libmgpu.so"))
    assert r.handle
    r.close()
    with pytest.raises(PluginError, match="failed to load"):
        load_dynamic_renderer(str(tmp_path / "missing.so"))
