"""The C-ABI library loads and exports every entry point include/*.h declares, and the Milton
plugin library exports the three entry points Milton resolves (no GPU calls)."""
import ctypes as C
import re
import subprocess
from pathlib import Path


ROOT = Path(__file__).resolve().parent.parent
DECL = re.compile(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b((?:mgpu|plugin)_\w+)\s*\(", re.M)


def declared(headers=("mgpu.h", "mgpu_server.h", "mgpu_renderer.h")):
    names = set()
    for h in headers:
        text = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / h).read_text(), flags=re.S)
        for m in DECL.finditer(text):
            if "typedef" not in text[max(0, m.start() - 40):m.start()]:
                names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_boundary():
    names = declared()
    for must in ("mgpu_accel_build", "mgpu_scene_create", "mgpu_trace_closest", "mgpu_trace_any", "mgpu_render",
                 "mgpu_film_read", "mgpu_last_error", "mgpu_renderer_create", "mgpu_renderer_init"):
        assert must in names
    assert declared(("milton_plugin.h",)) == ["plugin_delete", "plugin_new", "plugin_type"]


def test_library_exports_every_declared_symbol():
    from milton_gb300 import _native
    lib = _native.load()
    bound = {n for n, _, _ in _native.SIGNATURES}
    for name in declared():
        assert hasattr(lib, name), f"{name} not exported"
        assert name in bound, f"{name} has no ctypes signature"
    # the Milton plugin entry points live in the plugin library only
    for name in ("plugin_type", "plugin_new", "plugin_delete"):
        assert not hasattr(lib, name), f"libmgpu.so must not export {name}"


def _dynamic_symbols(path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_plugin_library_exports_the_milton_entry_points():
    from milton_gb300.plugin import PLUGIN_PATH
    syms = _dynamic_symbols(PLUGIN_PATH)
    for name in declared(("milton_plugin.h",)):
        assert name in syms, f"{name} not exported by {PLUGIN_PATH.name}"


def test_renderer_object_and_errors_without_gpu():
    from milton_gb300 import _native
    lib = _native.load()
    h = C.c_void_p()
    assert lib.mgpu_renderer_create(C.byref(h)) == 0 and h.value
    r = h.value
    # PropertyMap round trip and Renderer::init preconditions (host-only paths)
    assert lib.mgpu_renderer_set_value(r, b"noSuperSamples", b"16") == 0
    buf = C.create_string_buffer(32)
    assert lib.mgpu_renderer_get_value(r, b"noSuperSamples", buf, 32) == 0 and buf.value == b"16"
    assert lib.mgpu_renderer_init(r) == -1
    assert b"no scene" in lib.mgpu_last_error()
    assert lib.mgpu_renderer_render(r) == -1
    assert lib.mgpu_renderer_destroy(r) == 0
    assert lib.mgpu_renderer_create(None) == -1
    # argument validation happens before any device work
    assert lib.mgpu_accel_build(None, None, None) == -1
    assert lib.mgpu_trace_closest(None, None, None, 1, None) == -1
    assert lib.mgpu_render(None, None, None, None) == -1
    assert lib.mgpu_version() == 1


def test_kd_traversal_cost_default_is_one_value_everywhere():
    # the header's constant is what the plugins default to and what the Python host's KdSettings use
    from milton_gb300.pathtracer import KdSettings
    m = re.search(r"#define MGPU_KD_COST_TRAVERSAL ([0-9.]+)", (ROOT / "include" / "mgpu.h").read_text())
    assert m and float(m.group(1)) == KdSettings().cost_traversal
    for src in ("milton_gb300/csrc/plugin.cpp", "milton_gb300/milton_plugin/gpu_path_tracer.cpp"):
        assert 'num("kdCostTraversal", MGPU_KD_COST_TRAVERSAL)' in (ROOT / src).read_text()
