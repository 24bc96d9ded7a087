"""Milton's renderer plugin (libmgpu_milton.so) without a GPU: the stand-in Milton host loads it
as Milton's loader does (plugin_type, plugin_new, cast to Renderer*, dynamic_cast to
PointSampleRenderer, setOutput / getOutput through the vtable, init() without a scene); and,
where the reference tree is present, the plugin source compiles against Milton's own headers
(every `override` matches a Milton virtual function) and the re-declared classes keep every
vtable slot and data-member offset of Milton's."""
import subprocess
from pathlib import Path

import pytest

from oracle import milton_ref

ROOT = Path(__file__).resolve().parent.parent
PLUGIN_SRC = ROOT / "milton_gb300" / "milton_plugin" / "gpu_path_tracer.cpp"
LAYOUT_SRC = ROOT / "tests" / "native" / "milton_layout.cpp"


def test_host_loads_the_plugin_like_milton():
    from plugin_host import host_path
    from milton_gb300.plugin import PLUGIN_PATH
    r = subprocess.run([str(host_path()), "--check", str(PLUGIN_PATH)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert r.stdout.startswith("ok plugin_type=0 PointSampleRenderer")
    assert "init: no scene set" in r.stderr


def test_host_reports_the_loaders_errors(tmp_path):
    from plugin_host import host_path
    from milton_gb300._native import LIB_PATH
    r = subprocess.run([str(host_path()), "--check", str(tmp_path / "missing.so")], capture_output=True, text=True)
    assert r.returncode == 1 and "plugin failed to load" in r.stderr
    # libmgpu.so is the C ABI, not a Milton plugin: no plugin_type symbol
    r = subprocess.run([str(host_path()), "--check", str(LIB_PATH)], capture_output=True, text=True)
    assert r.returncode == 1 and "could not find plugin_type symbol" in r.stderr


needs_ref = pytest.mark.skipif(not milton_ref.available(), reason="the reference tree is not present")


@needs_ref
def test_plugin_compiles_against_milton_headers():
    from oracle.milton_ref import build as rb
    r = subprocess.run(["g++", "-std=gnu++17", "-DNDEBUG", "-DPOSIX", "-DMGPU_WITH_MILTON_HEADERS", "-fsyntax-only",
                        "-w", *rb.include_flags(), str(PLUGIN_SRC)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@needs_ref
def test_redeclared_classes_keep_miltons_layout(tmp_path):
    from oracle.milton_ref import build as rb
    rb.build()
    compat = tmp_path / "layout_compat"
    real = tmp_path / "layout_milton"
    subprocess.run(["g++", "-std=gnu++17", "-w", str(LAYOUT_SRC), "-o", str(compat)], check=True)
    obj = tmp_path / "layout_milton.o"
    subprocess.run(["g++", "-std=gnu++17", "-w", "-DNDEBUG", "-DPOSIX", "-DMGPU_WITH_MILTON_HEADERS",
                    *rb.include_flags(), "-c", str(LAYOUT_SRC), "-o", str(obj)], check=True)
    subprocess.run(["g++", "-no-pie", "-o", str(real), str(obj), *map(str, rb.objects())], check=True)
    a = subprocess.run([str(compat)], capture_output=True, text=True, check=True).stdout
    b = subprocess.run([str(real)], capture_output=True, text=True, check=True).stdout
    assert a == b
    assert "Renderer::init 24" in a and "PointSampleRenderer::setOutput 88" in a
