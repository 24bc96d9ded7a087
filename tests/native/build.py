"""Builds the native test harnesses: tests/_build/libhostcheck.so (see hostcheck.cpp) and
tests/_build/milton_host, the stand-in Milton host that loads the renderer plugin (see
milton_host.cpp)."""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
OUT = HERE.parent / "_build" / "libhostcheck.so"
SRCS = [HERE / "hostcheck.cpp", ROOT / "milton_gb300" / "csrc" / "kdbuild.cpp"]
DEPS = SRCS + list((ROOT / "milton_gb300" / "csrc").glob("hd_*.h")) + [ROOT / "milton_gb300" / "csrc" / "kdbuild.h"]


def build() -> Path:
    OUT.parent.mkdir(exist_ok=True)
    if OUT.exists() and OUT.stat().st_mtime >= max(p.stat().st_mtime for p in DEPS):
        return OUT
    tmp = OUT.with_suffix(".so.tmp")
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", *map(str, SRCS), "-o", str(tmp),
           "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("hostcheck build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, OUT)
    return OUT


HOST = HERE.parent / "_build" / "milton_host"
HOST_DEPS = [HERE / "milton_host.cpp", ROOT / "milton_gb300" / "milton_plugin" / "milton_compat.h",
             ROOT / "include" / "mgpu.h"]


def build_host() -> Path:
    """The stand-in host exports its milton:: definitions (-rdynamic) for the plugin it loads."""
    HOST.parent.mkdir(exist_ok=True)
    if HOST.exists() and HOST.stat().st_mtime >= max(p.stat().st_mtime for p in HOST_DEPS):
        return HOST
    tmp = HOST.with_suffix(".tmp")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-rdynamic", str(HOST_DEPS[0]), "-o", str(tmp), "-ldl"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("milton_host build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, HOST)
    return HOST
