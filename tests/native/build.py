"""Builds tests/_build/libhostcheck.so (test harness; see hostcheck.cpp)."""
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
