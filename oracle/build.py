"""Build the oracle (test infrastructure): oracle/oracle.c -> oracle/_build/liborc.so.

Compiled with gcc at -O3 (the reference's OPT level, mlt/src/.make/defines.mk:144-148) and
-ffp-contract=off so that the FP64 restatement rounds the same way on x86-64 and aarch64 (the
kd-tree comparison against the product builder is bit-exact); no -march=native, so the one
build runs on both hosts.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "oracle.c"
OUT = HERE / "_build" / "liborc.so"


def build(force: bool = False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    if not force and OUT.exists() and OUT.stat().st_mtime >= SRC.stat().st_mtime:
        return OUT
    tmp = OUT.with_suffix(".so.tmp")
    cmd = ["gcc", "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-Wall", str(SRC), "-o", str(tmp),
           "-lm", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
