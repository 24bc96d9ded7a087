"""Build libmgpu.so in-tree (milton_gb300/lib/) for sm_103a, and beside it libmgpu_milton.so,
Milton's dynamic renderer plugin (milton_plugin/gpu_path_tracer.cpp, linked against libmgpu.so).

Each translation unit is compiled in parallel: .cu files with nvcc
(-gencode arch=compute_103a,code=sm_103a), .cpp files with g++, then linked with nvcc
-shared against the CUDA runtime.  Host code is compiled with -ffp-contract=off so the SAH
cost arithmetic of the kd builder rounds the same way on x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
OUT_DIR = PKG / "lib"
LIB = OUT_DIR / "libmgpu.so"
PLUGIN_SRC = PKG / "milton_plugin" / "gpu_path_tracer.cpp"
PLUGIN = OUT_DIR / "libmgpu_milton.so"
BUILD_DIR = PKG / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-O3", "-fPIC", "-ffp-contract=off", "-std=c++17", "-Wall"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmgpu.so")


def _cuda_home(nvcc: str) -> Path:
    return Path(nvcc).resolve().parent.parent


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def build(verbose: bool = False, force: bool = False, extra_nvcc: list[str] | None = None) -> Path:
    nvcc = _nvcc()
    BUILD_DIR.mkdir(exist_ok=True)
    OUT_DIR.mkdir(exist_ok=True)
    srcs = sources()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    newest_header = max((h.stat().st_mtime for h in headers), default=0.0)
    jobs = []
    objs = []
    for src in srcs:
        obj = BUILD_DIR / (src.name + ".o")
        objs.append(obj)
        stale = force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, newest_header)
        if not stale:
            continue
        if src.suffix == ".cu":
            cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr",
                   "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v" if verbose else "-O3",
                   "-I", str(INCLUDE), *(extra_nvcc or []), "-c", str(src), "-o", str(obj)]
        else:
            cmd = ["g++", *HOST_FLAGS, "-I", str(INCLUDE), "-I", str(_cuda_home(nvcc) / "include"),
                   "-c", str(src), "-o", str(obj)]
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-lpthread"])
        os.replace(tmp, LIB)
    build_plugin()
    return LIB


def build_plugin() -> Path:
    """libmgpu_milton.so: the plugin's Milton base-class members stay undefined here and resolve
    against the host (Milton's library, or the stand-in host of the tests) when it is loaded."""
    deps = [PLUGIN_SRC, LIB, *(PKG / "milton_plugin").glob("*.h"), INCLUDE / "mgpu.h"]
    if PLUGIN.exists() and PLUGIN.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        return PLUGIN
    tmp = PLUGIN.with_suffix(".so.tmp")
    _run(["g++", *HOST_FLAGS, "-shared", "-o", str(tmp), str(PLUGIN_SRC), f"-L{OUT_DIR}", "-lmgpu",
          "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, PLUGIN)
    return PLUGIN


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
