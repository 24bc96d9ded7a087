"""Build Milton's own intersection code into a test-oracle program: oracle/_ref/milton_ref.

Test infrastructure.  The reference's kd-tree, shape and math sources are compiled unmodified
from the reference tree (MILTON_REFERENCE, default /root/reference) with g++; the external
headers they include and that this image lacks (Boost any / shared_ptr / random /
static_assert, QtCore's mutex and thread storage, OpenGL) come from the stand-ins in
oracle/milton_ref/shim, and oracle/milton_ref/driver.cpp reads a flattened scene and a ray
batch and answers Scene::getIntersection / Scene::intersects with them.  Flags are the
reference's OPT mode (mlt/src/.make/defines.mk:144-148: -O3 -DNDEBUG) without -march=native
(portable x86-64, so no FMA contraction), gnu++17 for its `typeof` and `register`.  Linked
without PIE: kdTreeAccel keeps child pointers in 32 bits (mlt/src/milton/accel/kdTreeAccel.cpp:
78-85), which holds for a heap below 4 GiB.  The outputs go to oracle/_ref/ only; nothing here
is shipped or used on the product path.  Returns None when the reference tree is absent.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT_DIR = HERE.parent / "_ref"
EXE = OUT_DIR / "milton_ref"
OBJ_DIR = OUT_DIR / "obj"

# the reference sources this oracle links (paths inside mlt/src/milton): the kd-tree and its
# primitives, plus what their vtables and statics pull in (materials, samplers, filters)
SOURCES = [
    "accel/kdTreeAccel.cpp", "accel/NaiveSpatialAccel.cpp", "accel/SpatialAccel.cpp", "accel/AABB.cpp",
    "shapes/Mesh.cpp", "shapes/MeshTriangle.cpp", "shapes/Triangle.cpp", "shapes/ShapeSet.cpp",
    "shapes/Shape.cpp", "shapes/Transformable.cpp", "shapes/Intersectable.cpp", "shapes/Plane.cpp",
    "shapes/Implicit.cpp",
    "common/math/Matrix.cpp", "common/math/Point.cpp", "common/math/Vector.cpp",
    "utils/PropertyMap.cpp", "utils/Log.cpp", "utils/SpectralSampleSet.cpp", "utils/GLState.cpp",
    "core/SurfacePoint.cpp",
    "materials/Material.cpp", "materials/BSDF.cpp", "materials/Emitter.cpp", "materials/Sensor.cpp",
    "materials/IndexOfRefraction.cpp",
    "materials/bsdfs/DiffuseBSDF.cpp", "materials/bsdfs/ModifiedPhongBSDF.cpp", "materials/bsdfs/DielectricBSDF.cpp",
    "materials/bsdfs/AbsorbentBSDF.cpp", "materials/bsdfs/AggregateBSDF.cpp",
    "materials/emitters/OrientedEmitter.cpp", "materials/emitters/OmniEmitter.cpp",
    "materials/emitters/NullEmitter.cpp", "materials/emitters/EnvironmentMap.cpp", "materials/sensors/NullSensor.cpp",
    "stats/Random.cpp", "stats/Event.cpp", "stats/JointEvent.cpp", "stats/Sampler.cpp",
    "stats/MultipleImportanceSampler.cpp",
    "stats/samplers/ContUniformSampler.cpp", "stats/samplers/DiscreteUniformSampler.cpp",
    "stats/samplers/EmitterSampler.cpp", "stats/samplers/ExponentialSampler.cpp",
    "stats/samplers/JointContUniformSampler.cpp", "stats/samplers/JointSampler.cpp",
    "stats/samplers/UniformOnSphereSampler.cpp", "stats/samplers/UniformSampler.cpp",
    "filters/Filter.cpp", "filters/KernelFilter.cpp", "filters/BoxFilter.cpp", "filters/TriangleFilter.cpp",
    "filters/GaussianFilter.cpp", "filters/MitchellFilter.cpp", "filters/LanczosSincFilter.cpp",
    "cameras/Camera.cpp",
]

# this directory's own sources linked in: the query driver and the statics Milton's host keeps
OWN = ["host_statics.cpp", "driver.cpp"]

FLAGS = ["-std=gnu++17", "-O3", "-DNDEBUG", "-DPOSIX", "-fno-pie", "-w"]


def reference_root() -> Path:
    return Path(os.environ.get("MILTON_REFERENCE", "/root/reference"))


def milton_dir() -> Path:
    return reference_root() / "mlt" / "src" / "milton"


def available() -> bool:
    return (milton_dir() / "accel" / "kdTreeAccel.cpp").exists()


def _includes(m: Path) -> list[str]:
    dirs = [HERE / "shim"]
    for d in sorted(p for p in m.rglob("*") if p.is_dir()):
        rel = d.relative_to(m).parts
        if any(x.startswith(".") or x in ("third-party", "scratch") for x in rel):
            continue
        dirs.append(d)
    dirs += [m, m.parent]
    return [f"-I{d}" for d in dirs]


def include_flags() -> list[str]:
    """-I flags (stand-ins first) for compiling other test sources against Milton's headers."""
    return _includes(milton_dir())


def objects(with_driver: bool = False) -> list[Path]:
    """The compiled reference objects (and host_statics), after build()."""
    names = [rel.replace("/", "_") + ".o" for rel in SOURCES + OWN if with_driver or rel != "driver.cpp"]
    return [OBJ_DIR / n for n in names]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False) -> Path | None:
    if not available():
        return None
    m = milton_dir()
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    inc = _includes(m)
    shim_mtime = max(p.stat().st_mtime for p in (HERE / "shim").rglob("*") if p.is_file())
    jobs, objs = [], []
    for rel in SOURCES + OWN:
        src = HERE / rel if rel in OWN else m / rel
        obj = OBJ_DIR / (rel.replace("/", "_") + ".o")
        objs.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, shim_mtime):
            jobs.append(["g++", *FLAGS, *inc, "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if jobs or not EXE.exists():
        tmp = EXE.with_suffix(".tmp")
        _run(["g++", "-no-pie", "-o", str(tmp), *map(str, objs)])
        os.replace(tmp, EXE)
    return EXE


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
