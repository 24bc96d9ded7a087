"""Writes tests/golden/milton_hits.npz: closest hits and any-hit answers of Milton's OWN
intersection code on the ray batches of tests/milton_cases.py (test infrastructure).

The answers come from oracle/_ref/milton_ref, the reference's kdTreeAccel, Mesh, MeshTriangle,
Triangle and ShapeSet compiled unmodified from the reference tree (oracle/milton_ref/build.py),
so this script runs only where that tree is present.  Per case it stores

  {case}_t     closest-hit t (float64, inf on a miss)       Scene::getIntersection
  {case}_id    global primitive id (int32, -1 on a miss)    (pt.shape, pt.index) flattened
  {case}_occ   any-hit answer per segment (uint8)           Scene::intersects(ray, tMax)
  {case}_scene_sha, {case}_rays_sha, {case}_any_sha          hashes of the inputs it was made on

Regenerate deliberately with

    python tests/golden/make_milton_hits.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
for p in (HERE.parents[1], HERE.parent):
    sys.path.insert(0, str(p))
import milton_cases as mc  # noqa: E402
from oracle import milton_ref  # noqa: E402


def main():
    out = {}
    for case in mc.CASES:
        s = mc.scene(case)
        cr = mc.closest_rays(case, s)
        t, pid = milton_ref.closest(s, cr[:, 0:3], cr[:, 4:7])
        ar = mc.any_rays(case, s)
        occ = milton_ref.any_hit(s, ar[:, 0:3], ar[:, 4:7], ar[:, 7])
        out[f"{case}_t"] = t
        out[f"{case}_id"] = pid.astype(np.int32)
        out[f"{case}_occ"] = occ.astype(np.uint8)
        out[f"{case}_scene_sha"] = np.array(mc.sha(s.tri_v))
        out[f"{case}_rays_sha"] = np.array(mc.sha(cr))
        out[f"{case}_any_sha"] = np.array(mc.sha(ar))
        print(case, "hits", float((pid >= 0).mean()), "occluded", float(occ.mean()))
    np.savez_compressed(HERE / "milton_hits.npz", **out)


if __name__ == "__main__":
    main()
