"""Closest-hit primitive ids and any-hit answers of the sm_103a kernels against Milton's OWN
intersection code (tests/golden/milton_hits.npz: the reference's kdTreeAccel, Mesh,
MeshTriangle and Triangle compiled unmodified, on the ray batches of tests/milton_cases.py).

Bar: the same primitive id as Milton on every ray, except reported ties -- the two nearest hits
within 1e-6 relative t (found by the oracle's brute force, itself equal to Milton's answers on
these batches, tests/test_milton_ref.py), or the GPU's t within 1e-6 of Milton's (a shared edge
or vertex).  The t error of agreeing hits is stated.  Any hit: the same answer except where the
segment ends within the FP32 margin of the closest surface."""
import numpy as np
import pytest

import milton_cases as mc
from gpu_util import gpu_any, gpu_trace
from milton_gb300 import pathtracer as pt
from raygen import classify

pytestmark = pytest.mark.gpu

FIX = mc.__file__.rsplit("/", 1)[0] + "/golden/milton_hits.npz"


@pytest.fixture(scope="module")
def fix():
    return dict(np.load(FIX))


@pytest.mark.parametrize("case", mc.CASES)
def test_hit_ids_match_milton(cuda, oracle, fix, case):
    s = mc.scene(case)
    rays = mc.closest_rays(case, s)
    assert str(fix[f"{case}_rays_sha"]) == mc.sha(rays)
    same_scene = str(fix[f"{case}_scene_sha"]) == mc.sha(s.tri_v)
    ds = pt.DeviceScene(s, pt.Accel(s))
    h, _ = gpu_trace(cuda, ds, rays)
    pg, tg = h[:, 1].view(np.int32).astype(np.int64), h[:, 0].astype(np.float64)
    pm, tm = fix[f"{case}_id"].astype(np.int64), fix[f"{case}_t"]
    bad = np.nonzero(pg != pm)[0]
    t2 = np.full(len(rays), np.inf)
    if bad.size:
        _, _, t2b, _ = oracle.trace_closest(None, s.tri_v, s.tri_flags, rays[bad])
        t2[bad] = t2b
    r = classify(pm, tm, t2, pg, tg)
    hit = (pm >= 0) & (pg == pm)
    rel = np.abs(tg[hit] - tm[hit]) / tm[hit]
    print(f"{case}: {r['n']} rays, {r['exact']} identical ids, {r['ties']} ties, {r['mismatches']} mismatches, "
          f"t error max {rel.max():.2e} / mean {rel.mean():.2e} relative (scene bit-identical to the "
          f"fixture's: {same_scene})")
    assert r["mismatches"] == 0, r["bad_idx"][:10]
    assert r["ties"] <= 0.002 * r["n"]
    assert np.all(np.abs(tg[hit] - tm[hit]) <= 1e-5 * np.maximum(tm[hit], 1.0))


@pytest.mark.parametrize("case", mc.CASES)
def test_any_hit_matches_milton(cuda, oracle, fix, case):
    s = mc.scene(case)
    ar = mc.any_rays(case, s)
    assert str(fix[f"{case}_any_sha"]) == mc.sha(ar)
    ds = pt.DeviceScene(s, pt.Accel(s))
    occ = gpu_any(cuda, ds, ar).astype(bool)
    ref = fix[f"{case}_occ"].astype(bool)
    diff = np.nonzero(occ != ref)[0]
    if diff.size:
        # only segments that end within the FP32 margin of their closest surface may differ
        tc, _, _, _ = oracle.trace_closest(None, s.tri_v, s.tri_flags, ar[diff])
        tmax = ar[diff, 7].astype(np.float64)
        assert np.all(np.abs(tc - tmax) <= 1e-4 * tmax + 1e-5), diff[:10]
    print(f"{case}: {len(ar)} segments, {int(ref.sum())} occluded in Milton, {diff.size} differ (all at the "
          f"segment's end)")
    assert diff.size <= 0.001 * len(ar)
