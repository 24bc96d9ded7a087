"""The oracle pinned to Milton itself.

tests/golden/milton_hits.npz holds the answers of the reference's own kdTreeAccel, Mesh,
MeshTriangle and Triangle (compiled unmodified into oracle/_ref/milton_ref) on the ray batches of
tests/milton_cases.py.  The oracle's FP64 restatement must reproduce them: the same primitive
ids and the same t, bit for bit, on the plain box (culled Triangles, brute force) and on the
1,000,010-triangle mid scene (Milton's two-level kd-trees against the oracle's one tree over
the flattened soup).  Where the reference tree is present the fixture is re-derived from it, and
Milton's kd-tree is checked against its own brute force (NaiveSpatialAccel).
"""
import numpy as np
import pytest

import milton_cases as mc
from oracle import milton_ref

ROOT_FIX = mc.__file__.rsplit("/", 1)[0] + "/golden/milton_hits.npz"


@pytest.fixture(scope="module")
def fix():
    return dict(np.load(ROOT_FIX))


@pytest.fixture(scope="module")
def scenes():
    return {c: mc.scene(c) for c in mc.CASES}


def _same_inputs(fix, case, s):
    assert str(fix[f"{case}_rays_sha"]) == mc.sha(mc.closest_rays(case, s))
    assert str(fix[f"{case}_any_sha"]) == mc.sha(mc.any_rays(case, s))
    return str(fix[f"{case}_scene_sha"]) == mc.sha(s.tri_v)


def test_oracle_brute_force_equals_milton_plain(oracle, fix, scenes):
    s = scenes["plain_culled"]
    assert _same_inputs(fix, "plain_culled", s)
    rays = mc.closest_rays("plain_culled", s)
    t, p, _, _ = oracle.trace_closest(None, s.tri_v, s.tri_flags, rays)
    assert np.array_equal(p, fix["plain_culled_id"])
    hit = p >= 0
    assert np.array_equal(t[hit], fix["plain_culled_t"][hit])
    # any hit: Milton's window is (EPSILON, tMax - 2 EPSILON) with the traversal clipped at
    # tMax - EPSILON (Scene.cpp:110-114, Intersectable.cpp:20-25); the oracle takes the clip
    ar = mc.any_rays("plain_culled", s)
    occ = oracle.trace_any(None, s.tri_v, s.tri_flags, ar)
    diff = occ.astype(bool) != fix["plain_culled_occ"].astype(bool)
    if diff.any():
        tc, _, _, _ = oracle.trace_closest(None, s.tri_v, s.tri_flags, ar[diff])
        assert np.all(np.abs(tc - ar[diff, 7]) <= 1e-6 * ar[diff, 7])
    assert diff.sum() <= 2


def test_oracle_kd_equals_milton_mid(oracle, fix, scenes):
    """Milton's per-Mesh kd-trees under a kd-tree of shapes against the oracle's single SAH tree
    over the flattened soup: identical closest primitives and t on 32,768 rays."""
    s = scenes["mid"]
    identical_scene = _same_inputs(fix, "mid", s)
    rays = mc.closest_rays("mid", s)
    tree = oracle.Tree(s.tri_v)
    t, p, _, _ = oracle.trace_closest(tree, s.tri_v, s.tri_flags, rays)
    same = p == fix["mid_id"]
    if identical_scene:
        assert same.all()
        hit = p >= 0
        assert np.array_equal(t[hit], fix["mid_t"][hit])
    else:
        # the scene generator's trigonometry rounded differently on this machine: ids may only
        # differ where the ray passes within rounding of a triangle edge
        assert same.mean() >= 0.9999
    ar = mc.any_rays("mid", s)
    occ = oracle.trace_any(tree, s.tri_v, s.tri_flags, ar)
    assert (occ.astype(bool) != fix["mid_occ"].astype(bool)).sum() <= (0 if identical_scene else 4)


@pytest.mark.skipif(not milton_ref.available(), reason="the reference tree is not present")
def test_fixture_is_milton_output_and_kd_equals_brute_force(fix, scenes):
    s = scenes["plain_culled"]
    rays = mc.closest_rays("plain_culled", s)
    t, p = milton_ref.closest(s, rays[:, 0:3], rays[:, 4:7])
    assert np.array_equal(p, fix["plain_culled_id"].astype(np.int64))
    assert np.array_equal(t, fix["plain_culled_t"])
    tn, pn = milton_ref.closest(s, rays[:, 0:3], rays[:, 4:7], naive=True)
    assert np.array_equal(pn, p) and np.array_equal(tn, t)
    ar = mc.any_rays("plain_culled", s)
    occ = milton_ref.any_hit(s, ar[:, 0:3], ar[:, 4:7], ar[:, 7])
    assert np.array_equal(occ, fix["plain_culled_occ"].astype(bool))
    assert np.array_equal(milton_ref.any_hit(s, ar[:, 0:3], ar[:, 4:7], ar[:, 7], naive=True), occ)


@pytest.mark.skipif(not milton_ref.available(), reason="the reference tree is not present")
def test_milton_drops_a_mesh_whose_bounds_compare_fuzzy_equal(oracle):
    """A reference defect, recorded: SpatialAccel::init unions primitive boxes with AABB::add,
    which skips a box whose min and max are equal under the fuzzy EQ macro
    (mlt/src/milton/accel/AABB.inl:67-72, mlt/src/milton/common/utilities.h:240).  By that macro's
    operator precedence EQ(-1, 1) holds (|a - b / a| = 0), so a flat Mesh spanning [-1, 1] in x
    and z -- the plain box's floor -- gets an empty root box and no ray ever hits it, while the
    same quad as a Milton Triangle is hit.  The oracle and the GPU follow the geometry."""
    from milton_gb300 import scenegen
    s = scenegen.plain(0)
    floor = [sh for sh in s.shapes if sh[0] == "floor"][0]
    o = np.array([[0.85, 1.0, -0.85], [-0.85, 1.0, 0.85]])
    d = np.array([[0.0, -1.0, 0.0], [0.05, -1.0, 0.03]])
    t, p = milton_ref.closest(s, o, d)
    assert np.all(p == -1)
    s.tri_flags = np.ones_like(s.tri_flags)
    s.shapes = [(f"triangle{i}", i, 1) for i in range(s.ntri)]
    t, p = milton_ref.closest(s, o, d)
    assert np.all((p >= floor[1]) & (p < floor[1] + floor[2]))
