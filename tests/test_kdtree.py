"""The product's host SAH kd builder against the oracle's restatement of kdTreeAccel:
node-by-node identical trees and identical build logs."""
import numpy as np
import pytest

from milton_gb300 import scenegen
from milton_gb300.pathtracer import Accel, KdSettings
from milton_gb300.scene import Scene


def _soup(seed, n, degenerate=True):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-5, 5, (n, 1, 3))
    v = (c + rng.normal(scale=0.3, size=(n, 3, 3))).astype(np.float32)
    if degenerate:
        k = n // 20
        v[:k, 1] = v[:k, 0]                      # sliver / line triangles
        v[k:2 * k, :, 1] = v[k:2 * k, :1, 1]     # axis-planar triangles (SPLIT_PLANE events)
        v[2 * k:3 * k] = v[2 * k:3 * k, :1]      # point triangles (dropped from the tree)
        v[3 * k:4 * k] = v[4 * k:5 * k]          # duplicates
        v = np.round(v * 8) / 8                  # shared coordinates -> equal split positions
    return v.astype(np.float32)


def _scene_from_v(v):
    T = v.shape[0]
    return Scene(tri_v=v, tri_n=np.zeros_like(v), tri_mat=np.zeros(T, np.int32), tri_light=-np.ones(T, np.int32),
                 tri_flags=np.zeros(T, np.uint32), materials=np.zeros((1, 16), np.float32),
                 lights=np.zeros((0, 16), np.float32), camera=np.zeros(11, np.float32))


def _same(oracle, v, kd: KdSettings):
    tree = oracle.Tree(v, kd.min_prims, kd.max_depth, kd.cost_traversal, kd.empty_bias)
    acc = Accel(_scene_from_v(v), kd)
    ko, kp = tree.serialize(), acc.serialize()
    for name, a, b in zip(("kind", "split", "count", "prims"), ko, kp):
        assert a.shape == b.shape and np.array_equal(a, b), name
    so, sp = tree.stats(), acc.stats()
    for k, val in so.items():
        assert sp[k] == val, k
    return acc


@pytest.mark.parametrize("scene", ["plain", "random"])
@pytest.mark.parametrize("kd", [KdSettings.milton(), KdSettings()], ids=["milton_defaults", "renderer_defaults"])
def test_identical_to_oracle_on_scenes(oracle, scene, kd):
    s = scenegen.plain(0) if scene == "plain" else scenegen.random_scene(2, 30000)
    _same(oracle, s.tri_v, kd)


def test_milton_defaults_except_the_traversal_cost():
    m, d = KdSettings.milton(), KdSettings()
    assert (m.min_prims, m.max_depth, m.cost_traversal, m.empty_bias) == (3, 24, 1.0, 0.9)  # kdTreeAccel.h:97-104
    assert (d.min_prims, d.max_depth, d.empty_bias) == (3, 24, 0.9) and d.cost_traversal == 3.0


@pytest.mark.parametrize("kd", [KdSettings(), KdSettings.milton(), KdSettings(min_prims=1), KdSettings(min_prims=8, max_depth=12),
                                KdSettings(max_depth=32, empty_bias=1.0), KdSettings(cost_traversal=0.25),
                                KdSettings(max_depth=0)])
def test_identical_to_oracle_with_degenerate_soup(oracle, kd):
    _same(oracle, _soup(1, 3000), kd)


def test_empty_and_tiny_inputs(oracle):
    for n in (1, 2, 3, 4):
        _same(oracle, _soup(5, n, degenerate=False), KdSettings())


def test_thread_count_does_not_change_the_tree():
    s = scenegen.random_scene(4, 60000)
    a1 = Accel(s, KdSettings(threads=1)).serialize()
    a8 = Accel(s, KdSettings(threads=8)).serialize()
    for x, y in zip(a1, a8):
        assert np.array_equal(x, y)


def test_flattened_layout_invariants():
    s = scenegen.random_scene(6, 20000)
    acc = Accel(s)
    st = acc.stats()
    assert st["bytes_nodes"] == 16 * st["node_pairs"]          # 16-byte sibling-pair records
    assert st["node_pairs"] == st["no_internal"] + 1           # one pair per interior node + root pair
    kind, split, count, prims = acc.serialize()
    assert prims.size == st["sum_prims"]
    assert prims.min() >= 0 and prims.max() < s.ntri


def test_rejects_too_deep_trees():
    from milton_gb300._native import MgpuError
    with pytest.raises(MgpuError):
        Accel(scenegen.plain(0), KdSettings(max_depth=65))


def test_identical_to_oracle_on_a_large_soup(oracle):
    # 300,000 triangles: the root's axes are evaluated on parallel threads and its event lists
    # are radix sorted (the small cases above take std::sort); the tree must not change
    _same(oracle, _soup(7, 300_000), KdSettings(threads=4))


def test_oracle_adopts_a_serialised_tree(oracle):
    """For scenes too large for the restated build (the 20 M-triangle large configuration) the
    oracle traverses the product's tree read from its serialisation; on a scene where both run,
    that tree serialises back identically and answers every ray as the oracle's own build does."""
    import raygen
    s = scenegen.random_scene(5, 30000)
    own = oracle.Tree(s.tri_v)
    acc = Accel(s, KdSettings.milton())
    adopted = oracle.Tree.from_serial(s.tri_v, *acc.serialize())
    for a, b in zip(own.serialize(), adopted.serialize()):
        assert np.array_equal(a, b)
    assert np.array_equal(own.bounds(), adopted.bounds())
    lo, hi = s.tri_v.reshape(-1, 3).min(0), s.tri_v.reshape(-1, 3).max(0)
    rays = np.concatenate([raygen.camera_rays(s.camera, 4096, 3), raygen.sphere_rays(lo, hi, 4096, 4)])
    t1, p1, _, _ = oracle.trace_closest(own, s.tri_v, s.tri_flags, rays)
    t2, p2, _, _ = oracle.trace_closest(adopted, s.tri_v, s.tri_flags, rays)
    assert np.array_equal(p1, p2) and np.array_equal(t1, t2)
    with pytest.raises(ValueError):
        k, sp, c, pr = acc.serialize()
        oracle.Tree.from_serial(s.tri_v, k[:-3], sp[:-3], c[:-3], pr)
