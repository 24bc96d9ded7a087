"""Batched rendering: requests of different scenes, resolutions and sample counts share waves;
every film must hold exactly the image its own mgpu_render gives (bit for bit), whatever the
wave packing, with or without the CUDA graph."""
import numpy as np
import pytest

from milton_gb300 import pathtracer as pt
from milton_gb300 import scenegen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scenes(cuda):
    out = []
    for s in (scenegen.plain(0), scenegen.random_scene(31, 3000), scenegen.random_scene(32, 40000),
              scenegen.random_scene(33, 800)):
        out.append((s, pt.DeviceScene(s, pt.Accel(s))))
    return out


def _requests(scenes):
    shapes = [(40, 32, 16, 5), (64, 48, 4, 8), (96, 96, 8, 6), (24, 40, 9, 3), (64, 64, 16, 8)]
    reqs = []
    for k, (w, h, spp, depth) in enumerate(shapes):
        s, ds = scenes[k % len(scenes)]
        reqs.append((ds, pt.RenderSettings(w, h, spp, max_depth=depth, rr_start_depth=3, seed=100 + k, stream_id=k)))
    return reqs


def _solo(reqs):
    out = []
    for ds, st in reqs:
        f = pt.Film(st.width, st.height)
        pt.render(ds, st, f)
        out.append(f.raw())
    return out


@pytest.mark.parametrize("wave_paths,use_graph", [(0, True), (0, False), (9000, True), (4096, False)])
def test_batch_equals_individual_renders(cuda, scenes, wave_paths, use_graph):
    reqs = _requests(scenes)
    want = _solo(reqs)
    batch = pt.Batch(wave_paths=wave_paths, use_graph=use_graph)
    films = []
    for ds, st in reqs:
        f = pt.Film(st.width, st.height)
        batch.add(ds, st, f)
        films.append(f)
    batch.render()
    for f, w in zip(films, want):
        assert np.array_equal(f.raw(), w)


def test_batch_progressive_and_unlimited_depth(cuda, scenes):
    # later passes added by a second batch render continue each film exactly
    reqs = _requests(scenes)[:3]
    want = _solo(reqs)
    films = [pt.Film(st.width, st.height) for _, st in reqs]
    for half in (0, 1):
        b = pt.Batch()
        for (ds, st), f in zip(reqs, films):
            n = st.spp // 2
            part = pt.RenderSettings(st.width, st.height, st.spp, sample_begin=half * n,
                                     sample_count=n if half == 0 else st.spp - n, max_depth=st.max_depth,
                                     rr_start_depth=3, seed=st.seed, stream_id=st.stream_id)
            b.add(ds, part, f)
        b.render()
    for f, w in zip(films, want):
        assert np.array_equal(f.raw(), w)
    # Milton's default estimator (no depth cap) cannot be graph-captured; the batch drains it
    ds, _ = scenes[0][1], None
    st = pt.RenderSettings(32, 32, 4, max_depth=0, rr_start_depth=2, seed=7)
    f_solo = pt.Film(32, 32)
    pt.render(ds, st, f_solo)
    b = pt.Batch()
    f_b = pt.Film(32, 32)
    b.add(ds, st, f_b)
    b.render()
    assert np.array_equal(f_b.raw(), f_solo.raw())
