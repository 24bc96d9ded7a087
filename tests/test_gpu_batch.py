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


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_mixing_image_maps_spheres_and_plain_scenes(cuda, use_graph):
    # waves that mix scenes with image maps and a background, scenes with analytic spheres and
    # plain ones run the kernel variants that carry those branches; every film still equals its
    # own render
    from milton_gb300.scene import SceneBuilder, dielectric, diffuse
    tex = scenegen.textured(6)
    tex.background_le = np.array([0.2, 0.3, 0.4], np.float32)
    s0 = scenegen.plain(7)
    b = SceneBuilder()
    for name, first, count in s0.shapes:
        b.add(name, s0.tri_v[first:first + count], s0.tri_n[first:first + count],
              b.material(s0.materials[s0.tri_mat[first]]),
              light=int(s0.tri_light[first]) if s0.tri_light[first] >= 0 else -1)
    for rec, ext in zip(s0.lights, s0.light_ext):
        b.add_light(rec, ext)
    b.add_sphere((0.0, 0.4, 0.0), 0.35, b.material(dielectric(1.5)))
    b.add_sphere((0.5, 1.2, -0.4), 0.1, b.material(diffuse(0.2)), radiance=5.0)
    sph = b.build(s0.camera)
    plain = scenegen.plain(8)
    reqs = []
    for k, (s, (w, h, spp)) in enumerate(zip((tex, sph, plain, tex), ((40, 32, 8), (48, 40, 8), (32, 32, 4), (24, 24, 16)))):
        ds = pt.DeviceScene(s, pt.Accel(s))
        reqs.append((ds, pt.RenderSettings(w, h, spp, max_depth=5, rr_start_depth=3, seed=50 + k, stream_id=k)))
    want = _solo(reqs)
    batch = pt.Batch(wave_paths=12000, use_graph=use_graph)
    films = [pt.Film(st.width, st.height) for _, st in reqs]
    for (ds, st), f in zip(reqs, films):
        batch.add(ds, st, f)
    batch.render()
    for f, w in zip(films, want):
        assert np.array_equal(f.raw(), w)
