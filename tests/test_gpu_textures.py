"""Image maps on the GPU against the oracle: the device's filtered texels (one KernelFilter::apply
per texel, computed when the scene is created) against the oracle's per-lookup convolution for
every filter kind and for bump gradients, and per-path radiance of textured scenes (kd, ks,
transparency and bump maps; uvs of quads and spheres) against the oracle's paths."""
import numpy as np
import pytest

from milton_gb300 import pathtracer as pt
from milton_gb300 import scene as S
from milton_gb300 import scenegen
from gpu_util import gpu_render_paths

pytestmark = pytest.mark.gpu

FILTERS = [("box", 2.0, {}), ("triangle", 2.0, {}), ("triangle", 5.0, {}), ("gaussian", 3.0, {"sigma": 0.8}),
           ("mitchell", 2.0, {"B": 1 / 3, "C": 1 / 3}), ("lanczosSinc", 3.0, {"tau": 3.0})]


def _center_lookups(oracle, tex: S.Texture) -> np.ndarray:
    h, w, _ = tex.rgb.shape
    unit = S.Texture(tex.rgb, tex.kind, tex.filter, 1.0, 1.0, tex.bump_intensity)
    out = np.zeros((h, w, 2 if tex.kind == S.TEX_BUMP else 3))
    for y in range(h):
        for x in range(w):
            r = oracle.texture_lookup(unit, (x + 0.5) / w, (y + 0.5) / h)
            out[y, x] = r[:out.shape[2]]
    return out


@pytest.mark.parametrize("flt", FILTERS, ids=lambda f: f"{f[0]}-{f[1]}")
def test_device_texels_match_oracle_filter(cuda, oracle, flt):
    sc = scenegen.textured(3, filters=flt)
    ds = pt.DeviceScene(sc, pt.Accel(sc))
    for i, tex in enumerate(sc.textures):
        dev = ds.texels(i)
        ref = _center_lookups(oracle, tex)
        got = dev[..., :ref.shape[2]].astype(np.float64)
        # FP32 accumulation of at most (ceil(support) | 1)^2 products against FP64
        assert np.allclose(got, ref, rtol=2e-5, atol=2e-6), (i, np.abs(got - ref).max())


@pytest.mark.parametrize("flt", [FILTERS[1], FILTERS[3], FILTERS[5]], ids=lambda f: f[0])
def test_textured_scene_per_path(cuda, oracle, flt):
    sc = scenegen.textured(1, filters=flt)
    st = pt.RenderSettings(48, 48, 16, no_direct_samples=1, max_depth=5, rr_start_depth=3, seed=11)
    mean_g, paths_g, _ = gpu_render_paths(cuda, sc, st)
    tree = oracle.Tree(sc.tri_v)
    mean_o, paths_o, _ = oracle.render(sc, tree, st.width, st.height, st.spp, nds=1, max_depth=5, rr_start=3,
                                       seed=11, per_path=True)
    close = np.abs(paths_g - paths_o) <= 1e-4 + 2e-3 * np.maximum(np.abs(paths_g), np.abs(paths_o))
    agree = np.all(close, axis=-1).mean()
    print(f"textured ({flt[0]}): path agreement {agree:.5f}, mean {mean_g.mean():.5f} / {mean_o.mean():.5f}")
    assert agree >= 0.97
    assert abs(mean_g.mean() - mean_o.mean()) < 0.02 * mean_o.mean()


def test_textures_change_the_image(cuda):
    # the same scene with every texture slot cleared renders differently (the maps are used)
    sc = scenegen.textured(2)
    plain = scenegen.textured(2)
    plain.materials[:, 10:14] = 0
    st = pt.RenderSettings(32, 32, 4, max_depth=4, rr_start_depth=3, seed=5)
    a, _, _ = gpu_render_paths(cuda, sc, st)
    b, _, _ = gpu_render_paths(cuda, plain, st)
    assert np.abs(a - b).max() > 0.05


def test_texture_validation(cuda):
    sc = scenegen.textured(0)
    bad = scenegen.textured(0)
    bad.materials[0, 13] = 1  # a colour map in the bump slot
    with pytest.raises(Exception, match="colour map as bump map"):
        pt.DeviceScene(bad, pt.Accel(bad))
    bad = scenegen.textured(0, filters=("box", 1.0, {}))  # a 1x1 box kernel at (-1/2, -1/2): weight 0
    with pytest.raises(Exception, match="zero total weight"):
        pt.DeviceScene(bad, pt.Accel(bad))
    emit = sc.tri_light >= 0
    sc.materials[sc.tri_mat[emit][0], 13] = 1 + [t.kind for t in sc.textures].index(S.TEX_BUMP)
    with pytest.raises(Exception, match="bump-mapped emitter"):
        pt.DeviceScene(sc, pt.Accel(sc))


@pytest.mark.parametrize("kind", ["environment", "constant"])
def test_background_per_path(cuda, oracle, kind):
    # the plain box is open toward the camera: camera rays and bounces that leave it see the
    # background (an environment map, or an omni background's constant radiance)
    sc = scenegen.plain(2)
    rng = np.random.default_rng(9)
    if kind == "environment":
        env = rng.uniform(0.0, 2.0, (24, 48, 3)).astype(np.float32)
        sc.textures = [S.Texture(env, S.TEX_COLOR, ("gaussian", 3.0, {"sigma": 1.0}))]
        sc.background_tex = 1
    else:
        sc.background_le = np.array([0.4, 0.5, 0.8], np.float32)
    st = pt.RenderSettings(48, 48, 16, max_depth=5, rr_start_depth=3, seed=3)
    mean_g, paths_g, _ = gpu_render_paths(cuda, sc, st)
    tree = oracle.Tree(sc.tri_v)
    mean_o, paths_o, _ = oracle.render(sc, tree, st.width, st.height, st.spp, nds=1, max_depth=5, rr_start=3, seed=3,
                                       per_path=True)
    close = np.abs(paths_g - paths_o) <= 1e-4 + 2e-3 * np.maximum(np.abs(paths_g), np.abs(paths_o))
    agree = np.all(close, axis=-1).mean()
    print(f"background ({kind}): path agreement {agree:.5f}, mean {mean_g.mean():.5f} / {mean_o.mean():.5f}")
    assert agree >= 0.98
    black, _, _ = gpu_render_paths(cuda, scenegen.plain(2), st)
    assert mean_g.mean() > black.mean() + 0.02  # the background reaches the film
