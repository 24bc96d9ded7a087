"""Milton's renderer plugin end to end on the GPU: the stand-in Milton host loads
libmgpu_milton.so as Milton's scene loader does, copies the renderer keys into its
PropertyMap, sets output, scene and camera, and calls init() and render() through
milton::Renderer*; every pixel of its RenderOutput must equal mgpu_render's film mean for the
same keys, bit for bit, from exactly one sample per pixel."""
import numpy as np
import pytest

from milton_gb300 import pathtracer as pt
from milton_gb300 import scenegen
from milton_gb300.plugin import PLUGIN_PATH
from plugin_host import run

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["plain", "random"])
def test_plugin_renders_what_mgpu_render_renders(cuda, kind):
    s = scenegen.plain(0) if kind == "plain" else scenegen.random_scene(3, 20000)
    W, H = (48, 40) if kind == "plain" else (64, 64)
    props = dict(noSuperSamples=9, maxDepth=5, rrStartDepth=3, seed=11, efficientDirect=True)
    vals, cnt, _ = run(PLUGIN_PATH, s, W, H, props)
    assert np.all(cnt == 1)
    f = pt.Film(W, H)
    pt.render(pt.DeviceScene(s, pt.Accel(s)), pt.RenderSettings(W, H, 9, max_depth=5, rr_start_depth=3, seed=11), f)
    ref = f.mean()
    assert ref.mean() > 0.01
    assert np.array_equal(vals, ref)


def test_plugin_keys_change_the_render(cuda):
    s = scenegen.plain(1)
    a, _, _ = run(PLUGIN_PATH, s, 16, 16, dict(noSuperSamples=4, maxDepth=5, seed=1))
    b, _, _ = run(PLUGIN_PATH, s, 16, 16, dict(noSuperSamples=4, maxDepth=5, seed=2))
    c, _, _ = run(PLUGIN_PATH, s, 16, 16, dict(noSuperSamples=4, maxDepth=1, seed=1))
    assert not np.array_equal(a, b) and not np.array_equal(a, c)
