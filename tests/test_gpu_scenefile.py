"""Milton scene files loaded by milton_gb300.sceneloader render on the GPU like the oracle:
tests/scenes/box.js (unit-plane light, culled planes, a Phong cube, a dielectric OBJ mesh) and
tests/scenes/emitters.js (triangle, mesh and plane lights), tests/scenes/spheres.js (analytic
spheres tessellated by the loader), tests/scenes/textures.js (image maps) and
tests/scenes/points.js (point lights, omni emitters)."""
from pathlib import Path

import numpy as np
import pytest

from milton_gb300 import sceneloader
from gpu_util import gpu_render_paths

pytestmark = pytest.mark.gpu
HERE = Path(__file__).resolve().parent


@pytest.mark.parametrize("name,tess", [("box.js", None), ("emitters.js", None), ("spheres.js", (32, 17)),
                                       ("spheres.js", None), ("textures.js", None), ("points.js", None)])
def test_scene_file_renders_like_the_oracle(cuda, oracle, name, tess):
    # emitters.js: plane, triangle (two uv frames) and mesh lights, 4 light samples per vertex;
    # spheres.js: tessellated spheres (Phong, dielectric, a named sphere and its instance);
    # textures.js: kd / ks / bump maps from PNG and PPM files, plane, cube and mesh uvs;
    # points.js: omni and oriented point lights, omni plane and mesh emitters
    sf = sceneloader.load(str(HERE / "scenes" / name), tessellate=tess)  # spheres.js: analytic or tessellated
    r = sceneloader.path_tracer(sf)
    st = r.settings()
    mean_g, paths_g, _ = gpu_render_paths(cuda, sf.scene, st)
    tree = oracle.Tree(sf.scene.tri_v)
    mean_o, paths_o, _ = oracle.render(sf.scene, tree, st.width, st.height, st.spp, nds=st.no_direct_samples,
                                       max_depth=st.max_depth, rr_start=st.rr_start_depth, seed=st.seed,
                                       per_path=True)
    close = np.abs(paths_g - paths_o) <= 1e-4 + 2e-3 * np.maximum(np.abs(paths_g), np.abs(paths_o))
    agree = np.all(close, axis=-1).mean()
    print(f"{name}: path agreement {agree:.5f}, mean {mean_g.mean():.5f} / {mean_o.mean():.5f}")
    assert agree >= 0.97
    assert mean_g.mean() > 0.01  # the light reaches the film


def test_path_tracer_object_from_scene_file(cuda):
    sf = sceneloader.load(str(HERE / "scenes" / "box.js"))
    r = sceneloader.path_tracer(sf)
    r.init()
    r.render()
    img = r.output()
    assert img.shape == (sf.height, sf.width, 3) and np.isfinite(img).all() and img.mean() > 0.01
