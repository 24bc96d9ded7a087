"""Wavefront renderer parity against the FP64 PathTracer oracle, called through the C ABI.

* per path: the GPU and the oracle draw the same Philox numbers, so most paths follow the same
  vertices; a path may diverge where FP32 and FP64 take different discrete decisions (Russian
  roulette or lobe thresholds, hits within FP32 precision of an edge);
* per pixel: independent estimates (different seeds) agree in a z-test on per-pixel means;
* film: deterministic, independent of wave size and of how sample passes are split.
"""
import numpy as np
import pytest

from milton_gb300 import pathtracer as pt
from milton_gb300 import scenegen
from gpu_util import gpu_render_paths

pytestmark = pytest.mark.gpu

PATH_RTOL = 2e-3   # per-path radiance tolerance (relative, FP32 vs FP64)
PATH_ATOL = 1e-4


def _path_agreement(a, b):
    ok = np.all(np.abs(a - b) <= PATH_ATOL + PATH_RTOL * np.maximum(np.abs(a), np.abs(b)), axis=-1)
    return ok.mean()


@pytest.mark.parametrize("mode", ["config", "reference"])
def test_plain_per_path(cuda, oracle, mode):
    s = scenegen.plain(0)
    kw = dict(max_depth=5, rr_start=3) if mode == "config" else dict(max_depth=0, rr_start=2)
    W = H = 64
    spp = 16
    st = pt.RenderSettings(W, H, spp, max_depth=kw["max_depth"], rr_start_depth=kw["rr_start"], seed=3)
    mean_g, paths_g, _ = gpu_render_paths(cuda, s, st)
    tree = oracle.Tree(s.tri_v)
    mean_o, paths_o, ost = oracle.render(s, tree, W, H, spp, seed=3, per_path=True, **kw)
    agree = _path_agreement(paths_g, paths_o)
    rmse = np.sqrt(((mean_g - mean_o) ** 2).mean())
    print(f"plain {mode}: path agreement {agree:.5f}, image rmse {rmse:.3e}, mean {mean_g.mean():.5f}/{mean_o.mean():.5f}")
    assert agree >= 0.98
    assert rmse <= 0.02 * mean_o.mean()
    assert np.allclose(mean_g, paths_g.mean(axis=2), rtol=1e-5, atol=1e-6)


def test_materials_per_path(cuda, oracle):
    # spheres with Lambertian, modified Phong and dielectric BSDFs, several lights
    s = scenegen.random_scene(11, 30000)
    W = H = 48
    st = pt.RenderSettings(W, H, 8, max_depth=8, rr_start_depth=3, seed=5)
    mean_g, paths_g, _ = gpu_render_paths(cuda, s, st)
    tree = oracle.Tree(s.tri_v)
    mean_o, paths_o, _ = oracle.render(s, tree, W, H, 8, max_depth=8, rr_start=3, seed=5, per_path=True)
    agree = _path_agreement(paths_g, paths_o)
    print(f"materials: path agreement {agree:.5f}")
    assert agree >= 0.95


def test_plain_independent_estimates_z_test(cuda, oracle):
    s = scenegen.plain(0)
    W = H = 32
    spp = 256
    st = pt.RenderSettings(W, H, spp, max_depth=5, rr_start_depth=3, seed=101)
    _, pg, _ = gpu_render_paths(cuda, s, st)
    tree = oracle.Tree(s.tri_v)
    _, po, _ = oracle.render(s, tree, W, H, spp, max_depth=5, rr_start=3, seed=202, per_path=True)
    mg, mo = pg.mean(2), po.mean(2)
    se = np.sqrt(pg.var(2, ddof=1) / spp + po.var(2, ddof=1) / spp)
    z = np.where(se > 0, (mg - mo) / np.maximum(se, 1e-12), 0.0)
    frac = (np.abs(z) > 4).mean()
    print(f"z-test: |z|>4 fraction {frac:.4f}, mean |z| {np.abs(z).mean():.3f}")
    assert frac <= 0.01
    assert abs(np.abs(z).mean() - 0.8) < 0.25  # E|z| = sqrt(2/pi) for a standard normal


def test_film_determinism_and_pass_splits(cuda):
    s = scenegen.plain(0)
    acc = pt.Accel(s)
    ds = pt.DeviceScene(s, acc)
    W = H = 40  # not a multiple of the 8x8 tile
    base = pt.RenderSettings(W, H, 16, max_depth=5, rr_start_depth=3, seed=9)
    f1 = pt.Film(W, H)
    pt.render(ds, base, f1)
    f2 = pt.Film(W, H)
    pt.render(ds, base, f2)
    raw1, raw2 = f1.raw(), f2.raw()
    assert np.array_equal(raw1, raw2)
    # the same passes in two calls, and with tiny waves
    f3 = pt.Film(W, H)
    pt.render(ds, pt.RenderSettings(W, H, 16, sample_begin=0, sample_count=7, max_depth=5, rr_start_depth=3, seed=9), f3)
    pt.render(ds, pt.RenderSettings(W, H, 16, sample_begin=7, sample_count=9, max_depth=5, rr_start_depth=3, seed=9), f3)
    assert np.array_equal(raw1, f3.raw())
    f4 = pt.Film(W, H)
    pt.render(ds, pt.RenderSettings(W, H, 16, max_depth=5, rr_start_depth=3, seed=9, wave_paths=4096), f4)
    assert np.array_equal(raw1, f4.raw())
    assert np.all(raw1[0, ..., 3] == 16)  # sample count per pixel
    stats = pt.render_stats()
    assert stats["paths"] == W * H * 16 and stats["extension_rays"] >= W * H * 16


def test_tuning_knobs_do_not_change_the_image(cuda):
    # queue binning, persistent traversal and warp-shared leaf tests reorder work, never the result
    s = scenegen.random_scene(12, 20000)
    acc = pt.Accel(s)
    ds = pt.DeviceScene(s, acc)
    st = pt.RenderSettings(48, 40, 8, max_depth=6, rr_start_depth=3, seed=4)
    raws = []
    saved = {k: pt.tune_get(k) for k in ("persistent", "coop_leaf", "bin_shadow", "bin_extension", "bin_min_paths",
                                         "trav_block", "carveout")}
    assert saved["carveout"] == -2  # per-kernel automatic carveout by default
    pt.tune("bin_min_paths", 0)  # bin even this small wave
    try:
        for shape in ("grid", "persistent", "coop_shadow", "coop_both"):
            for bins in ((0, 0), (1, 0), (1, 1)):
                pt.tune("persistent", int(shape == "persistent"))
                pt.tune("coop_leaf", {"grid": 0, "persistent": 0, "coop_shadow": 1, "coop_both": 3}[shape])
                pt.tune("bin_shadow", bins[0])
                pt.tune("bin_extension", bins[1])
                f = pt.Film(48, 40)
                pt.render(ds, st, f)
                raws.append(f.raw())
        for blk in (64, 256):  # threads per traversal block
            pt.tune("persistent", 0)
            pt.tune("trav_block", blk)
            for coop in (0, 1, 3):
                pt.tune("coop_leaf", coop)
                f = pt.Film(48, 40)
                pt.render(ds, st, f)
                raws.append(f.raw())
        for cv in (-1, 0, 20, 100, -2):  # L1 / shared-memory split: the driver's, fixed, automatic
            pt.tune("carveout", cv)
            f = pt.Film(48, 40)
            pt.render(ds, st, f)
            raws.append(f.raw())
    finally:
        for k, v in saved.items():
            pt.tune(k, v)
    for r in raws[1:]:
        assert np.array_equal(raws[0], r)


@pytest.mark.parametrize("kind", ["plain", "textured"])
def test_renderer_object(cuda, kind):
    # the C renderer object (include/mgpu_renderer.h) owns copies of every scene array (image
    # maps, uvs and a background included) and renders what mgpu_render renders
    from milton_gb300.plugin import RendererObject
    s = scenegen.plain(0) if kind == "plain" else scenegen.textured(4)
    if kind == "textured":
        s.background_le = np.array([0.3, 0.2, 0.1], np.float32)
    r = RendererObject()
    r.set_scene(s)
    r.set_output(32, 32)
    for k, v in dict(noSuperSamples=4, maxDepth=5, rrStartDepth=3, seed=9).items():
        r[k] = v
    r.init()
    r.render()
    out = r.output()
    acc = pt.Accel(s)
    ds = pt.DeviceScene(s, acc)
    f = pt.Film(32, 32)
    pt.render(ds, pt.RenderSettings(32, 32, 4, max_depth=5, rr_start_depth=3, seed=9), f)
    assert np.array_equal(out, f.mean())
    r.close()


def test_thin_lens_per_path(cuda, oracle):
    # ThinLensCamera::getWorldRay with an aperture: same lens samples, same paths as the oracle
    from milton_gb300.scene import camera
    s = scenegen.plain(0)
    c = s.camera
    s.camera = camera(eye=c[0:3], look=c[3:6], up=c[6:9], height_angle=float(c[9]), aspect=float(c[10]),
                      aperture=0.08, focal_length=0.6, focal_distance=2.5)
    W = H = 48
    st = pt.RenderSettings(W, H, 8, max_depth=5, rr_start_depth=3, seed=7)
    mean_g, paths_g, _ = gpu_render_paths(cuda, s, st)
    tree = oracle.Tree(s.tri_v)
    mean_o, paths_o, _ = oracle.render(s, tree, W, H, 8, max_depth=5, rr_start=3, seed=7, per_path=True)
    agree = _path_agreement(paths_g, paths_o)
    print(f"thin lens: path agreement {agree:.5f}")
    assert agree >= 0.98


def test_autofocus_and_unresolved_lens(cuda, oracle):
    s = scenegen.plain(0)
    acc = pt.Accel(s)
    ds = pt.DeviceScene(s, acc)
    cam = s.camera.copy()
    cam[11], cam[12], cam[13], cam[14], cam[15] = 0.05, 0.6, -1.0, 0.5, 0.5
    f = pt.Film(16, 16)
    with pytest.raises(pt.N.MgpuError, match="thin lens"):
        pt.render(ds, pt.RenderSettings(16, 16, 1), f, camera=cam)
    c2 = pt.resolve_autofocus(cam, ds)
    # the centre ray's hit distance, from the oracle's closest hit
    d = oracle.camera_dir(s.camera, 0.5, 0.5)
    t, _, _, _ = oracle.trace_closest(None, s.tri_v, s.tri_flags,
                                      np.array([[*s.camera[:3], 0, *d, np.inf]], np.float32))
    assert c2[13] == pytest.approx(t[0], rel=1e-5)
    pt.render(ds, pt.RenderSettings(16, 16, 1), f, camera=c2)


def test_film_mean_is_the_fp64_mean_of_the_compensated_sums(cuda):
    # mgpu_film_read: (sum - compensation) / count per pixel in FP64, 0 where nothing was drawn
    s = scenegen.plain(0)
    ds = pt.DeviceScene(s, pt.Accel(s))
    W, H = 72, 40
    f = pt.Film(W, H)
    pt.render(ds, pt.RenderSettings(W, H, 9, max_depth=5, rr_start_depth=3, seed=12), f)
    raw = f.raw().astype(np.float64)
    cnt = raw[0, ..., 3:4]
    host = np.where(cnt > 0, (raw[0, ..., :3] - raw[1, ..., :3]) / np.where(cnt > 0, cnt, 1.0), 0.0)
    assert np.array_equal(f.mean(), host)
    empty = pt.Film(W, H)
    assert np.array_equal(empty.mean(), np.zeros((H, W, 3)))


def test_device_tonemap_matches_host_model(cuda, tmp_path):
    from milton_gb300 import imageio
    from oracle import tonemap
    s = scenegen.plain(0)
    acc = pt.Accel(s)
    ds = pt.DeviceScene(s, acc)
    f = pt.Film(64, 48)
    pt.render(ds, pt.RenderSettings(64, 48, 16, max_depth=5, rr_start_depth=3, seed=2), f)
    dev = f.tonemap()
    host = tonemap.reinhard(f.mean())
    diff = np.abs(dev.astype(int) - host.astype(int))
    assert diff.max() <= 1 and (diff == 0).mean() >= 0.99
    p = tmp_path / "plain.png"
    imageio.write_png(str(p), dev)
    assert np.array_equal(imageio.read_png(str(p)), dev)


@pytest.mark.parametrize("kind,support,params", [("box", 2.0, {}), ("triangle", 2.0, {}),
                                                 ("gaussian", 3.0, {"sigma": 0.8}),
                                                 ("mitchell", 2.0, {"B": 1 / 3, "C": 1 / 3}),
                                                 ("lanczosSinc", 2.0, {"tau": 3.0})])
def test_reconstruction_filters(cuda, kind, support, params):
    from oracle import filters, pyoracle
    s = scenegen.plain(0)
    acc = pt.Accel(s)
    ds = pt.DeviceScene(s, acc)
    W, H, spp = 20, 16, 4
    st = pt.RenderSettings(W, H, spp, max_depth=5, rr_start_depth=3, seed=3)
    mean_g, paths_g, _ = gpu_render_paths(cuda, s, st, accel=acc, dscene=ds)
    f = pt.Film(W, H)
    f.set_filter(kind, support, **params)
    pt.render(ds, st, f)
    got = f.mean()
    want = filters.splat(paths_g, spp, 0, 3, 0, kind, support, params, pyoracle.uniforms)
    assert np.allclose(got, want, rtol=2e-5, atol=1e-6)
    # the splat sums are order-independent: the same image from tiny waves and split passes
    f2 = pt.Film(W, H)
    f2.set_filter(kind, support, **params)
    pt.render(ds, pt.RenderSettings(W, H, spp, sample_count=1, max_depth=5, rr_start_depth=3, seed=3,
                                    wave_paths=64), f2)
    pt.render(ds, pt.RenderSettings(W, H, spp, sample_begin=1, max_depth=5, rr_start_depth=3, seed=3), f2)
    assert np.array_equal(f2.mean(), got)


def test_point_light_known_answer(cuda):
    # an omni point light of power P at height h above a Lambertian floor: radiance at the
    # point below it is kd / pi * (P / 4 pi) / h^2, one shadow ray per path
    from milton_gb300.scene import SceneBuilder, camera, diffuse
    kd, P, hgt = 0.6, 10.0, 1.5
    b = SceneBuilder()
    fm = b.material(diffuse(kd))
    h = 50.0
    b.add("floor", np.array([[[-h, 0, h], [h, 0, h], [h, 0, -h]], [[-h, 0, h], [h, 0, -h], [-h, 0, -h]]],
                            np.float32), None, fm)
    rec = np.zeros(16, np.float32)
    rec[0:3] = (0.0, hgt, 0.0)
    rec[13:16] = P / (4 * np.pi)
    ext = np.zeros(16, np.float32)
    ext[0] = 3
    b.add_light(rec, ext)
    s = b.build(camera(eye=(0.0, 0.5, 0.0), look=(0.0, -1.0, 0.0), up=(0, 0, 1), height_angle=0.05, aspect=1.0))
    st = pt.RenderSettings(4, 4, 16, no_direct_samples=4, max_depth=1, seed=2)
    mean, paths, _ = gpu_render_paths(cuda, s, st)
    want = kd / np.pi * P / (4 * np.pi) / hgt ** 2
    assert np.allclose(mean, want, rtol=1e-4), (mean.mean(), want)
    assert pt.render_stats()["shadow_rays"] == 4 * 4 * 16


def test_dispersive_dielectric_per_path(cuda, oracle):
    # a per-channel IOR: every path refracts with its colour channel's index
    from milton_gb300.scene import dielectric
    s = scenegen.plain(1)
    for name, first, count in s.shapes:
        if name in ("tallBox", "shortBox"):
            s.materials[s.tri_mat[first]] = dielectric([1.4, 1.55, 1.8], transparency=0.9)
    st = pt.RenderSettings(48, 48, 16, max_depth=6, rr_start_depth=3, seed=8)
    mean_g, paths_g, _ = gpu_render_paths(cuda, s, st)
    mean_o, paths_o, _ = oracle.render(s, oracle.Tree(s.tri_v), 48, 48, 16, max_depth=6, rr_start=3, seed=8,
                                       per_path=True)
    agree = _path_agreement(paths_g, paths_o)
    print(f"dispersive: path agreement {agree:.5f}, mean {mean_g.mean():.5f} / {mean_o.mean():.5f}")
    assert agree >= 0.97


@pytest.mark.parametrize("w,h,spp,nds", [(1, 1, 1, 1), (13, 7, 7, 3), (9, 17, 2, 2)])
def test_ragged_sizes_and_non_square_sample_counts(cuda, oracle, w, h, spp, nds):
    # image sides that are not multiples of the 8 x 8 slot tiles, sample counts that are not
    # squares (strata of side floor(sqrt(spp)) reused), several light samples
    s = scenegen.plain(3)
    st = pt.RenderSettings(w, h, spp, no_direct_samples=nds, max_depth=5, rr_start_depth=3, seed=21)
    mean_g, paths_g, _ = gpu_render_paths(cuda, s, st)
    mean_o, paths_o, _ = oracle.render(s, oracle.Tree(s.tri_v), w, h, spp, nds=nds, max_depth=5, rr_start=3, seed=21,
                                       per_path=True)
    assert paths_g.shape == paths_o.shape == (h, w, spp, 3)
    assert _path_agreement(paths_g, paths_o) >= (0.97 if w * h * spp > 50 else 1.0)


def test_scenes_without_geometry_or_lights(cuda):
    from milton_gb300.scene import SceneBuilder, camera, diffuse, quad_light
    cam = camera(eye=(0, 0, 3), look=(0, 0, -1), up=(0, 1, 0), height_angle=40.0, aspect=1.0)
    # a light record but no triangles: every ray misses, the film is black (no background)
    b = SceneBuilder()
    b.material(diffuse(0.5))
    b.add_light(quad_light((0, 1, 0), (1, 0, 0), (0, 0, 1), 5.0))
    empty = b.build(cam)
    assert empty.ntri == 0
    mean, paths, _ = gpu_render_paths(cuda, empty, pt.RenderSettings(8, 8, 4, max_depth=3, seed=1))
    assert np.all(mean == 0) and np.all(paths == 0)
    # with a constant background the misses see it
    empty.background_le = np.array([0.25, 0.5, 1.0], np.float32)
    mean, _, _ = gpu_render_paths(cuda, empty, pt.RenderSettings(8, 8, 4, max_depth=3, seed=1))
    assert np.allclose(mean, [0.25, 0.5, 1.0])
    # geometry without lights: black
    s = scenegen.plain(0)
    dark = type(s)(tri_v=s.tri_v, tri_n=s.tri_n, tri_mat=s.tri_mat, tri_light=np.full(s.ntri, -1, np.int32),
                   tri_flags=s.tri_flags, materials=s.materials, lights=np.zeros((0, 16), np.float32), camera=s.camera)
    mean, _, _ = gpu_render_paths(cuda, dark, pt.RenderSettings(16, 16, 4, max_depth=5, rr_start_depth=3, seed=1))
    assert np.all(mean == 0)


def test_emitting_and_plain_spheres_per_path(cuda, oracle):
    # analytic spheres in the plain box: a glass one, a Phong one, and an emitting one whose light
    # samples follow Sphere::getPosition (a patch off its surface, area pi) and whose surface
    # emits at hits
    from milton_gb300.scene import SceneBuilder, camera, dielectric, diffuse, phong
    s0 = scenegen.plain(4)
    b = SceneBuilder()
    for name, first, count in s0.shapes:
        if name == "light":
            continue
        mi = b.material(s0.materials[s0.tri_mat[first]])
        b.add(name, s0.tri_v[first:first + count], s0.tri_n[first:first + count], mi)
    b.add_sphere((-0.4, 0.35, 0.3), 0.3, b.material(dielectric(1.5)))
    b.add_sphere((0.45, 0.25, -0.2), 0.25, b.material(phong(0.3, 0.4, 40.0)))
    rot = np.array([[0, 0, 1], [0, 1, 0], [-1, 0, 0]], np.float64)  # object +z toward world -x
    b.add_sphere((0.2, 1.5, 0.0), 0.15, b.material(diffuse(0.5)), rotation=rot, radiance=[20.0, 18.0, 15.0])
    s = b.build(s0.camera)
    assert len(s.lights) == 1 and s.light_ext[0, 0] == 4 and s.sphere_light.tolist() == [-1, -1, 0]
    st = pt.RenderSettings(40, 40, 16, no_direct_samples=2, max_depth=5, rr_start_depth=3, seed=13)
    mean_g, paths_g, _ = gpu_render_paths(cuda, s, st)
    mean_o, paths_o, _ = oracle.render(s, oracle.Tree(s.tri_v), 40, 40, 16, nds=2, max_depth=5, rr_start=3,
                                       seed=13, per_path=True)
    agree = _path_agreement(paths_g, paths_o)
    print(f"spheres: path agreement {agree:.5f}, mean {mean_g.mean():.5f} / {mean_o.mean():.5f}")
    assert agree >= 0.97 and mean_g.mean() > 0.01


def test_large_frame_and_many_passes(cuda, oracle):
    # a 4096 x 4096 frame (16.8 M paths in one call: several waves when the wave is capped) and a
    # tiny one with 1024 passes: a band of rows and every pixel match the oracle's paths
    s = scenegen.plain(5)
    ds = pt.DeviceScene(s, pt.Accel(s))
    f = pt.Film(4096, 4096)
    st = pt.RenderSettings(4096, 4096, 1, max_depth=5, rr_start_depth=3, seed=17, wave_paths=1 << 22)
    pt.render(ds, st, f)
    img = f.mean()
    mean_o, _, _ = oracle.render(s, oracle.Tree(s.tri_v), 4096, 4096, 1, max_depth=5, rr_start=3, seed=17,
                                 rows=(2048, 2052))
    band = img[2048:2052]
    close = np.abs(band - mean_o) <= 1e-4 + 2e-3 * np.maximum(np.abs(band), np.abs(mean_o))
    assert np.all(close, axis=-1).mean() >= 0.98
    st = pt.RenderSettings(3, 2, 1024, max_depth=5, rr_start_depth=3, seed=19)
    mean_g, paths_g, _ = gpu_render_paths(cuda, s, st)
    mean_o, paths_o, _ = oracle.render(s, oracle.Tree(s.tri_v), 3, 2, 1024, max_depth=5, rr_start=3, seed=19,
                                       per_path=True)
    assert _path_agreement(paths_g, paths_o) >= 0.98
    assert np.allclose(mean_g, mean_o, rtol=3e-2, atol=5e-3)  # a diverged path moves a mean by at most its share


def test_read_bandwidth_probe(cuda):
    # the roofline denominators: an L2-resident buffer reads faster than one 16x the L2
    l2 = pt.measure_read_bandwidth(32 << 20, 50)
    hbm = pt.measure_read_bandwidth(2 << 30, 3)
    print(f"read bandwidth: L2-resident {l2:.0f} GB/s, HBM {hbm:.0f} GB/s")
    assert hbm > 1000 and l2 > hbm
