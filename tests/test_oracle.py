"""The oracle pinned: Philox known answers, kd traversal against brute force, BSDF property
checks modelled on the reference's material tests, and analytic known-answer scenes."""
import numpy as np
import pytest

from milton_gb300 import scenegen
from milton_gb300.scene import SceneBuilder, camera, dielectric, diffuse, phong
from raygen import camera_rays, classify, sphere_rays


# Random123 known-answer vectors for philox4x32-10 (kat_vectors of the Random123 library)
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,want", PHILOX_KAT)
def test_philox_known_answers(oracle, ctr, key, want):
    assert tuple(int(x) for x in oracle.philox(ctr, key)) == want


def test_uniform_mapping(oracle):
    u = oracle.uniforms(7, 3, 12345, 2, 1)
    w = oracle.philox([12345, 0, (2 << 16) | 1, 3], [7, 0])
    assert np.array_equal(u, (w >> 8).astype(np.float64) / 16777216.0)
    assert np.all((u >= 0) & (u < 1))


def test_kd_traversal_matches_brute_force(oracle):
    s = scenegen.plain(0)
    flags = s.tri_flags.copy()
    flags[::3] = 1
    rays = np.concatenate([camera_rays(s.camera, 20000, 0), sphere_rays((-1, 0, -1), (1, 2, 1), 20000, 1)])
    tree = oracle.Tree(s.tri_v)
    t, p, t2, _ = oracle.trace_closest(None, s.tri_v, flags, rays)
    tk, pk, _, _ = oracle.trace_closest(tree, s.tri_v, flags, rays)
    r = classify(p, t, t2, pk, tk)
    assert r["mismatches"] == 0, r
    assert r["exact"] >= 0.99 * r["n"]
    # any-hit: kd and brute force agree
    rays2 = rays.copy()
    rays2[:, 7] = np.where(np.isfinite(t), t * 1.5, 4.0)
    assert np.array_equal(oracle.trace_any(tree, s.tri_v, flags, rays2), oracle.trace_any(None, s.tri_v, flags, rays2))


def test_kd_traversal_matches_brute_force_spheres(oracle):
    s = scenegen.random_scene(5, 12000)
    lo, hi = s.tri_v.reshape(-1, 3).min(0), s.tri_v.reshape(-1, 3).max(0)
    rays = np.concatenate([camera_rays(s.camera, 4000, 3), sphere_rays(lo, hi, 4000, 4)])
    tree = oracle.Tree(s.tri_v)
    t, p, t2, _ = oracle.trace_closest(None, s.tri_v, s.tri_flags, rays)
    tk, pk, _, _ = oracle.trace_closest(tree, s.tri_v, s.tri_flags, rays)
    r = classify(p, t, t2, pk, tk)
    assert r["mismatches"] == 0, r


def test_culled_triangle_semantics(oracle):
    # Triangle.cpp:245-248: det = e1 . (d x e2) must exceed EPSILON
    v = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]]], np.float32)  # (v1-v0)x(v2-v0) = +z
    rays = np.zeros((2, 8), np.float32)
    rays[0, :3] = (0.2, 0.2, 1.0); rays[0, 4:7] = (0, 0, -1); rays[0, 7] = np.inf   # from the +z side
    rays[1, :3] = (0.2, 0.2, -1.0); rays[1, 4:7] = (0, 0, 1); rays[1, 7] = np.inf   # from the -z side
    t_two, p_two, _, _ = oracle.trace_closest(None, v, np.array([0], np.uint32), rays)
    t_cul, p_cul, _, _ = oracle.trace_closest(None, v, np.array([1], np.uint32), rays)
    assert list(p_two) == [0, 0]
    assert list(p_cul) == [0, -1]
    assert np.allclose(t_two, [1.0, 1.0])


def _hemi_samples(oracle, mat, ns, wi, n=20000, seed=0):
    rng = np.random.default_rng(seed)
    evs, wos, fss = [], [], []
    for k in range(n):
        ev, wo, fs = oracle.bsdf_sample(mat, ns, wi, k % 3, rng.random(3))
        evs.append(ev); wos.append(wo); fss.append(fs)
    return np.array(evs), np.array(wos), np.array(fss)


def test_diffuse_sampling_properties(oracle):
    # mlt/src/tests/materials/basic: unit wo in the upper hemisphere; E[f/pdf] = kd
    ns = np.array([0.0, 1.0, 0.0])
    wi = np.array([0.3, -1.0, 0.2]); wi /= np.linalg.norm(wi)
    kd = np.array([0.7, 0.4, 0.2])
    ev, wo, fs = _hemi_samples(oracle, diffuse(kd), ns, wi)
    assert np.all(ev == 1)
    assert np.allclose(np.linalg.norm(wo, axis=1), 1.0, atol=1e-12)
    assert np.all(wo @ ns >= 0)
    assert np.allclose(fs.mean(0), kd.astype(np.float32), rtol=1e-9)  # f / pdf = (kd/pi) / (1/pi) exactly
    # cosine-weighted: E[cos] = 2/3
    assert abs((wo @ ns).mean() - 2.0 / 3.0) < 0.01
    # back-face hit is absorbed (DiffuseBSDF.cpp:21-24)
    ev_b, _, _ = oracle.bsdf_sample(diffuse(kd), ns, -wi, 0, np.array([0.5, 0.5, 0.5]))
    assert ev_b == 0


def test_energy_conservation_and_reciprocity(oracle):
    # mlt/src/tests/materials/physicallyValid: E[reflected] <= 1 + eps; fuzzy reciprocity
    ns = np.array([0.0, 0.0, 1.0])
    rng = np.random.default_rng(3)
    for mat in (diffuse([0.9, 0.5, 0.1]), phong([0.3, 0.2, 0.1], [0.4, 0.5, 0.6], 50.0)):
        for _ in range(5):
            wi = rng.normal(size=3); wi[2] = -abs(wi[2]) - 0.1; wi /= np.linalg.norm(wi)
            ev, wo, fs = _hemi_samples(oracle, mat, ns, wi, n=4000, seed=int(rng.integers(1 << 30)))
            ok = ev > 0
            assert np.all(fs[ok] >= 0)
            if mat[0] == 0:
                assert np.all(fs.mean(0) <= 1.0 + 1e-9)
        for _ in range(50):
            a = rng.normal(size=3); a[2] = abs(a[2]) + 0.05; a /= np.linalg.norm(a)
            b = rng.normal(size=3); b[2] = abs(b[2]) + 0.05; b /= np.linalg.norm(b)
            f_ab = oracle.bsdf_eval(mat, ns, -a, b)
            f_ba = oracle.bsdf_eval(mat, ns, -b, a)
            assert np.allclose(f_ab, f_ba, rtol=1e-9, atol=1e-12)


def test_dielectric_fresnel_split(oracle):
    # refraction probability = transparency * (1 - Fr); fs = ks on reflection, ks*e_index on refraction
    ns = np.array([0.0, 1.0, 0.0])
    wi = np.array([0.0, -1.0, 0.0])
    mat = dielectric(1.5)
    rng = np.random.default_rng(1)
    evs = np.array([oracle.bsdf_sample(mat, ns, wi, 1, rng.random(3))[0] for _ in range(20000)])
    fr = ((1.0003 - 1.5) / (1.0003 + 1.5)) ** 2
    assert abs((evs == 3).mean() - fr) < 0.01
    ev, wo, fs = oracle.bsdf_sample(mat, ns, wi, 1, np.array([0.99, 0, 0]))
    assert ev == 3 and np.allclose(wo, [0, 1, 0]) and np.allclose(fs, [1, 1, 1])
    ev, wo, fs = oracle.bsdf_sample(mat, ns, wi, 1, np.array([0.0, 0, 0]))
    assert ev == 4 and np.allclose(wo, [0, -1, 0]) and np.allclose(fs, [0, 1, 0])
    # total internal reflection from inside at grazing incidence
    wi_in = np.array([0.9, 0.1, 0.0]); wi_in /= np.linalg.norm(wi_in)
    ev, wo, _ = oracle.bsdf_sample(mat, ns, wi_in, 0, np.array([0.0, 0, 0]))
    assert ev == 3


def _single_plane_scene(kd=0.5, light_radiance=1.0, light_half=0.5, light_h=1.0):
    """Lambertian floor under a square light facing down: a direct-lighting known answer."""
    b = SceneBuilder()
    fm = b.material(diffuse(kd))
    h = 50.0
    b.add("floor", np.array([[[-h, 0, h], [h, 0, h], [h, 0, -h]], [[-h, 0, h], [h, 0, -h], [-h, 0, -h]]],
                            np.float32), None, fm)
    lm = b.material(diffuse(0.0))
    b.add_quad_light("light", (0.0, light_h, 0.0), (2 * light_half, 0, 0), (0, 0, -2 * light_half), light_radiance, lm)
    cam = camera(eye=(0.0, 0.5, 0.0), look=(0.0, -1.0, 0.0), up=(0, 0, 1), height_angle=0.5, aspect=1.0)
    return b.build(cam, name="plane_under_light")


def _form_factor_point_to_square(a, h):
    """Irradiance factor E / L at the centre below a square light of half-side a at height h
    (closed form for a parallel axis-aligned rectangle, unit radiance)."""
    def f(x, y):
        return (x / np.sqrt(x * x + h * h) * np.arctan(y / np.sqrt(x * x + h * h))
                + y / np.sqrt(y * y + h * h) * np.arctan(x / np.sqrt(y * y + h * h)))
    return 4 * 0.5 * f(a, a)  # four quadrants, each x, y in [0, a]; E/L = pi * F, F = f / (2 pi)


def test_direct_lighting_known_answer(oracle):
    # camera looks straight down at the floor point below the light centre: the first hit's
    # radiance is kd/pi * E with E = L * (closed-form form factor); Russian roulette is off
    # by capping depth at 1 so only direct light counts
    kd, L, a, hgt = 0.5, 2.0, 0.5, 1.0
    s = _single_plane_scene(kd, L, a, hgt)
    tree = oracle.Tree(s.tri_v)
    mean, paths, st = oracle.render(s, tree, 4, 4, 4096, max_depth=1, nds=1, seed=11, threads=4)
    E = L * _form_factor_point_to_square(a, hgt)
    want = kd / np.pi * E
    got = mean.mean()
    assert abs(got - want) < 0.01 * want, (got, want)


def test_render_is_thread_count_independent(oracle):
    s = scenegen.plain(0)
    tree = oracle.Tree(s.tri_v)
    m1, _, s1 = oracle.render(s, tree, 24, 24, 4, max_depth=5, rr_start=3, threads=1)
    m8, _, s8 = oracle.render(s, tree, 24, 24, 4, max_depth=5, rr_start=3, threads=8)
    assert np.array_equal(m1, m8) and s1 == s8


def test_point_light_known_answer(oracle):
    # an omni point light of power P at height h above a Lambertian floor: the point below it
    # receives E = (P / 4 pi) / h^2 (DirectIllumination's point branch: one sample, cosine 1 at
    # the light, no area factor); radiance kd / pi * E
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
    cam = camera(eye=(0.0, 0.5, 0.0), look=(0.0, -1.0, 0.0), up=(0, 0, 1), height_angle=0.05, aspect=1.0)
    s = b.build(cam, name="floor_under_point")
    tree = oracle.Tree(s.tri_v)
    mean, _, st = oracle.render(s, tree, 2, 2, 4, max_depth=1, nds=4, seed=3, threads=2)
    want = kd / np.pi * P / (4 * np.pi) / hgt ** 2
    assert np.allclose(mean, want, rtol=1e-4), (mean.mean(), want)
    # one shadow ray per path for the point light, whatever noDirectSamples is
    assert st["shadow_rays"] == 2 * 2 * 4


def test_sphere_intersection_known_answers(oracle):
    # Sphere::getIntersection: unit-diameter sphere under T(c) R S(2r); the nearest root beyond
    # EPSILON, else the far one (a ray from inside), else none
    sp = np.array([1.0, 2.0, -3.0, 0.5, 0.0, 0.0, 0.0, 1.0], np.float32)
    assert np.isclose(oracle.sphere_closest(sp, [1, 2, 0], [0, 0, -1]), 2.5)
    assert np.isclose(oracle.sphere_closest(sp, [1, 2, -3], [0, 1, 0]), 0.5)
    assert np.isinf(oracle.sphere_closest(sp, [1, 2.6, 0], [0, 0, -1]))
    assert np.isinf(oracle.sphere_closest(sp, [1, 2, -4], [0, 0, -1]))  # sphere behind
    # a grazing ray at distance 0.4 from the centre: chord half-length 0.3
    assert np.isclose(oracle.sphere_closest(sp, [1, 2.4, 0], [0, 0, -1]), 3.0 - 0.3)
    # a rotation does not move the surface
    q = np.array([0.2, 0.4, -0.1, 0.8]); q /= np.linalg.norm(q)
    sp2 = sp.copy(); sp2[4:8] = q
    assert np.isclose(oracle.sphere_closest(sp2, [1, 2.4, 0], [0, 0, -1]), 2.7)


def test_oracle_matches_its_golden_fixtures(oracle):
    # regression pins of the oracle's own outputs (tests/golden/make_golden.py); FP64 libm may
    # differ in the last bits between hosts, hence the tolerance
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    import make_golden as G
    here = Path(__file__).resolve().parent / "golden"
    for name, fn in (("oracle_plain.npz", G.plain_case), ("oracle_textured.npz", G.textured_case)):
        want = np.load(here / name)
        got = fn()
        for k in want.files:
            if want[k].dtype.kind == "f":
                assert np.allclose(got[k], want[k], rtol=1e-9, atol=1e-12), (name, k)
            else:
                assert np.array_equal(got[k], want[k]), (name, k)
