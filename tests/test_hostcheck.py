"""The FP32 arithmetic the kernels run (milton_gb300/csrc/hd_*.h, compiled for the host by the
test harness in tests/native) against the FP64 oracle -- runs without a GPU."""
import numpy as np
import pytest

from milton_gb300 import scenegen
from milton_gb300.scene import dielectric, diffuse, phong
from raygen import camera_rays, classify, sphere_rays


def _p(a):
    return None if a is None else a.ctypes.data


def hc_trace(lib, v, flags, rays, top=1, max_depth=24):
    n = rays.shape[0]
    hits = np.zeros((n, 4), np.float32)
    occ = np.zeros(n, np.uint8)
    cnt = np.zeros((n, 4), np.uint32)
    v = np.ascontiguousarray(v, np.float32)
    fl = None if flags is None else np.ascontiguousarray(flags, np.uint32)
    rays = np.ascontiguousarray(rays, np.float32)
    assert lib.hc_trace(_p(v), _p(fl), v.reshape(-1, 9).shape[0], _p(rays), n, _p(hits), _p(occ), _p(cnt),
                        max_depth, top) == 0
    return hits, occ, cnt


@pytest.mark.parametrize("top", [0, 1])
def test_fp32_traversal_plain(oracle, hostcheck, top):
    s = scenegen.plain(0)
    flags = s.tri_flags.copy()
    flags[::3] = 1
    rays = np.concatenate([camera_rays(s.camera, 30000, 0), sphere_rays((-1, 0, -1), (1, 2, 1), 30000, 1)])
    t, p, t2, _ = oracle.trace_closest(None, s.tri_v, flags, rays)
    h, occ, cnt = hc_trace(hostcheck, s.tri_v, flags, rays, top=top)
    r = classify(p, t, t2, h[:, 1].view(np.int32), h[:, 0])
    assert r["mismatches"] == 0, r
    assert r["ties"] <= 0.005 * r["n"]
    # any-hit with tmax just short of the closest hit sees nothing; beyond it sees the hit
    r2 = rays.copy()
    hit = np.isfinite(t)
    r2[:, 7] = np.where(hit, t * (1 - 1e-4), 10.0)
    _, occ_short, _ = hc_trace(hostcheck, s.tri_v, flags, r2, top=top)
    assert occ_short.sum() <= 2
    r2[:, 7] = np.where(hit, t * (1 + 1e-4), 10.0)
    _, occ_long, _ = hc_trace(hostcheck, s.tri_v, flags, r2, top=top)
    assert np.array_equal(occ_long.astype(bool)[hit], np.ones(hit.sum(), bool)) or \
        (occ_long.astype(bool)[hit].mean() > 0.999)


def test_fp32_traversal_spheres(oracle, hostcheck):
    s = scenegen.random_scene(8, 40000)
    lo, hi = s.tri_v.reshape(-1, 3).min(0), s.tri_v.reshape(-1, 3).max(0)
    rays = np.concatenate([camera_rays(s.camera, 20000, 5), sphere_rays(lo, hi, 20000, 6)])
    tree = oracle.Tree(s.tri_v)
    t, p, _, _ = oracle.trace_closest(tree, s.tri_v, s.tri_flags, rays)
    h, _, cnt = hc_trace(hostcheck, s.tri_v, s.tri_flags, rays)
    pg = h[:, 1].view(np.int32)
    bad = np.nonzero(pg != p)[0]
    # every disagreement must be a tie in the brute-force oracle
    if bad.size:
        tb, pb, t2b, _ = oracle.trace_closest(None, s.tri_v, s.tri_flags, rays[bad])
        r = classify(pb, tb, t2b, pg[bad], h[bad, 0])
        assert r["mismatches"] == 0, r
    assert bad.size <= 0.01 * len(rays)
    assert cnt[:, 3].max() <= 24


def test_uniforms_match_oracle(oracle, hostcheck):
    rng = np.random.default_rng(0)
    for _ in range(200):
        seed, stream, path = int(rng.integers(1 << 62)), int(rng.integers(1 << 31)), int(rng.integers(1 << 60))
        depth, block = int(rng.integers(0, 0x10000)), int(rng.integers(0, 0x10000))
        u32 = np.zeros(4, np.float32)
        hostcheck.hc_uniforms(seed, stream, path, depth, block, u32.ctypes.data)
        assert np.array_equal(u32.astype(np.float64), oracle.uniforms(seed, stream, path, depth, block))


@pytest.mark.parametrize("mat", [diffuse([0.6, 0.5, 0.4]), phong([0.3, 0.2, 0.25], [0.5, 0.6, 0.4], 80.0),
                                 phong([0.05, 0.05, 0.05], [0.9, 0.9, 0.9], 200.0), dielectric(1.5),
                                 dielectric([1.45, 1.6, 1.9], transparency=0.8)],
                         ids=["diffuse", "phong", "phong-sharp", "dielectric", "dielectric-dispersive"])
def test_fp32_bsdf_matches_fp64(oracle, hostcheck, mat):
    rng = np.random.default_rng(2)
    agree = 0
    N = 3000
    for k in range(N):
        ns = rng.normal(size=3); ns /= np.linalg.norm(ns)
        wi = rng.normal(size=3); wi /= np.linalg.norm(wi)
        if rng.random() < 0.8:
            wi = wi - 2 * max(0.0, wi @ ns) * ns  # mostly front-side hits
            wi /= np.linalg.norm(wi)
        u = rng.random(3)
        ns32, wi32, u32 = ns.astype(np.float32), wi.astype(np.float32), u.astype(np.float32)
        ev64, wo64, fs64 = oracle.bsdf_sample(mat, ns32, wi32, k % 3, u32)
        wo = np.zeros(3, np.float32)
        fs = np.zeros(3, np.float32)
        ev32 = hostcheck.hc_bsdf_sample(mat.ctypes.data, ns32.ctypes.data, wi32.ctypes.data, k % 3, u32.ctypes.data,
                                        wo.ctypes.data, fs.ctypes.data)
        if ev32 == ev64 and np.allclose(wo, wo64, atol=2e-4) and np.allclose(fs, fs64, rtol=2e-3, atol=1e-4):
            agree += 1
    # lobe decisions can flip only on FP32/FP64 rounding near a threshold
    assert agree >= 0.995 * N, agree


def test_offset_moves_off_the_surface(hostcheck):
    rng = np.random.default_rng(1)
    for _ in range(1000):
        p = (rng.normal(size=3) * 10 ** rng.uniform(-3, 3)).astype(np.float32)
        n = rng.normal(size=3).astype(np.float32); n /= np.linalg.norm(n)
        out = np.zeros(3, np.float32)
        hostcheck.hc_offset(p.ctypes.data, n.ctypes.data, out.ctypes.data)
        assert float((out.astype(np.float64) - p) @ n) > 0


def test_light_point_types(hostcheck):
    """light_point (shared by the GPU kernels) against the reference's formulas, restated here
    in FP64: Plane::getPosition, Triangle::getPosition (uv frame, magnitudes of 2-D cross
    products) and Mesh::getPosition (triangle floor(u n), barycentrics (r1, v, r2) / sum)."""
    from pathlib import Path
    from milton_gb300 import sceneloader as L
    sf = L.load(str(Path(__file__).resolve().parent / "scenes" / "emitters.js"))
    s = sf.scene
    rng = np.random.default_rng(5)
    tv = np.ascontiguousarray(s.tri_v, np.float32)
    tn = np.ascontiguousarray(s.tri_n, np.float32)
    for li in range(len(s.lights)):
        rec, ext = s.lights[li], s.light_ext[li]
        for _ in range(50):
            uvr = rng.uniform(0, 1, 4).astype(np.float32)
            out = np.zeros(6, np.float32)
            hostcheck.hc_light_point(_p(rec), _p(ext), _p(uvr), _p(tv), _p(tn), _p(out))
            u, v, r1, r2 = (float(x) for x in uvr)
            kind = int(ext[0])
            if kind == 0:
                p = rec[0:3] + rec[3:6] * (u - 0.5) + rec[6:9] * (v - 0.5)
                n = rec[9:12]
            elif kind == 1:
                c = np.array([u - ext[1], v - ext[2]], np.float64)
                a, b = ext[3:5].astype(np.float64), ext[5:7].astype(np.float64)
                pb = abs(c[0] * b[1] - c[1] * b[0]) * ext[7]
                pc = abs(c[0] * a[1] - c[1] * a[0]) * ext[7]
                p = rec[0:3] + rec[3:6] * pb + rec[6:9] * pc
                n = rec[9:12]
            else:
                first, count = ext.view(np.uint32)[8:10]
                t = first + min(int(np.floor(u * count)), count - 1)
                bary = np.array([r1, v, r2]) / (r1 + v + r2)
                p = bary @ s.tri_v[t].astype(np.float64)
                n = bary @ s.tri_n[t].astype(np.float64)
                n = n / np.linalg.norm(n)
            assert np.allclose(out[:3], p, atol=1e-5), (li, kind)
            assert np.allclose(out[3:], n / np.linalg.norm(n), atol=1e-5), (li, kind)


def test_thin_lens_camera_rays(hostcheck, oracle):
    """camera_ray (kernels, FP32) against the oracle's ThinLensCamera::getWorldRay (FP64)."""
    from milton_gb300.scene import camera
    rng = np.random.default_rng(9)
    for aperture, fl, fd in ((0.0, 0.0, 1.0), (0.05, 0.7, 3.0), (0.2, 0.5, 1.2)):
        cam = camera(eye=(0.3, 1.1, 3.5), focus=(0.0, 0.8, 0.0), height_angle=40.0, aspect=1.25, aperture=aperture,
                     focal_length=fl, focal_distance=fd)
        for _ in range(200):
            x, y, u1, u2 = rng.uniform(0, 1, 4)
            out = np.zeros(6, np.float32)
            hostcheck.hc_camera_ray(_p(cam), x, y, u1, u2, _p(out))
            o, d = oracle.camera_ray(cam, x, y, u1, u2)
            assert np.allclose(out[:3], o, atol=2e-6) and np.allclose(out[3:], d, atol=2e-6)
            if aperture == 0.0:
                assert np.allclose(out[:3], cam[:3])
    # rays of one film point converge on the focal plane (distance fd along the view axis)
    cam = camera(eye=(0, 0, 0), look=(0, 0, -1), aperture=0.1, focal_length=0.5, focal_distance=2.0)
    pts = []
    for u1, u2 in rng.uniform(0, 1, (16, 2)):
        o, d = oracle.camera_ray(cam, 0.3, 0.6, u1, u2)
        t = (-2.0 - o[2]) / d[2]
        pts.append(o + t * d)
    assert np.ptp(np.array(pts), axis=0).max() < 1e-9


def test_dispersion_refracts_each_channel_with_its_ior(oracle, hostcheck):
    # a path refracts with its colour channel's IOR (DielectricBSDF.cpp:79-87): the refracted
    # directions of channels 0, 1, 2 bend by their own indices (Snell's law)
    mat = dielectric([1.3, 1.6, 2.2], transparency=1.0)
    ns = np.array([0.0, 1.0, 0.0], np.float32)
    wi = np.array([0.6, -0.8, 0.0], np.float32)
    sin_i = 0.6
    for ch, ior in enumerate((1.3, 1.6, 2.2)):
        for u0 in np.linspace(0.001, 0.5, 20):  # small u: the refraction lobe (probability T (1 - Fr))
            u = np.array([u0, 0.5, 0.5], np.float32)
            ev, wo, fs = oracle.bsdf_sample(mat, ns, wi, ch, u)
            if ev != 4:
                continue
            sin_t = np.hypot(wo[0], wo[2])
            assert abs(sin_t - 1.0003 * sin_i / ior) < 1e-6  # float32 inputs
            wo32 = np.zeros(3, np.float32)
            fs32 = np.zeros(3, np.float32)
            ev32 = hostcheck.hc_bsdf_sample(mat.ctypes.data, ns.ctypes.data, wi.ctypes.data, ch, u.ctypes.data,
                                            wo32.ctypes.data, fs32.ctypes.data)
            assert ev32 == 4 and np.allclose(wo32, wo, atol=1e-5)
            break
        else:
            raise AssertionError("no refraction sampled")
