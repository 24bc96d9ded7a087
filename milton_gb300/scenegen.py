"""Seeded synthetic scenes for the benchmark configurations (no external assets).

* ``plain``  closed box of 5 axis-aligned quads (10 triangles, open toward the camera), two boxes
             rotated about y at seeded angles (24 triangles), one 0.25-area quad light of
             radiance 15, Lambertian albedos U[0.2, 0.8] per RGB, pinhole camera with a 40 degree
             vertical field of view; rendered at 256x256, 16 spp, max depth 5, RR from depth 3.
* ``mid``    400 seeded UV spheres (50 x 26 segments = 2,500 triangles each, smooth normals) with
             log-uniform radii in [0.05, 1.0], resting without overlap on a 20 x 20 ground quad;
             materials 60% Lambertian / 30% modified Phong (n ~ U[10, 200], kd + ks <= 1) / 10%
             dielectric (IOR 1.5); 4 quad lights; 1024x1024, 64 spp, depth 8.
* ``batch``  many independent scenes of uneven size built from the same recipes.
* ``textured`` the plain box with image maps: a checker ``kd`` map repeated on the floor, a
             noise ``ks`` map on a Phong sphere, a ``transparency`` map on a dielectric sphere
             and a bump map on the back wall (seeded procedural images, material filters of
             every kind).
* ``large``  a displaced-grid terrain (fBm heights; 2,800 x 2,800 cells = 15,680,000 triangles
             by default: a 4096^2 vertex grid would be 33.5 M triangles, above the configuration's
             stated ~20 M total) plus 2,000 copied UV spheres of 2,160 triangles resting on it
             (4,320,000 triangles; modified Phong or dielectric), 16 quad lights in a 4 x 4 grid;
             about 20 M triangles; rendered at 2048x2048, 128 spp, depth 16.

Every generator is a pure function of its seed (numpy PCG64).
"""
from __future__ import annotations

import numpy as np

from .scene import TEX_BUMP, TEX_COLOR, SceneBuilder, Scene, Texture, camera, dielectric, diffuse, phong


# ------------------------------------------------------------------------------------------
# primitives

def quad_tris(p0, p1, p2, p3) -> np.ndarray:
    """Two triangles of the quad p0 p1 p2 p3 (counter-clockwise seen from the front)."""
    return np.array([[p0, p1, p2], [p0, p2, p3]], np.float32)


def box_tris(center, size, angle_y: float) -> tuple[np.ndarray, np.ndarray]:
    """12 triangles of a box resting on y = center[1], rotated by angle_y about +y; outward
    flat normals (each face has its own vertices, as a mesh with per-face normals)."""
    cx, cy, cz = center
    sx, sy, sz = (s / 2 for s in size)
    c, s = np.cos(angle_y), np.sin(angle_y)

    def P(x, y, z):
        return np.array([cx + c * x + s * z, cy + y, cz - s * x + c * z], np.float64)

    y0, y1 = 0.0, 2 * sy
    faces = [
        (P(-sx, y0, sz), P(sx, y0, sz), P(sx, y1, sz), P(-sx, y1, sz)),     # +z
        (P(sx, y0, -sz), P(-sx, y0, -sz), P(-sx, y1, -sz), P(sx, y1, -sz)),  # -z
        (P(sx, y0, sz), P(sx, y0, -sz), P(sx, y1, -sz), P(sx, y1, sz)),     # +x
        (P(-sx, y0, -sz), P(-sx, y0, sz), P(-sx, y1, sz), P(-sx, y1, -sz)),  # -x
        (P(-sx, y1, sz), P(sx, y1, sz), P(sx, y1, -sz), P(-sx, y1, -sz)),   # +y
        (P(-sx, y0, -sz), P(sx, y0, -sz), P(sx, y0, sz), P(-sx, y0, sz)),   # -y
    ]
    tris = np.concatenate([quad_tris(*f) for f in faces]).astype(np.float32)
    fn = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0]).astype(np.float64)
    fn /= np.linalg.norm(fn, axis=1, keepdims=True)
    return tris, np.repeat(fn[:, None, :], 3, axis=1).astype(np.float32)


def uv_sphere(center, radius, nu: int = 50, nv: int = 26) -> tuple[np.ndarray, np.ndarray]:
    """UV sphere: nu segments, nv rings -> 2 * nu * (nv - 2) + 2 * nu triangles, radial normals
    (what Mesh::computeNormals' vertex averaging converges to, Mesh.cpp:335-377)."""
    c = np.asarray(center, np.float64)
    th = np.linspace(0.0, np.pi, nv + 1)
    ph = np.linspace(0.0, 2 * np.pi, nu + 1)
    T, PH = np.meshgrid(th, ph, indexing="ij")
    dirs = np.stack([np.sin(T) * np.cos(PH), np.cos(T), np.sin(T) * np.sin(PH)], -1)
    dirs[:, -1] = dirs[:, 0]
    pts = c + radius * dirs
    tris, nrms = [], []
    for i in range(nv):
        for j in range(nu):
            a, b = pts[i, j], pts[i, j + 1]
            cc, d = pts[i + 1, j + 1], pts[i + 1, j]
            na, nb, nc, nd = dirs[i, j], dirs[i, j + 1], dirs[i + 1, j + 1], dirs[i + 1, j]
            if i != 0:           # skip the degenerate triangle at the north pole
                tris.append((a, d, b)); nrms.append((na, nd, nb))
            if i != nv - 1:      # and at the south pole
                tris.append((b, d, cc)); nrms.append((nb, nd, nc))
    return np.asarray(tris, np.float32), np.asarray(nrms, np.float32)


def _uv_sphere_fast(center, radius, nu: int = 50, nv: int = 26):
    """Vectorised uv_sphere (same triangles, same order)."""
    c = np.asarray(center, np.float64)
    th = np.linspace(0.0, np.pi, nv + 1)
    ph = np.linspace(0.0, 2 * np.pi, nu + 1)
    T, PH = np.meshgrid(th, ph, indexing="ij")
    dirs = np.stack([np.sin(T) * np.cos(PH), np.cos(T), np.sin(T) * np.sin(PH)], -1)
    dirs[:, -1] = dirs[:, 0]
    pts = c + radius * dirs
    i, j = np.meshgrid(np.arange(nv), np.arange(nu), indexing="ij")
    a, b, cc, d = (i, j), (i, j + 1), (i + 1, j + 1), (i + 1, j)
    t1 = np.stack([pts[a], pts[d], pts[b]], -2)
    n1 = np.stack([dirs[a], dirs[d], dirs[b]], -2)
    t2 = np.stack([pts[b], pts[d], pts[cc]], -2)
    n2 = np.stack([dirs[b], dirs[d], dirs[cc]], -2)
    keep1 = (i != 0)
    keep2 = (i != nv - 1)
    # interleave per cell as uv_sphere does: [t1 (if kept), t2 (if kept)]
    T2 = np.stack([t1, t2], 2)           # (nv, nu, 2, 3, 3)
    N2 = np.stack([n1, n2], 2)
    K2 = np.stack([keep1, keep2], 2)     # (nv, nu, 2)
    return T2[K2].astype(np.float32), N2[K2].astype(np.float32)


# ------------------------------------------------------------------------------------------
# configurations

PLAIN = dict(width=256, height=256, spp=16, max_depth=5, rr_start=3, nds=1)
MID = dict(width=1024, height=1024, spp=64, max_depth=8, rr_start=3, nds=1)


def plain(seed: int = 0) -> Scene:
    rng = np.random.default_rng(seed)
    b = SceneBuilder()
    alb = lambda: rng.uniform(0.2, 0.8, 3)  # noqa: E731
    # closed box x in [-1, 1], y in [0, 2], z in [-1, 1], open toward +z; normals face inward
    walls = {
        "floor": ((-1, 0, 1), (1, 0, 1), (1, 0, -1), (-1, 0, -1)),
        "ceiling": ((-1, 2, -1), (1, 2, -1), (1, 2, 1), (-1, 2, 1)),
        "back": ((-1, 0, -1), (1, 0, -1), (1, 2, -1), (-1, 2, -1)),
        "left": ((-1, 0, 1), (-1, 0, -1), (-1, 2, -1), (-1, 2, 1)),
        "right": ((1, 0, -1), (1, 0, 1), (1, 2, 1), (1, 2, -1)),
    }
    for name, pts in walls.items():
        m = b.material(diffuse(alb()))
        b.add(name, quad_tris(*[np.asarray(p, np.float32) for p in pts]), None, m)
    for name, center, size in (("tallBox", (-0.35, 0.0, -0.3), (0.6, 1.2, 0.6)),
                               ("shortBox", (0.4, 0.0, 0.3), (0.6, 0.6, 0.6))):
        ang = rng.uniform(-np.pi / 4, np.pi / 4)
        tris, nrm = box_tris(center, size, ang)
        b.add(name, tris, nrm, b.material(diffuse(alb())))
    lm = b.material(diffuse(0.0))
    # 0.5 x 0.5 quad just below the ceiling, emitting downward (normal = ez x ex = -y)
    b.add_quad_light("light", (0.0, 1.999, 0.0), (0.5, 0.0, 0.0), (0.0, 0.0, -0.5), 15.0, lm)
    cam = camera(eye=(0.0, 1.0, 3.75), look=(0.0, 0.0, -1.0), up=(0, 1, 0), height_angle=40.0, aspect=1.0)
    return b.build(cam, name="plain")


def textured(seed: int = 0, filters=("triangle", 2.0, {})) -> Scene:
    """The plain box with image maps (module docstring).  filters: the colour maps' filter
    (kind, support, params)."""
    rng = np.random.default_rng(seed)
    b = SceneBuilder()
    uv_quad = np.array([[(0, 0), (1, 0), (1, 1)], [(0, 0), (1, 1), (0, 1)]], np.float32)
    # checker with seeded colours, 16 x 12 texels, repeated 3 x 2 times over the floor
    cells = (np.add.outer(np.arange(12) // 3, np.arange(16) // 4) % 2).astype(bool)
    c0, c1 = rng.uniform(0.1, 0.4, 3), rng.uniform(0.5, 0.9, 3)
    checker = np.where(cells[..., None], c1, c0).astype(np.float32)
    checker += rng.uniform(-0.05, 0.05, checker.shape).astype(np.float32)
    kd_tex = b.texture(Texture(np.clip(checker, 0, 1), TEX_COLOR, filters, repeat_u=3.0, repeat_v=2.0))
    floor = diffuse(0.5)
    floor[10] = kd_tex
    walls = {
        "floor": (((-1, 0, 1), (1, 0, 1), (1, 0, -1), (-1, 0, -1)), floor),
        "ceiling": (((-1, 2, -1), (1, 2, -1), (1, 2, 1), (-1, 2, 1)), diffuse(rng.uniform(0.3, 0.7, 3))),
        "left": (((-1, 0, 1), (-1, 0, -1), (-1, 2, -1), (-1, 2, 1)), diffuse(rng.uniform(0.3, 0.7, 3))),
        "right": (((1, 0, -1), (1, 0, 1), (1, 2, 1), (1, 2, -1)), diffuse(rng.uniform(0.3, 0.7, 3))),
    }
    for name, (pts, rec) in walls.items():
        b.add(name, quad_tris(*[np.asarray(p, np.float32) for p in pts]), None, b.material(rec), uv=uv_quad)
    # bump-mapped back wall: seeded height field, 40 x 40 texels
    heights = rng.uniform(0, 1, (10, 10))
    heights = np.kron(heights, np.ones((4, 4)))
    bump = b.texture(Texture(np.repeat(heights[..., None], 3, 2).astype(np.float32), TEX_BUMP,
                             repeat_u=1.0, repeat_v=1.0, bump_intensity=3.0))
    back = diffuse(rng.uniform(0.4, 0.8, 3))
    back[13] = bump
    b.add("back", quad_tris(*[np.asarray(p, np.float32) for p in ((-1, 0, -1), (1, 0, -1), (1, 2, -1), (-1, 2, -1))]),
          None, b.material(back), uv=uv_quad)
    # Phong sphere with a ks map, dielectric sphere with a transparency map (uvs: Sphere::_getUV)
    noise = rng.uniform(0.1, 0.5, (8, 8, 3)).astype(np.float32)
    ks_tex = b.texture(Texture(noise, TEX_COLOR, filters))
    ph = phong((0.3, 0.3, 0.3), (0.4, 0.4, 0.4), 30.0)
    ph[11] = ks_tex
    tr_tex = b.texture(Texture(rng.uniform(0.2, 1.0, (6, 10, 3)).astype(np.float32), TEX_COLOR, filters,
                               repeat_u=2.0))
    di = dielectric(1.5)
    di[12] = tr_tex
    for name, center, r, rec in (("phongSphere", (-0.45, 0.35, -0.2), 0.35, ph),
                                 ("glassSphere", (0.45, 0.3, 0.3), 0.3, di)):
        tris, nrm = _uv_sphere_fast(center, r, 24, 13)
        d = (tris.reshape(-1, 3) - np.asarray(center, np.float32)) / r
        u = 1.0 - np.arctan2(d[:, 2], d[:, 0]) / (2 * np.pi)
        v = 0.5 - np.arcsin(np.clip(d[:, 1], -1, 1)) / np.pi
        uv = np.stack([u, v], -1).reshape(-1, 3, 2)
        # keep each triangle on one side of the seam (a lookup only uses the fractional part)
        span = uv[:, :, 0].max(1) - uv[:, :, 0].min(1)
        fix = (span > 0.5)[:, None] & (uv[:, :, 0] < 1.0)
        uv[:, :, 0] += fix
        b.add(name, tris, nrm, b.material(rec), uv=uv.astype(np.float32))
    lm = b.material(diffuse(0.0))
    b.add_quad_light("light", (0.0, 1.999, 0.0), (0.5, 0.0, 0.0), (0.0, 0.0, -0.5), 15.0, lm)
    cam = camera(eye=(0.0, 1.0, 3.75), look=(0.0, 0.0, -1.0), up=(0, 1, 0), height_angle=40.0, aspect=1.0)
    return b.build(cam, name="textured")


def _place_spheres(rng, n, rmin, rmax, half_extent, max_tries=200000):
    radii = np.exp(rng.uniform(np.log(rmin), np.log(rmax), n))
    radii = np.sort(radii)[::-1]
    centers = []
    placed_r = []
    for r in radii:
        for _ in range(max_tries):
            x = rng.uniform(-half_extent + r, half_extent - r)
            z = rng.uniform(-half_extent + r, half_extent - r)
            ok = True
            for (cx, cz), pr in zip(centers, placed_r):
                if (x - cx) ** 2 + (z - cz) ** 2 < (r + pr + 1e-3) ** 2:
                    ok = False
                    break
            if ok:
                centers.append((x, z))
                placed_r.append(r)
                break
        else:
            raise RuntimeError("could not place spheres without overlap")
    return [(x, r, z) for (x, z), r in zip(centers, placed_r)], placed_r


def mid(seed: int = 0, n_spheres: int = 400, nu: int = 50, nv: int = 26, n_lights: int = 4,
        ground: float = 20.0) -> Scene:
    rng = np.random.default_rng(seed)
    b = SceneBuilder()
    h = ground / 2
    gm = b.material(diffuse(rng.uniform(0.3, 0.7, 3)))
    b.add("ground", quad_tris(np.array((-h, 0, h), np.float32), np.array((h, 0, h), np.float32),
                              np.array((h, 0, -h), np.float32), np.array((-h, 0, -h), np.float32)), None, gm)
    centers, radii = _place_spheres(rng, n_spheres, 0.05, 1.0, h)
    for k, (c, r) in enumerate(zip(centers, radii)):
        u = rng.uniform()
        if u < 0.6:
            m = diffuse(rng.uniform(0.2, 0.8, 3))
        elif u < 0.9:
            kd = rng.uniform(0.05, 0.5, 3)
            ks = rng.uniform(0.1, 0.45, 3)
            m = phong(kd, ks, rng.uniform(10.0, 200.0))
        else:
            m = dielectric(1.5)
        tris, nrm = _uv_sphere_fast(c, r, nu, nv)
        b.add(f"sphere{k}", tris, nrm, b.material(m))
    lm = b.material(diffuse(0.0))
    # lights: 2 x 2 quads at height 8 over the four quadrants, facing down, radiance 10
    for i in range(n_lights):
        ang = 2 * np.pi * (i + 0.5) / n_lights
        cx, cz = 5.0 * np.cos(ang), 5.0 * np.sin(ang)
        b.add_quad_light(f"light{i}", (cx, 8.0, cz), (2.0, 0.0, 0.0), (0.0, 0.0, -2.0), 10.0, lm)
    cam = camera(eye=(0.0, 7.0, 17.0), focus=(0.0, 0.0, 0.0), up=(0, 1, 0), height_angle=40.0, aspect=1.0)
    return b.build(cam, name="mid")


def random_scene(seed: int, target_tris: int) -> Scene:
    """Spheres and boxes on a ground quad with one to four quad lights, about target_tris
    triangles (batched / serving workloads)."""
    rng = np.random.default_rng(seed)
    b = SceneBuilder()
    gm = b.material(diffuse(rng.uniform(0.3, 0.7, 3)))
    h = 10.0
    b.add("ground", quad_tris(np.array((-h, 0, h), np.float32), np.array((h, 0, h), np.float32),
                              np.array((h, 0, -h), np.float32), np.array((-h, 0, -h), np.float32)), None, gm)
    per_sphere = 2500
    n_sph = max(1, target_tris // per_sphere)
    nu = 50 if target_tris >= per_sphere else max(4, int(np.sqrt(target_tris / 2)))
    nv = 26 if target_tris >= per_sphere else max(3, nu // 2)
    if n_sph > 400:
        # 400 spheres fill the ground; beyond ~1M triangles they are tessellated finer
        # (a UV sphere of nu x nv has 2 nu (nv - 1) triangles, nu = 2 (nv - 1))
        nv = int(round(np.sqrt(target_tris / 400 / 4.0))) + 1
        nu = 2 * (nv - 1)
        n_sph = 400
    centers, radii = _place_spheres(rng, n_sph, 0.05, 1.0, h)
    for k, (c, r) in enumerate(zip(centers, radii)):
        u = rng.uniform()
        if u < 0.6:
            m = diffuse(rng.uniform(0.2, 0.8, 3))
        elif u < 0.9:
            m = phong(rng.uniform(0.05, 0.5, 3), rng.uniform(0.1, 0.45, 3), rng.uniform(10.0, 200.0))
        else:
            m = dielectric(1.5)
        tris, nrm = _uv_sphere_fast(c, r, nu, nv)
        b.add(f"sphere{k}", tris, nrm, b.material(m))
    for k in range(int(rng.integers(0, 4))):
        tris, nrm = box_tris((rng.uniform(-8, 8), 0.0, rng.uniform(-8, 8)), rng.uniform(0.3, 1.5, 3),
                             rng.uniform(-np.pi, np.pi))
        b.add(f"box{k}", tris, nrm, b.material(diffuse(rng.uniform(0.2, 0.8, 3))))
    lm = b.material(diffuse(0.0))
    nl = int(rng.integers(1, 5))
    for i in range(nl):
        ang = 2 * np.pi * (i + 0.5) / nl
        b.add_quad_light(f"light{i}", (5.0 * np.cos(ang), 8.0, 5.0 * np.sin(ang)), (2.0, 0.0, 0.0),
                         (0.0, 0.0, -2.0), 10.0, lm)
    cam = camera(eye=(0.0, 6.0, 15.0), focus=(0.0, 0.0, 0.0), height_angle=40.0, aspect=1.0)
    return b.build(cam, name=f"random{seed}")


def _fbm(x, z, rng, octaves: int = 7):
    """Fractional Brownian motion heights: a sum of octaves of randomly phased, randomly
    oriented sinusoid pairs, amplitude halving and frequency doubling per octave."""
    h = np.zeros(np.broadcast(x, z).shape, np.float64)
    amp, freq = 1.0, 0.05
    for _ in range(octaves):
        for _ in range(3):
            a = rng.uniform(0, 2 * np.pi)
            ph = rng.uniform(0, 2 * np.pi, 2)
            u = np.cos(a) * x + np.sin(a) * z
            w = -np.sin(a) * x + np.cos(a) * z
            h += amp * np.sin(freq * u * 2 * np.pi + ph[0]) * np.cos(freq * w * 2 * np.pi + ph[1]) / 3.0
        amp *= 0.5
        freq *= 2.0
    return h


def large(seed: int = 0, cells: int = 2800, n_objects: int = 2000, extent: float = 100.0, height: float = 6.0,
          obj_nu: int = 40, obj_nv: int = 28, n_lights: int = 16) -> Scene:
    rng = np.random.default_rng(seed)
    b = SceneBuilder()
    # terrain: (cells + 1)^2 vertices over [-extent/2, extent/2]^2, two triangles per cell
    g = np.linspace(-extent / 2, extent / 2, cells + 1)
    X, Z = np.meshgrid(g, g, indexing="ij")
    Y = height * _fbm(X, Z, rng)
    P = np.stack([X, Y, Z], -1)
    # vertex normals from central differences of the height field
    dx = extent / cells
    gy, gx = np.gradient(Y, dx, dx)
    N = np.stack([-gy, np.ones_like(Y), -gx], -1)
    N /= np.linalg.norm(N, axis=-1, keepdims=True)
    i, j = np.meshgrid(np.arange(cells), np.arange(cells), indexing="ij")
    a, bb, c, d = (i, j), (i + 1, j), (i + 1, j + 1), (i, j + 1)
    t1 = np.stack([P[a], P[d], P[c]], -2)
    n1 = np.stack([N[a], N[d], N[c]], -2)
    t2 = np.stack([P[a], P[c], P[bb]], -2)
    n2 = np.stack([N[a], N[c], N[bb]], -2)
    tv = np.stack([t1, t2], 2).reshape(-1, 3, 3).astype(np.float32)
    tn = np.stack([n1, n2], 2).reshape(-1, 3, 3).astype(np.float32)
    del t1, t2, n1, n2, P, N
    gm = b.material(diffuse(rng.uniform(0.3, 0.6, 3)))
    b.add("terrain", tv, tn, gm)
    del tv, tn
    # 2,000 copied objects (glossy or dielectric spheres) resting on the terrain
    def height_at(x, z):
        fi = (x + extent / 2) / dx
        fj = (z + extent / 2) / dx
        i0 = np.clip(np.floor(fi).astype(int), 0, cells - 1)
        j0 = np.clip(np.floor(fj).astype(int), 0, cells - 1)
        return Y[i0:i0 + 2, j0:j0 + 2].max()
    mats = [b.material(phong(rng.uniform(0.05, 0.4, 3), rng.uniform(0.2, 0.5, 3), rng.uniform(20, 300)))
            for _ in range(16)] + [b.material(dielectric(1.5))]
    placed = np.zeros((0, 3))
    for k in range(n_objects):
        for _ in range(1000):  # no two objects overlap
            r = float(np.exp(rng.uniform(np.log(0.3), np.log(1.5))))
            x, z = rng.uniform(-extent / 2 + 2, extent / 2 - 2, 2)
            if not len(placed) or np.all((placed[:, 0] - x) ** 2 + (placed[:, 1] - z) ** 2 > (placed[:, 2] + r) ** 2):
                break
        placed = np.vstack([placed, (x, z, r)])
        y = float(height_at(x, z)) + r
        m = mats[-1] if rng.uniform() < 0.3 else mats[int(rng.integers(16))]
        tris, nrm = _uv_sphere_fast((x, y, z), r, obj_nu, obj_nv)
        b.add(f"object{k}", tris, nrm, m)
    lm = b.material(diffuse(0.0))
    side = int(round(np.sqrt(n_lights)))
    for li in range(n_lights):
        cx = (li % side + 0.5) / side * extent * 0.8 - extent * 0.4
        cz = (li // side + 0.5) / side * extent * 0.8 - extent * 0.4
        b.add_quad_light(f"light{li}", (cx, 40.0, cz), (4.0, 0.0, 0.0), (0.0, 0.0, -4.0), 40.0, lm)
    cam = camera(eye=(0.0, 35.0, 75.0), focus=(0.0, 0.0, 0.0), height_angle=45.0, aspect=1.0)
    return b.build(cam, name="large")
