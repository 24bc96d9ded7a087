"""Image maps on the host: the oracle's texture lookup (Material::getSample with
KernelFilter::apply, the bump map of Material::_initShadingNormal) against an independent numpy
restatement, the PNG / PPM readers, and the scene loader's texture slots and uvs."""
import math
import struct
import zlib

import numpy as np
import pytest

from milton_gb300 import imageio
from milton_gb300 import scene as S
from milton_gb300 import sceneloader as L
from oracle import filters as F

KINDS = [("box", 2.0, {}), ("triangle", 2.0, {}), ("triangle", 4.0, {}), ("gaussian", 3.0, {"sigma": 0.7}),
         ("mitchell", 2.0, {"B": 0.5, "C": 0.25}), ("lanczosSinc", 3.0, {"tau": 2.0})]


def _np_lookup(tex: S.Texture, u: float, v: float) -> np.ndarray:
    """KernelFilter::apply at Material::getSample's texel, restated with numpy."""
    h, w, _ = tex.rgb.shape
    s, t = u * tex.repeat_u, v * tex.repeat_v
    x = int(math.floor(min(max((s - math.floor(s)) * w, 0.0), w - 1)))
    y = int(math.floor(min(max((t - math.floor(t)) * h, 0.0), h - 1)))
    kind, support, params = tex.filter
    kw = int(math.ceil(support)) | 1
    half = kw >> 1
    ker = np.array([[F.weight(kind, support, params, i - kw / 2.0, j - kw / 2.0) for j in range(kw)]
                    for i in range(kw)])
    rows = np.clip(np.arange(-half, half + 1) + y, 0, h - 1)
    cols = np.clip(np.arange(-half, half + 1) + x, 0, w - 1)
    win = tex.rgb.astype(np.float64)[np.ix_(rows, cols)]
    return (win * ker[..., None]).sum((0, 1)) / ker.sum()


@pytest.mark.parametrize("flt", KINDS, ids=lambda f: f"{f[0]}-{f[1]}")
def test_oracle_lookup_matches_numpy(oracle, flt):
    rng = np.random.default_rng(7)
    tex = S.Texture(rng.random((9, 13, 3)).astype(np.float32), S.TEX_COLOR, flt, repeat_u=2.5, repeat_v=1.5)
    for u, v in list(rng.uniform(-2, 2, (40, 2))) + [(0.0, 0.0), (0.9999, 0.9999), (1.0, 1.0), (0.4, 1e-9)]:
        # the filter parameters cross the C boundary as float32
        assert np.allclose(oracle.texture_lookup(tex, u, v), _np_lookup(tex, u, v), rtol=1e-6, atol=1e-9)


def test_triangle_kernel_is_sampled_half_a_texel_off(oracle):
    # KernelFilter::_computeKernel evaluates at i - width / 2: for the default triangle filter
    # (support 2, width 3) the weights are (2.5, 1.5, 0.5) per axis, favouring the upper left
    img = np.zeros((5, 5, 3), np.float32)
    img[1, 1] = 1.0  # one lit texel up and left of the centre texel (2, 2)
    tex = S.Texture(img)
    got = oracle.texture_lookup(tex, 2.5 / 5, 2.5 / 5)
    assert np.allclose(got, 2.5 * 2.5 / 4.5 ** 2)


def test_oracle_bump_normal(oracle):
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, (6, 7, 3)).astype(np.float32) / 255
    tex = S.Texture(img, S.TEX_BUMP, bump_intensity=2.0)
    lum = img @ np.array([0.2126, 0.7152, 0.0722])
    for (x, y) in [(0, 0), (3, 2), (6, 5), (6, 0)]:
        gx = lum[y, x - (x > 0)] - lum[y, x + (x < 6)]
        gy = lum[y - (y > 0), x] - lum[y + (y < 5), x]
        n = np.array([0.3, 0.8, -0.2])
        n /= np.linalg.norm(n)
        r = oracle.texture_lookup(tex, (x + 0.5) / 7, (y + 0.5) / 6, normal=n)
        assert np.allclose(r[:2], (gx, gy), atol=1e-12)
        up = np.array([0.0, 1.0, 0.0]) if abs(n[1]) <= 0.8 else np.array([1.0, 0.0, 0.0])
        U = np.cross(up, n)
        U /= np.linalg.norm(U)
        V = np.cross(n, U)
        want = n + 2.0 * (gx * U + gy * V)
        assert np.allclose(r[2:], want / np.linalg.norm(want), atol=1e-12)
    flat = S.Texture(np.full((4, 4, 3), 0.5, np.float32), S.TEX_BUMP)
    assert np.allclose(oracle.texture_lookup(flat, 0.3, 0.6, normal=[0, 0, 1])[2:], [0, 0, 1])


# --- image files ---------------------------------------------------------------------------

def _png(rows: np.ndarray, ctype: int, filters, plte=None) -> bytes:
    """Encodes 8-bit rows (H, W*channels) with the given per-row filter types."""
    h, stride = rows.shape
    bpp = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    raw = bytearray()
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        cur = rows[y].astype(np.int32)
        f = filters[y % len(filters)]
        a = np.concatenate([np.zeros(bpp, np.int32), cur[:-bpp]])
        c = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        b = prev
        if f == 0:
            p = np.zeros(stride, np.int32)
        elif f == 1:
            p = a
        elif f == 2:
            p = b
        elif f == 3:
            p = (a + b) // 2
        else:
            pa, pb, pc = np.abs(b - c), np.abs(a - c), np.abs(a + b - 2 * c)
            p = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
        raw += bytes([f]) + ((cur - p) & 0xFF).astype(np.uint8).tobytes()
        prev = cur
    w = stride // bpp

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)
    out = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
    if plte is not None:
        out += chunk(b"PLTE", plte.astype(np.uint8).tobytes())
    return out + chunk(b"IDAT", zlib.compress(bytes(raw))) + chunk(b"IEND", b"")


@pytest.mark.parametrize("ctype", [0, 2, 3, 4, 6])
def test_png_colour_types_and_filters(tmp_path, ctype):
    rng = np.random.default_rng(ctype)
    h, w = 7, 9
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    px = rng.integers(0, 256 if ctype != 3 else 5, (h, w, ch)).astype(np.uint8)
    plte = rng.integers(0, 256, (5, 3)) if ctype == 3 else None
    p = tmp_path / "t.png"
    p.write_bytes(_png(px.reshape(h, w * ch), ctype, [0, 1, 2, 3, 4], plte))
    rgb = imageio.read_png(str(p), rgb=True)
    want = {0: np.repeat(px, 3, 2), 2: px, 3: None if plte is None else plte[px[..., 0]],
            4: np.repeat(px[..., :1], 3, 2), 6: px[..., :3]}[ctype]
    assert rgb.dtype == np.uint8 and np.array_equal(rgb, want)
    assert np.allclose(imageio.read_image(str(p)), want / 255.0)


def test_pnm_reader(tmp_path):
    rng = np.random.default_rng(1)
    px = rng.integers(0, 256, (4, 5, 3)).astype(np.uint8)
    (tmp_path / "a.ppm").write_bytes(b"P6\n# comment\n5 4\n255\n" + px.tobytes())
    assert np.array_equal(imageio.read_pnm(str(tmp_path / "a.ppm")), px)
    g = px[..., 0]
    (tmp_path / "b.pgm").write_text("P2 5 4 255\n" + " ".join(str(int(x)) for x in g.reshape(-1)))
    assert np.array_equal(imageio.read_pnm(str(tmp_path / "b.pgm")), np.repeat(g[..., None], 3, 2))
    with pytest.raises(ValueError):
        imageio.read_image(str(tmp_path / "c.jpg"))


# --- scene loader ----------------------------------------------------------------------------

def _scene(body: str) -> str:
    return '{ "scenefile" : { "scene" : { ' + body + ' } } }'


def test_loader_texture_slots_filter_and_uvs(tmp_path):
    rng = np.random.default_rng(5)
    img = rng.integers(0, 256, (3, 4, 3)).astype(np.uint8)
    (tmp_path / "kd.ppm").write_bytes(b"P6 4 3 255\n" + img.tobytes())
    (tmp_path / "bump.ppm").write_bytes(b"P6 4 3 255\n" + img[::-1].tobytes())
    text = _scene('"material" : { "repeatU" : 2.0, "bumpMap" : "bump.ppm", "bumpIntensity" : 0.5, '
                  '"filter" : { "type" : "gaussian", "support" : 3, "sigma" : 0.5 }, '
                  '"bsdf" : { "type" : "diffuse", "kd" : "kd.ppm" }, '
                  '"plane" : { }, "triangle" : { "vertices" : [0,0,0, 1,0,0, 0,0,1], "uvs" : [0,0, 1,0, 0,1] }, '
                  '"cube" : { } }, '
                  '"material" : { "bsdf" : { "type" : "phong", "ks" : "kd.ppm", "n" : 10 }, "triangle" : { } }, '
                  '"material" : { "bsdf" : { "type" : "dielectric", "transparency" : "missing.ppm" }, '
                  '"triangle" : { } }')
    with pytest.warns(UserWarning, match="missing.ppm"):
        sf = L.loads(text, base_dir=str(tmp_path))
    s = sf.scene
    assert len(s.textures) == 3
    kd, bump, ks = s.textures
    assert np.allclose(kd.rgb, img / 255.0) and kd.kind == S.TEX_COLOR
    assert kd.filter == ("gaussian", 3.0, {"sigma": 0.5}) and (kd.repeat_u, kd.repeat_v) == (2.0, 1.0)
    assert bump.kind == S.TEX_BUMP and bump.bump_intensity == 0.5
    assert ks.filter == ("triangle", 2.0, {}) and ks.repeat_u == 1.0  # the default filter
    m0 = s.materials[s.tri_mat[0]]
    assert tuple(m0[10:14]) == (1, 0, 0, 2)
    m_ph = s.materials[s.tri_mat[-2]]
    assert tuple(m_ph[10:14]) == (0, 3, 0, 0)
    m_di = s.materials[s.tri_mat[-1]]
    assert tuple(m_di[10:14]) == (0, 0, 0, 0) and m_di[9] == np.float32(0.7)  # failed image: 0.7
    # shapes in key order: cube (triangles 0-11), plane (12, 13), triangle (14)
    # unit plane: (x + 1/2, z + 1/2) of the object-space corners
    for k in (12, 13):
        for c in range(3):
            p = s.tri_v[k, c]
            assert np.allclose(s.tri_uv[k, c], (p[0] + 0.5, p[2] + 0.5))
    assert np.allclose(s.tri_uv[14], [(0, 0), (1, 0), (0, 1)])  # the triangle's own uvs
    # cube: Cube::_getUV of each corner's world position (here the object space)
    for t in range(12):
        n = np.cross(s.tri_v[t, 1] - s.tri_v[t, 0], s.tri_v[t, 2] - s.tri_v[t, 0])
        axis = int(np.argmax(np.abs(n)))
        case = axis if n[axis] > 0 else 4 + axis
        for c in range(3):
            P = s.tri_v[t, c].astype(np.float64)
            side = case & 3
            v = P[(side + 1) % 3] + 0.5
            u = P[(side + 2) % 3] + 0.5
            if side == 2:
                u, v = 1 - v, u
            if case & 4:
                v = 1 - v
            if not case & 5:
                u, v = 1 - u, 1 - v
            assert np.allclose(s.tri_uv[t, c], (u, v)), (t, c)


def test_obj_texture_coordinates_of_the_first_vertex(tmp_path):
    (tmp_path / "q.obj").write_text("v 0 0 0\nv 1 0 0\nv 1 0 1\nv 0 0 1\nvt 0.1 0.2\nvt 0.3 0.4\nvt 0.5 0.6\n"
                                    "vn 0 1 0\nf 1/2/1 2/1/1 3/3/1 4/1/1\nf 1//1 3//1 4//1\n")
    v, f, n, nf, uv = L.load_mesh(str(tmp_path / "q.obj"), with_uv=True)
    # Mesh::_getUV takes the first vertex's texture index for the whole triangle; faces without
    # texture indices use index 0
    assert np.allclose(uv, [(0.3, 0.4), (0.3, 0.4), (0.1, 0.2)])
    (tmp_path / "t.png").write_bytes(imageio.png_bytes(np.full((2, 2, 4), 200, np.uint8)))
    sf = L.loads(_scene('"material" : { "bsdf" : { "type" : "diffuse", "kd" : "t.png" }, '
                        '"mesh" : { "path" : "q.obj" } }'), base_dir=str(tmp_path))
    assert np.allclose(sf.scene.tri_uv, np.repeat(uv[:, None, :], 3, 1))
    assert np.allclose(sf.scene.textures[0].rgb, 200 / 255.0)


def test_untextured_scene_has_no_uvs():
    sf = L.loads(_scene('"triangle" : { }'))
    assert sf.scene.tri_uv is None and sf.scene.textures == []


def test_bump_mapped_emitter_refused(tmp_path):
    (tmp_path / "b.ppm").write_bytes(b"P6 1 1 255\n\x10\x20\x30")
    with pytest.raises(L.SceneFileError, match="bump-mapped emitter"):
        L.loads(_scene('"material" : { "bumpMap" : "b.ppm", "emitter" : { "type" : "oriented" }, "plane" : { } }'),
                base_dir=str(tmp_path))


# --- backgrounds ---------------------------------------------------------------------------------

def _rgbe_bytes(img: np.ndarray, rle_rows=()) -> bytes:
    """Radiance RGBE encoding of (H, W, 3) floats; rows in rle_rows as new-style RLE scanlines
    (one literal run and one repeat run per channel), the others flat."""
    h, w, _ = img.shape
    m = img.max(axis=2)
    mant, ex = np.frexp(m)
    scale = np.where(m > 1e-32, mant * 256.0 / np.where(m > 0, m, 1), 0.0)
    px = np.zeros((h, w, 4), np.uint8)
    px[..., :3] = np.clip(img * scale[..., None], 0, 255).astype(np.uint8)
    px[..., 3] = np.where(m > 1e-32, ex + 128, 0).astype(np.uint8)
    out = bytearray(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n" + f"-Y {h} +X {w}\n".encode())
    for y in range(h):
        if y in rle_rows:
            out += bytes([2, 2, w >> 8, w & 0xFF])
            for c in range(4):
                lit = px[y, : w // 2, c]
                out += bytes([len(lit)]) + lit.tobytes()
                rest = px[y, w // 2:, c]
                px[y, w // 2:, c] = rest[0]  # the repeat run carries the first value
                out += bytes([128 + len(rest), int(rest[0])])
        else:
            out += px[y].tobytes()
    return bytes(out), px


def test_hdr_reader(tmp_path):
    rng = np.random.default_rng(2)
    img = (rng.random((5, 12, 3)) * 20).astype(np.float32)
    img[1, 3] = 0.0
    # a scanline that does not start with the RLE marker makes the rest of the file flat pixels
    # (rgbe.cpp's RGBE_ReadPixels_RLE), so files are all flat or all run-length encoded
    for name, rows in (("flat.hdr", ()), ("rle.hdr", range(5))):
        data, px = _rgbe_bytes(img, rle_rows=rows)
        (tmp_path / name).write_bytes(data)
        got = imageio.read_image(str(tmp_path / name))
        e = px[..., 3].astype(np.int64)
        want = np.where(e[..., None] > 0, px[..., :3] * np.ldexp(1.0, e - 136)[..., None], 0.0)
        assert got.shape == (5, 12, 3) and np.array_equal(got, want.astype(np.float32)), name
        if not rows:
            # 8-bit mantissas with a shared exponent: error below max(r, g, b) / 128
            assert np.all(np.abs(got - img) <= img.max(axis=2, keepdims=True) / 128 + 1e-6)


def _np_env_uv(d):
    w = -np.asarray(d, np.float64)
    rho, mag = math.hypot(w[0], w[2]), np.linalg.norm(w)
    theta = math.acos(rho / mag) * (1 if w[1] >= 0 else -1) if rho < abs(w[1]) else math.asin(w[1] / mag)
    phi = 0.0 if (w[0] == 0 and w[2] == 0) else math.atan2(w[0], w[2])
    return phi / (-2 * math.pi) + 0.5, theta / -math.pi + 0.5


def test_oracle_background(oracle):
    rng = np.random.default_rng(4)
    env = S.Texture(rng.random((16, 32, 3)).astype(np.float32) * 3)
    for d in list(rng.normal(size=(30, 3))) + [np.array([0.0, 1.0, 0.0]), np.array([0.0, -1.0, 0.0])]:
        d = d / np.linalg.norm(d)
        u, v = _np_env_uv(d)
        assert np.allclose(oracle.background(d, env), _np_lookup(env, u, v), rtol=1e-6, atol=1e-9)
    assert np.allclose(oracle.background([0, 0, 1], le=(0.5, 1.0, 2.0)), (0.5, 1.0, 2.0))


def test_loader_background(tmp_path):
    (tmp_path / "sky.ppm").write_bytes(b"P6 2 1 255\n\x10\x20\x30\x40\x50\x60")
    sf = L.loads(_scene('"background" : { "emitter" : { "type" : "environment", "path" : "sky.ppm" } }, '
                        '"triangle" : { }'), base_dir=str(tmp_path))
    s = sf.scene
    assert s.background_tex == 1 and s.textures[0].filter == ("triangle", 2.0, {})
    assert np.allclose(s.textures[0].rgb[0, 1], np.array([0x40, 0x50, 0x60]) / 255)
    sf = L.loads(_scene('"background" : { "emitter" : { "type" : "omni", "power" : [1, 2, 4] } }, "triangle" : { }'))
    assert sf.scene.background_tex == 0 and np.allclose(sf.scene.background_le, np.array([1, 2, 4]) / (4 * math.pi))
    assert np.all(L.loads(_scene('"background" : { }, "triangle" : { }')).scene.background_le == 0)
    with pytest.warns(UserWarning, match="nope.hdr"), pytest.raises(L.SceneFileError, match="failed to load environment"):
        L.loads(_scene('"background" : { "emitter" : { "type" : "environment", "path" : "nope.hdr" } }'))
    with pytest.raises(L.SceneFileError, match="must contain a 'path'"):
        L.loads(_scene('"background" : { "emitter" : { "type" : "environment" } }'))
    with pytest.raises(L.SceneFileError, match="at most one background"):
        L.loads(_scene('"background" : { }, "background" : { }'))
    with pytest.raises(L.SceneFileError, match="exactly one child emitter"):
        L.loads(_scene('"background" : { "emitter" : { "type" : "null" }, "x" : 1 }'))
    with pytest.raises(L.SceneFileError, match="oriented background"):
        L.loads(_scene('"background" : { "emitter" : { "type" : "oriented" } }'))
