"""Writes the image maps tests/scenes/textures.js uses (seeded, procedural):
checker.png (24 x 16 RGBA checker), bumps.ppm (32 x 32 grey height steps) and sky.hdr
(32 x 16 Radiance RGBE latitude-longitude environment: a bright band over a gradient).

    python tests/scenes/make_textures.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
from milton_gb300 import imageio  # noqa: E402


def main():
    rng = np.random.default_rng(2024)
    cells = (np.add.outer(np.arange(16) // 4, np.arange(24) // 4) % 2).astype(bool)
    a, b = rng.integers(30, 110, 3), rng.integers(150, 240, 3)
    rgba = np.full((16, 24, 4), 255, np.uint8)
    rgba[..., :3] = np.where(cells[..., None], b, a)
    (HERE / "checker.png").write_bytes(imageio.png_bytes(rgba))
    steps = np.kron(rng.integers(0, 256, (8, 8)), np.ones((4, 4), np.int64)).astype(np.uint8)
    (HERE / "bumps.ppm").write_bytes(b"P6\n32 32\n255\n" + np.repeat(steps[..., None], 3, 2).tobytes())
    v = (np.arange(16) + 0.5) / 16
    sky = np.zeros((16, 32, 3))
    sky[...] = (0.2 + 0.6 * (1 - v))[:, None, None] * np.array([0.5, 0.7, 1.0])
    sky[4:6, 8:14] = (6.0, 5.5, 4.0)  # a sun-like band above the horizon
    sky += rng.uniform(0, 0.05, sky.shape)
    m = sky.max(axis=2)
    mant, ex = np.frexp(m)
    px = np.zeros((16, 32, 4), np.uint8)
    px[..., :3] = (sky * (mant * 256.0 / m)[..., None]).astype(np.uint8)
    px[..., 3] = (ex + 128).astype(np.uint8)
    (HERE / "sky.hdr").write_bytes(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 16 +X 32\n" + px.tobytes())


if __name__ == "__main__":
    main()
