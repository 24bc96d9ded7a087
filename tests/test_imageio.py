"""PNG output of tone-mapped films and the tone map's host model (CPU)."""
import numpy as np

from milton_gb300 import imageio
from oracle import tonemap


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (7, 5, 4), dtype=np.uint8)
    p = tmp_path / "x.png"
    imageio.write_png(str(p), img)
    assert np.array_equal(imageio.read_png(str(p)), img)


def test_reinhard_gray_and_black():
    # a uniform gray image maps every pixel to the same value; its luminance is the key,
    # so L = 0.18 and, with white = 1 / g^2, Y' = 0.18 (1 + 0.18 / g^2) / 1.18
    g = 0.4
    out = tonemap.reinhard(np.full((4, 4, 3), g))
    y = 0.18 * (1 + 0.18 / (g * g)) / 1.18
    expect = int(255 * y ** (1 / 2.22))  # gray stays gray (D65 white point), within rounding
    assert np.all(np.abs(out[..., :3].astype(int) - expect) <= 1) and np.all(out[..., 3] == 255)
    # black pixels (0/0 chromaticity) become 0, as the reference's NaN conversion does
    img = np.full((2, 2, 3), 0.3)
    img[0, 0] = 0
    out = tonemap.reinhard(img)
    assert out[0, 0, :3].tolist() == [0, 0, 0] and out[1, 1, 0] > 0
