"""FP64 restatement of Milton's Reinhard tone map (test infrastructure: the checker of
mgpu_film_tonemap, never used by the product).

ReinhardToneMap::map, mlt/src/milton/renderers/tonemaps/ReinhardToneMap.cpp:25-94, with the
sRGB <-> XYZ matrices of mlt/src/milton/utils/ColorUtils.cpp:115-133 and the CLAMP macro of
mlt/src/milton/common/utilities.h:195-200; pixels visited in the reference's reverse order for
the key's log sum.  A NaN channel (an all-black pixel's chromaticity is 0/0) converts to 0.
"""
from __future__ import annotations

import numpy as np

RGB_TO_XYZ = np.array([[0.41245322014416, 0.35757958129350, 0.18042258997054],
                       [0.21267112134122, 0.71515920531078, 0.07216877677613],
                       [0.01933381646199, 0.11919354020663, 0.95022692228971]])
XYZ_TO_RGB = np.array([[3.240479, -1.537150, -0.498535],
                       [-0.969256, 1.875992, 0.041556],
                       [0.055648, -0.204043, 1.057311]])
EPSILON = 1e-7


def reinhard(mean_rgb: np.ndarray) -> np.ndarray:
    """(H, W, 3) radiance means -> (H, W, 4) uint8 RGBA."""
    img = np.asarray(mean_rgb, np.float64)
    h, w, _ = img.shape
    xyz = img.reshape(-1, 3) @ RGB_TO_XYZ.T
    with np.errstate(invalid="ignore", divide="ignore"):
        s = xyz.sum(1)
        cx, cy, Y = xyz[:, 0] / s, xyz[:, 1] / s, xyz[:, 1]
    key = 0.0
    for v in np.log(EPSILON + Y)[::-1]:
        key += v
    key = np.exp(key / Y.shape[0])
    ymax = max(0.0, float(Y.max())) if Y.size else 0.0
    white = 0.0 if ymax <= 0 else 1.0 / (ymax * ymax)
    scale = 0.0 if key <= 0 else 0.18 / key
    lum = scale * Y
    Yd = lum * (1.0 + lum * white) / (1.0 + lum)
    with np.errstate(invalid="ignore", divide="ignore"):
        Xd = Yd * cx / cy
        Zd = Yd * (1.0 - cx - cy) / cy
        rgb = np.stack([Xd, Yd, Zd], 1) @ XYZ_TO_RGB.T
        rgb = 255.0 * np.power(rgb, 1.0 / 2.22)
    out = np.where(rgb >= 255, 255.0, np.where(rgb <= 0, 0.0, rgb))
    out = np.where(np.isnan(out), 0.0, out)
    rgba = np.full((h * w, 4), 255, np.uint8)
    rgba[:, :3] = out.astype(np.uint8)
    return rgba.reshape(h, w, 4)
