"""FP64 restatement of Milton's reconstruction splat (test infrastructure: the checker of the
film's filtered output, never used by the product).

ReconstructionRenderOutput::addSample (mlt/src/milton/renderers/outputs/
ReconstructionRenderOutput.cpp:30-83) with the kernel filters of mlt/src/milton/filters/
(BoxFilter.cpp, TriangleFilter.cpp, GaussianFilter.cpp, MitchellFilter.cpp, LanczosSincFilter.cpp;
widths from KernelFilter.h:28).  Sample film positions are the jittered strata the renderers
draw (counter RNG, depth 0xFFFF): the oracle's uniforms reproduce them.
"""
from __future__ import annotations

import math

import numpy as np

EPSILON = 1e-7


def weight(kind, support, params, dx, dy):
    if kind == "box":
        return 1.0 if 2.0 * math.sqrt(dx * dx + dy * dy) < support else 0.0
    if kind == "triangle":
        r = support / 2.0
        return max(0.0, 1.0 - dx / r) * max(0.0, 1.0 - dy / r)
    if kind == "gaussian":
        s = params.get("sigma", 1.0)
        return max(0.0, (1.0 / (math.sqrt(2 * math.pi) * s)) * math.exp(-0.5 / (s * s) * (dx * dx + dy * dy)))
    if kind == "mitchell":
        B, C = params.get("B", 1 / 3), params.get("C", 1 / 3)

        def m(x):
            x = abs(2.0 * x / support)
            if x > 1.0:
                return (((-B / 6 - C) * x + (B + 5 * C)) * x + (-2 * B - 8 * C)) * x + (4.0 / 3.0 * B + 4 * C)
            return x * x * ((2 - 1.5 * B - C) * x + (-3 + 2 * B + C)) + (1 - B / 3)
        return m(dx) * m(dy)
    if kind == "lanczosSinc":
        tau = params.get("tau", 3.0)

        def l(x):
            x = abs(x / support)
            if x < EPSILON:
                return 1.0
            if x > 1:
                return 0.0
            x *= math.pi
            return math.sin(x * tau) / (x * tau) * math.sin(x) / x
        return l(dx) * l(dy)
    raise ValueError(kind)


def splat(paths_rgb, spp, sample_begin, seed, stream, kind, support, params, uniforms):
    """paths_rgb: (H, W, S, 3) radiance of samples sample_begin .. sample_begin + S - 1;
    uniforms(seed, stream, path, depth, block) -> 4 uniforms.  Returns the filtered (H, W, 3)."""
    h, w, ns, _ = paths_rgb.shape
    side = max(1, int(math.sqrt(spp)))
    s2 = side * side
    half = (int(math.ceil(support)) | 1) >> 1
    num = np.zeros((h, w, 3))
    den = np.zeros((h, w))
    for y in range(h):
        for x in range(w):
            pix = y * w + x
            for si in range(ns):
                s = sample_begin + si
                k = s % s2
                j = uniforms(seed, stream, pix * s2 + k, 0xFFFF, 0)
                cx = x + ((k % side) + j[0]) / side
                cy = y + ((k // side) + j[1]) / side
                for yy in range(max(0, y - half), min(h - 1, y + half) + 1):
                    for xx in range(max(0, x - half), min(w - 1, x + half) + 1):
                        wt = weight(kind, support, params, xx - cx, yy - cy)
                        if wt > 0:
                            num[yy, xx] += wt * paths_rgb[y, x, si]
                            den[yy, xx] += wt
    return np.where(den[..., None] > 0, num / np.maximum(den, 1e-300)[..., None], 0.0)
