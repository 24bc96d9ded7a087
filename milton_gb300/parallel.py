"""Multi-GPU rendering as replicas: sample passes split across ranks, one film reduction.

Paths are independent, so ranks never exchange data while they render.  A job's spp passes are
split into contiguous ranges (one per rank, `pass_range`); each rank renders its range into its
own compensated film, and the one collective of the job adds the films at the end
(`reduce_films`): per pixel the Kahan-corrected rgb sums (sum - compensation, in FP64) and the
sample counts, then mean = sum / count -- the same per-pixel mean a single film over all passes
holds (ProgressiveFilterValue, mlt/src/milton/filters/ProgressiveFilterValue.h:18-38).
"""
from __future__ import annotations

import numpy as np


def pass_range(spp: int, world: int, rank: int) -> tuple[int, int]:
    """(sample_begin, sample_count) of rank's contiguous share of spp passes."""
    if not (0 <= rank < world) or world <= 0:
        raise ValueError("rank must be in [0, world)")
    lo = spp * rank // world
    hi = spp * (rank + 1) // world
    return lo, hi - lo


def film_partials(raw: np.ndarray) -> np.ndarray:
    """Raw film (2, H, W, 4) float32 -> (H, W, 4) float64: corrected rgb sums and count."""
    raw = np.asarray(raw)
    s, c = raw[0].astype(np.float64), raw[1].astype(np.float64)
    out = np.empty(s.shape, np.float64)
    out[..., :3] = s[..., :3] - c[..., :3]
    out[..., 3] = s[..., 3]
    return out


def reduce_films(raw: np.ndarray, group=None) -> np.ndarray:
    """Sum every rank's film partials (torch.distributed all_reduce) and return the per-pixel
    mean (H, W, 3) float64 on every rank.  Works with gloo (CPU) and NCCL (device) groups."""
    import torch
    import torch.distributed as dist
    part = torch.from_numpy(film_partials(raw))
    if dist.is_available() and dist.is_initialized():
        backend = dist.get_backend(group)
        if backend == "nccl":
            part = part.cuda()
        dist.all_reduce(part, op=dist.ReduceOp.SUM, group=group)
        part = part.cpu()
    p = part.numpy()
    cnt = p[..., 3:4]
    return np.where(cnt > 0, p[..., :3] / np.maximum(cnt, 1.0), 0.0)


def kahan_film(paths_rgb: np.ndarray) -> np.ndarray:
    """Host model of the device film: Kahan-add per-path radiance (H, W, S, 3) in FP32 sample
    order, as k_accumulate does, with the plain FP32 sum of squared luminance (r+g+b)/3;
    returns the raw (2, H, W, 4) float32 film."""
    h, w, n, _ = paths_rgb.shape
    S = np.zeros((h, w, 3), np.float32)
    C = np.zeros((h, w, 3), np.float32)
    Q = np.zeros((h, w), np.float32)
    third = np.float32(1.0 / 3.0)
    for k in range(n):
        L = paths_rgb[:, :, k, :].astype(np.float32)
        y = L - C
        t = (S + y).astype(np.float32)
        C = ((t - S).astype(np.float32) - y).astype(np.float32)
        S = t
        lum = (((L[..., 0] + L[..., 1]).astype(np.float32) + L[..., 2]).astype(np.float32) * third).astype(np.float32)
        Q = (Q + (lum * lum).astype(np.float32)).astype(np.float32)
    raw = np.zeros((2, h, w, 4), np.float32)
    raw[0, ..., :3] = S
    raw[0, ..., 3] = n
    raw[1, ..., :3] = C
    raw[1, ..., 3] = Q
    return raw
