"""Autotuner for the wavefront renderer: picks the wave size (paths in flight, i.e. queue
capacity), the traversal kernel shape (grid-stride or persistent warps), queue binning and the
traversal block size by timing a short calibration render of the actual requests (wave size x
shape first, then the block size of the best), and caches the choice per workload size class.  Results never depend on these knobs (every path draws its own counter-based random
numbers and each film sums its samples in sample order), only speed does."""
from __future__ import annotations

import itertools
import math

from . import pathtracer as pt

WAVES = (1 << 21, 1 << 22, 1 << 23, 1 << 24, 1 << 25, 1 << 26)
SHAPES = ((0, 1, 1), (0, 1, 0), (0, 0, 1), (1, 1, 1), (0, 0, 0))  # (persistent, bin_shadow, bin_extension)
BLOCKS = (64, 128, 256)  # threads per traversal block (grid-stride shapes)

_cache: dict = {}


def _size_class(requests) -> tuple:
    paths = sum(st.width * st.height for _, st in requests)
    tris = sum(ds.scene.ntri for ds, _ in requests)
    return (int(math.log2(max(paths, 1))), int(math.log2(max(tris, 1))))


def tune(requests, stream=None, calib_samples: int = 4, waves=WAVES, shapes=SHAPES, blocks=BLOCKS) -> dict:
    """requests: list of (DeviceScene, RenderSettings).  Returns {"wave_paths", "persistent",
    "bin_shadow", "bin_extension", "trav_block", "ms"} for the fastest calibration render and
    applies the kernel-shape knobs process-wide."""
    key = _size_class(requests)
    if key in _cache:
        best = _cache[key]
        _apply(best)
        return best
    films = [pt.Film(st.width, st.height) for _, st in requests]
    best = None
    for wave, shape in itertools.product(waves, shapes):
        cfg = {"persistent": shape[0], "bin_shadow": shape[1], "bin_extension": shape[2], "trav_block": 256}
        ms = _time(requests, films, wave, cfg, stream, calib_samples)
        if ms is not None and (best is None or ms < best["ms"]):
            best = {"wave_paths": wave, **cfg, "ms": ms}
    if best is not None and not best["persistent"]:
        for blk in blocks:
            if blk == 256:
                continue
            cfg = {k: best[k] for k in ("persistent", "bin_shadow", "bin_extension")}
            cfg["trav_block"] = blk
            ms = _time(requests, films, best["wave_paths"], cfg, stream, calib_samples)
            if ms is not None and ms < best["ms"]:
                best = {"wave_paths": best["wave_paths"], **cfg, "ms": ms}
    for f in films:
        f.close()
    _cache[key] = best
    _apply(best)
    return best


def _time(requests, films, wave, cfg, stream, calib_samples):
    """ms of one calibration batch (after a warm-up one), or None if its workspace does not fit."""
    import torch
    _apply(cfg)
    b = pt.Batch(wave_paths=wave, use_graph=True)
    for (ds, st), f in zip(requests, films):
        c = pt.RenderSettings(st.width, st.height, st.spp, sample_begin=0, sample_count=min(calib_samples, st.spp),
                              max_depth=st.max_depth or 8, rr_start_depth=st.rr_start_depth, seed=st.seed)
        b.add(ds, c, f)
    try:
        b.render(stream)  # warm
        torch.cuda.synchronize()
    except pt.N.MgpuError:  # a wave whose workspace does not fit the device: skip it
        b.close()
        return None
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    b.render(stream)
    e1.record()
    torch.cuda.synchronize()
    b.close()
    return e0.elapsed_time(e1)


def _apply(cfg: dict) -> None:
    for k in ("persistent", "bin_shadow", "bin_extension", "trav_block"):
        pt.tune(k, int(cfg.get(k, 256 if k == "trav_block" else 0)))
