"""Helpers for the GPU parity tests (device buffers through torch; compute through libmgpu)."""
from __future__ import annotations

import numpy as np

from milton_gb300 import pathtracer as pt


def to_dev(torch, a: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def gpu_trace(torch, dscene, rays: np.ndarray, counts=False):
    r = to_dev(torch, rays.astype(np.float32))
    if counts:
        c = torch.zeros((rays.shape[0], 4), dtype=torch.int32, device="cuda")
        h = pt.trace_closest(dscene, r, counts=c)
        torch.cuda.synchronize()
        return h.cpu().numpy(), c.cpu().numpy().view(np.uint32)
    h = pt.trace_closest(dscene, r)
    torch.cuda.synchronize()
    return h.cpu().numpy(), None


def gpu_any(torch, dscene, rays: np.ndarray):
    occ = pt.trace_any(dscene, to_dev(torch, rays.astype(np.float32)))
    torch.cuda.synchronize()
    return occ.cpu().numpy()


def gpu_render_paths(torch, scene, settings: pt.RenderSettings, accel=None, dscene=None):
    """Renders and returns (film mean (h, w, 3), per-path radiance (h, w, samples, 3), flags)."""
    accel = accel or pt.Accel(scene)
    dscene = dscene or pt.DeviceScene(scene, accel)
    film = pt.Film(settings.width, settings.height)
    ns = settings.sample_count if settings.sample_count is not None else settings.spp - settings.sample_begin
    out = torch.zeros((settings.width * settings.height * ns, 4), dtype=torch.float32, device="cuda")
    pt.render(dscene, settings, film, path_out=out)
    torch.cuda.synchronize()
    o = out.cpu().numpy().reshape(settings.height, settings.width, ns, 4)
    return film.mean(), o[..., :3].astype(np.float64), o[..., 3].view(np.uint32)
