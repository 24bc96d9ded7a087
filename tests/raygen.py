"""Seeded ray batches for parity tests: camera rays and uniform-sphere rays."""
from __future__ import annotations

import numpy as np


def camera_rays(camera: np.ndarray, n: int, seed: int = 0) -> np.ndarray:
    """n pinhole-camera rays through uniform random film points (ThinLensCamera::getWorldRay)."""
    rng = np.random.default_rng(seed)
    c = np.asarray(camera, np.float64)
    eye, look, up = c[0:3], c[3:6], c[6:9]
    nn = -look / np.linalg.norm(look)
    u = np.cross(up, nn); u /= np.linalg.norm(u)
    v = np.cross(nn, u)
    th = np.tan(np.radians(c[9]) / 2); tw = c[10] * th
    x, y = rng.random(n), rng.random(n)
    d = (tw * (2 * x - 1))[:, None] * u + (th * (1 - 2 * y))[:, None] * v - nn
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = eye
    r[:, 3] = 0.0
    r[:, 4:7] = d
    r[:, 7] = np.inf
    return r


def sphere_rays(lo, hi, n: int, seed: int = 1) -> np.ndarray:
    """Origins uniform in the box [lo, hi], directions uniform on the unit sphere."""
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    o = lo + (hi - lo) * rng.random((n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = o
    r[:, 4:7] = d
    r[:, 7] = np.inf
    # normalise in float32 so the ray the oracle sees is the ray the GPU sees
    dd = r[:, 4:7].astype(np.float64)
    r[:, 4:7] = (dd / np.linalg.norm(dd, axis=1, keepdims=True)).astype(np.float32)
    return r


def classify(prim_ref, t_ref, t2_ref, prim_gpu, t_gpu, rel_tie=1e-6):
    """Compare closest-hit ids.  A mismatch is a reported tie when the reference's two nearest
    hits lie within rel_tie relative t, or the GPU's t is within rel_tie of the reference's
    (a hit on a shared edge or vertex of two triangles)."""
    with np.errstate(invalid="ignore", divide="ignore"):
        return _classify(prim_ref, t_ref, t2_ref, prim_gpu, t_gpu, rel_tie)


def _classify(prim_ref, t_ref, t2_ref, prim_gpu, t_gpu, rel_tie):
    prim_ref = np.asarray(prim_ref, np.int64)
    prim_gpu = np.asarray(prim_gpu, np.int64)
    t_ref = np.asarray(t_ref, np.float64)
    t_gpu = np.asarray(t_gpu, np.float64)
    same = prim_ref == prim_gpu
    both = (prim_ref >= 0) & (prim_gpu >= 0)
    tie2 = np.isfinite(t2_ref) & (np.abs(t2_ref - t_ref) <= rel_tie * np.abs(t_ref))
    tie_t = both & (np.abs(t_gpu - t_ref) <= rel_tie * np.maximum(np.abs(t_ref), 1e-30))
    ties = ~same & (tie2 | tie_t)
    bad = ~same & ~ties
    terr = np.where(same & both, np.abs(t_gpu - t_ref) / np.maximum(np.abs(t_ref), 1e-30), 0.0)
    return dict(n=int(same.size), exact=int(same.sum()), ties=int(ties.sum()), mismatches=int(bad.sum()),
                max_rel_t_err=float(terr.max()) if terr.size else 0.0, bad_idx=np.nonzero(bad)[0])
