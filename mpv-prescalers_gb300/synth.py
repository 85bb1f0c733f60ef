"""Seeded synthetic video planes (the prescaler benchmark inputs).

No public dataset is involved: every plane is generated from
``numpy.random.default_rng(seed)`` as

* 8 random-orientation sinusoids ``0.5 + sum A sin(2 pi (x cos phi + y sin phi)/P + psi)``
  with ``phi ~ U(0, pi)``, ``P`` log-uniform in [4, 64] px, ``A ~ U(0.02, 0.1)``,
  ``psi ~ U(0, 2 pi)``;
* 20 random polygons (3-8 vertices at sorted random angles around a centre,
  radius ``U(8, 0.25 min(W, H))``) painted in order with a constant random
  intensity, filled by the even-odd rule at pixel centres;
* Gaussian noise sigma 0.01, then a clamp to [0, 1].

RGB frames mix one shared plane with three independent ones
(``c_i = sqrt(0.8) S + sqrt(0.2) N_i`` on standardised planes, pairwise
correlation 0.8) and rescale to [0, 1]; YUV 4:4:4 frames are three planes
from independent seeds.  The seed of frame ``f`` of benchmark config ``k``
is ``1000 k + f``.
"""
from __future__ import annotations

import numpy as np


def _polygon_mask(h: int, w: int, vx: np.ndarray, vy: np.ndarray):
    """Even-odd fill at pixel centres; returns (y0, x0, mask) over the bbox."""
    x0b = int(max(0, np.floor(vx.min())))
    x1b = int(min(w, np.ceil(vx.max()) + 1))
    y0b = int(max(0, np.floor(vy.min())))
    y1b = int(min(h, np.ceil(vy.max()) + 1))
    if x1b <= x0b or y1b <= y0b:
        return 0, 0, np.zeros((0, 0), dtype=bool)
    yy, xx = np.mgrid[y0b:y1b, x0b:x1b]
    px = xx + 0.5
    py = yy + 0.5
    inside = np.zeros(px.shape, dtype=bool)
    n = len(vx)
    for i in range(n):
        x0, y0 = vx[i], vy[i]
        x1, y1 = vx[(i + 1) % n], vy[(i + 1) % n]
        if y0 == y1:
            continue
        cond = (py >= min(y0, y1)) & (py < max(y0, y1))
        xint = x0 + (py - y0) * (x1 - x0) / (y1 - y0)
        inside ^= cond & (px < xint)
    return y0b, x0b, inside


def luma_plane(h: int, w: int, seed: int) -> np.ndarray:
    """One [h][w] float32 plane in [0, 1]."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    img = np.full((h, w), 0.5)
    for _ in range(8):
        phi = rng.uniform(0.0, np.pi)
        period = np.exp(rng.uniform(np.log(4.0), np.log(64.0)))
        amp = rng.uniform(0.02, 0.1)
        psi = rng.uniform(0.0, 2.0 * np.pi)
        img += amp * np.sin(2.0 * np.pi * (xx * np.cos(phi) + yy * np.sin(phi)) / period + psi)
    rmax = max(8.0, 0.25 * min(w, h))
    for _ in range(20):
        nv = int(rng.integers(3, 9))
        cx = rng.uniform(0, w)
        cy = rng.uniform(0, h)
        rad = rng.uniform(min(8.0, rmax), rmax)
        ang = np.sort(rng.uniform(0.0, 2.0 * np.pi, nv))
        val = rng.uniform(0.0, 1.0)
        y0b, x0b, mask = _polygon_mask(h, w, cx + rad * np.cos(ang), cy + rad * np.sin(ang))
        sub = img[y0b:y0b + mask.shape[0], x0b:x0b + mask.shape[1]]
        sub[mask] = val
    img += rng.normal(0.0, 0.01, size=(h, w))
    return np.clip(img, 0.0, 1.0).astype(np.float32)


def rgb_frame(h: int, w: int, seed: int) -> np.ndarray:
    """[3][h][w] float32 RGB with 0.8 pairwise channel correlation."""
    base = luma_plane(h, w, seed).astype(np.float64)
    out = []
    for c in range(3):
        nz = luma_plane(h, w, seed * 7919 + c + 1).astype(np.float64)
        s = (base - base.mean()) / (base.std() + 1e-12)
        n = (nz - nz.mean()) / (nz.std() + 1e-12)
        out.append(np.sqrt(0.8) * s + np.sqrt(0.2) * n)
    x = np.stack(out)
    x = (x - x.min()) / (x.max() - x.min() + 1e-12)
    return x.astype(np.float32)


def yuv_frame(h: int, w: int, seed: int) -> np.ndarray:
    """[3][h][w] float32 4:4:4 planes from independent seeds."""
    return np.stack([luma_plane(h, w, seed * 7919 + c + 101) for c in range(3)])


def frame(h: int, w: int, seed: int, channels: str = "luma") -> np.ndarray:
    if channels == "luma":
        return luma_plane(h, w, seed)[None]
    if channels == "rgb":
        return rgb_frame(h, w, seed)
    if channels == "yuv":
        return yuv_frame(h, w, seed)
    raise ValueError(channels)
