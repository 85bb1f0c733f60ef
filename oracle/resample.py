"""FP64 restatement of the host scaler steps around a prescaler (TEST
INFRASTRUCTURE ONLY): the //!OFFSET shift correction and the chroma
upsampling that precedes a NATIVE hook.

The hook files only announce these steps; the host performs them:
``ravu-r3.hook:424`` (``//!OFFSET -0.500000 -0.500000``),
``nnedi3-nns16-win8x4.hook:95,185`` (``0 -0.5`` then ``-0.5 0``) and
``compute/ravu-r2-yuv.hook:15`` (``//!HOOK NATIVE``: planes merged after
``--cscale``, ``README.md:50-56``).  The interpolation itself is the
textbook separable form with texel centres at integer coordinates and
edge-replicating borders:

    out(x, y) = sum_i sum_j k(u - i) k(v - j) in(clamp(i), clamp(j)),
    u = sx * x + ox,  v = sy * y + oy,

k = tent (bilinear) or Keys' cubic convolution kernel with a = -1/2
(Catmull-Rom).
"""
from __future__ import annotations

import numpy as np


def _cubic(t):
    t = np.abs(t)
    return np.where(t < 1, 1.5 * t**3 - 2.5 * t**2 + 1,
                    np.where(t < 2, -0.5 * t**3 + 2.5 * t**2 - 4 * t + 2, 0.0))


def _tent(t):
    return np.maximum(0.0, 1.0 - np.abs(t))


def _axis_matrix(n_out: int, n_in: int, s: float, o: float, filt: str) -> np.ndarray:
    """[n_out][n_in] interpolation matrix of one axis (clamped borders fold
    the weight of every outside tap onto the edge texel)."""
    u = s * np.arange(n_out, dtype=np.float64) + o
    base = np.floor(u)
    taps = (0, 1) if filt == "bilinear" else (-1, 0, 1, 2)
    k = _tent if filt == "bilinear" else _cubic
    M = np.zeros((n_out, n_in))
    rows = np.arange(n_out)
    for d in taps:
        i = base + d
        w = k(u - i)
        np.add.at(M, (rows, np.clip(i, 0, n_in - 1).astype(np.int64)), w)
    return M


def resample(plane: np.ndarray, out_w: int, out_h: int, sx: float, ox: float, sy: float, oy: float,
             filt: str = "catmull_rom") -> np.ndarray:
    if filt not in ("bilinear", "catmull_rom"):
        raise ValueError(filt)
    p = np.asarray(plane, dtype=np.float64)
    My = _axis_matrix(out_h, p.shape[0], sy, oy, filt)
    Mx = _axis_matrix(out_w, p.shape[1], sx, ox, filt)
    return My @ p @ Mx.T


def shift(plane: np.ndarray, ox: float, oy: float, filt: str = "catmull_rom") -> np.ndarray:
    """Correct an announced //!OFFSET (ox, oy): out(x, y) = in(x + ox, y + oy)."""
    h, w = plane.shape
    return resample(plane, w, h, 1.0, ox, 1.0, oy, filt)
