"""FP64 restatement of the NNEDI3 shader arithmetic -- test infrastructure.

Transcribes ``nnedi3-nns16-win8x4.hook`` (and every nnsN/win8xK sibling):

* ``double_y`` (``:15-104``): for the gap between rows j and j+1, the 8x4
  (or 8x6) window around it is normalised (``:20-29``), every neuron pair k
  evaluates ``e_k = exp(<x,A_k> * invstd + a_k)`` and
  ``s_k = <x,B_k> * invstd + b_k``, accumulating ``wsum += e_k`` and
  ``vsum += e_k * s_k / (1 + |s_k|)`` (macros ``:31-33``), and the result is
  ``clamp(mean + 5 * vsum / wsum * std, 0, 1)`` (``:50``).
* ``combine_y`` (``:105-119``) interleaves: output row 2j = input row j,
  row 2j+1 = the interpolated row.
* ``double_x``/``combine_x`` (``:120-210``) repeat this on the row-doubled
  image with the transposed window (the weights are the same, transposed).

Weights come from the model in canonical tap order (row-major window,
``dy`` outer, ``dx`` inner, in the double_y orientation).
"""
from __future__ import annotations

from typing import Dict, Tuple

import numpy as np

FLT_EPS = 1.192092896e-7
FP32_BUDGET = 256.0 * 2.0 ** -24


def nnedi3_double(model, plane: np.ndarray, chunk: int = 1 << 16) -> Tuple[np.ndarray, Dict]:
    """One double_y pass: ``[H][W]`` -> interpolated rows ``[H][W]``.

    Row j of the result lies between input rows j and j+1.
    """
    p = np.asarray(plane, dtype=np.float64)
    H, W = p.shape
    taps = np.asarray(model.taps)
    A = np.asarray(model.weights_a, dtype=np.float64)
    B = np.asarray(model.weights_b, dtype=np.float64)
    ba = np.asarray(model.bias_a, dtype=np.float64)
    bb = np.asarray(model.bias_b, dtype=np.float64)
    T = taps.shape[0]
    yy, xx = np.mgrid[0:H, 0:W]
    yy = yy.ravel()
    xx = xx.ravel()
    out = np.empty(H * W)
    bnd = np.zeros(H * W, dtype=bool)
    for s in range(0, H * W, chunk):
        ys = yy[s:s + chunk]
        xs = xx[s:s + chunk]
        X = np.stack([p[np.clip(ys + dy, 0, H - 1), np.clip(xs + dx, 0, W - 1)] for dx, dy in taps], axis=1)
        mstd0 = X.sum(1) / T
        var = (X * X).sum(1) / T - mstd0 * mstd0
        with np.errstate(divide="ignore", invalid="ignore"):
            invstd = np.where(var >= FLT_EPS, 1.0 / np.sqrt(np.maximum(var, 1e-300)), 0.0)
            std = var * invstd
            s1 = (X @ A) * invstd[:, None] + ba
            e = np.exp(s1)
            s2 = (X @ B) * invstd[:, None] + bb
            wsum = e.sum(1)
            vsum = (e * (s2 / (1.0 + np.abs(s2)))).sum(1)
            out[s:s + chunk] = np.clip(mstd0 + 5.0 * vsum / wsum * std, 0.0, 1.0)
        # the variance gate is the only threshold in NNEDI3
        bnd[s:s + chunk] = np.abs(var - FLT_EPS) <= FP32_BUDGET * (X * X).sum(1) / T + 1e-12
    return out.reshape(H, W), {"boundary": bnd.reshape(H, W)}


def nnedi3_upscale(model, plane: np.ndarray, axes: str = "yx") -> Tuple[np.ndarray, Dict]:
    """Full 2x NNEDI3: double_y + combine_y, then double_x + combine_x.

    ``axes`` selects the enabled passes (``//!WHEN`` per axis): "yx", "y"
    or "x".  Returns the upscaled plane and boundary masks per pass.
    """
    p = np.asarray(plane, dtype=np.float64)
    if p.ndim == 3:
        if p.shape[0] != 1:
            raise ValueError("NNEDI3 is luma-only")
        p = p[0]
    info = {}
    if "y" in axes:
        iy, inf = nnedi3_double(model, p)
        H, W = p.shape
        q = np.empty((2 * H, W))
        q[0::2] = p
        q[1::2] = iy
        p = q
        info["boundary_y"] = inf["boundary"]
    if "x" in axes:
        ix, inf = nnedi3_double(model, p.T)
        H, W = p.shape
        q = np.empty((H, 2 * W))
        q[:, 0::2] = p
        q[:, 1::2] = ix.T
        p = q
        info["boundary_x"] = inf["boundary"].T
    return p[None], info
