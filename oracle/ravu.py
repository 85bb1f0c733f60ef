"""FP64 restatement of the RAVU shader arithmetic -- test infrastructure.

Transcribes the root ``.hook`` files of the reference:

* ravu-lite / ravu-lite-ar: ``ravu-lite-r3.hook:22-131`` and
  ``ravu-lite-ar-r3.hook:22-183`` (window, structure tensor, key, keyed
  filter, anti-ringing, 2x2 shuffle).
* ravu (4-pass lattice form): ``ravu-r3.hook:15-437`` (int11, int10, int01,
  combine; yuv ``ravu-r3-yuv.hook``, rgb ``ravu-r3-rgb.hook``).
* ravu-zoom / ravu-zoom-ar: ``ravu-zoom-r2.hook:15-139``,
  ``ravu-zoom-ar-r2.hook`` (arbitrary ratio, bilinear LUT, AR LUT).
* ravu-3x: ``compute/ravu-3x-r2.hook:15-115`` (the only form of ravu-3x).

Planes are float arrays ``[C][H][W]`` (C = 1 luma, 3 for yuv/rgb), values
in [0, 1].  Out-of-range reads replicate the edge texel (clamp-to-edge, the
mpv texture border mode).  Every key evaluation also records whether its
continuous inputs sit within an FP32 rounding bound of a quantisation
threshold; such *boundary* keys may legitimately differ in an FP32
evaluation and are counted rather than failed.
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Tuple

import numpy as np

FLT_EPS = 1.192092896e-7          # the shaders' epsilon literal
PI = 3.141592653589793            # the shaders' pi literal
# Relative rounding budget of an FP32 evaluation of one key (2^-24 * 256),
# in units of the structure tensor's scale T = a + d (see key_margin).  The
# CUDA kernels' key flips, measured on full-size frames, needed at most 1.5
# units (ravu-lite-r3, 9 gradient points), 77 (ravu-r3 int11, 16 points) and
# 137 (ravu-lite-ar-r4, 25 points summed as packed pairs with the stencil
# scales folded into the weights); 256 covers the largest with a 1.9x factor.
FP32_BUDGET = 256.0 * 2.0 ** -24
REC709 = (0.2126, 0.7152, 0.0722)  # ravu-r2-rgb.hook:21 color_primary


# ------------------------------------------------------------------ utils --

def _as_planes(x) -> np.ndarray:
    a = np.asarray(x, dtype=np.float64)
    if a.ndim == 2:
        a = a[None]
    if a.ndim != 3:
        raise ValueError("planes must be [H][W] or [C][H][W]")
    return a


def _fetch(plane: np.ndarray, ys: np.ndarray, xs: np.ndarray) -> np.ndarray:
    """plane[clamp(y)][clamp(x)] for integer index grids (clamp-to-edge)."""
    H, W = plane.shape[-2:]
    return plane[..., np.clip(ys, 0, H - 1), np.clip(xs, 0, W - 1)]


def _luma(vals: np.ndarray, channels: str) -> np.ndarray:
    """Key input: the plane itself (luma), .x (yuv), Rec.709 dot (rgb)."""
    if channels == "luma":
        return vals[0]
    if channels == "yuv":
        return vals[0]            # ravu-r2-yuv.hook: gradients use sampleN.x
    return vals[0] * REC709[0] + vals[1] * REC709[1] + vals[2] * REC709[2]


def _window_size(family: str, radius: int) -> int:
    # ravu-lite-r3.hook:23-47 (5x5 = 2r-1); ravu-r3.hook:22-57 (6x6 = 2r)
    return 2 * radius - 1 if family in ("lite", "3x") else 2 * radius


def _deriv(lum: List[np.ndarray], n: int, four_tap: bool, px: int, py: int, axis: int) -> np.ndarray:
    """Gradient stencil of the shaders at grid (px, py).

    One-sided at the window border (``ravu-lite-r2.hook:34-35``), central
    ``/2.0`` inside (``ravu-lite-r3.hook:50``), 4-tap ``/12.0`` for
    ravu/zoom where both distance-2 neighbours exist (``ravu-r3.hook:63``).
    """
    p = px if axis == 0 else py

    def s(q):
        return lum[q * n + py] if axis == 0 else lum[px * n + q]

    if p == 0:
        return s(1) - s(0)
    if p == n - 1:
        return s(n - 1) - s(n - 2)
    if four_tap and 2 <= p <= n - 3:
        return (-s(p + 2) + 8.0 * s(p + 1) - 8.0 * s(p - 1) + s(p - 2)) / 12.0
    return (s(p + 1) - s(p - 1)) / 2.0


def structure_key(lum: List[np.ndarray], model) -> Dict[str, np.ndarray]:
    """Key row and boundary flag for every pixel of a window stack.

    ``lum[k]`` is the key-input value of window sample ``k`` (grid
    ``(k // n, k % n)``).  Transcribes ``ravu-lite-r3.hook:48-88`` (and the
    ravu/zoom/3x variants: ``ravu-r3.hook:121-125``,
    ``ravu-zoom-r2.hook:110-124``, ``compute/ravu-3x-r2.hook:70-81``).
    """
    family, radius = model.family, model.radius
    n = _window_size(family, radius)
    four = family in ("ravu", "zoom")
    pts = range(n) if n <= 4 else range(1, n - 1)
    w = list(model.grad_weights)
    a = np.zeros_like(lum[0])
    b = np.zeros_like(lum[0])
    d = np.zeros_like(lum[0])
    i = 0
    for px in pts:
        for py in pts:
            gx = _deriv(lum, n, four, px, py, 0)
            gy = _deriv(lum, n, four, px, py, 1)
            a += gx * gx * w[i]
            b += gx * gy * w[i]
            d += gy * gy * w[i]
            i += 1
    with np.errstate(invalid="ignore", divide="ignore"):
        T = a + d
        D = a * d - b * b
        delta = np.sqrt(np.maximum(T * T / 4.0 - D, 0.0))
        L1 = T / 2.0 + delta
        L2 = T / 2.0 - delta
        sqrtL1 = np.sqrt(L1)
        sqrtL2 = np.sqrt(L2)                      # NaN when L2 < 0, as on a GPU
        t0 = np.arctan2(L1 - a, b) + PI
        theta = np.where(np.abs(b) < FLT_EPS, 0.0, t0 - PI * np.floor(t0 / PI))
        lam = sqrtL1
        ssum = sqrtL1 + sqrtL2
        mu = np.where(ssum < FLT_EPS, 0.0, (sqrtL1 - sqrtL2) / ssum)
        angle = np.floor(theta * 24.0 / PI)
        kind = model.strength[0]
        if kind == "log2":
            q = np.log2(lam * model.strength[1] + FLT_EPS)
            strength = np.clip(np.floor(q), 0.0, model.strength[2])
            nstr = int(model.strength[2]) + 1
        else:
            ts = model.strength[1]
            if len(ts) == 3:   # mix(mix(0,1,l>=t0), mix(2,3,l>=t2), l>=t1)
                strength = np.where(lam >= ts[1], np.where(lam >= ts[2], 3.0, 2.0),
                                    np.where(lam >= ts[0], 1.0, 0.0))
            else:              # mix(mix(0,1,l>=t0), 2, l>=t1)
                strength = np.where(lam >= ts[1], 2.0, np.where(lam >= ts[0], 1.0, 0.0))
            nstr = len(ts) + 1
        c0, c1 = model.coherence
        coherence = np.where(mu >= c1, 2.0, np.where(mu >= c0, 1.0, 0.0))
        key = ((angle * nstr + strength) * 3.0 + coherence).astype(np.int64)   # raw, may reach rows

        margin = key_margin(a, b, d, T, L1, L2, theta, lam, mu, ssum, q if kind == "log2" else None, model)
        bnd = margin <= FP32_BUDGET
    return {"key": key, "boundary": bnd, "margin": margin, "theta": theta, "lambda": lam, "mu": mu,
            "rows": 24 * nstr * 3}


def key_margin(a, b, d, T, L1, L2, theta, lam, mu, ssum, q, model) -> np.ndarray:
    """Distance of a key from its nearest quantisation decision, in units of
    a relative error budget B of the structure tensor.

    An FP32 evaluation perturbs (a, b, d) by about B * T (T = a + d, the
    tensor's scale) with B a small multiple of 2^-24; each threshold test
    moves by that perturbation times its first-order sensitivity (angle:
    2 E / |(L1 - a, b)|; lambda: E / (2 lambda); log2 strength:
    E / (2 L1 ln 2) + B; coherence: E / |L2| + E / L1; the eps gates: E).
    The margin is, over all tests of the key, the smallest B at which the
    test's threshold lies within reach; a key is a *boundary* key when its
    margin is at most FP32_BUDGET.  A flat window (T = 0) is exact in any
    precision: margin +inf.
    """
    inf = np.inf
    with np.errstate(invalid="ignore", divide="ignore"):
        Ts = np.maximum(T, 1e-300)

        def m_of(dist, sens, const=0.0):
            m = (np.abs(dist) - const) / sens
            return np.where(np.isfinite(m), np.maximum(m, 0.0), inf)

        r = np.hypot(L1 - a, b)
        qa = theta * 24.0 / PI
        m = m_of(qa - np.round(qa), (24.0 / PI) * 2.0 * Ts / np.maximum(r, 1e-300), 1e-9)
        m = np.minimum(m, m_of(np.abs(b) - FLT_EPS, Ts))
        kind = model.strength[0]
        if kind == "log2":
            sens = (Ts / np.maximum(2.0 * L1, 1e-300)) / math.log(2.0) + 1.0
            inrange = (q > -0.5) & (q < model.strength[2] + 0.5)
            m = np.minimum(m, np.where(inrange, m_of(q - np.round(q), sens), inf))
        else:
            for t in model.strength[1]:
                m = np.minimum(m, m_of(lam - t, Ts / (2.0 * t) + t))
        m = np.minimum(m, m_of(L2, Ts))
        sens_mu = Ts / np.maximum(np.abs(L2), 1e-300) + Ts / np.maximum(L1, 1e-300)
        for c in model.coherence:
            m = np.minimum(m, m_of(mu - c, sens_mu, 1e-9))
        m = np.minimum(m, m_of(ssum * ssum - FLT_EPS * FLT_EPS, 2.0 * Ts))
        return np.where(T > 0.0, m, inf)


def _row(key: np.ndarray, rows: int) -> np.ndarray:
    """NEAREST LUT row of a key: ``(key + 0.5) / rows`` clamped to the edge."""
    return np.clip(key, 0, rows - 1)


def _ar_powers(v):
    """(0.1+v)^32, (0.1+v)^33, (1.1-v)^32, (1.1-v)^33 by 5 squarings
    (``ravu-lite-ar-r3.hook:91-98``)."""
    hi1 = 0.1 + v
    lo1 = 1.1 - v
    hi32 = hi1
    lo32 = lo1
    for _ in range(5):
        hi32 = hi32 * hi32
        lo32 = lo32 * lo32
    return hi32, hi32 * hi1, lo32, lo32 * lo1


def _finish_ar(res, lo, hi, lo2, hi2, strength):
    """``lo = 1.1 - lo2/lo; hi = hi2/hi - 0.1; res = mix(res, clamp(res,lo,hi), s)``
    (``ravu-lite-ar-r3.hook:178-181``)."""
    with np.errstate(invalid="ignore", divide="ignore"):
        lo_b = 1.1 - lo2 / lo
        hi_b = hi2 / hi - 0.1
        cl = np.minimum(np.maximum(res, lo_b), hi_b)
        return res * (1.0 - strength) + cl * strength


# ---------------------------------------------------------- ravu-lite -----

def ravu_lite(model, planes, keys: Optional[np.ndarray] = None):
    """2x ravu-lite(-ar) of a luma plane; returns (out [1][2H][2W], info).

    ``keys`` forces the LUT rows (e.g. those an FP32 evaluation chose) so
    that filter arithmetic can be compared independently of key flips.
    """
    x = _as_planes(planes)
    if x.shape[0] != 1:
        raise ValueError("ravu-lite is luma-only")
    p = x[0]
    H, W = p.shape
    r = model.radius
    n = 2 * r - 1
    lo = -(r - 1)
    S = n * n
    yy, xx = np.mgrid[0:H, 0:W]
    # ravu-lite-r3.hook:23-47: lumaK = HOOKED_texOff(vec2(K/n - 2, K%n - 2))
    lum = [_fetch(p, yy + (k % n + lo), xx + (k // n + lo)) for k in range(S)]
    info = structure_key(lum, model)
    key = info["key"] if keys is None else np.asarray(keys, dtype=np.int64).reshape(H, W)
    key = _row(key, info["rows"])
    lut = np.asarray(model.lut, dtype=np.float64)          # [rows][cols][4]
    res = np.zeros((4, H, W))
    ar = float(model.ar)
    if ar:
        lo_s = np.zeros((4, H, W)); hi_s = np.zeros((4, H, W))
        lo2 = np.zeros((4, H, W)); hi2 = np.zeros((4, H, W))
        ar_cols = model.ar_taps
    for c in range(S // 2):
        w = np.moveaxis(lut[key, c, :], -1, 0)              # ravu-lite-r3.hook:90
        res += lum[c] * w + lum[S - 1 - c] * w[::-1]        # w.wzyx
        if ar and ar_cols[c]:
            wg = np.maximum(0.0, w)                         # ravu-lite-ar-r3.hook:94
            h1, h2, l1, l2 = _ar_powers(lum[c])
            H1, H2, L1_, L2_ = _ar_powers(lum[S - 1 - c])
            hi_s += h1 * wg + H1 * wg[::-1]
            lo_s += l1 * wg + L1_ * wg[::-1]
            hi2 += h2 * wg + H2 * wg[::-1]
            lo2 += l2 * wg + L2_ * wg[::-1]
    c = S // 2
    w = np.moveaxis(lut[key, c, :], -1, 0)
    res += lum[c] * w
    if ar:
        wg = np.maximum(0.0, w)
        h1, h2, l1, l2 = _ar_powers(lum[c])
        hi_s += h1 * wg; lo_s += l1 * wg; hi2 += h2 * wg; lo2 += l2 * wg
        res = _finish_ar(res, lo_s, hi_s, lo2, hi2, ar)     # no [0,1] clamp after AR
    else:
        res = np.clip(res, 0.0, 1.0)                        # ravu-lite-r3.hook:117
    # step2 shuffle (ravu-lite-r3.hook:124-130): idx = (dx>0)*2 + (dy>0)
    out = np.empty((1, 2 * H, 2 * W))
    out[0, 0::2, 0::2] = res[0]
    out[0, 1::2, 0::2] = res[1]
    out[0, 0::2, 1::2] = res[2]
    out[0, 1::2, 1::2] = res[3]
    info["key"] = key if keys is None else info["key"]
    return out, info


# ------------------------------------------------------------ ravu-3x -----

def ravu_3x(model, planes, keys: Optional[np.ndarray] = None):
    """3x ravu-3x of luma/yuv/rgb planes (``compute/ravu-3x-r2.hook:82-114``)."""
    x = _as_planes(planes)
    C, H, W = x.shape
    r = model.radius
    n = 2 * r - 1
    lo = -(r - 1)
    S = n * n
    yy, xx = np.mgrid[0:H, 0:W]
    vals = [_fetch(x, yy + (k % n + lo), xx + (k // n + lo)) for k in range(S)]   # [C][H][W] each
    lum = [_luma(v, model.channels) for v in vals]
    info = structure_key(lum, model)
    key = info["key"] if keys is None else np.asarray(keys, dtype=np.int64).reshape(H, W)
    key = _row(key, info["rows"])
    lut = np.asarray(model.lut, dtype=np.float64)
    res0 = np.zeros((C, 4, H, W))
    res1 = np.zeros((C, 4, H, W))
    for c in range(S // 2):
        w0 = np.moveaxis(lut[key, 2 * c, :], -1, 0)
        w1 = np.moveaxis(lut[key, 2 * c + 1, :], -1, 0)
        a = vals[c][:, None]
        bq = vals[S - 1 - c][:, None]
        res0 += a * w0 + bq * w1[::-1]
        res1 += a * w1 + bq * w0[::-1]
    c = S // 2
    res0 += vals[c][:, None] * np.moveaxis(lut[key, 2 * c, :], -1, 0)
    res1 += vals[c][:, None] * np.moveaxis(lut[key, 2 * c + 1, :], -1, 0)
    res0 = np.clip(res0, 0.0, 1.0)
    res1 = np.clip(res1, 0.0, 1.0)
    out = np.empty((C, 3 * H, 3 * W))
    # imageStore(gid*3 + ivec2(dx, dy)): res0 -> (0,0),(0,1),(0,2),(1,0);
    # centre copy (1,1); res1 -> (1,2),(2,0),(2,1),(2,2)
    place = [(0, 0, res0[:, 0]), (0, 1, res0[:, 1]), (0, 2, res0[:, 2]), (1, 0, res0[:, 3]),
             (1, 1, vals[c]), (1, 2, res1[:, 0]), (2, 0, res1[:, 1]), (2, 1, res1[:, 2]),
             (2, 2, res1[:, 3])]
    for dx, dy, v in place:
        out[:, dy::3, dx::3] = v
    return out, info


# ------------------------------------------------- ravu (lattice form) ----

def _lattice_source(n: int, k: int, lattice: str):
    """Where rotated-window sample k of an int10/int01 pass reads from.

    ``ravu-r3.hook:155-189`` (int10) and ``:289-323`` (int01): the window is
    the 45-degree lattice that interleaves input pixels and int11 pixels.
    Returns (0 = input, 1 = int11, dx, dy).
    """
    kx, ky = k // n, k % n
    s = kx + ky - (n - 1)
    d = ky - kx
    if lattice == "int10":
        if s % 2:
            return 0, (s + 1) // 2, d // 2
        return 1, s // 2, (d - 1) // 2
    if s % 2 == 0:
        return 0, s // 2, (d + 1) // 2
    return 1, (s - 1) // 2, d // 2


def _ravu_pass(model, vals, keys_forced):
    """One keyed ravu pass over a window stack (``ravu-r3.hook:58-146``)."""
    C = vals[0].shape[0]
    S = len(vals)
    lum = [_luma(v, model.channels) for v in vals]
    info = structure_key(lum, model)
    key = info["key"] if keys_forced is None else keys_forced
    key = _row(key, info["rows"])
    lut = np.asarray(model.lut, dtype=np.float64).reshape(model.lut.shape[0], -1)   # [rows][4*cols]
    res = np.zeros_like(vals[0])
    for i in range(S // 2):
        res += (vals[i] + vals[S - 1 - i]) * lut[key, i][None]
    return np.clip(res, 0.0, 1.0), info


def ravu_lattice(model, planes, keys: Optional[np.ndarray] = None, int11: Optional[np.ndarray] = None):
    """2x ravu (luma/yuv/rgb), all four passes of ``ravu-r3.hook``.

    Output pixel (2i, 2j) is the input, (2i+1, 2j) int10, (2i, 2j+1) int01,
    (2i+1, 2j+1) int11 (``ravu-r3.hook:424-437`` with ``OFFSET -0.5 -0.5``).
    ``keys`` (optional) is ``[3][H][W]``: int11, int10, int01 rows.
    ``int11`` (optional, ``[C][H][W]``) replaces the computed int11 plane as
    the input of the two lattice passes, so that they can be checked on
    exactly the int11 values another implementation produced.
    """
    x = _as_planes(planes)
    C, H, W = x.shape
    r = model.radius
    n = 2 * r
    lo = -(r - 1)
    S = n * n
    yy, xx = np.mgrid[0:H, 0:W]
    kf = None if keys is None else np.asarray(keys, dtype=np.int64).reshape(3, H, W)
    vals = [_fetch(x, yy + (k % n + lo), xx + (k // n + lo)) for k in range(S)]
    own11, i11 = _ravu_pass(model, vals, None if kf is None else kf[0])
    if int11 is None:
        src11 = own11
    else:
        src11 = np.asarray(int11, dtype=np.float64).reshape(C, H, W)
    out_keys = [i11["key"]]
    bnd = [i11["boundary"]]
    margins = [i11["margin"]]
    results = {}
    for li, lattice in ((1, "int10"), (2, "int01")):
        vals = []
        for k in range(S):
            src, dx, dy = _lattice_source(n, k, lattice)
            vals.append(_fetch(x if src == 0 else src11, yy + dy, xx + dx))
        results[lattice], inf = _ravu_pass(model, vals, None if kf is None else kf[li])
        out_keys.append(inf["key"])
        bnd.append(inf["boundary"])
        margins.append(inf["margin"])
    out = np.empty((C, 2 * H, 2 * W))
    out[:, 0::2, 0::2] = x
    out[:, 0::2, 1::2] = results["int10"]
    out[:, 1::2, 0::2] = results["int01"]
    out[:, 1::2, 1::2] = own11
    return out, {"key": np.stack(out_keys), "boundary": np.stack(bnd), "margin": np.stack(margins)}


# ----------------------------------------------------------- ravu-zoom ----

def _bilinear(lut: np.ndarray, tx: np.ndarray, ty: np.ndarray, comp: int, frac_steps=None) -> np.ndarray:
    """FILTER LINEAR fetch of one component at texel coordinates (centre = k);
    ``frac_steps`` rounds the fractions to multiples of 1/frac_steps, as a
    texture unit's fixed-point weights are (256: 8 fractional bits)."""
    h, w = lut.shape[:2]
    x0 = np.floor(tx)
    y0 = np.floor(ty)
    fx = tx - x0
    fy = ty - y0
    if frac_steps:
        fx = np.rint(fx * frac_steps) / frac_steps
        fy = np.rint(fy * frac_steps) / frac_steps
    x0 = x0.astype(np.int64)
    y0 = y0.astype(np.int64)
    xa = np.clip(x0, 0, w - 1); xb = np.clip(x0 + 1, 0, w - 1)
    ya = np.clip(y0, 0, h - 1); yb = np.clip(y0 + 1, 0, h - 1)
    v00 = lut[ya, xa, comp]; v01 = lut[ya, xb, comp]
    v10 = lut[yb, xa, comp]; v11 = lut[yb, xb, comp]
    return (v00 * (1 - fx) + v01 * fx) * (1 - fy) + (v10 * (1 - fx) + v11 * fx) * fy


def ravu_zoom(model, planes, out_w: int, out_h: int, keys: Optional[np.ndarray] = None, frac_steps=None):
    """Arbitrary-ratio ravu-zoom(-ar) (``ravu-zoom-r2.hook:24-138``).

    Output pixel (X, Y) samples the input around
    ``pos = (X+0.5, Y+0.5) * in_size / out_size`` (centre-aligned,
    ``//!OFFSET ALIGN``); ``subpix = fract(pos - 0.5)`` selects the bilinear
    LUT position inside the key's 9x9 block.
    """
    x = _as_planes(planes)
    C, H, W = x.shape
    r = model.radius
    n = 2 * r
    lo = -(r - 1)
    S = n * n
    Y, X = np.mgrid[0:out_h, 0:out_w]
    # pos - 0.5 = ((2X+1) W - OW) / (2 OW), taken exactly: anchor = floor,
    # subpix = fract (ravu-zoom-r2.hook:25-27)
    numx = (2 * X.astype(np.int64) + 1) * W - out_w
    numy = (2 * Y.astype(np.int64) + 1) * H - out_h
    ix = numx // (2 * out_w)
    iy = numy // (2 * out_h)
    spx = (numx - ix * 2 * out_w) / (2.0 * out_w)
    spy = (numy - iy * 2 * out_h) / (2.0 * out_h)
    vals = [_fetch(x, iy + (k % n + lo), ix + (k // n + lo)) for k in range(S)]
    lum = [_luma(v, model.channels) for v in vals]
    info = structure_key(lum, model)
    key = info["key"] if keys is None else np.asarray(keys, dtype=np.int64).reshape(out_h, out_w)
    lut = np.asarray(model.lut, dtype=np.float64)
    # LUTPOS(s, 9) then /vec2(blocks, 288): texel x = block*9 + 8*s, y = key*9 + 8*s
    ty_sub = key * 9.0 + 8.0 * spy
    ty_inv = key * 9.0 + 8.0 * (1.0 - spy)
    res = np.zeros((C, out_h, out_w))
    ar = float(model.ar)
    if ar:
        lut_ar = np.asarray(model.lut_ar, dtype=np.float64)
        lo_s = np.zeros_like(res); hi_s = np.zeros_like(res)
        lo2 = np.zeros_like(res); hi2 = np.zeros_like(res)
    for i in range(S // 2):
        blk, comp = i // 4, i % 4
        w_sub = _bilinear(lut, blk * 9.0 + 8.0 * spx, ty_sub, comp, frac_steps)
        w_inv = _bilinear(lut, blk * 9.0 + 8.0 * (1.0 - spx), ty_inv, comp, frac_steps)
        res += vals[i] * w_sub + vals[S - 1 - i] * w_inv
        if ar:
            a_sub = _bilinear(lut_ar, blk * 9.0 + 8.0 * spx, ty_sub, comp, frac_steps)
            a_inv = _bilinear(lut_ar, blk * 9.0 + 8.0 * (1.0 - spx), ty_inv, comp, frac_steps)
            for v, wa in ((vals[i], a_sub), (vals[S - 1 - i], a_inv)):
                h1, h2, l1, l2 = _ar_powers(v)
                hi_s += h1 * wa; lo_s += l1 * wa; hi2 += h2 * wa; lo2 += l2 * wa
    if ar:
        res = _finish_ar(res, lo_s, hi_s, lo2, hi2, ar)
    else:
        res = np.clip(res, 0.0, 1.0)
    return res, info


def mpv_form(model, round_ar: bool = True):
    """The model as the mpv host holds it: every LUT value rounded to FP16
    (the //!TEXTURE blocks are uploaded as ``//!FORMAT rgba16f``,
    ``ravu-lite-r3.hook:134``).  Use with ``frac_steps=256`` for ravu-zoom
    and FP16 planes to restate what the host computes.  ``round_ar=False``
    leaves ravu-zoom-ar's anti-ringing LUT exact (the library's fast form)."""
    import copy
    m = copy.copy(model)
    m.lut = np.asarray(model.lut, dtype=np.float32).astype(np.float16).astype(np.float32)
    if round_ar and getattr(model, "lut_ar", None) is not None:
        m.lut_ar = np.asarray(model.lut_ar, dtype=np.float32).astype(np.float16).astype(np.float32)
    return m


def keyed_upscale(model, planes, out_size: Optional[Tuple[int, int]] = None, keys=None, int11=None,
                  frac_steps=None):
    """Dispatch on the model family; ``out_size`` = (w, h) for ravu-zoom;
    ``int11`` overrides the int11 plane fed to the ravu lattice passes;
    ``frac_steps`` quantises ravu-zoom's LUT bilinear fractions."""
    fam = model.family
    if fam == "lite":
        return ravu_lite(model, planes, keys)
    if fam == "3x":
        return ravu_3x(model, planes, keys)
    if fam == "ravu":
        return ravu_lattice(model, planes, keys, int11)
    if fam == "zoom":
        if out_size is None:
            raise ValueError("ravu-zoom needs an output size")
        return ravu_zoom(model, planes, out_size[0], out_size[1], keys, frac_steps)
    raise ValueError(fam)
