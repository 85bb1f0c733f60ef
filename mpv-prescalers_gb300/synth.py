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


# ------------------------------------------------------------------ models --

_WHEN_2X = "HOOKED.w OUTPUT.w / 0.707106 < HOOKED.h OUTPUT.h / 0.707106 < *"
_WHEN_3X = "HOOKED.w OUTPUT.w / 0.471404 < HOOKED.h OUTPUT.h / 0.471404 < *"
_WHEN_ZOOM = "HOOKED.w OUTPUT.w < HOOKED.h OUTPUT.h < *"


def _parse_name(name: str):
    import re
    m = re.fullmatch(r"nnedi3-nns(\d+)-win8x([46])", name)
    if m:
        return {"family": "nnedi3", "nns": int(m.group(1)), "win_h": int(m.group(2))}
    m = re.fullmatch(r"ravu(-lite|-zoom|-3x)?(-ar)?-r([234])(?:-(yuv|rgb))?", name)
    if not m:
        raise ValueError(f"not a prescaler name: {name!r}")
    fam = {None: "ravu", "-lite": "lite", "-zoom": "zoom", "-3x": "3x"}[m.group(1)]
    return {"family": fam, "ar": 0.8 if m.group(2) else 0.0, "radius": int(m.group(3)),
            "channels": m.group(4) or "luma"}


def synthetic_model(name: str, seed: int = 0):
    """A canonical model with the shapes and structure of the named hook
    file but seeded random LUT / neuron weights.  For tests and benchmarks
    on machines without the ``.hook`` files: the CUDA path and the oracle do
    not depend on the weight values."""
    from . import geometry as geo
    from .hookfile import Pass
    from .models import Nnedi3Model, RavuModel

    info = _parse_name(name)
    rng = np.random.default_rng(seed + sum(map(ord, name)))

    # hook point and //!OFFSET as in the real files: luma files hook LUMA,
    # yuv NATIVE, rgb MAIN (compute/ravu-r2-yuv.hook:15, ravu-r2-rgb.hook:16);
    # ravu ends with OFFSET -0.5 -0.5 (ravu-r3.hook:424), zoom with ALIGN
    # (ravu-zoom-r2.hook:21), the NNEDI3 combine passes with 0 -0.5 and
    # -0.5 0 (nnedi3-nns16-win8x4.hook:95,185)
    hook = {"luma": "LUMA", "yuv": "NATIVE", "rgb": "MAIN"}[info.get("channels", "luma")]

    def mkpass(desc, when, save=None, offset=None, width=None, height=None):
        return Pass(desc=desc, hooks=[hook], binds=["HOOKED"], save=save, width=width, height=height,
                    offset=offset, when=when, components=None, compute=None, body=[], line=0, body_line=0)

    if info["family"] == "nnedi3":
        nns, wh = info["nns"], info["win_h"]
        T = 8 * wh
        A = rng.normal(0.0, 0.15, size=(T, nns))
        B = rng.normal(0.0, 0.15, size=(T, nns))
        A -= A.mean(0)
        B -= B.mean(0)
        passes = [mkpass(f"NNEDI3 (double_y, nns{nns}, win8x{wh})", "HOOKED.h OUTPUT.h / 0.707106 <", "nnedi3_int"),
                  mkpass(f"NNEDI3 (combine_y, nns{nns}, win8x{wh})", "HOOKED.h OUTPUT.h / 0.707106 <",
                         offset=(0.0, -0.5), height="2 HOOKED.h *"),
                  mkpass(f"NNEDI3 (double_x, nns{nns}, win8x{wh})", "HOOKED.w OUTPUT.w / 0.707106 <", "nnedi3_int"),
                  mkpass(f"NNEDI3 (combine_x, nns{nns}, win8x{wh})", "HOOKED.w OUTPUT.w / 0.707106 <",
                         offset=(-0.5, 0.0), width="2 HOOKED.w *")]
        return Nnedi3Model(name=name, nns=nns, win_w=8, win_h=wh,
                           taps=np.asarray(geo.nnedi3_taps(8, wh), dtype=np.int32),
                           weights_a=A.astype(np.float32), weights_b=B.astype(np.float32),
                           bias_a=rng.normal(0, 0.5, nns).astype(np.float32),
                           bias_b=rng.normal(0, 0.5, nns).astype(np.float32),
                           passes=passes, style="synthetic", path="<synthetic>")
    fam, r = info["family"], info["radius"]
    n = geo.window_size(fam, r)
    S = n * n
    if fam == "ravu":
        strength = ("log2", 2000.0, 8.0)
    elif fam == "3x":
        strength = ("thr", (0.005, 0.02))
    else:
        strength = ("thr", (0.004, 0.016, 0.05))
    ns = int(strength[2]) + 1 if strength[0] == "log2" else len(strength[1]) + 1
    rows = 24 * ns * 3
    if fam == "lite":
        w = rng.normal(0.0, 0.05, size=(rows, S, 4)) + np.exp(-rng.random((1, S, 1)) * 3) * 0.1
        # fold to the paired layout: column c holds tap c, tap S-1-c reads it reversed
        lut = np.zeros((rows, (S + 1) // 2, 4))
        for c in range(S // 2):
            lut[:, c] = w[:, c]
        lut[:, S // 2] = w[:, S // 2]
        tot = lut[:, : S // 2].sum(1) + lut[:, : S // 2, ::-1].sum(1) + lut[:, S // 2]
        lut[:, S // 2] += 1.0 - tot
    elif fam == "3x":
        lut = rng.normal(0.0, 0.05, size=(rows, 2 * ((S + 1) // 2), 4))
        lut[:, S - 1] += 0.5
        lut[:, S - 2] += 0.5
    elif fam == "ravu":
        ncols = (S // 2 + 3) // 4
        wt = rng.normal(0.0, 0.03, size=(rows, 4 * ncols))
        wt[:, S // 2:] = 0.0
        wt[:, : S // 2] += (0.5 - wt[:, : S // 2].sum(1, keepdims=True)) / (S // 2)
        lut = wt.reshape(rows, ncols, 4)
    else:  # zoom
        nb = (S // 2 + 3) // 4
        lut = rng.normal(0.0, 0.03, size=(rows * 9, 9 * nb, 4)) + 1.0 / S
    lut = lut.astype(np.float32)
    lut_ar = None
    if fam == "zoom" and info["ar"]:
        lut_ar = (rng.random(lut.shape) * 0.1).astype(np.float32)
    when = _WHEN_ZOOM if fam == "zoom" else (_WHEN_3X if fam == "3x" else _WHEN_2X)
    if info["channels"] == "yuv":
        when += " LUMA.w 0 > *"   # yuv files need a luma plane (compute/ravu-r2-yuv.hook:19)
    scale = {"zoom": None, "3x": "3"}.get(fam, "2")
    passes = [mkpass(f"synthetic {name}", when, offset={"ravu": (-0.5, -0.5), "zoom": "ALIGN"}.get(fam),
                     width=f"{scale} HOOKED.w *" if scale else "OUTPUT.w",
                     height=f"{scale} HOOKED.h *" if scale else "OUTPUT.h")]
    return RavuModel(name=name, family=fam, radius=r, channels=info["channels"], ar=info["ar"], lut=lut,
                     lut_ar=lut_ar, grad_weights=np.asarray(geo.grad_weights(fam, r)), strength=strength,
                     coherence=(0.25, 0.5), passes=passes, style="synthetic", path="<synthetic>",
                     ar_taps=geo.lite_ar_taps(r) if fam == "lite" and info["ar"] else None)


def model_for(name: str):
    """(HookModel, source): the parsed model from the package cache when
    present ("parsed"), else :func:`synthetic_model` ("synthetic")."""
    from .prescaler import HookModel, cached_model
    try:
        return cached_model(name), "parsed"
    except FileNotFoundError:
        return HookModel(synthetic_model(name)), "synthetic"
