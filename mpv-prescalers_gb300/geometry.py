"""Window geometry rules shared by the host and the CUDA kernels.

The generated shaders follow a small set of rules.  They are written out
here once; :mod:`.models` checks every parsed file against them, and the
CUDA templates in ``csrc/`` implement the same rules at compile time.

* Window: ``n = 2r-1`` taps per axis for ravu-lite and ravu-3x
  (``ravu-lite-r3.hook:23-47``: offsets -2..2), ``n = 2r`` for ravu and
  ravu-zoom (``ravu-r3.hook:22-57``: offsets -2..3).  Offsets start at
  ``-(r-1)``.  Sample index ``k`` sits at grid ``(k // n, k % n)``.
* Gradient points: the whole window when ``n <= 4``, otherwise the window
  minus a one-tap border (``ravu-lite-r3.hook:50-76`` uses the inner 3x3,
  ``ravu-r2.hook`` all 16).  Points run x-major, y inner.
* Derivative along an axis at grid position ``p``: one-sided difference at
  the window border (``ravu-lite-r2.hook:34``), ``(s[p+1]-s[p-1])/2``
  inside, and for ravu/ravu-zoom the 4-tap ``(-s[p+2]+8s[p+1]-8s[p-1]+s[p-2])/12``
  wherever both neighbours at distance 2 exist (``ravu-r3.hook:63``).
* Gaussian weights ``exp(-d^2/8)`` around the window centre, normalised to
  sum 1 over the gradient points (``ravu-lite-r3.hook:52,55,67``:
  0.1018..., 0.1154..., 0.1308...).
* ravu lattice passes (int10/int01, ``ravu-r3.hook:148-281``) read a window
  rotated by 45 degrees: index ``(kx, ky)`` lies at
  ``((s)/2, (d)/2)`` from the target with ``s = kx+ky-(n-1)``,
  ``d = ky-kx``, alternating between original pixels and int11 pixels.
* NNEDI3 windows are 8 wide and 4 or 6 tall around the gap being filled
  (``nnedi3-nns16-win8x4.hook:56-87``: x -3..4, y -1..2).
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Tuple

import numpy as np


def window_size(family: str, radius: int) -> int:
    if family in ("lite", "3x"):
        return 2 * radius - 1
    if family in ("ravu", "zoom"):
        return 2 * radius
    raise ValueError(family)


def window_lo(family: str, radius: int) -> int:
    return -(radius - 1)


def window_pos(family: str, radius: int, idx: int) -> Tuple[int, int]:
    n = window_size(family, radius)
    return (idx // n, idx % n)


def grad_points(family: str, radius: int) -> List[Tuple[int, int]]:
    n = window_size(family, radius)
    rng = range(n) if n <= 4 else range(1, n - 1)
    return [(px, py) for px in rng for py in rng]


def derivative(family: str, radius: int, p: int) -> Tuple[Dict[int, float], float]:
    """Stencil along one axis at grid position ``p``: ({grid: coef}, divisor)."""
    n = window_size(family, radius)
    if p == 0:
        return {1: 1.0, 0: -1.0}, 1.0
    if p == n - 1:
        return {n - 1: 1.0, n - 2: -1.0}, 1.0
    if family in ("ravu", "zoom") and p >= 2 and p <= n - 3:
        return {p + 2: -1.0, p + 1: 8.0, p - 1: -8.0, p - 2: 1.0}, 12.0
    return {p + 1: 1.0, p - 1: -1.0}, 2.0


def grad_weights(family: str, radius: int) -> List[float]:
    n = window_size(family, radius)
    c = (n - 1) / 2.0
    raw = [math.exp(-((px - c) ** 2 + (py - c) ** 2) / 8.0) for px, py in grad_points(family, radius)]
    s = math.fsum(raw)
    return [v / s for v in raw]


def sample_source(family: str, radius: int, idx: int, lattice: Optional[str] = None):
    """(texture, dx, dy) that sample ``idx`` of a pass reads.

    ``lattice`` is None for passes on the input grid, ``"int10"`` or
    ``"int01"`` for the two rotated ravu passes.
    """
    n = window_size(family, radius)
    kx, ky = idx // n, idx % n
    lo = window_lo(family, radius)
    if lattice is None:
        return ("HOOKED", float(kx + lo), float(ky + lo))
    s = kx + ky - (n - 1)
    d = ky - kx
    if lattice == "int10":
        if s % 2:
            return ("HOOKED", float((s + 1) // 2), float(d // 2))
        return ("ravu_int11", float(s // 2), float((d - 1) // 2))
    if lattice == "int01":
        if s % 2 == 0:
            return ("HOOKED", float(s // 2), float((d + 1) // 2))
        return ("ravu_int11", float((s - 1) // 2), float(d // 2))
    raise ValueError(lattice)


def lite_ar_taps(radius: int) -> np.ndarray:
    """Columns of a ravu-lite LUT whose tap pair enters the anti-ringing sums."""
    n = window_size("lite", radius)
    S = n * n
    lo = window_lo("lite", radius)
    ncols = (S + 1) // 2
    out = np.zeros(ncols, dtype=bool)
    for c in range(ncols):
        dx, dy = c // n + lo, c % n + lo
        out[c] = radius == 2 or abs(dx) + abs(dy) <= 2
    return out


def nnedi3_taps(win_w: int, win_h: int) -> List[Tuple[int, int]]:
    """Canonical NNEDI3 tap order: row-major (dy outer, dx inner)."""
    xs = range(-(win_w // 2 - 1), win_w // 2 + 1)
    ys = range(-(win_h // 2 - 1), win_h // 2 + 1)
    return [(dx, dy) for dy in ys for dx in xs]
