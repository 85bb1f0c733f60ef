"""Canonical prescaler models built from parsed ``.hook`` files.

Every ``.hook`` variant of one algorithm (root fragment shaders, ``compute/``
and ``gather/``) encodes the same arithmetic with a different sample order.
This module reduces a parsed file to one canonical model:

* :class:`RavuModel` for ravu-lite(-ar), ravu (two-pass lattice), ravu-zoom(-ar)
  and ravu-3x, in luma / yuv / rgb flavours.  It holds the LUT texture(s) as
  float32 ``[rows][cols][4]`` exactly as embedded, the gradient geometry
  (window taps, per-point derivative stencils, Gaussian weights), the key
  quantisation constants and the anti-ringing strength.
* :class:`Nnedi3Model` for nnedi3-nnsN-win8xK: the two neuron weight banks in
  canonical tap order plus their biases.

The gradient geometry is generated from a rule (:mod:`.geometry`) and every
file is checked against it: root files stencil by stencil, compute/gather
files by their weights, thresholds and (for NNEDI3) their full weight sets
remapped to canonical taps.  A file that disagrees is rejected with a
:class:`~.hookfile.HookParseError` naming the line.
"""
from __future__ import annotations

import dataclasses
import os
import re
import struct
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import geometry as geo
from .hookfile import HookFile, HookParseError, Pass, parse_hook_file, rpn_eval

_NUM = r"[-+]?\d+(?:\.\d*)?(?:[eE][-+]?\d+)?"


@dataclasses.dataclass
class RavuModel:
    name: str
    family: str                 # "lite" | "ravu" | "zoom" | "3x"
    radius: int
    channels: str               # "luma" | "yuv" | "rgb"
    ar: float                   # anti-ringing strength, 0.0 when absent
    lut: np.ndarray             # float32 [rows][cols][4]
    lut_ar: Optional[np.ndarray]
    grad_weights: np.ndarray    # float64 [n_points] in geometry order
    strength: Tuple             # ("thr", (t0, t1, ...)) or ("log2", scale, max)
    coherence: Tuple[float, float]
    passes: List[Pass]
    style: str
    path: str
    ar_taps: Optional[np.ndarray] = None   # bool [cols]: lite columns with AR

    kind = "ravu"

    @property
    def window(self) -> int:
        return geo.window_size(self.family, self.radius)

    @property
    def n_strength(self) -> int:
        if self.strength[0] == "log2":
            return int(self.strength[2]) + 1
        return len(self.strength[1]) + 1

    @property
    def rows(self) -> int:
        return 24 * self.n_strength * 3

    @property
    def scale(self) -> Optional[int]:
        return {"lite": 2, "ravu": 2, "3x": 3}.get(self.family)

    @property
    def offset(self):
        """Output shift reported by the last pass (``//!OFFSET``)."""
        for p in reversed(self.passes):
            if p.offset is not None:
                return p.offset
        return (0.0, 0.0)


@dataclasses.dataclass
class Nnedi3Model:
    name: str
    nns: int
    win_w: int                  # 8
    win_h: int                  # 4 or 6
    taps: np.ndarray            # int [T,2] (dx, dy) in double_y orientation
    weights_a: np.ndarray       # float32 [T][nns] (softmax branch)
    weights_b: np.ndarray       # float32 [T][nns] (elliott branch)
    bias_a: np.ndarray          # float32 [nns]
    bias_b: np.ndarray          # float32 [nns]
    passes: List[Pass]
    style: str
    path: str

    kind = "nnedi3"
    family = "nnedi3"
    channels = "luma"

    @property
    def n_taps(self) -> int:
        return self.win_w * self.win_h


# ----------------------------------------------------------- helpers -------

def _desc_info(p: Pass) -> Tuple[str, Dict[str, str]]:
    m = re.match(r"(RAVU-Lite-AR|RAVU-Lite|RAVU-Zoom-AR|RAVU-Zoom|RAVU-3x|RAVU|NNEDI3)\s*\((.*)\)$", p.desc)
    if not m:
        raise HookParseError("", p.line, f"unrecognised pass DESC {p.desc!r}")
    return m.group(1), {"args": m.group(2)}


def _find(body: List[str], pattern: str, path: str, p: Pass, what: str) -> Tuple[re.Match, int]:
    rx = re.compile(pattern)
    for k, ln in enumerate(body):
        m = rx.search(ln)
        if m:
            return m, p.body_line + k
    raise HookParseError(path, p.line, f"{what} not found in pass {p.desc!r}")


def _parse_strength(p: Pass, path: str) -> Tuple[Tuple, Tuple[float, float], bool]:
    m, _ = _find(p.body, r"float strength = (.*);", path, p, "strength line")
    s = m.group(1)
    m4 = re.fullmatch(rf"mix\(mix\(0\.0, 1\.0, lambda >= ({_NUM})\), mix\(2\.0, 3\.0, lambda >= ({_NUM})\), lambda >= ({_NUM})\)", s)
    m3 = re.fullmatch(rf"mix\(mix\(0\.0, 1\.0, lambda >= ({_NUM})\), 2\.0, lambda >= ({_NUM})\)", s)
    ml = re.fullmatch(rf"clamp\(floor\(log2\(lambda \* ({_NUM}) \+ ({_NUM})\)\), 0\.0, ({_NUM})\)", s)
    if m4:
        strength = ("thr", (float(m4.group(1)), float(m4.group(3)), float(m4.group(2))))
    elif m3:
        strength = ("thr", (float(m3.group(1)), float(m3.group(2))))
    elif ml:
        strength = ("log2", float(ml.group(1)), float(ml.group(3)))
    else:
        raise HookParseError(path, p.line, f"unrecognised strength expression {s!r}")
    mc, _ = _find(p.body, rf"float coherence = mix\(mix\(0\.0, 1\.0, mu >= ({_NUM})\), 2\.0, mu >= ({_NUM})\);", path, p, "coherence line")
    coherence = (float(mc.group(1)), float(mc.group(2)))
    mk, ln = _find(p.body, r"float coord_y = \(\(angle \* (\d+)\.0 \+ strength\) \* 3\.0 \+ coherence( \+ 0\.5)?\) / (\d+)\.0;", path, p, "coord_y line")
    nstr = int(mk.group(1))
    rows = int(mk.group(3))
    ns = int(strength[2]) + 1 if strength[0] == "log2" else len(strength[1]) + 1
    if nstr != ns or rows != 24 * ns * 3:
        raise HookParseError(path, ln, f"key layout {nstr}/{rows} does not match strength levels {ns}")
    return strength, coherence, mk.group(2) is not None


def _parse_abd_weights(p: Pass) -> List[float]:
    return [float(m.group(1)) for m in
            (re.match(rf"abd \+= vec3\(gx \* gx, gx \* gy, gy \* gy\) \* ({_NUM});", ln) for ln in p.body) if m]


def _parse_linear(expr: str) -> Tuple[Dict[int, float], float]:
    """'(-s10+8.0*s9-8.0*s7+s6)/12.0' -> ({10:-1, 9:8, 7:-8, 6:1}, 12)."""
    expr = expr.strip()
    m = re.fullmatch(rf"\((.*)\)(?:/({_NUM}))?", expr)
    if not m:
        raise ValueError(expr)
    inner, div = m.group(1), float(m.group(2) or 1.0)
    coefs: Dict[int, float] = {}
    pos = 0
    for t in re.finditer(r"([+-]?)(?:(\d+\.\d*)\*)?(?:luma|sample)(\d+)(?:\.x)?", inner):
        if t.start() != pos:
            raise ValueError(expr)
        pos = t.end()
        c = float(t.group(2) or 1.0) * (-1.0 if t.group(1) == "-" else 1.0)
        coefs[int(t.group(3))] = coefs.get(int(t.group(3)), 0.0) + c
    if pos != len(inner):
        raise ValueError(expr)
    return coefs, div


def _check_root_gradients(p: Pass, path: str, family: str, radius: int,
                          sample_pos: Dict[int, Tuple[float, float]]) -> None:
    """Compare every ``gx``/``gy`` stencil of a root pass with the rule.

    ``sample_pos`` maps the pass's sample index to its physical position
    in window coordinates (already rotated for the ravu lattice passes).
    """
    n = geo.window_size(family, radius)
    points = geo.grad_points(family, radius)
    # inverse map: window grid position -> sample index
    grid: Dict[Tuple[int, int], int] = {}
    for idx, (wx, wy) in sample_pos.items():
        grid[(int(round(wx)), int(round(wy)))] = idx
    gx_lines = [(k, ln) for k, ln in enumerate(p.body) if ln.startswith("gx = ")]
    gy_lines = [(k, ln) for k, ln in enumerate(p.body) if ln.startswith("gy = ")]
    if len(gx_lines) != len(points) or len(gy_lines) != len(points):
        raise HookParseError(path, p.line, f"expected {len(points)} gradient points, found {len(gx_lines)}")
    for (px, py), (kx, lx), (ky, ly) in zip(points, gx_lines, gy_lines):
        for axis, (k, ln) in (("x", (kx, lx)), ("y", (ky, ly))):
            try:
                coefs, div = _parse_linear(ln.split("=", 1)[1].rstrip(";"))
            except ValueError:
                raise HookParseError(path, p.body_line + k, f"unparsable gradient {ln!r}")
            want_c, want_div = geo.derivative(family, radius, px if axis == "x" else py)
            want = {}
            for off, c in want_c.items():
                wpos = (off, py) if axis == "x" else (px, off)
                if wpos not in grid:
                    raise HookParseError(path, p.body_line + k, f"rule needs window position {wpos} with no sample")
                want[grid[wpos]] = c
            if want != coefs or want_div != div:
                raise HookParseError(path, p.body_line + k,
                                     f"gradient at {(px, py)} axis {axis}: file {coefs}/{div}, rule {want}/{want_div}")


def _root_sample_map(p: Pass, path: str) -> Dict[int, Tuple[str, float, float]]:
    """sample index -> (source texture, dx, dy) from the declarations."""
    out: Dict[int, Tuple[str, float, float]] = {}
    rx = re.compile(rf"^(?:float|vec3) (?:luma|sample)(\d+) = (\w+?)_texOff\(vec2\(({_NUM}), ({_NUM})\)\)\.(?:x|xyz);")
    rz = re.compile(rf"^(?:float|vec3) sample(\d+) = HOOKED_tex\(\(pos \+ vec2\(({_NUM}),({_NUM})\)\) \* HOOKED_pt\)\.(?:x|xyz);")
    for ln in p.body:
        m = rx.match(ln)
        if m:
            out[int(m.group(1))] = (m.group(2), float(m.group(3)), float(m.group(4)))
            continue
        m = rz.match(ln)
        if m:
            out[int(m.group(1))] = ("HOOKED", float(m.group(2)), float(m.group(3)))
    return out


def _check_lut_columns_lite(p: Pass, path: str, lut_name: str, ncols: int, S: int,
                            three_x: bool) -> Optional[np.ndarray]:
    """Check the lite/3x filter texture layout; return the AR column mask."""
    body = p.body
    cols_seen = []
    for k, ln in enumerate(body):
        m = re.match(rf"w[01]? = texture\({lut_name}, vec2\(({_NUM}), coord_y\)\);", ln)
        if m:
            x = float(m.group(1))
            cols_seen.append(int(round(x * ncols - 0.5)))
    if cols_seen != list(range(ncols)):
        raise HookParseError(path, p.line, f"LUT columns read in order {cols_seen[:6]}..., expected 0..{ncols - 1}")
    # sample pairing: lite 'res += lumaA * w + lumaB * w.wzyx;'
    pairs = []
    for ln in body:
        m = re.match(r"res0? \+= (?:luma|sample)(\d+) \* w0? \+ (?:luma|sample)(\d+) \* w[01]?\.wzyx;", ln)
        if m:
            pairs.append((int(m.group(1)), int(m.group(2))))
    npairs = S // 2
    if pairs != [(c, S - 1 - c) for c in range(npairs)]:
        raise HookParseError(path, p.line, "tap pairing differs from t <-> S-1-t")
    ar = np.zeros(ncols if not three_x else ncols // 2, dtype=bool)
    for ln in body:
        m = re.match(r"cg4 = vec4\(0\.1 \+ (?:luma|sample)(\d+), 1\.1 - (?:luma|sample)\d+, 0\.1 \+ (?:luma|sample)(\d+), 1\.1 - (?:luma|sample)\d+\);", ln)
        if m:
            a, b = int(m.group(1)), int(m.group(2))
            if b != S - 1 - a:
                raise HookParseError(path, p.line, "AR pair is not t <-> S-1-t")
            ar[a] = True
        m = re.match(r"vec2 cg2 = vec2\(0\.1 \+ (?:luma|sample)(\d+), 1\.1 - (?:luma|sample)\d+\);", ln)
        if m:
            ar[int(m.group(1))] = True
    return ar if ar.any() else None


def _ar_strength(passes: List[Pass]) -> float:
    for p in passes:
        for ln in p.body:
            m = re.search(rf"res = mix\(res, clamp\(res, lo, hi\), ({_NUM})\);", ln)
            if m:
                return float(m.group(1))
    return 0.0


# ----------------------------------------------------------- RAVU ----------

def _ravu_from_hook(h: HookFile) -> RavuModel:
    path = h.path
    first = h.passes[0]
    fam_desc, info = _desc_info(first)
    args = [a.strip() for a in info["args"].split(",")]
    radius = None
    channels = "luma"
    for a in args:
        if re.fullmatch(r"r\d", a):
            radius = int(a[1])
        elif a in ("luma", "yuv", "rgb"):
            channels = a
    if radius is None:
        raise HookParseError(path, first.line, "radius missing from DESC")
    family = {"RAVU-Lite": "lite", "RAVU-Lite-AR": "lite", "RAVU": "ravu",
              "RAVU-Zoom": "zoom", "RAVU-Zoom-AR": "zoom", "RAVU-3x": "3x"}[fam_desc]
    lut_names = [t for t in h.textures if not t.endswith("_ar")]
    if len(lut_names) != 1:
        raise HookParseError(path, first.line, f"expected one LUT texture, found {lut_names}")
    lut_tex = h.textures[lut_names[0]]
    ar_tex = h.textures.get(lut_names[0] + "_ar")
    strength, coherence, half = _parse_strength(first, path)
    if half != (family != "zoom"):
        raise HookParseError(path, first.line, "key +0.5 row centring does not match the family")
    rows = 24 * ((int(strength[2]) + 1) if strength[0] == "log2" else len(strength[1]) + 1) * 3
    if lut_tex.height != rows * (9 if family == "zoom" else 1):
        raise HookParseError(path, lut_tex.line, f"LUT height {lut_tex.height} vs {rows} keys")
    weights = _parse_abd_weights(first)
    want_w = geo.grad_weights(family, radius)
    if len(weights) != len(want_w):
        raise HookParseError(path, first.line, f"{len(weights)} gradient weights, rule has {len(want_w)}")
    if h.style == "gather":
        ok = np.allclose(sorted(weights), sorted(want_w), rtol=1e-13, atol=0)
    else:
        ok = np.allclose(weights, want_w, rtol=1e-13, atol=0)
    if not ok:
        raise HookParseError(path, first.line, "gradient weights differ from the Gaussian rule")
    S = geo.window_size(family, radius) ** 2
    ar_taps = None
    if h.style == "root":
        # full stencil check of every keyed pass
        keyed = [p for p in h.passes if any(ln.startswith("gx = ") for ln in p.body)]
        for p in keyed:
            smap = _root_sample_map(p, path)
            if len(smap) != S:
                raise HookParseError(path, p.line, f"{len(smap)} samples declared, window has {S}")
            pos = {}
            rotated = family == "ravu" and p is not keyed[0]
            for idx, (src, dx, dy) in smap.items():
                want = geo.sample_source(family, radius, idx, lattice=_lattice_of(p) if rotated else None)
                if (src, dx, dy) != want:
                    raise HookParseError(path, p.line, f"sample{idx} reads {src}{(dx, dy)}, rule says {want}")
                pos[idx] = geo.window_pos(family, radius, idx)
            _check_root_gradients(p, path, family, radius, pos)
            if family in ("lite", "3x"):
                ncols = lut_tex.width
                ar_taps = _check_lut_columns_lite(p, path, lut_tex.name, ncols, S, family == "3x")
        if family == "lite" and ar_taps is not None:
            want_ar = geo.lite_ar_taps(radius)
            if not np.array_equal(ar_taps, want_ar):
                raise HookParseError(path, first.line, "anti-ringing tap set differs from the rule")
    ar = _ar_strength(h.passes)
    if family == "lite" and ar:
        ar_taps = geo.lite_ar_taps(radius)
    if family == "zoom" and (ar_tex is not None) != bool(ar):
        raise HookParseError(path, first.line, "zoom AR strength and _ar LUT must come together")
    name = os.path.basename(path)[:-5] if path.endswith(".hook") else path
    return RavuModel(name=name, family=family, radius=radius, channels=channels, ar=ar,
                     lut=lut_tex.data, lut_ar=None if ar_tex is None else ar_tex.data,
                     grad_weights=np.asarray(want_w, dtype=np.float64), strength=strength,
                     coherence=coherence, passes=h.passes, style=h.style, path=path,
                     ar_taps=ar_taps)


def _lattice_of(p: Pass) -> str:
    if p.save == "ravu_int10":
        return "int10"
    if p.save == "ravu_int01":
        return "int01"
    raise HookParseError("", p.line, f"ravu lattice pass saving {p.save!r}")


# ----------------------------------------------------------- NNEDI3 --------

def _i2f(i: int) -> float:
    return struct.unpack("<f", struct.pack("<i", i))[0]


def _nnedi3_slots(p: Pass, path: str, style: str, nvec: int) -> List[Tuple[int, int]]:
    """(dx, dy) of each of the 4*nvec scalar sample slots of a double pass."""
    slots: List[Optional[Tuple[int, int]]] = [None] * (4 * nvec)
    if style == "root":
        for ln in p.body:
            m = re.match(rf"samples\[(\d+)\]\[(\d)\] = HOOKED_texOff\(vec2\(({_NUM}), ({_NUM})\)\)\.x;", ln)
            if m:
                slots[int(m.group(1)) * 4 + int(m.group(2))] = (int(float(m.group(3))), int(float(m.group(4))))
    elif style == "compute":
        mh, _ = _find(p.body, r"int local_pos = int\(gl_LocalInvocationID\.x\) \* (\d+) \+ int\(gl_LocalInvocationID\.y\);", path, p, "tile stride")
        H = int(mh.group(1))
        mo, _ = _find(p.body, r"group_base\.x\+x-\((\d+)\)\)\+0\.5,float\(group_base\.y\+y-\((\d+)\)\)", path, p, "tile origin")
        ox, oy = int(mo.group(1)), int(mo.group(2))
        for ln in p.body:
            m = re.match(r"samples\[(\d+)\]\[(\d)\] = inp\[local_pos \+ (\d+)\];", ln)
            if m:
                k = int(m.group(3))
                slots[int(m.group(1)) * 4 + int(m.group(2))] = (k // H - ox, k % H - oy)
    else:  # gather: components x,y,z,w = (0,1),(1,1),(1,0),(0,0) from the offset
        comp = [(0, 1), (1, 1), (1, 0), (0, 0)]
        for ln in p.body:
            m = re.match(r"samples\[(\d+)\] = HOOKED_mul \* textureGatherOffset\(HOOKED_raw, HOOKED_pos, ivec2\((-?\d+), (-?\d+)\), 0\);", ln)
            if m:
                i, ox, oy = int(m.group(1)), int(m.group(2)), int(m.group(3))
                for c, (ax, ay) in enumerate(comp):
                    slots[i * 4 + c] = (ox + ax, oy + ay)
    if any(s is None for s in slots):
        raise HookParseError(path, p.line, "could not place every NNEDI3 sample slot")
    return slots  # type: ignore[return-value]


def _nnedi3_weights(p: Pass, path: str, nvec: int, nns: int):
    rows = [(k, ln) for k, ln in enumerate(p.body) if ln.startswith("sum1=")]
    if len(rows) != nns:
        raise HookParseError(path, p.line, f"{len(rows)} neuron lines, DESC says nns{nns}")
    A = np.zeros((nns, 4 * nvec), dtype=np.float32)
    B = np.zeros((nns, 4 * nvec), dtype=np.float32)
    ba = np.zeros(nns, dtype=np.float32)
    bb = np.zeros(nns, dtype=np.float32)
    wrx = re.compile(r"W\((\d+),(-?\d+),(-?\d+),(-?\d+),(-?\d+)\)")
    for j, (k, ln) in enumerate(rows):
        m = re.fullmatch(r"sum1=(.*);sum2=(.*);WS\((-?\d+),(-?\d+)\);", ln)
        if not m:
            raise HookParseError(path, p.body_line + k, "malformed neuron line")
        for dst, part in ((A, m.group(1)), (B, m.group(2))):
            terms = wrx.findall(part)
            if len(terms) != nvec:
                raise HookParseError(path, p.body_line + k, "neuron does not cover every sample vector")
            for t in terms:
                i = int(t[0])
                for c in range(4):
                    dst[j, 4 * i + c] = _i2f(int(t[1 + c]))
        ba[j] = _i2f(int(m.group(3)))
        bb[j] = _i2f(int(m.group(4)))
    return A, B, ba, bb


def _nnedi3_from_hook(h: HookFile) -> Nnedi3Model:
    path = h.path
    dy_pass = next((p for p in h.passes if "double_y" in p.desc), None)
    dx_pass = next((p for p in h.passes if "double_x" in p.desc), None)
    if dy_pass is None or dx_pass is None:
        raise HookParseError(path, h.passes[0].line, "NNEDI3 file needs double_y and double_x passes")
    m = re.search(r"nns(\d+), win(\d+)x(\d+)", dy_pass.desc)
    if not m:
        raise HookParseError(path, dy_pass.line, "nns/win missing from DESC")
    nns, ww, wh = int(m.group(1)), int(m.group(2)), int(m.group(3))
    T = ww * wh
    nvec = T // 4
    taps = geo.nnedi3_taps(ww, wh)
    index = {tuple(t): i for i, t in enumerate(taps)}
    banks = []
    for p, transpose in ((dy_pass, False), (dx_pass, True)):
        slots = _nnedi3_slots(p, path, h.style, nvec)
        A, B, ba, bb = _nnedi3_weights(p, path, nvec, nns)
        perm = np.empty(T, dtype=np.int64)
        for s, (dx, dy) in enumerate(slots):
            key = (dy, dx) if transpose else (dx, dy)
            if key not in index:
                raise HookParseError(path, p.line, f"sample offset {(dx, dy)} outside the {ww}x{wh} window")
            perm[index[key]] = s
        banks.append((A[:, perm].T.copy(), B[:, perm].T.copy(), ba, bb))
    (A, B, ba, bb), (A2, B2, ba2, bb2) = banks
    if not (np.array_equal(A, A2) and np.array_equal(B, B2) and np.array_equal(ba, ba2) and np.array_equal(bb, bb2)):
        raise HookParseError(path, dx_pass.line, "double_x weights are not the transpose of double_y")
    name = os.path.basename(path)[:-5] if path.endswith(".hook") else path
    return Nnedi3Model(name=name, nns=nns, win_w=ww, win_h=wh, taps=np.asarray(taps, dtype=np.int32),
                       weights_a=A, weights_b=B, bias_a=ba, bias_b=bb, passes=h.passes,
                       style=h.style, path=path)


def model_from_hook(h: HookFile):
    fam, _ = _desc_info(h.passes[0])
    if fam == "NNEDI3":
        return _nnedi3_from_hook(h)
    return _ravu_from_hook(h)


def load_model(path: str):
    return model_from_hook(parse_hook_file(path))


# ----------------------------------------------------------- WHEN ----------

def pass_enabled(p: Pass, in_w: int, in_h: int, out_w: int, out_h: int, luma_w: int = 1) -> bool:
    """Evaluate a pass's ``//!WHEN`` for a given input/output size."""
    if p.when is None:
        return True
    env = {"HOOKED.w": in_w, "HOOKED.h": in_h, "OUTPUT.w": out_w, "OUTPUT.h": out_h,
           "LUMA.w": luma_w, "LUMA.h": luma_w, "NATIVE.w": in_w, "NATIVE.h": in_h,
           "MAIN.w": in_w, "MAIN.h": in_h}
    return rpn_eval(p.when, env) != 0.0
