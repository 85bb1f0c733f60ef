"""Writer for mpv ``.hook`` files: canonical models back to hook text.

Two levels, both the inverse of the reader:

* :func:`format_hook` turns a parsed :class:`~.hookfile.HookFile` back into
  text.  Pass directives are written in the order the prescaler files use
  (``DESC, HOOK, BIND.., SAVE, WIDTH, HEIGHT, OFFSET, WHEN, COMPONENTS,
  COMPUTE``; e.g. ``ravu-r3.hook:148-154``), ``//!OFFSET`` with ``%f``
  fields, textures after the passes with their float32 texels as one line
  of lower-case little-endian hex (``ravu-lite-r3.hook:132-136``).  For the
  prescaler files this reproduces the file byte for byte.
* :func:`model_to_hook` writes a canonical model's numbers into a template
  file of the same kind: the LUT texture(s) of a :class:`~.models.RavuModel`,
  or the neuron lines (``sum1=W(..)+..;sum2=..;WS(a,b);``, weights as the
  int bits of float32, ``nnedi3-nns16-win8x4.hook:32-34``) of both passes of
  a :class:`~.models.Nnedi3Model`, in each pass's own sample-slot order.
  Everything else (the GLSL, thresholds, stencils) is the template's; a
  model whose structure differs from the template's is refused.

``parse(write(m)) == m`` for every model the reader accepts, which makes the
pair a regression check on the file format.
"""
from __future__ import annotations

import copy
import dataclasses
import struct
from typing import List, Union

import numpy as np

from .hookfile import HookFile, HookParseError, Pass, Texture, parse_hook_text
from . import models as _models


def _fmt_offset(off) -> str:
    if isinstance(off, str):
        return off
    return f"{off[0]:f} {off[1]:f}"


def _pass_lines(p: Pass) -> List[str]:
    out = [f"//!DESC {p.desc}"]
    out += [f"//!HOOK {h}" for h in p.hooks]
    out += [f"//!BIND {b}" for b in p.binds]
    if p.save is not None:
        out.append(f"//!SAVE {p.save}")
    if p.width is not None:
        out.append(f"//!WIDTH {p.width}")
    if p.height is not None:
        out.append(f"//!HEIGHT {p.height}")
    if p.offset is not None:
        out.append(f"//!OFFSET {_fmt_offset(p.offset)}")
    if p.when is not None:
        out.append(f"//!WHEN {p.when}")
    if p.components is not None:
        out.append(f"//!COMPONENTS {p.components}")
    if p.compute is not None:
        out.append("//!COMPUTE " + " ".join(str(v) for v in p.compute))
    return out + list(p.body)


def encode_texels(data: np.ndarray) -> str:
    """float32 texels ``[h][w][4]`` as one line of little-endian hex."""
    return np.ascontiguousarray(data, dtype="<f4").tobytes().hex()


def _texture_lines(t: Texture) -> List[str]:
    if t.data.shape != (t.height, t.width, 4):
        raise ValueError(f"texture {t.name}: data {t.data.shape} vs SIZE {t.width}x{t.height}")
    return [f"//!TEXTURE {t.name}", f"//!SIZE {t.width} {t.height}", f"//!FORMAT {t.fmt}",
            f"//!FILTER {t.filt}", encode_texels(t.data)]


def format_hook(h: HookFile) -> str:
    """The text of a parsed hook file (passes, then textures)."""
    lines = list(h.preamble)
    for p in h.passes:
        lines += _pass_lines(p)
    for t in h.textures.values():
        lines += _texture_lines(t)
    return "\n".join(lines) + "\n"


# ------------------------------------------------------------ models -------

def _f2i(v: float) -> int:
    return struct.unpack("<i", struct.pack("<f", float(v)))[0]


def _ravu_into(m: "_models.RavuModel", t: HookFile) -> HookFile:
    ref = _models.model_from_hook(t)
    if not isinstance(ref, _models.RavuModel):
        raise ValueError("template is not a RAVU file")
    same = (ref.family, ref.radius, ref.channels, ref.ar, ref.strength, ref.coherence) == \
        (m.family, m.radius, m.channels, m.ar, m.strength, m.coherence)
    if not same or not np.array_equal(ref.grad_weights, m.grad_weights):
        raise ValueError(f"model {m.name} does not have the structure of template {t.path}")
    out = copy.deepcopy(t)
    names = [n for n in out.textures if not n.endswith("_ar")]
    for name, data in ((names[0], m.lut), (names[0] + "_ar", m.lut_ar)):
        if data is None:
            if name in out.textures:
                raise ValueError(f"template has {name}, model has no such LUT")
            continue
        tex = out.textures.get(name)
        if tex is None:
            raise ValueError(f"template has no texture {name}")
        data = np.asarray(data, dtype=np.float32)
        if data.shape != tex.data.shape:
            raise ValueError(f"LUT {name}: model {data.shape} vs template {tex.data.shape}")
        out.textures[name] = dataclasses.replace(tex, data=data.copy())
    return out


def _neuron_line(A_slots: np.ndarray, B_slots: np.ndarray, ba: float, bb: float) -> str:
    nvec = A_slots.shape[0] // 4

    def terms(v):
        return "+".join(f"W({i}," + ",".join(str(_f2i(v[4 * i + c])) for c in range(4)) + ")"
                        for i in range(nvec))
    return f"sum1={terms(A_slots)};sum2={terms(B_slots)};WS({_f2i(ba)},{_f2i(bb)});"


def _nnedi3_into(m: "_models.Nnedi3Model", t: HookFile) -> HookFile:
    ref = _models.model_from_hook(t)
    if not isinstance(ref, _models.Nnedi3Model):
        raise ValueError("template is not an NNEDI3 file")
    if (ref.nns, ref.win_w, ref.win_h) != (m.nns, m.win_w, m.win_h):
        raise ValueError(f"model nns{m.nns} win{m.win_w}x{m.win_h} vs template "
                         f"nns{ref.nns} win{ref.win_w}x{ref.win_h}")
    out = copy.deepcopy(t)
    T = m.n_taps
    nvec = T // 4
    index = {tuple(int(v) for v in tap): i for i, tap in enumerate(m.taps)}
    for p in out.passes:
        transpose = "double_x" in p.desc
        if "double_y" not in p.desc and not transpose:
            continue
        slots = _models._nnedi3_slots(p, t.path, t.style, nvec)
        tap_of_slot = [index[(dy, dx) if transpose else (dx, dy)] for dx, dy in slots]
        A = np.asarray(m.weights_a, dtype=np.float32)[tap_of_slot]     # [slots][nns]
        B = np.asarray(m.weights_b, dtype=np.float32)[tap_of_slot]
        rows = [k for k, ln in enumerate(p.body) if ln.startswith("sum1=")]
        if len(rows) != m.nns:
            raise HookParseError(t.path, p.line, f"{len(rows)} neuron lines in template, model has {m.nns}")
        for j, k in enumerate(rows):
            p.body[k] = _neuron_line(A[:, j], B[:, j], m.bias_a[j], m.bias_b[j])
    return out


def model_to_hook(model, template: HookFile) -> HookFile:
    """The template file with ``model``'s LUT(s) or neuron weights written in."""
    if isinstance(model, _models.Nnedi3Model):
        return _nnedi3_into(model, template)
    if isinstance(model, _models.RavuModel):
        return _ravu_into(model, template)
    raise TypeError(f"not a prescaler model: {type(model).__name__}")


def write_hook(obj: Union[HookFile, "_models.RavuModel", "_models.Nnedi3Model"], path: str,
               template: HookFile = None) -> str:
    """Write a hook file (or a model into ``template``) to ``path``; returns the text."""
    h = obj if isinstance(obj, HookFile) else model_to_hook(obj, template)
    text = format_hook(h)
    parse_hook_text(text, path)          # what is written must read back
    with open(path, "w", encoding="utf-8") as f:
        f.write(text)
    return text
