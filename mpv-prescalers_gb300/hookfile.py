"""Parser for mpv user-shader ``.hook`` files (the prescaler file format).

A ``.hook`` file is a sequence of blocks.  A *pass* block starts with
``//!DESC`` and carries directives (``//!HOOK``, ``//!BIND``, ``//!SAVE``,
``//!WIDTH``/``//!HEIGHT`` as RPN, ``//!OFFSET``, ``//!WHEN`` as RPN,
``//!COMPONENTS``, ``//!COMPUTE``) followed by GLSL.  A *texture* block starts
with ``//!TEXTURE`` and carries ``//!SIZE w h``, ``//!FORMAT``, ``//!FILTER``
and one line of hex: little-endian float32 texels, 4 components each, row
after row (x fastest).  Examples of both: ``ravu-lite-r3.hook:15-131`` (two
passes), ``ravu-lite-r3.hook:132-136`` (texture block),
``compute/ravu-r3.hook:155-164`` (compute directives).

This module only splits and decodes; :mod:`.models` turns the result into
the canonical prescaler models the CUDA library consumes.
"""
from __future__ import annotations

import dataclasses
import os
import re
from typing import Dict, List, Optional, Tuple

import numpy as np


class HookParseError(ValueError):
    """A ``.hook`` file that does not follow the grammar; names file:line."""

    def __init__(self, path: str, line: int, msg: str):
        super().__init__(f"{path}:{line}: {msg}")
        self.path = path
        self.line = line


@dataclasses.dataclass
class Texture:
    name: str
    width: int
    height: int
    fmt: str
    filt: str
    data: np.ndarray          # float32 [height][width][4]
    line: int                 # line of the //!TEXTURE directive


@dataclasses.dataclass
class Pass:
    desc: str
    hooks: List[str]
    binds: List[str]
    save: Optional[str]
    width: Optional[str]      # RPN text or None (same as HOOKED)
    height: Optional[str]
    offset: Optional[Tuple[float, float] | str]
    when: Optional[str]
    components: Optional[int]
    compute: Optional[Tuple[int, ...]]
    body: List[str]           # GLSL lines
    line: int                 # line of //!DESC
    body_line: int            # line number of body[0]

    def body_text(self) -> str:
        return "\n".join(self.body)


@dataclasses.dataclass
class HookFile:
    path: str
    passes: List[Pass]
    textures: Dict[str, Texture]
    preamble: List[str] = dataclasses.field(default_factory=list)   # lines before the first block

    @property
    def style(self) -> str:
        """'compute', 'gather' or 'root' (plain fragment shaders)."""
        if any(p.compute for p in self.passes):
            return "compute"
        if any("textureGatherOffset" in p.body_text() for p in self.passes):
            return "gather"
        return "root"


_FORMAT_COMPONENTS = {"rgba16f": 4, "rgba16hf": 4, "rgba32f": 4}


def _decode_texture(path: str, line: int, name: str, w: int, h: int,
                    fmt: str, hexline: str) -> np.ndarray:
    ncomp = _FORMAT_COMPONENTS.get(fmt)
    if ncomp is None:
        raise HookParseError(path, line, f"unsupported texture FORMAT {fmt!r}")
    hexline = hexline.strip()
    need = w * h * ncomp * 4 * 2
    if len(hexline) != need:
        raise HookParseError(
            path, line,
            f"texture {name}: {len(hexline)} hex chars, SIZE {w}x{h} "
            f"{fmt} as float32 needs {need}")
    try:
        raw = bytes.fromhex(hexline)
    except ValueError as e:
        raise HookParseError(path, line, f"texture {name}: bad hex ({e})")
    return np.frombuffer(raw, dtype="<f4").reshape(h, w, ncomp).copy()


def parse_hook_text(text: str, path: str = "<string>") -> HookFile:
    lines = text.split("\n")
    passes: List[Pass] = []
    textures: Dict[str, Texture] = {}
    cur: Optional[dict] = None
    tex: Optional[dict] = None
    preamble: List[str] = []
    seen_block = False

    def close_pass():
        nonlocal cur
        if cur is not None:
            body = cur["body"]
            while body and not body[-1].strip():
                body.pop()
            passes.append(Pass(**cur))
            cur = None

    i = 0
    n = len(lines)
    while i < n:
        ln = lines[i]
        lineno = i + 1
        if ln.startswith("//!"):
            m = re.match(r"//!(\w+)\s*(.*)$", ln)
            if not m:
                raise HookParseError(path, lineno, "malformed directive")
            key, val = m.group(1), m.group(2).strip()
            seen_block = seen_block or key in ("DESC", "TEXTURE")
            if key == "DESC":
                close_pass()
                tex = None
                cur = dict(desc=val, hooks=[], binds=[], save=None, width=None,
                           height=None, offset=None, when=None, components=None,
                           compute=None, body=[], line=lineno, body_line=lineno + 1)
            elif key == "TEXTURE":
                close_pass()
                tex = dict(name=val, line=lineno, size=None, fmt=None, filt="NEAREST")
            elif tex is not None:
                if key == "SIZE":
                    parts = val.split()
                    if len(parts) != 2:
                        raise HookParseError(path, lineno, "only 2-D textures are supported")
                    tex["size"] = (int(parts[0]), int(parts[1]))
                elif key == "FORMAT":
                    tex["fmt"] = val
                elif key == "FILTER":
                    tex["filt"] = val
                elif key in ("BORDER",):
                    tex[key.lower()] = val
                else:
                    raise HookParseError(path, lineno, f"unknown texture directive {key}")
                # the payload follows the last directive
                if i + 1 < n and not lines[i + 1].startswith("//!"):
                    if tex["size"] is None or tex["fmt"] is None:
                        raise HookParseError(path, lineno, "texture payload before SIZE/FORMAT")
                    w, h = tex["size"]
                    data = _decode_texture(path, i + 2, tex["name"], w, h, tex["fmt"], lines[i + 1])
                    textures[tex["name"]] = Texture(tex["name"], w, h, tex["fmt"], tex["filt"],
                                                    data, tex["line"])
                    tex = None
                    i += 1
            elif cur is not None:
                if key == "HOOK":
                    cur["hooks"].append(val)
                elif key == "BIND":
                    cur["binds"].append(val)
                elif key == "SAVE":
                    cur["save"] = val
                elif key == "WIDTH":
                    cur["width"] = val
                elif key == "HEIGHT":
                    cur["height"] = val
                elif key == "OFFSET":
                    if val == "ALIGN":
                        cur["offset"] = "ALIGN"
                    else:
                        a, b = val.split()
                        cur["offset"] = (float(a), float(b))
                elif key == "WHEN":
                    cur["when"] = val
                elif key == "COMPONENTS":
                    cur["components"] = int(val)
                elif key == "COMPUTE":
                    cur["compute"] = tuple(int(v) for v in val.split())
                else:
                    raise HookParseError(path, lineno, f"unknown pass directive {key}")
                cur["body_line"] = lineno + 1
            else:
                raise HookParseError(path, lineno, f"directive {key} outside a block")
        elif cur is not None:
            cur["body"].append(ln)
        elif tex is not None and ln.strip():
            raise HookParseError(path, lineno, "unexpected text inside texture block")
        elif not seen_block:
            preamble.append(ln)
        i += 1
    close_pass()
    if not passes:
        raise HookParseError(path, 1, "no //!DESC pass blocks")
    for p in passes:
        for b in p.binds:
            if b in ("HOOKED",) or b in textures:
                continue
            if any(q.save == b for q in passes):
                continue
            raise HookParseError(path, p.line, f"pass binds unknown texture {b!r}")
    return HookFile(path=path, passes=passes, textures=textures, preamble=preamble)


def parse_hook_file(path: str) -> HookFile:
    with open(path, "r", encoding="utf-8") as f:
        return parse_hook_text(f.read(), os.fspath(path))


# ---------------------------------------------------------------- RPN ------

def rpn_eval(expr: str, env: Dict[str, float]) -> float:
    """Evaluate a WIDTH/HEIGHT/WHEN expression (reverse Polish notation).

    Tokens are numbers, ``TEX.w``/``TEX.h`` (looked up in ``env`` as
    ``"TEX.w"``) and the operators ``+ - * / > < = !`` as used by e.g.
    ``ravu-lite-r3.hook:20`` (``HOOKED.w OUTPUT.w / 0.707106 < ... *``).
    Comparisons yield 1.0/0.0; ``!`` is logical not.
    """
    stack: List[float] = []
    for tok in expr.split():
        if tok in ("+", "-", "*", "/", ">", "<", "="):
            if len(stack) < 2:
                raise ValueError(f"RPN underflow at {tok!r} in {expr!r}")
            b = stack.pop()
            a = stack.pop()
            if tok == "+":
                stack.append(a + b)
            elif tok == "-":
                stack.append(a - b)
            elif tok == "*":
                stack.append(a * b)
            elif tok == "/":
                stack.append(a / b)
            elif tok == ">":
                stack.append(1.0 if a > b else 0.0)
            elif tok == "<":
                stack.append(1.0 if a < b else 0.0)
            else:
                stack.append(1.0 if a == b else 0.0)
        elif tok == "!":
            if not stack:
                raise ValueError(f"RPN underflow at '!' in {expr!r}")
            stack.append(0.0 if stack.pop() else 1.0)
        elif re.fullmatch(r"[-+]?\d+(\.\d*)?([eE][-+]?\d+)?", tok):
            stack.append(float(tok))
        else:
            if tok not in env:
                raise KeyError(f"RPN variable {tok!r} not provided")
            stack.append(float(env[tok]))
    if len(stack) != 1:
        raise ValueError(f"RPN expression {expr!r} left {len(stack)} values")
    return stack[0]
