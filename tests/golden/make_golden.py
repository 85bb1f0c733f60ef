"""Generate golden input/output vectors from the reference's own shader text.

Builds (via ``oracle/build_ref.py``) the ``.hook`` files listed below -- root
fragment-shader files and ``compute/`` compute-shader files (ravu-3x exists
only there) -- as C++ in double precision, runs them on small seeded
synthetic planes and a few edge shapes, and stores
``tests/golden/<hook>__<case>.npz`` (``compute/x`` is stored as ``compute.x``)
with

* ``input``  float32 ``[C][H][W]`` (the exact values fed to the shader),
* ``output`` float64 ``[C][OH][OW]`` (what the shader text computed),
* ``out_w``, ``out_h``.

Needs the reference checkout (default ``/root/reference``) and g++; run from
the repository root::

    python tests/golden/make_golden.py [--force]

Existing files are kept unless ``--force`` is given (each case's seed is
fixed by its position in CASES, so appended cases leave earlier ones as they
were).
"""
from __future__ import annotations

import ctypes
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import build_ref  # noqa: E402


def _synth():
    root = os.path.join(REPO, "mpv-prescalers_gb300")
    spec = importlib.util.spec_from_file_location("_synth", os.path.join(root, "synth.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


# (hook stem, channels, [(case, H, W, scale or (OW, OH))])
CASES = [
    ("ravu-lite-r2", "luma", [("synth", 13, 19, 2), ("tiny", 3, 5, 2)]),
    ("ravu-lite-r3", "luma", [("synth", 13, 19, 2), ("tiny", 1, 1, 2), ("const", 7, 6, 2)]),
    ("ravu-lite-r4", "luma", [("synth", 13, 19, 2)]),
    ("ravu-lite-ar-r2", "luma", [("synth", 13, 19, 2)]),
    ("ravu-lite-ar-r3", "luma", [("synth", 13, 19, 2), ("tiny", 3, 5, 2)]),
    ("ravu-lite-ar-r4", "luma", [("synth", 13, 19, 2)]),
    ("ravu-r2", "luma", [("synth", 13, 19, 2)]),
    ("ravu-r3", "luma", [("synth", 13, 19, 2), ("tiny", 3, 5, 2)]),
    ("ravu-r4", "luma", [("synth", 13, 19, 2)]),
    ("ravu-r2-rgb", "rgb", [("synth", 11, 14, 2)]),
    ("ravu-r3-rgb", "rgb", [("synth", 11, 14, 2)]),
    ("ravu-r3-yuv", "yuv", [("synth", 11, 14, 2)]),
    ("ravu-r4-yuv", "yuv", [("synth", 11, 14, 2)]),
    ("ravu-zoom-r2", "luma", [("x1.5", 12, 16, (24, 18)), ("x2.25", 9, 13, (29, 20))]),
    ("ravu-zoom-r3", "luma", [("x1.75", 12, 16, (28, 21))]),
    ("ravu-zoom-ar-r2", "luma", [("x1.5", 12, 16, (24, 18)), ("x2.25", 9, 13, (29, 20))]),
    ("ravu-zoom-ar-r2-rgb", "rgb", [("x1.5", 10, 12, (18, 15))]),
    ("ravu-zoom-ar-r2-yuv", "yuv", [("x1.75", 10, 12, (21, 17))]),
    ("ravu-zoom-r3-rgb", "rgb", [("x2.25", 8, 10, (22, 18))]),
    ("nnedi3-nns16-win8x4", "luma", [("synth", 13, 19, 2), ("const", 6, 7, 2)]),
    ("nnedi3-nns32-win8x6", "luma", [("synth", 13, 19, 2)]),
    ("nnedi3-nns64-win8x4", "luma", [("synth", 11, 12, 2)]),
    ("nnedi3-nns128-win8x6", "luma", [("synth", 11, 12, 2)]),
    # compute-shader forms: ravu-3x (compute only), and the compute geometry of
    # the other families (shared-memory tiles, two-pass ravu, zoom rectangle)
    ("compute/ravu-3x-r2", "luma", [("synth", 13, 19, 3), ("tiny", 2, 3, 3)]),
    ("compute/ravu-3x-r3", "luma", [("synth", 13, 19, 3)]),
    ("compute/ravu-3x-r4", "luma", [("synth", 11, 14, 3)]),
    ("compute/ravu-3x-r2-yuv", "yuv", [("synth", 11, 14, 3)]),
    ("compute/ravu-3x-r3-rgb", "rgb", [("synth", 11, 14, 3)]),
    ("compute/ravu-3x-r4-yuv", "yuv", [("synth", 9, 12, 3)]),
    ("compute/ravu-3x-r4-rgb", "rgb", [("synth", 9, 12, 3)]),
    ("compute/ravu-lite-ar-r3", "luma", [("synth", 13, 19, 2)]),
    ("compute/ravu-r3", "luma", [("synth", 13, 19, 2)]),
    ("compute/ravu-r2-yuv", "yuv", [("synth", 11, 14, 2)]),
    ("compute/ravu-zoom-ar-r2", "luma", [("x1.5", 12, 16, (24, 18))]),
    ("compute/nnedi3-nns32-win8x6", "luma", [("synth", 13, 19, 2)]),
]


def make_input(synth, channels: str, case: str, H: int, W: int, seed: int) -> np.ndarray:
    if case == "const":
        return np.full((1 if channels == "luma" else 3, H, W), 0.3725, dtype=np.float32)
    return synth.frame(H, W, seed, channels).astype(np.float32)


def run_ref(so: str, x: np.ndarray, ow: int, oh: int) -> np.ndarray:
    lib = ctypes.CDLL(so)
    lib.ref_run.restype = ctypes.c_int
    C, H, W = x.shape
    xin = np.ascontiguousarray(x, dtype=np.float64)
    cap = C * ow * oh
    out = np.zeros(cap)
    dims = (ctypes.c_int * 2)()
    rc = lib.ref_run(xin.ctypes.data_as(ctypes.c_void_p), C, H, W, ow, oh,
                     out.ctypes.data_as(ctypes.c_void_p), cap, dims)
    if rc != 0:
        raise RuntimeError(f"ref_run failed for {so}")
    return out[: C * dims[0] * dims[1]].reshape(C, dims[0], dims[1])


def main(argv=None) -> int:
    force = "--force" in (sys.argv[1:] if argv is None else argv)
    synth = _synth()
    todo, seed = [], 7
    for stem, channels, cases in CASES:
        for case, H, W, scale in cases:
            seed += 1
            fn = os.path.join(HERE, f"{build_ref.out_stem(stem)}__{case}.npz")
            if force or not os.path.exists(fn):
                todo.append((stem, channels, case, H, W, scale, seed, fn))
    if not todo:
        return 0
    if build_ref.main(sorted({t[0] for t in todo})) != 0:
        return 1
    for stem, channels, case, H, W, scale, seed, fn in todo:
        so = os.path.join(build_ref.OUT, build_ref.out_stem(stem) + ".so")
        x = make_input(synth, channels, case, H, W, seed)
        ow, oh = (W * scale, H * scale) if isinstance(scale, int) else scale
        y = run_ref(so, x, ow, oh)
        np.savez_compressed(fn, input=x, output=y, out_w=ow, out_h=oh)
        print(f"{os.path.relpath(fn, REPO)}: in {x.shape} -> out {y.shape}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
