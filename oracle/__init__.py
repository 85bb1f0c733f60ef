"""FP64 CPU oracle for the prescaler hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in NumPy float64, the per-pixel arithmetic of the
mpv ``.hook`` prescaler shaders (RAVU family and NNEDI3).  It follows the
root (fragment-shader) files of the reference; each function cites the
lines it transcribes.  It is the checker for the CUDA library, and its
NumPy form is also the timed CPU baseline in ``bench.py``.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import it.  The product (``mpv-prescalers_gb300``) never does: its
device path fails loudly when the CUDA library is missing.

Parity pin: ``oracle/build_ref.py`` compiles the reference's own shader
text (the GLSL bodies of the root ``.hook`` files, read in place) as C++
against the GLSL shim in ``oracle/glsl_shim.hpp``; ``tests/golden/`` holds
input/output vectors produced by that build, and ``tests/test_oracle.py``
checks this restatement against them.
"""
from .ravu import ravu_lite, ravu_3x, ravu_lattice, ravu_zoom, keyed_upscale, mpv_form  # noqa: F401
from .nnedi3 import nnedi3_double, nnedi3_upscale  # noqa: F401
