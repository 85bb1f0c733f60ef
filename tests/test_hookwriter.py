"""Hook-file writer: parsed files and canonical models back to ``.hook`` text."""
import glob
import os

import numpy as np
import pytest

from mpv_prescalers_gb300 import hookfile, hookwriter, models

SYNTH = """// preamble comment
// second line

//!DESC Example (step1, r2)
//!HOOK LUMA
//!BIND HOOKED
//!BIND example_lut
//!SAVE example_int
//!WHEN HOOKED.w OUTPUT.w / 0.707106 <
//!COMPONENTS 4
vec4 hook() {
    return HOOKED_texOff(vec2(0.0, 0.0));
}
//!DESC Example (step2, r2)
//!HOOK LUMA
//!BIND HOOKED
//!BIND example_int
//!WIDTH 2 HOOKED.w *
//!HEIGHT 2 HOOKED.h *
//!OFFSET -0.500000 0.000000
//!WHEN HOOKED.w OUTPUT.w / 0.707106 <
//!COMPUTE 32 8
void hook() {
}
//!TEXTURE example_lut
//!SIZE 3 2
//!FORMAT rgba16f
//!FILTER NEAREST
"""


def _synth_text():
    data = np.random.default_rng(3).normal(size=(2, 3, 4)).astype("<f4")
    return SYNTH + data.tobytes().hex() + "\n", data


def test_format_roundtrip_synthetic():
    text, data = _synth_text()
    h = hookfile.parse_hook_text(text, "synth.hook")
    assert h.preamble == ["// preamble comment", "// second line", ""]
    assert hookwriter.format_hook(h) == text
    h2 = hookfile.parse_hook_text(hookwriter.format_hook(h), "synth.hook")
    assert [p.body for p in h2.passes] == [p.body for p in h.passes]
    assert h2.passes[1].offset == (-0.5, 0.0) and h2.passes[1].compute == (32, 8)
    assert np.array_equal(h2.textures["example_lut"].data, data)


def test_texture_data_must_match_its_size():
    text, _ = _synth_text()
    h = hookfile.parse_hook_text(text, "synth.hook")
    h.textures["example_lut"].data = np.zeros((3, 3, 4), np.float32)
    with pytest.raises(ValueError, match="SIZE 3x2"):
        hookwriter.format_hook(h)


def test_write_hook_checks_what_it_writes(tmp_path):
    text, _ = _synth_text()
    h = hookfile.parse_hook_text(text, "synth.hook")
    out = tmp_path / "x.hook"
    assert hookwriter.write_hook(h, str(out)) == text
    assert out.read_text() == text


def _all_hooks(ref):
    return sorted(glob.glob(os.path.join(ref, "**", "*.hook"), recursive=True))


def test_every_reference_file_is_rewritten_byte_for_byte(reference_dir):
    files = _all_hooks(reference_dir)
    assert len(files) == 99
    for f in files:
        text = open(f, encoding="utf-8").read()
        assert hookwriter.format_hook(hookfile.parse_hook_text(text, f)) == text, f


def test_unchanged_models_write_back_the_same_file(reference_dir):
    for f in _all_hooks(reference_dir):
        text = open(f, encoding="utf-8").read()
        h = hookfile.parse_hook_text(text, f)
        m = models.model_from_hook(h)
        assert hookwriter.format_hook(hookwriter.model_to_hook(m, h)) == text, f


@pytest.mark.parametrize("rel", ["ravu-lite-ar-r4.hook", "compute/ravu-r3-rgb.hook", "gather/ravu-zoom-r2.hook",
                                 "compute/ravu-zoom-ar-r2-yuv.hook", "compute/ravu-3x-r3.hook",
                                 "nnedi3-nns32-win8x6.hook", "compute/nnedi3-nns64-win8x4.hook",
                                 "gather/nnedi3-nns16-win8x4.hook"])
def test_changed_models_read_back_exactly(reference_dir, rel):
    f = os.path.join(reference_dir, rel)
    h = hookfile.parse_hook_file(f)
    m = models.model_from_hook(h)
    rng = np.random.default_rng(11)
    if isinstance(m, models.Nnedi3Model):
        m.weights_a = (m.weights_a * rng.uniform(0.5, 1.5, m.weights_a.shape)).astype(np.float32)
        m.weights_b = -m.weights_b
        m.bias_a = (m.bias_a + 0.125).astype(np.float32)
        m.bias_b = rng.normal(size=m.bias_b.shape).astype(np.float32)
    else:
        m.lut = (m.lut + rng.normal(0, 0.01, m.lut.shape)).astype(np.float32)
        if m.lut_ar is not None:
            m.lut_ar = np.abs(m.lut_ar[::-1]).copy()
    text = hookwriter.format_hook(hookwriter.model_to_hook(m, h))
    m2 = models.model_from_hook(hookfile.parse_hook_text(text, f))
    if isinstance(m, models.Nnedi3Model):
        for k in ("weights_a", "weights_b", "bias_a", "bias_b"):
            assert np.array_equal(getattr(m, k), getattr(m2, k)), k
    else:
        assert np.array_equal(m.lut, m2.lut)
        assert (m.lut_ar is None) == (m2.lut_ar is None)
        if m.lut_ar is not None:
            assert np.array_equal(m.lut_ar, m2.lut_ar)


def test_structure_mismatch_is_refused(reference_dir):
    lite3 = models.load_model(os.path.join(reference_dir, "ravu-lite-r3.hook"))
    with pytest.raises(ValueError, match="structure"):
        hookwriter.model_to_hook(lite3, hookfile.parse_hook_file(os.path.join(reference_dir, "ravu-lite-r4.hook")))
    nn16 = models.load_model(os.path.join(reference_dir, "nnedi3-nns16-win8x4.hook"))
    with pytest.raises(ValueError, match="nns16"):
        hookwriter.model_to_hook(nn16, hookfile.parse_hook_file(os.path.join(reference_dir,
                                                                             "nnedi3-nns32-win8x4.hook")))
    with pytest.raises(ValueError, match="not an NNEDI3"):
        hookwriter.model_to_hook(nn16, hookfile.parse_hook_file(os.path.join(reference_dir, "ravu-r2.hook")))
