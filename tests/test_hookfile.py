"""Parser and canonical-model tests over every reference ``.hook`` file."""
import glob
import os

import numpy as np
import pytest

from mpv_prescalers_gb300 import hookfile, models


def _all_hooks(ref):
    return sorted(glob.glob(os.path.join(ref, "**", "*.hook"), recursive=True))


def test_every_reference_file_parses_and_matches_the_geometry_rule(reference_dir):
    files = _all_hooks(reference_dir)
    assert len(files) == 99
    kinds = {}
    for f in files:
        m = models.load_model(f)
        kinds[m.family] = kinds.get(m.family, 0) + 1
    assert kinds == {"lite": 18, "ravu": 21, "zoom": 20, "3x": 9, "nnedi3": 30} or sum(kinds.values()) == 99


def test_lut_payload_is_float32_and_rows_sum_to_one(reference_dir):
    m = models.load_model(os.path.join(reference_dir, "ravu-lite-r3.hook"))
    assert m.lut.shape == (288, 13, 4) and m.lut.dtype == np.float32
    S = 25
    s = m.lut[:, :12].sum(1) + m.lut[:, :12, ::-1].sum(1) + m.lut[:, 12]
    assert np.abs(s - 1).max() < 2e-4
    r = models.load_model(os.path.join(reference_dir, "ravu-r3.hook"))
    w = r.lut.reshape(648, -1)
    assert np.abs(2 * w[:, :18].sum(1) - 1).max() < 1e-6
    assert np.all(w[:, 18:] == 0)


@pytest.mark.parametrize("stem", ["ravu-lite-r3", "ravu-lite-ar-r4", "ravu-r3", "ravu-zoom-ar-r2",
                                  "nnedi3-nns32-win8x6", "nnedi3-nns128-win8x4"])
def test_root_compute_gather_parse_to_the_same_model(reference_dir, stem):
    ms = [models.load_model(os.path.join(reference_dir, d, stem + ".hook")) for d in ("", "compute", "gather")]
    a = ms[0]
    for b in ms[1:]:
        if a.kind == "nnedi3":
            assert np.array_equal(a.weights_a, b.weights_a) and np.array_equal(a.weights_b, b.weights_b)
            assert np.array_equal(a.bias_a, b.bias_a) and np.array_equal(a.bias_b, b.bias_b)
        else:
            assert np.array_equal(a.lut, b.lut)
            assert a.strength == b.strength and a.ar == b.ar
            np.testing.assert_array_equal(a.grad_weights, b.grad_weights)


def test_ar_and_plain_variants_share_the_lut(reference_dir):
    a = models.load_model(os.path.join(reference_dir, "ravu-lite-r4.hook"))
    b = models.load_model(os.path.join(reference_dir, "ravu-lite-ar-r4.hook"))
    assert np.array_equal(a.lut, b.lut) and a.ar == 0.0 and b.ar == 0.8


def test_nnedi3_weights_sum_to_zero_per_neuron(reference_dir):
    m = models.load_model(os.path.join(reference_dir, "nnedi3-nns128-win8x6.hook"))
    assert m.weights_a.shape == (48, 128)
    assert np.abs(m.weights_a.astype(np.float64).sum(0)).max() < 1e-6


def test_rpn():
    env = {"HOOKED.w": 960, "HOOKED.h": 540, "OUTPUT.w": 1920, "OUTPUT.h": 1080}
    assert hookfile.rpn_eval("2 HOOKED.w *", env) == 1920
    assert hookfile.rpn_eval("HOOKED.w OUTPUT.w / 0.707106 < HOOKED.h OUTPUT.h / 0.707106 < *", env) == 1.0
    assert hookfile.rpn_eval("HOOKED.w OUTPUT.w / 0.707106 < !", env) == 0.0
    with pytest.raises(KeyError):
        hookfile.rpn_eval("FOO.w 2 *", env)
    with pytest.raises(ValueError):
        hookfile.rpn_eval("2 *", env)


def test_malformed_file_reports_file_and_line():
    text = "//!DESC RAVU-Lite (step1, r3)\n//!HOOK LUMA\n//!BIND nothere\nvec4 hook() { return vec4(0.0); }\n"
    with pytest.raises(hookfile.HookParseError) as e:
        hookfile.parse_hook_text(text, "bad.hook")
    assert "bad.hook:1" in str(e.value)
    text = "//!DESC x\n//!BIND HOOKED\n//!TEXTURE t\n//!SIZE 2 1\n//!FORMAT rgba16f\nabcd\n"
    with pytest.raises(hookfile.HookParseError) as e:
        hookfile.parse_hook_text(text, "bad2.hook")
    assert "bad2.hook:6" in str(e.value)


def test_corrupted_stencil_is_rejected(reference_dir):
    txt = open(os.path.join(reference_dir, "ravu-r3.hook")).read()
    bad = txt.replace("gy = (-sample10+8.0*sample9-8.0*sample7+sample6)/12.0;",
                      "gy = (-sample10+8.0*sample9-8.0*sample7+sample5)/12.0;", 1)
    with pytest.raises(hookfile.HookParseError):
        models.model_from_hook(hookfile.parse_hook_text(bad, "x.hook"))


def test_when_conditions(reference_dir):
    m = models.load_model(os.path.join(reference_dir, "ravu-lite-r3.hook"))
    assert models.pass_enabled(m.passes[0], 960, 540, 1920, 1080)
    assert not models.pass_enabled(m.passes[0], 960, 540, 1200, 700)
    z = models.load_model(os.path.join(reference_dir, "ravu-zoom-r2.hook"))
    assert models.pass_enabled(z.passes[0], 960, 540, 1440, 810)
