"""The FP64 oracle against the reference's own shader text (golden vectors)
and against the invariants the shaders guarantee."""
import glob
import os

import numpy as np
import pytest

import oracle
from mpv_prescalers_gb300 import models, synth

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def _model(reference_dir, stem):
    """The model of a reference file stem; golden files name compute/x as compute.x."""
    return models.load_model(os.path.join(reference_dir, stem.replace(".", "/") + ".hook"))


def _run(m, x, out_w, out_h):
    if m.kind == "nnedi3":
        return oracle.nnedi3_upscale(m, x)
    return oracle.keyed_upscale(m, x, (out_w, out_h))


def test_golden_vectors_exist():
    assert len(GOLDEN) >= 44
    assert sum("compute.ravu-3x" in p for p in GOLDEN) >= 8   # ravu-3x exists only as compute shaders


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference_shader_text(reference_dir, path):
    g = np.load(path)
    stem = os.path.basename(path).split("__")[0]
    m = _model(reference_dir, stem)
    y, _ = _run(m, g["input"], int(g["out_w"]), int(g["out_h"]))
    assert y.shape == g["output"].shape
    np.testing.assert_allclose(y, g["output"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("stem", ["ravu-lite-r3", "ravu-lite-ar-r3", "ravu-r3", "ravu-zoom-ar-r2"])
def test_constant_plane_gives_key_zero(reference_dir, stem):
    m = _model(reference_dir, stem)
    c = np.full((1, 9, 11), 0.4375)
    y, info = _run(m, c, 17, 14)
    assert np.all(info["key"] == 0)
    # output = c * sum(weights of row 0)
    assert np.abs(y - 0.4375).max() < 2e-4


def test_nnedi3_constant_plane_is_exact(reference_dir):
    m = _model(reference_dir, "nnedi3-nns64-win8x4")
    y, _ = oracle.nnedi3_upscale(m, np.full((1, 6, 9), 0.3))
    assert np.array_equal(y, np.full((1, 12, 18), 0.3))


def test_ravu_lite_180_degree_rotation_equivariance(reference_dir):
    m = _model(reference_dir, "ravu-lite-r3")
    x = synth.luma_plane(17, 23, 5)
    y, _ = oracle.ravu_lite(m, x)
    yr, _ = oracle.ravu_lite(m, x[::-1, ::-1].copy())
    np.testing.assert_allclose(yr[0], y[0, ::-1, ::-1], atol=1e-12)


def test_forced_keys_reproduce_own_keys(reference_dir):
    m = _model(reference_dir, "ravu-r3")
    x = synth.luma_plane(12, 15, 3)
    y, info = oracle.ravu_lattice(m, x)
    y2, _ = oracle.ravu_lattice(m, x, keys=info["key"])
    assert np.array_equal(y, y2)


def test_planted_oracle_mistake_is_caught(reference_dir):
    """A wrong stencil in the oracle must break the golden comparison."""
    g = np.load([p for p in GOLDEN if "ravu-lite-r3__synth" in p][0])
    m = _model(reference_dir, "ravu-lite-r3")
    orig = oracle.ravu._deriv

    def wrong(lum, n, four, px, py, axis):
        v = orig(lum, n, four, px, py, axis)
        return v * 1.01 if (px, py) == (2, 2) else v
    oracle.ravu._deriv = wrong
    try:
        y, _ = oracle.ravu_lite(m, g["input"])
    finally:
        oracle.ravu._deriv = orig
    assert np.abs(y - g["output"]).max() > 1e-6


def test_mpv_form_rounds_luts_to_fp16_and_steps_zoom_fractions():
    from mpv_prescalers_gb300 import synth
    m = synth.synthetic_model("ravu-zoom-ar-r2")
    f = oracle.mpv_form(m)
    assert np.array_equal(f.lut, m.lut.astype(np.float16).astype(np.float32))
    assert np.array_equal(f.lut_ar, m.lut_ar.astype(np.float16).astype(np.float32))
    assert f.lut is not m.lut and m.lut.dtype == np.float32
    x = synth.luma_plane(12, 14, 3)
    a, _ = oracle.ravu_zoom(m, x, 25, 21)
    b, _ = oracle.ravu_zoom(m, x, 25, 21, frac_steps=256)
    c, _ = oracle.ravu_zoom(m, x, 25, 21, frac_steps=1 << 30)
    assert 0 < np.abs(a - b).max() < 1e-2      # 1/256 steps move the weights a little
    assert np.abs(a - c).max() < 1e-7          # ever finer steps converge to exact
