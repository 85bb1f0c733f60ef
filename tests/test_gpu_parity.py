"""GPU parity: the CUDA path (through the C ABI) against the FP64 oracle.

For every family the plain FP32 form must
* pick the same LUT key as the oracle for every key evaluation, except keys
  the oracle flags as sitting on a quantisation boundary (counted), and
* with the keys it picked, produce pixels within 1e-5 max-abs of the
  oracle's arithmetic (the oracle re-run with those keys forced).
"""
import json
import os

import numpy as np
import pytest

import oracle
from mpv_prescalers_gb300 import synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-5          # max-abs, plain FP32 form vs FP64 oracle
TOL_FP16_MAXABS = 2e-3   # FP16 planes vs oracle on the same FP16-rounded input
TOL_FP16_PSNR = 55.0
ULP = 2.0 ** -24
# NNEDI3's only threshold is the variance gate (invstd = 0 below FLT_EPS):
# where FP32 and FP64 take different sides of it, the output moves by at
# most 5 * |vsum / wsum| * std < 5 * sqrt(FLT_EPS) (|vsum / wsum| < 1)
NN_GATE_BOUND = 5.0 * np.sqrt(oracle.nnedi3.FLT_EPS * (1.0 + 1e-3)) + TOL_FP32


def report(tag, stats):
    """Print the parity figures of a case; with $PRESCALER_PARITY_REPORT
    set, also append them as one JSON line to that file."""
    print(f"[parity] {tag}: " + ", ".join(f"{k}={v}" for k, v in stats.items()))
    path = os.environ.get("PRESCALER_PARITY_REPORT")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps({"case": tag, **stats}) + "\n")


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    yield


def _model(name):
    hm, _src = synth.model_for(name)
    return hm


def _psnr(a, b):
    mse = float(np.mean((a - b) ** 2))
    return float("inf") if mse == 0 else 10.0 * np.log10(1.0 / mse)


def _run_gpu(hm, x, out_size, dtype=torch.float32, precision="fp32", int11=None):
    """The GPU's output and raw keys; for the ravu lattice with `int11` a
    list, also the FP32 int11 plane it kept between its two launches (the
    caller scratch passed in opts.scratch)."""
    xt = torch.from_numpy(np.ascontiguousarray(x)).to("cuda", dtype)
    if hm.family != "ravu" or int11 is None:
        y, keys = hm.upscale(xt, out_size=out_size, precision=precision, return_keys=True)
    else:
        C, H, W = xt.shape
        scratch = torch.empty((C, H, W), dtype=torch.float32, device="cuda")
        y = torch.empty((C, 2 * H, 2 * W), dtype=dtype, device="cuda")
        keys = torch.empty(hm.key_shape(W, H, 2 * W, 2 * H), dtype=torch.int32, device="cuda")
        hm.run_raw(list(xt.unbind(0)), list(y.unbind(0)), out_size=(2 * W, 2 * H), precision=precision,
                   keys=keys, scratch=scratch)
        torch.cuda.synchronize()
        int11.append(scratch.double().cpu().numpy())
    torch.cuda.synchronize()
    return y.float().cpu().numpy().astype(np.float64), keys.cpu().numpy()


def flip_mask(family, mism, out_hw):
    """Output pixels whose own LUT key differs from the oracle's: the 2x2
    (3x3) block of a flipped lite (3x) key, the lattice sample of a flipped
    int11 / int10 / int01 key, the pixel of a flipped zoom key."""
    if family == "ravu":
        m = np.zeros(out_hw, dtype=bool)
        m[1::2, 1::2] = mism[0]
        m[0::2, 1::2] = mism[1]
        m[1::2, 0::2] = mism[2]
        return m
    if family in ("lite", "3x"):
        s = 2 if family == "lite" else 3
        return np.repeat(np.repeat(mism, s, 0), s, 1)
    return mism.reshape(out_hw)


def key_stats(kg, info):
    """Key figures of a GPU run against the oracle's keys: evaluations,
    mismatches, boundary keys (the oracle's FP32 budget), mismatches off the
    boundary, and the largest margin (in units of 2^-24 of the structure
    tensor's scale) among the mismatched keys -- the budget the GPU's flips
    actually needed."""
    ref = info["key"]
    mism = kg.reshape(ref.shape) != ref
    bnd = info["boundary"]
    marg = info["margin"][mism] / ULP
    return {"keys": int(ref.size), "mismatch": int(mism.sum()), "boundary": int(bnd.sum()),
            "mismatch_off_boundary": int((mism & ~bnd).sum()),
            "max_mismatch_margin_ulp": float(marg.max()) if marg.size else 0.0,
            "mismatch_rate": float(mism.mean()), "boundary_rate": float(bnd.mean())}


def _check_keyed(hm, x, out_size, tol=TOL_FP32, dtype=torch.float32, precision="fp32", oracle_model=None):
    """Keys and values of the GPU against the oracle.

    For the ravu lattice the int10/int01 passes read int11; they are checked
    on the GPU's own int11 plane (the FP32 plane it keeps between its two
    launches, taken from the scratch the test passes in), so that each pass
    is compared on identical inputs (the int11 pass itself is checked on the
    original input).
    Returns the key figures (``key_stats``) plus the max-abs with identical
    keys and the max-abs and PSNR against the unforced oracle.
    """
    m = hm.model if oracle_model is None else oracle_model
    planes11 = []
    y, kg = _run_gpu(hm, x, out_size, dtype=dtype, precision=precision, int11=planes11)
    over = planes11[0] if planes11 else None
    ref, info = oracle.keyed_upscale(m, x, out_size, int11=over)
    forced, _ = oracle.keyed_upscale(m, x, out_size, keys=kg, int11=over)
    assert y.shape == ref.shape
    err = np.abs(y - forced).max()
    assert err <= tol, f"{m.name}: max-abs {err:.3e} with identical keys"
    st = key_stats(kg, info)
    assert st["mismatch_off_boundary"] == 0, \
        f"{m.name}: {st['mismatch_off_boundary']} key mismatches off the quantisation boundary"
    mism = kg.reshape(info["key"].shape) != info["key"]
    if m.family == "ravu":   # the unforced oracle's own int11 feeds its lattice passes
        ref, _ = oracle.keyed_upscale(m, x, out_size)
    d = np.abs(y - ref)
    keep = ~flip_mask(m.family, mism, y.shape[-2:])
    st.update({"max_abs_forced": float(err), "max_abs": float(d.max()),
               "max_abs_key_matched": float(d[:, keep].max()) if keep.any() else 0.0, "psnr_db": _psnr(y, ref)})
    return st


LITE = ["ravu-lite-r2", "ravu-lite-r3", "ravu-lite-r4", "ravu-lite-ar-r2", "ravu-lite-ar-r3", "ravu-lite-ar-r4"]
SIZES = [(37, 45), (16, 64), (1, 1), (3, 5), (9, 33), (144, 256)]


@pytest.mark.parametrize("name", LITE)
@pytest.mark.parametrize("hw", SIZES, ids=lambda s: f"{s[0]}x{s[1]}")
def test_ravu_lite_fp32(name, hw):
    hm = _model(name)
    H, W = hw
    x = synth.luma_plane(H, W, 11 + H)[None]
    _check_keyed(hm, x, (2 * W, 2 * H))


RAVU = ["ravu-r2", "ravu-r3", "ravu-r4", "ravu-r2-yuv", "ravu-r3-rgb", "ravu-r4-yuv", "ravu-r4-rgb"]


@pytest.mark.parametrize("name", RAVU)
@pytest.mark.parametrize("hw", [(37, 45), (1, 1), (4, 7), (72, 128)], ids=lambda s: f"{s[0]}x{s[1]}")
def test_ravu_lattice_fp32(name, hw):
    hm = _model(name)
    H, W = hw
    x = synth.frame(H, W, 21 + W, hm.channels)
    _check_keyed(hm, x, (2 * W, 2 * H))


THREE = ["ravu-3x-r2", "ravu-3x-r3", "ravu-3x-r4", "ravu-3x-r3-yuv", "ravu-3x-r2-rgb"]


@pytest.mark.parametrize("name", THREE)
@pytest.mark.parametrize("hw", [(29, 41), (2, 3), (64, 96)], ids=lambda s: f"{s[0]}x{s[1]}")
def test_ravu_3x_fp32(name, hw):
    hm = _model(name)
    H, W = hw
    x = synth.frame(H, W, 31 + W, hm.channels)
    _check_keyed(hm, x, (3 * W, 3 * H))


ZOOM = ["ravu-zoom-r2", "ravu-zoom-r3", "ravu-zoom-ar-r2", "ravu-zoom-ar-r2-rgb", "ravu-zoom-ar-r2-yuv",
        "ravu-zoom-r3-rgb", "ravu-zoom-r2-yuv"]


@pytest.mark.parametrize("name", ZOOM)
@pytest.mark.parametrize("geom", [((30, 40), (60, 45)), ((30, 40), (90, 67)), ((17, 23), (40, 39)),
                                  ((48, 64), (96, 128)), ((2, 3), (5, 7))],
                         ids=lambda g: f"{g[0][1]}x{g[0][0]}to{g[1][0]}x{g[1][1]}")
def test_ravu_zoom_fp32(name, geom):
    hm = _model(name)
    (H, W), out_size = geom
    x = synth.frame(H, W, 41 + W, hm.channels)
    _check_keyed(hm, x, out_size)


NN = ["nnedi3-nns16-win8x4", "nnedi3-nns32-win8x6", "nnedi3-nns64-win8x4", "nnedi3-nns128-win8x6",
      "nnedi3-nns256-win8x4", "nnedi3-nns256-win8x6"]


def _nn_pass_check(hm, x, y, axis):
    """One NNEDI3 pass of the GPU (output `y`, [H'][W']) against the oracle
    on the same input `x`: copied pixels exact, interpolated pixels within
    1e-5, except windows on the variance gate (oracle boundary), which are
    held to NN_GATE_BOUND each."""
    ref, info = oracle.nnedi3_upscale(hm.model, x, axes=axis)
    ref = ref[0]
    err = np.abs(y - ref)
    bnd = np.zeros(err.shape, dtype=bool)
    if axis == "y":
        bnd[1::2, :] = info["boundary_y"]
    else:
        bnd[:, 1::2] = info["boundary_x"]
    off = err[~bnd].max() if (~bnd).any() else 0.0
    on = err[bnd].max() if bnd.any() else 0.0
    assert off <= TOL_FP32, f"{hm.name}/{axis}: max-abs {off:.3e} off the variance gate"
    assert on <= NN_GATE_BOUND, f"{hm.name}/{axis}: max-abs {on:.3e} on the variance gate"
    return {"pixels": int(err.size), "gate_windows": int(bnd.sum()), "max_abs": float(off),
            "max_abs_on_gate": float(on), "psnr_db": _psnr(y, ref)}


def _check_nnedi3_fp32(hm, x, axes):
    """The plain FP32 form pass by pass: with both axes, the column pass is
    checked on the GPU's own row-doubled plane (and the two-pass call must
    equal the two single-axis calls bit for bit)."""
    H, W = x.shape
    xt = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    if axes != "yx":
        out_size = (2 * W if axes == "x" else W, 2 * H if axes == "y" else H)
        y = hm.upscale(xt, out_size=out_size).cpu().numpy().astype(np.float64)
        return {axes: _nn_pass_check(hm, x, y, axes)}
    rows = hm.upscale(xt, out_size=(W, 2 * H))
    both = hm.upscale(xt)
    cols = hm.upscale(rows, out_size=(2 * W, 2 * H))
    assert torch.equal(both, cols)
    r = rows.cpu().numpy().astype(np.float64)
    return {"y": _nn_pass_check(hm, x, r, "y"),
            "x": _nn_pass_check(hm, r, cols.cpu().numpy().astype(np.float64), "x")}


@pytest.mark.parametrize("name", NN)
@pytest.mark.parametrize("axes", ["y", "x", "yx"])
def test_nnedi3_fp32(name, axes):
    hm = _model(name)
    H, W = 27, 35
    x = synth.luma_plane(H, W, 51)
    _check_nnedi3_fp32(hm, x, axes)


def test_nnedi3_fp32_on_the_variance_gate():
    """Windows with variance near FLT_EPS: a plane of 0.5 with +-d
    perturbations on a few pixels so that var ~ eps; the bound per gate
    window holds."""
    hm = _model("nnedi3-nns32-win8x4")
    rng = np.random.default_rng(5)
    x = np.full((24, 40), 0.5, dtype=np.float32)
    idx = rng.integers(0, x.size, 40)
    # var of a 32-tap window with one sample at +-d: d^2 (1/32 - 1/32^2) ~ eps
    d = np.float32(np.sqrt(oracle.nnedi3.FLT_EPS / (1 / 32 - 1 / 1024)))
    x.flat[idx] += d * rng.choice([-1.0, 1.0], idx.size).astype(np.float32)
    st = _check_nnedi3_fp32(hm, x, "yx")
    report("nnedi3-nns32-win8x4 variance gate", {k + "_" + a: v for a, d_ in st.items() for k, v in d_.items()})


@pytest.mark.parametrize("name", ["ravu-lite-ar-r3", "ravu-lite-ar-r4", "ravu-r3", "ravu-r4-yuv",
                                  "ravu-zoom-ar-r2-rgb", "ravu-3x-r2"])
def test_fp16_planes_meet_quality_bar(name):
    """FP16 planes (FP32 math): against the oracle on the same FP16-rounded
    input, max-abs <= 2e-3 with the keys the GPU chose, key flips only on
    the quantisation boundary, PSNR >= 55 dB against the unforced oracle."""
    hm = _model(name)
    H, W = 64, 96
    x = synth.frame(H, W, 61, hm.channels)
    x16 = x.astype(np.float16).astype(np.float32)
    out_size = {"zoom": (150, 100), "3x": (3 * W, 3 * H)}.get(hm.family, (2 * W, 2 * H))
    st = _check_keyed(hm, x16, out_size, tol=TOL_FP16_MAXABS, dtype=torch.float16)
    assert st["psnr_db"] >= TOL_FP16_PSNR, f"{name}: PSNR {st['psnr_db']:.1f} dB"


FAST_RAVU = ["ravu-lite-r2", "ravu-lite-ar-r3", "ravu-lite-ar-r4", "ravu-3x-r2", "ravu-3x-r4-yuv", "ravu-3x-r3-rgb",
             "ravu-zoom-r3", "ravu-zoom-ar-r2", "ravu-zoom-ar-r2-rgb", "ravu-r3"]


@pytest.mark.parametrize("name", FAST_RAVU)
def test_ravu_fast_form_is_fp32_math_on_fp16_lut_texels(name):
    """precision="fast" reads the lite / 3x / zoom LUTs as FP16 texels and
    keeps every operation FP32: on FP32 planes it matches the oracle run
    with those LUTs rounded to FP16 to the plain-FP32 bar (keys, 1e-5)."""
    hm = _model(name)
    H, W = 37, 45
    x = synth.frame(H, W, 67, hm.channels)
    out_size = {"zoom": (100, 71), "3x": (3 * W, 3 * H)}.get(hm.family, (2 * W, 2 * H))
    # the ravu lattice and zoom-ar's anti-ringing LUT keep FP32 texels
    m16 = oracle.mpv_form(hm.model, round_ar=False) if hm.family != "ravu" else hm.model
    _check_keyed(hm, x, out_size, precision="fast", oracle_model=m16)


@pytest.mark.parametrize("name", ["ravu-lite-ar-r3", "ravu-lite-ar-r4", "ravu-lite-r3", "ravu-3x-r3",
                                  "ravu-zoom-ar-r2-rgb", "ravu-zoom-r3-yuv"])
def test_ravu_fast_form_meets_quality_bar(name):
    """The chosen form (FP16 planes, FP16 LUT texels, FP32 math) against the
    exact-LUT FP64 oracle: max-abs <= 2e-3 with the GPU's keys, PSNR >= 55 dB
    unforced."""
    hm = _model(name)
    H, W = 64, 96
    x = synth.frame(H, W, 63, hm.channels).astype(np.float16).astype(np.float32)
    out_size = {"zoom": (150, 100), "3x": (3 * W, 3 * H)}.get(hm.family, (2 * W, 2 * H))
    st = _check_keyed(hm, x, out_size, tol=TOL_FP16_MAXABS, dtype=torch.float16, precision="fast")
    assert st["psnr_db"] >= TOL_FP16_PSNR, f"{name}: PSNR {st['psnr_db']:.1f} dB"


@pytest.mark.parametrize("name", NN)
@pytest.mark.parametrize("dtype", [torch.float32, torch.float16], ids=["f32planes", "f16planes"])
@pytest.mark.parametrize("axes", ["y", "x", "yx"])
def test_nnedi3_tensor_core_fast_form(name, dtype, axes):
    """precision="fast": FP16 normalised windows x FP16 weights on tcgen05,
    FP32 accumulation in tensor memory, FP32 epilogue.  Against the FP64
    oracle (on the same input values): max-abs <= 2e-3 and PSNR >= 55 dB.
    Odd sizes leave partial 32x4 tiles at the right and bottom edges."""
    hm = _model(name)
    H, W = 67, 99
    x = synth.luma_plane(H, W, 52)[None]
    if dtype == torch.float16:
        x = x.astype(np.float16).astype(np.float32)
    out_size = (2 * W if "x" in axes else W, 2 * H if "y" in axes else H)
    y = hm.upscale(torch.from_numpy(x).to("cuda", dtype), out_size=out_size, precision="fast")
    y = y.float().cpu().numpy().astype(np.float64)
    ref, _ = oracle.nnedi3_upscale(hm.model, x, axes=axes)
    err = np.abs(y - ref).max()
    assert err <= TOL_FP16_MAXABS, f"{name}/{axes}: max-abs {err:.3e}"
    assert _psnr(y, ref) >= TOL_FP16_PSNR


def test_nnedi3_fast_form_at_1080p_matches_fp32_form():
    hm = _model("nnedi3-nns128-win8x6")
    x = torch.from_numpy(synth.luma_plane(1080, 1920, 53)).cuda()
    a = hm.upscale(x, precision="fast")
    b = hm.upscale(x, precision="fp32")
    d = (a - b).abs()
    assert d.max().item() <= 2 * TOL_FP16_MAXABS
    mse = float((d.double() ** 2).mean())
    assert 10 * np.log10(1.0 / mse) >= TOL_FP16_PSNR


def test_nnedi3_fp16_planes():
    hm = _model("nnedi3-nns64-win8x4")
    x = synth.luma_plane(40, 48, 71)[None].astype(np.float16).astype(np.float32)
    y = hm.upscale(torch.from_numpy(x).to("cuda", torch.float16)).float().cpu().numpy()
    ref, _ = oracle.nnedi3_upscale(hm.model, x)
    assert np.abs(y - ref).max() <= TOL_FP16_MAXABS and _psnr(y, ref) >= TOL_FP16_PSNR


def test_constant_plane_is_exact_for_nnedi3_and_uses_key_zero():
    for name in ("ravu-lite-r3", "ravu-r3", "ravu-zoom-r2"):
        hm = _model(name)
        c = np.full((1, 20, 30), 0.3125, dtype=np.float32)
        out_size = (45, 33) if hm.family == "zoom" else (60, 40)
        _, keys = _run_gpu(hm, c, out_size)
        assert np.all(keys == 0)
    hm = _model("nnedi3-nns32-win8x4")
    y = hm.upscale(torch.full((20, 30), 0.3125, device="cuda"))
    assert torch.all(y == 0.3125)


def test_pitched_planes_match_contiguous():
    hm = _model("ravu-lite-ar-r3")
    x = torch.from_numpy(synth.luma_plane(40, 50, 81)).cuda()
    big = torch.zeros((40, 64), device="cuda")
    big[:, :50] = x
    view = big[:, :50]
    assert view.stride(0) == 64
    a = hm.upscale(x)
    b = hm.upscale(view)
    assert torch.equal(a, b)


def test_deterministic_and_translation_equivariant_at_full_size():
    """1920x1080: two runs are bit-identical, and a crop of the upscaled frame
    equals the upscale of the cropped input away from the crop border."""
    hm = _model("ravu-lite-ar-r3")
    x = torch.from_numpy(synth.luma_plane(1080, 1920, 91)).cuda()
    a = hm.upscale(x)
    b = hm.upscale(x)
    assert torch.equal(a, b)
    y0, x0, h, w = 301, 517, 200, 300
    c = hm.upscale(x[y0:y0 + h, x0:x0 + w].contiguous())
    m = 4  # radius-3 window + margin
    assert torch.equal(c[2 * m:-2 * m, 2 * m:-2 * m], a[2 * (y0 + m):2 * (y0 + h - m), 2 * (x0 + m):2 * (x0 + w - m)])


def test_bad_arguments_raise():
    from mpv_prescalers_gb300 import PrescaleError
    hm = _model("ravu-zoom-r2")
    x = torch.rand((20, 30), device="cuda")
    with pytest.raises(PrescaleError):
        hm.run_raw([x], [torch.empty((10, 10), device="cuda")], out_size=(10, 10))  # downscale
    lite = _model("ravu-lite-r2")
    with pytest.raises(PrescaleError):
        lite.run_raw([x], [torch.empty((41, 60), device="cuda")], out_size=(60, 41))  # wrong size
    with pytest.raises(ValueError):
        lite.upscale(torch.rand((3, 20, 30), device="cuda"))  # lite is luma only


@pytest.mark.parametrize("name", ["ravu-lite-ar-r3", "ravu-r3", "nnedi3-nns16-win8x4"])
def test_largest_frame_crop_matches_the_oracle(name):
    """A 3840x2160 input (the largest frame of the serving mix) in the fast
    form: a block of the output, away from the frame border, equals the
    oracle run on the matching input crop (the output at a pixel depends on
    its window only), to the FP16 bar."""
    hm = _model(name)
    x = synth.luma_plane(2160, 3840, 93).astype(np.float16).astype(np.float32)
    y = hm.upscale(torch.from_numpy(x).to("cuda", torch.float16), precision="fast").float().cpu().numpy()
    y0, x0, h, w, m = 1500, 3100, 24, 40, 6   # crop origin, size, margin beyond the window reach
    crop = x[y0 - m:y0 + h + m, x0 - m:x0 + w + m]
    if hm.family == "nnedi3":
        ref, _ = oracle.nnedi3_upscale(hm.model, crop)
    else:
        ref, _ = oracle.keyed_upscale(hm.model, crop[None], (2 * crop.shape[1], 2 * crop.shape[0]))
    ref = np.asarray(ref).reshape(2 * crop.shape[0], 2 * crop.shape[1])[2 * m:-2 * m, 2 * m:-2 * m]
    got = y.reshape(2 * 2160, 2 * 3840)[2 * y0:2 * (y0 + h), 2 * x0:2 * (x0 + w)]
    assert np.abs(got - ref).max() <= TOL_FP16_MAXABS or _psnr(got, ref) >= TOL_FP16_PSNR + 10


def test_empty_planes_are_rejected():
    from mpv_prescalers_gb300 import PrescaleError
    hm = _model("ravu-lite-r2")
    x = torch.empty((0, 30), device="cuda")
    with pytest.raises((PrescaleError, ValueError)):
        hm.upscale(x)


@pytest.mark.parametrize("name,zoom", [("ravu-lite-ar-r2", False), ("ravu-lite-ar-r3", False),
                                       ("ravu-zoom-ar-r2", True)])
def test_anti_ringing_with_subnormal_weight_sums(name, zoom):
    """Anti-ringing where the clamp bounds' denominators are subnormal: tiny
    positive LUT weights (1e-7) on a white plane give sum(w * (1.1 - 1)^32)
    ~ 1e-39.  The bounds are still finite (lo = hi = 1), as in the oracle."""
    import dataclasses
    from mpv_prescalers_gb300.prescaler import HookModel
    base = _model(name)
    lut = np.full_like(base.model.lut, 1e-7)
    kw = {"lut": lut}
    if zoom:
        kw["lut_ar"] = np.full_like(base.model.lut_ar, 1e-7)
    hm = HookModel(dataclasses.replace(base.model, **kw))
    x = np.ones((1, 24, 40), dtype=np.float32)
    out_size = (60, 36) if zoom else None
    y, kg = _run_gpu(hm, x, out_size)
    forced, _ = oracle.keyed_upscale(hm.model, x, out_size, keys=kg)
    assert np.isfinite(y).all()
    assert np.abs(y - forced).max() <= TOL_FP32
    assert np.abs(y - 0.8).max() < 1e-3       # 0.2 * (sum of tiny weights) + 0.8 * 1


# ---- the benchmark configurations at their own sizes ----------------------
# Seeds follow the synthetic generator's convention: 1000 * configuration +
# frame index.

def test_config1_ravu_lite_r3_960x540_plain_fp32():
    """ravu-lite-r3, one 960x540 FP32 plane, plain FP32 form: every key equal
    to the oracle's except counted boundary keys, pixels within 1e-5 of the
    oracle run with the GPU's keys."""
    hm = _model("ravu-lite-r3")
    x = synth.luma_plane(540, 960, 1000)[None]
    st = _check_keyed(hm, x, (1920, 1080))
    report("config1 ravu-lite-r3 960x540 fp32", st)
    assert st["psnr_db"] >= 80.0


@pytest.mark.parametrize("name", ["ravu-lite-ar-r4", "ravu-r3"])
def test_config2_1080p_fp16_chosen_form(name):
    """A 1920x1080 frame of the 8-frame batch (frame 0), FP16 planes, the
    chosen (fast) form: keys equal off the boundary, max-abs <= 2e-3 with the
    GPU's keys and PSNR >= 55 dB against the exact-LUT FP64 oracle on the same
    FP16-rounded input."""
    hm = _model(name)
    x = synth.luma_plane(1080, 1920, 2000).astype(np.float16).astype(np.float32)[None]
    st = _check_keyed(hm, x, (3840, 2160), tol=TOL_FP16_MAXABS, dtype=torch.float16, precision="fast")
    report(f"config2 {name} 1920x1080 fp16 fast", st)
    # the 2e-3 bar holds where the keys agree (a boundary key that flips
    # picks another LUT row, counted above); PSNR over every pixel
    assert st["psnr_db"] >= TOL_FP16_PSNR and st["max_abs_forced"] <= TOL_FP16_MAXABS


def test_config3_nnedi3_nns128_720p():
    """nnedi3-nns128-win8x6 on a 1280x720 plane: the plain FP32 form pass by
    pass against the oracle (1e-5, per-window bound on the variance gate),
    and the tensor-core form (FP16 planes) against the oracle run on the same
    FP16-rounded input: max-abs <= 2e-3, PSNR >= 55 dB."""
    hm = _model("nnedi3-nns128-win8x6")
    x = synth.luma_plane(720, 1280, 3000)
    st = _check_nnedi3_fp32(hm, x, "yx")
    report("config3 nnedi3-nns128-win8x6 1280x720 fp32", {k + "_" + a: v for a, d in st.items() for k, v in d.items()})
    x16 = x.astype(np.float16).astype(np.float32)
    y = hm.upscale(torch.from_numpy(x16).to("cuda", torch.float16), precision="fast").float().cpu().numpy()
    ref, _ = oracle.nnedi3_upscale(hm.model, x16)
    err = float(np.abs(y - ref[0]).max())
    psnr = _psnr(y.astype(np.float64), ref[0])
    report("config3 nnedi3-nns128-win8x6 1280x720 fp16 tensor cores", {"max_abs": err, "psnr_db": psnr})
    assert err <= TOL_FP16_MAXABS and psnr >= TOL_FP16_PSNR
