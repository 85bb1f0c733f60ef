"""The "mpv" form: what the mpv host computes (FP16 LUTs, FP16 planes,
1/256-step zoom LUT weights), checked against the oracle restated the same
way, and its distance from the FP32 form."""
import numpy as np
import pytest

import oracle
from mpv_prescalers_gb300 import PrescaleError, synth
from mpv_prescalers_gb300 import batch as B

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    yield


CASES = [("ravu-lite-ar-r3", None), ("ravu-lite-r4", None), ("ravu-r3", None), ("ravu-r2-yuv", None),
         ("ravu-3x-r2", None), ("ravu-zoom-ar-r2", (101, 67)), ("ravu-zoom-r3-rgb", (130, 88)),
         ("nnedi3-nns16-win8x4", None)]


@pytest.mark.parametrize("name,osz", CASES)
def test_mpv_form_matches_the_oracle_restated_the_same_way(name, osz):
    hm, _ = synth.model_for(name)
    x16 = torch.from_numpy(synth.frame(40, 58, 31, hm.channels)).to("cuda", torch.float16)
    y, keys = hm.upscale(x16, out_size=osz, precision="mpv", return_keys=True)
    xin = x16.double().cpu().numpy()
    y = y.double().cpu().numpy()
    if hm.family == "nnedi3":
        # FP32 neurons; the row-doubled plane between the passes is FP16
        mid, _ = oracle.nnedi3_upscale(hm.model, xin, axes="y")
        mid = mid.astype(np.float16).astype(np.float64)
        ref, _ = oracle.nnedi3_upscale(hm.model, mid, axes="x")
        ref = ref.reshape(y.shape).astype(np.float16).astype(np.float64)
        assert np.abs(y - ref).max() <= 1e-3
        return
    m = oracle.mpv_form(hm.model)
    over = y[..., 1::2, 1::2] if hm.family == "ravu" else None
    if over is not None and over.ndim == 2:
        over = over[None]
    ref, _ = oracle.keyed_upscale(m, xin, osz, keys=keys.cpu().numpy(), int11=over,
                                  frac_steps=256 if hm.family == "zoom" else None)
    ref = np.asarray(ref).reshape(y.shape).astype(np.float16).astype(np.float64)
    err = np.abs(y - ref)
    assert err.max() <= 2e-3, err.max()
    assert np.mean(err > 1e-3) < 1e-3


def test_mpv_form_needs_fp16_planes():
    hm, _ = synth.model_for("ravu-lite-r3")
    with pytest.raises(PrescaleError, match="FP16"):
        hm.upscale(torch.rand((16, 16), device="cuda"), precision="mpv")


def test_mpv_form_in_a_batch_matches_single_calls():
    jobs, want = [], []
    for name, osz in (("ravu-zoom-ar-r2", (90, 60)), ("ravu-lite-ar-r3", None), ("ravu-r3", None)):
        hm, _ = synth.model_for(name)
        x = torch.from_numpy(synth.frame(36, 52, 8, hm.channels)).to("cuda", torch.float16)
        jobs.append(B.Job.make(hm, x, out_size=osz, precision="mpv"))
        want.append(hm.upscale(x, out_size=osz, precision="mpv"))
    b = B.Batch(jobs)
    b.launch()
    torch.cuda.synchronize()
    for j, w in zip(jobs, want):
        got = torch.stack(j.outputs) if len(j.outputs) > 1 else j.outputs[0]
        assert torch.equal(got.reshape(w.shape), w)


@pytest.mark.parametrize("name,osz", [("ravu-lite-ar-r3", None), ("ravu-zoom-ar-r2", (2880, 1620))])
def test_distance_between_the_mpv_and_fp32_forms(name, osz):
    """The FP32 form differs from what mpv computes by the FP16 LUT and
    weight rounding only: well above the 55 dB bar on a 1080p frame."""
    hm, _ = synth.model_for(name)
    x = torch.from_numpy(synth.luma_plane(1080, 1920, 2)).to("cuda", torch.float16)
    a = hm.upscale(x, out_size=osz, precision="mpv").double()
    b = hm.upscale(x, out_size=osz, precision="fp32").double()
    mse = float(((a - b) ** 2).mean())
    psnr = 10 * np.log10(1.0 / mse) if mse > 0 else float("inf")
    print(f"{name}: mpv form vs FP32 form {psnr:.1f} dB, max-abs {float((a - b).abs().max()):.2e}")
    assert psnr > 55.0
