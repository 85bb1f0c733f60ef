"""pz_resample against the FP64 oracle, and whole frames through hook chains."""
import numpy as np
import pytest

import oracle.resample as ores
from mpv_prescalers_gb300 import frame as F
from mpv_prescalers_gb300 import synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    yield


CASES = [  # out_w, out_h, sx, ox, sy, oy
    (53, 37, 1.0, -0.5, 1.0, -0.5),      # ravu / nnedi3 offset correction
    (53, 37, 1.0, 0.0, 1.0, -0.5),       # rows-only NNEDI3
    (106, 74, 0.5, 0.0, 0.5, -0.25),     # 4:2:0 chroma, left siting
    (106, 37, 0.5, -0.25, 1.0, 0.0),     # 4:2:2 chroma, centre siting
    (31, 22, 1.7, 0.35, 1.7, -3.0),      # downscale with an outside start
    (53, 37, 1.0, 0.0, 1.0, 0.0),        # identity
]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("filt", ["bilinear", "catmull_rom"])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float16])
def test_resample_matches_oracle(case, filt, dtype):
    ow, oh, sx, ox, sy, oy = case
    x = synth.luma_plane(37, 53, 71)
    if dtype == torch.float16:
        x = x.astype(np.float16).astype(np.float64)
    got = F.resample_plane(torch.from_numpy(x).to("cuda", dtype), ow, oh, sx, ox, sy, oy, filt).double().cpu().numpy()
    want = ores.resample(x, ow, oh, sx, ox, sy, oy, filt)
    tol = 2e-6 if dtype == torch.float32 else 1e-3
    assert np.abs(got - want).max() <= tol
    if case[1:] == (37, 1.0, 0.0, 1.0, 0.0):
        assert np.array_equal(got, x)


def test_resample_rejects_bad_arguments():
    x = torch.zeros((8, 8), device="cuda")
    with pytest.raises(Exception, match="out of range"):
        F.resample_plane(x, 8, 8, float("nan"), 0.0, 1.0, 0.0)
    with pytest.raises(ValueError, match="filter"):
        F.resample_plane(x, 8, 8, 1.0, 0.0, 1.0, 0.0, "lanczos")


def _yuv420(h, w, seed, dtype=torch.float32):
    y = torch.from_numpy(synth.luma_plane(h, w, seed)).to("cuda", dtype)
    u = torch.from_numpy(synth.luma_plane(h // 2, w // 2, seed + 1)).to("cuda", dtype)
    v = torch.from_numpy(synth.luma_plane(h // 2, w // 2, seed + 2)).to("cuda", dtype)
    return F.Frame([y, u, v], "yuv", "left")


@pytest.mark.parametrize("name", ["ravu-r3", "ravu-lite-ar-r3", "nnedi3-nns16-win8x4"])
def test_luma_hook_frame(name):
    hm, _ = synth.model_for(name)
    fr = _yuv420(36, 64, 5)
    out = F.prescale_frame(hm, fr)
    assert out.planes[1] is fr.planes[1] and out.planes[2] is fr.planes[2]
    y = hm.upscale(fr.planes[0])
    off = hm.chain_offset(64, 36)
    if off != (0.0, 0.0):
        y = F.resample_plane(y, 128, 72, 1.0, off[0], 1.0, off[1])
    assert torch.equal(out.planes[0], y) and out.offset == (0.0, 0.0)
    raw = F.prescale_frame(hm, fr, offset_filter=None)
    assert torch.equal(raw.planes[0], hm.upscale(fr.planes[0])) and raw.offset == off


def test_native_hook_frame_against_oracle_steps():
    """4:2:0 through ravu-r2-yuv: chroma merged bilinearly at left siting,
    upscaled, offset corrected -- each GPU step checked against the oracle
    steps on the same intermediate values."""
    import oracle
    hm, _ = synth.model_for("ravu-r2-yuv")
    fr = _yuv420(36, 64, 9)
    out = F.prescale_frame(hm, fr)
    assert [tuple(p.shape) for p in out.planes] == [(72, 128)] * 3
    # step 1: chroma merge
    u_full = F.resample_plane(fr.planes[1], 64, 36, 0.5, 0.0, 0.5, -0.25, "bilinear")
    want_u = ores.resample(fr.planes[1].double().cpu().numpy(), 64, 36, 0.5, 0.0, 0.5, -0.25, "bilinear")
    assert np.abs(u_full.double().cpu().numpy() - want_u).max() < 2e-6
    # step 2+3 on the GPU's merged planes
    v_full = F.resample_plane(fr.planes[2], 64, 36, 0.5, 0.0, 0.5, -0.25, "bilinear")
    merged = torch.stack([fr.planes[0], u_full, v_full])
    up = hm.upscale(merged)
    corrected = torch.stack([F.resample_plane(p, 128, 72, 1.0, -0.5, 1.0, -0.5) for p in up])
    assert torch.equal(torch.stack(out.planes), corrected)
    # the oracle on the same keys and int11 values (boundary keys may flip)
    _, keys = hm.upscale(merged, return_keys=True)
    over = up[:, 1::2, 1::2].double().cpu().numpy()
    ref_up, _ = oracle.keyed_upscale(hm.model, merged.double().cpu().numpy(), keys=keys.cpu().numpy(), int11=over)
    ref = np.stack([ores.shift(p, -0.5, -0.5) for p in ref_up])
    assert np.abs(torch.stack(out.planes).double().cpu().numpy() - ref).max() < 3e-5


def test_main_hook_frame_and_rgb_on_luma_model():
    rgb = torch.from_numpy(synth.rgb_frame(36, 64, 3)).cuda()
    fr = F.Frame(list(rgb.unbind(0)), "rgb")
    hm, _ = synth.model_for("ravu-r2-rgb")
    out = F.prescale_frame(hm, fr, offset_filter="bilinear")
    up = hm.upscale(rgb)
    for i in range(3):
        assert torch.equal(out.planes[i], F.resample_plane(up[i], 128, 72, 1.0, -0.5, 1.0, -0.5, "bilinear"))
    lite, _ = synth.model_for("ravu-lite-r3")
    same = F.prescale_frame(lite, fr)
    assert all(a is b for a, b in zip(same.planes, fr.planes))
