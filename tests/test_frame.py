"""Frame planning on the host: hook points, chroma handling and the chain's
announced offset (no device calls)."""
import glob
import os

import pytest

from mpv_prescalers_gb300 import frame as F
from mpv_prescalers_gb300 import synth
from mpv_prescalers_gb300.prescaler import HookModel
from mpv_prescalers_gb300 import models

YUV420 = [(64, 36), (32, 18), (32, 18)]
YUV444 = [(64, 36)] * 3
RGB = [(64, 36)] * 3


def m(name):
    return synth.model_for(name)[0]


@pytest.mark.parametrize("name,offset", [
    ("ravu-lite-ar-r3", (0.0, 0.0)), ("ravu-r3", (-0.5, -0.5)), ("ravu-3x-r3", (0.0, 0.0)),
    ("nnedi3-nns16-win8x4", (-0.5, -0.5)),
])
def test_luma_hook_on_420(name, offset):
    p = F.plan_frame(m(name), "yuv", YUV420)
    assert p.runs and p.prescaled == (0,) and p.passthrough == (1, 2) and not p.upsample_chroma
    assert p.offset == offset
    s = 3 if "3x" in name else 2
    assert p.out_size == (64 * s, 36 * s)


def test_luma_hook_on_gray_and_rgb():
    p = F.plan_frame(m("ravu-lite-r3"), "gray", [(64, 36)])
    assert p.runs and p.prescaled == (0,) and p.passthrough == ()
    p = F.plan_frame(m("ravu-lite-r3"), "rgb", RGB)
    assert not p.runs and "no luma" in p.reason


def test_zoom_aligns_itself():
    p = F.plan_frame(m("ravu-zoom-ar-r2"), "yuv", YUV420, out_size=(100, 60))
    assert p.runs and p.offset == "ALIGN" and p.out_size == (100, 60)


def test_nnedi3_offset_follows_the_enabled_axes():
    nn = m("nnedi3-nns16-win8x4")
    assert nn.chain_offset(64, 36) == (-0.5, -0.5)
    assert nn.chain_offset(64, 36, out_size=(64, 72)) == (0.0, -0.5)    # rows only
    assert nn.chain_offset(64, 36, out_size=(128, 36)) == (-0.5, 0.0)   # columns only
    assert nn.chain_offset(64, 36, out_size=(64, 36)) == (0.0, 0.0)     # nothing runs


def test_native_hook_merges_subsampled_chroma():
    p = F.plan_frame(m("ravu-r3-yuv"), "yuv", YUV420, chroma_loc="left")
    assert p.runs and p.upsample_chroma and p.prescaled == (0, 1, 2)
    assert p.chroma_scale == (0.5, 0.5) and p.chroma_origin == (0.0, 0.5)
    assert p.offset == (-0.5, -0.5)
    p = F.plan_frame(m("ravu-r3-yuv"), "yuv", YUV420, chroma_loc="center")
    assert p.chroma_origin == (0.5, 0.5)
    p = F.plan_frame(m("ravu-r3-yuv"), "yuv", YUV444)
    assert p.runs and not p.upsample_chroma and p.chroma_origin == (0.0, 0.0)
    p = F.plan_frame(m("ravu-r3-yuv"), "yuv", [(64, 36), (32, 36), (32, 36)])   # 4:2:2
    assert p.chroma_scale == (0.5, 1.0)


def test_native_hook_refuses_rgb_and_gray():
    p = F.plan_frame(m("ravu-zoom-r2-yuv"), "rgb", RGB, out_size=(100, 60))
    assert not p.runs and "LUMA.w" in p.reason
    with pytest.raises(ValueError, match="Y, U and V"):
        F.plan_frame(m("ravu-r3-yuv"), "gray", [(64, 36)])
    with pytest.raises(ValueError, match="differ"):
        F.plan_frame(m("ravu-r3-yuv"), "yuv", [(64, 36), (32, 18), (32, 36)])


def test_main_hook_needs_rgb():
    p = F.plan_frame(m("ravu-r3-rgb"), "rgb", RGB)
    assert p.runs and p.prescaled == (0, 1, 2) and p.offset == (-0.5, -0.5)
    with pytest.raises(ValueError, match="convert"):
        F.plan_frame(m("ravu-r3-rgb"), "yuv", YUV444)
    with pytest.raises(ValueError, match="one size"):
        F.plan_frame(m("ravu-r3-rgb"), "rgb", [(64, 36), (64, 36), (32, 18)])


def test_when_false_passes_everything_through():
    p = F.plan_frame(m("ravu-lite-r3"), "yuv", YUV420, out_size=(80, 45))   # 1.25x: below the 1/0.707 gate
    assert not p.runs and p.passthrough == (0, 1, 2)


def test_bad_frames():
    with pytest.raises(ValueError, match="kind"):
        F.plan_frame(m("ravu-lite-r3"), "xyz", YUV420)
    with pytest.raises(ValueError, match="plane"):
        F.plan_frame(m("ravu-lite-r3"), "yuv", YUV420[:2])
    with pytest.raises(ValueError, match="chroma location"):
        F.plan_frame(m("ravu-r3-yuv"), "yuv", YUV420, chroma_loc="bottom")


def test_chain_offset_of_every_reference_file(reference_dir):
    """Offsets derived from the parsed passes of root, compute and gather
    files agree with the family rule."""
    want = {"lite": (0.0, 0.0), "3x": (0.0, 0.0), "ravu": (-0.5, -0.5), "nnedi3": (-0.5, -0.5), "zoom": "ALIGN"}
    hooks = {"luma": "LUMA", "yuv": "NATIVE", "rgb": "MAIN"}
    for f in sorted(glob.glob(os.path.join(reference_dir, "**", "*.hook"), recursive=True)):
        hm = HookModel(models.load_model(f))
        osz = (200, 120) if hm.family == "zoom" else None
        assert hm.chain_offset(64, 36, osz) == want[hm.family], f
        assert hm.hook_point == hooks[hm.channels], f
    nn = HookModel(models.load_model(os.path.join(reference_dir, "compute", "nnedi3-nns32-win8x4.hook")))
    assert nn.chain_offset(64, 36, out_size=(64, 72)) == (0.0, -0.5)
