"""pz_nnedi3_run_static: NNEDI3 for hosts that may not allocate device memory.

Some callers cannot allocate while they render a frame (a render callback
working against a display deadline, a host that hands the library a fixed
device-memory budget at start-up).  They call pz_nnedi3_run_static, which
takes the plane between the row and column passes from a static array inside
the library instead of allocating it.  These tests call it through the C ABI
and compare it with pz_run, on consecutive calls that reuse the array.

This file is collected last on purpose: when a run stops at the first
failure, every other test has already run.
"""
import ctypes

import pytest

from mpv_prescalers_gb300 import _ffi, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-5  # the FP32 parity tolerance of the other GPU tests


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    yield


def _plane(t):
    dt = _ffi.PZ_F32 if t.dtype == torch.float32 else _ffi.PZ_F16
    return _ffi.Plane(t.data_ptr(), t.shape[1], t.shape[0], t.stride(0), dt)


def _run_static(hm, x, out, axes=0, precision="fp32"):
    o = _ffi.Opts()
    o.nnedi3_axes = axes
    o.precision = {"fp32": _ffi.PZ_PREC_FP32, "fast": _ffi.PZ_PREC_FAST, "mpv": _ffi.PZ_PREC_MPV}[precision]
    pin, pout = _plane(x), _plane(out)
    lib = _ffi.lib()
    rc = lib.pz_nnedi3_run_static(hm.device_handle(x.device.index), ctypes.byref(pin), ctypes.byref(pout),
                                  ctypes.byref(o), torch.cuda.current_stream().cuda_stream)
    return rc, lib.pz_last_error().decode()


@pytest.mark.parametrize("dtype", [torch.float32, torch.float16])
def test_static_entry_matches_pz_run_on_two_calls_in_a_row(dtype):
    hm, _ = synth.model_for("nnedi3-nns32-win8x6")
    for seed in (1, 2):  # the second call finds the first call's data in the array
        x = torch.from_numpy(synth.luma_plane(200, 360, seed)).to("cuda", dtype)
        ref = hm.upscale(x)  # pz_run
        out = torch.full_like(ref, float("nan"))
        rc, msg = _run_static(hm, x, out)
        assert rc == 0, msg
        torch.cuda.synchronize()
        assert torch.isfinite(out).all()
        assert (out.float() - ref.float()).abs().max().item() <= TOL


@pytest.mark.parametrize("dtype", [torch.float32, torch.float16])
def test_static_entry_fast_form_matches_pz_run_on_two_calls_in_a_row(dtype):
    """The tensor-core form: its column pass reads the row-doubled plane
    from the static array at pitch W; compared with pz_run in the same form
    (FP16 tensor-core neurons), which the parity tests compare with the
    oracle.  The tolerance is the fast form's (2e-3): both calls run the same
    kernels on the same input, so in practice they agree exactly."""
    hm, _ = synth.model_for("nnedi3-nns128-win8x6")
    for seed in (3, 4):
        x = torch.from_numpy(synth.luma_plane(180, 320, seed)).to("cuda", dtype)
        ref = hm.upscale(x, precision="fast")
        out = torch.full_like(ref, float("nan"))
        rc, msg = _run_static(hm, x, out, precision="fast")
        assert rc == 0, msg
        torch.cuda.synchronize()
        assert torch.isfinite(out).all()
        assert (out.float() - ref.float()).abs().max().item() <= 2e-3


def test_precision_is_checked_like_pz_run():
    hm, _ = synth.model_for("nnedi3-nns16-win8x4")
    x = torch.zeros((20, 30), device="cuda")
    out = torch.empty((40, 60), device="cuda")
    o = _ffi.Opts()
    o.precision = 7
    lib = _ffi.lib()
    rc = lib.pz_nnedi3_run_static(hm.device_handle(0), ctypes.byref(_plane(x)), ctypes.byref(_plane(out)),
                                  ctypes.byref(o), torch.cuda.current_stream().cuda_stream)
    assert rc == _ffi.PZ_EINVAL and b"precision" in lib.pz_last_error()
    rc, msg = _run_static(hm, x, out, precision="mpv")   # the mpv form takes FP16 planes only
    assert rc == _ffi.PZ_EINVAL and "FP16" in msg


def test_largest_fp32_frame_that_fits_and_single_axis():
    hm, _ = synth.model_for("nnedi3-nns16-win8x4")
    x = torch.from_numpy(synth.luma_plane(1080, 1920, 3)).cuda()  # 2*1080*1920*4 B <= 16 MiB
    ref = hm.upscale(x)
    out = torch.empty_like(ref)
    rc, msg = _run_static(hm, x, out)
    assert rc == 0, msg
    torch.cuda.synchronize()
    assert (out - ref).abs().max().item() <= TOL
    ref_y = hm.upscale(x, out_size=(1920, 2160))  # rows only: no intermediate plane at all
    out_y = torch.empty_like(ref_y)
    rc, msg = _run_static(hm, x, out_y, axes=1)
    assert rc == 0, msg
    torch.cuda.synchronize()
    assert (out_y - ref_y).abs().max().item() <= TOL


def test_frames_beyond_the_static_array_are_rejected():
    hm, _ = synth.model_for("nnedi3-nns16-win8x4")
    x = torch.zeros((1200, 1920), device="cuda")  # needs 18.4 MB > 16 MiB
    out = torch.empty((2400, 3840), device="cuda")
    rc, msg = _run_static(hm, x, out)
    assert rc == _ffi.PZ_EINVAL
    assert "static array" in msg
