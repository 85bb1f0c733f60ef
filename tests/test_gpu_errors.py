"""Device-side errors reach the host.

Every wait inside the kernels (TMA copy completion, tensor-core MMA
completion) is bounded in time; when one runs out, the kernel abandons the
tile, records the failure in the device error word and returns instead of
hanging the GPU.  pz_check_device_error reads and clears that word.

The test makes a wait run out without any real copy or MMA involved:
pz_selftest_wait launches a one-CTA kernel that waits on an mbarrier nothing
ever arrives at (no TMA, no MMA in flight), with a limit of 0 or 1 ms.
"""
import ctypes

import numpy as np
import pytest

from mpv_prescalers_gb300 import _ffi, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    yield


def _stream():
    return torch.cuda.current_stream().cuda_stream


@pytest.mark.parametrize("limit_ns", [0, 1_000_000])
def test_a_wait_that_runs_out_is_reported_once(limit_ns):
    lib = _ffi.lib()
    assert lib.pz_check_device_error(_stream()) == _ffi.PZ_OK
    assert lib.pz_selftest_wait(limit_ns, _stream()) == _ffi.PZ_OK
    rc = lib.pz_check_device_error(_stream())
    assert rc == _ffi.PZ_ETIMEDOUT, lib.pz_last_error()
    assert b"bounded" in lib.pz_last_error()
    assert lib.pz_check_device_error(_stream()) == _ffi.PZ_OK   # read and cleared


def test_the_device_stays_usable_after_a_timeout():
    lib = _ffi.lib()
    assert lib.pz_selftest_wait(0, _stream()) == _ffi.PZ_OK
    with pytest.raises(_ffi.PrescaleError) as e:
        _ffi.check_device()
    assert e.value.code == _ffi.PZ_ETIMEDOUT
    hm, _ = synth.model_for("ravu-lite-ar-r3")
    x = torch.from_numpy(synth.luma_plane(40, 64, 5)).cuda()
    a = hm.upscale(x, staging="ldg")
    b = hm.upscale(x, staging="tma")
    _ffi.check_device()                      # no error from real launches
    assert torch.equal(a, b)
    nn, _ = synth.model_for("nnedi3-nns32-win8x4")
    y = nn.upscale(x, precision="fast")
    _ffi.check_device()
    assert torch.isfinite(y).all()


def test_negative_limit_is_rejected_on_the_host():
    lib = _ffi.lib()
    assert lib.pz_selftest_wait(-1, _stream()) == _ffi.PZ_EINVAL


def test_static_entry_shares_the_error_word():
    """pz_nnedi3_run_static reports into the same word (it allocates
    nothing, not even an error word of its own)."""
    lib = _ffi.lib()
    hm, _ = synth.model_for("nnedi3-nns16-win8x4")
    x = torch.from_numpy(synth.luma_plane(30, 40, 7)).cuda()
    out = torch.empty((60, 80), device="cuda")
    pin = _ffi.Plane(x.data_ptr(), 40, 30, 40, _ffi.PZ_F32)
    pout = _ffi.Plane(out.data_ptr(), 80, 60, 80, _ffi.PZ_F32)
    o = _ffi.Opts()
    assert lib.pz_selftest_wait(0, _stream()) == _ffi.PZ_OK
    rc = lib.pz_nnedi3_run_static(hm.device_handle(0), ctypes.byref(pin), ctypes.byref(pout), ctypes.byref(o),
                                  _stream())
    assert rc == _ffi.PZ_OK, lib.pz_last_error()
    assert lib.pz_check_device_error(_stream()) == _ffi.PZ_ETIMEDOUT   # the self-test's, not cleared by the call
    ref = hm.upscale(x)
    assert np.abs((out - ref).cpu().numpy()).max() <= 1e-5
