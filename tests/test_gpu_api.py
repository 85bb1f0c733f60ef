"""Public API behaviour on the GPU: batches, host pipelines, //!WHEN."""
import numpy as np
import pytest

from mpv_prescalers_gb300 import synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    yield


@pytest.mark.parametrize("name", ["ravu-lite-ar-r3", "ravu-r3-yuv", "nnedi3-nns32-win8x4"])
def test_host_pipeline_matches_device_calls(name):
    hm, _ = synth.model_for(name)
    C = hm.n_planes
    frames = torch.stack([torch.from_numpy(synth.frame(36, 52, 100 + i, hm.channels)) for i in range(5)])
    frames = frames.to(torch.float16).pin_memory()
    got = hm.upscale_host(frames)
    assert got.shape == (5, C, 72, 104)
    for i in range(5):
        ref = hm.upscale(frames[i].cuda()).cpu()
        assert torch.equal(got[i], ref)


def test_host_pipelines_of_two_models_overlap_and_match():
    """wait=False queues the work and returns an event: two models' host
    pipelines in flight together give the same frames as device calls."""
    a, _ = synth.model_for("ravu-lite-ar-r4")
    b, _ = synth.model_for("nnedi3-nns16-win8x4")
    frames = torch.stack([torch.from_numpy(synth.luma_plane(30, 44, 300 + i))[None] for i in range(4)])
    frames = frames.to(torch.float16).pin_memory()
    ya, ea = a.upscale_host(frames, precision="fast", wait=False)
    yb, eb = b.upscale_host(frames, precision="fast", wait=False)
    ea.synchronize()
    eb.synchronize()
    for i in range(4):
        assert torch.equal(ya[i], a.upscale(frames[i].cuda(), precision="fast").cpu())
        assert torch.equal(yb[i], b.upscale(frames[i].cuda(), precision="fast").cpu())


def test_host_pipelines_of_one_model_back_to_back_match():
    """Several wait=False calls of one model and frame size in flight
    together: each call gets a work buffer no queued call still uses (its
    copies start at once, on the library's copy streams), and finished
    buffers are handed out again."""
    hm, _ = synth.model_for("ravu-lite-ar-r3")
    sets = [torch.stack([torch.from_numpy(synth.luma_plane(192, 320, 500 + 10 * k + i))[None] for i in range(6)])
            .to(torch.float16).pin_memory() for k in range(3)]
    keys0 = set(hm._host_work)
    res = [hm.upscale_host(f, precision="fast", wait=False) for f in sets]
    for f, (y, ev) in zip(sets, res):
        ev.synchronize()
        for i in range(6):
            assert torch.equal(y[i], hm.upscale(f[i].cuda(), precision="fast").cpu())
    (key,) = set(hm._host_work) - keys0
    pool = hm._host_work[key]
    # one buffer per call still in flight when the next was queued (how many
    # overlapped depends on timing), never one buffer twice
    assert 1 <= len(pool) <= 3 and len({w.data_ptr() for _, w in pool}) == len(pool)
    n = len(pool)
    y = hm.upscale_host(sets[0], precision="fast")       # reuses a finished buffer
    assert len(hm._host_work[key]) == n
    assert torch.equal(y, res[0][0])


@pytest.mark.parametrize("shape", [(3, 240, 320), (2, 3, 120, 160)], ids=["planes", "batch"])
def test_upscale_on_a_side_stream(shape):
    """With ``stream=`` the results are allocated and gathered on that stream
    (the [C][H][W] result is one tensor whose planes the kernels write; a
    batch is stacked after its kernels), so they equal the default-stream run."""
    hm, _ = synth.model_for("ravu-r3-yuv")
    x = torch.from_numpy(np.stack([synth.frame(shape[-2], shape[-1], 700 + i, hm.channels)
                                   for i in range(shape[0] if len(shape) == 4 else 1)]))
    x = (x if len(shape) == 4 else x[0]).to("cuda", torch.float16)
    want = hm.upscale(x, precision="fast")
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    got = hm.upscale(x, precision="fast", stream=s)
    s.synchronize()
    assert got.shape == want.shape and got.is_contiguous()
    assert torch.equal(got, want)


def test_host_pipeline_c_abi_checks_work_and_layout():
    import ctypes
    from mpv_prescalers_gb300 import _ffi, PrescaleError
    hm, _ = synth.model_for("ravu-r3-yuv")
    frames = torch.from_numpy(synth.yuv_frame(20, 28, 5))[None].to(torch.float16).pin_memory()
    out = torch.empty((1, 3, 40, 56), dtype=torch.float16).pin_memory()
    o = _ffi.Opts()
    o.out_width, o.out_height = 56, 40
    L = _ffi.lib()
    h = hm.device_handle(0)
    need = L.pz_run_host_work_bytes(h, 28, 20, _ffi.PZ_F16, ctypes.byref(o))
    assert need >= 3 * (3 * 20 * 28 * 2 + 3 * 40 * 56 * 2) and need % 3 == 0
    work = torch.empty(need, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    slot = need // 3   # one frame in flight: one of the three slots
    rc = L.pz_run_host(h, frames.data_ptr(), out.data_ptr(), 1, 28, 20, _ffi.PZ_F16, ctypes.byref(o),
                       work.data_ptr(), slot - 256, 0, s.cuda_stream)
    assert rc == _ffi.PZ_EINVAL and b"work" in L.pz_last_error()
    _ffi.check(L.pz_run_host(h, frames.data_ptr(), out.data_ptr(), 1, 28, 20, _ffi.PZ_F16, ctypes.byref(o),
                             work.data_ptr(), slot, 0, s.cuda_stream))
    s.synchronize()
    assert torch.equal(out[0], hm.upscale(frames[0].cuda()).cpu())
    with pytest.raises(ValueError, match="contiguous"):
        hm.upscale_host(frames.transpose(2, 3))


def test_host_pipeline_when_false_passes_frames_through():
    hm, _ = synth.model_for("ravu-lite-r3")
    frames = torch.rand((2, 1, 20, 30)).pin_memory()
    y = hm.upscale_host(frames, out_size=(33, 22))   # below the //!WHEN ratio
    assert torch.equal(y, frames)


def test_batch_of_frames_matches_frame_by_frame():
    hm, _ = synth.model_for("ravu-zoom-ar-r2-rgb")
    x = torch.stack([torch.from_numpy(synth.rgb_frame(30, 40, 7 + i)) for i in range(3)]).cuda()
    y = hm.upscale(x, out_size=(70, 51))
    assert y.shape == (3, 3, 51, 70)
    for i in range(3):
        assert torch.equal(y[i], hm.upscale(x[i], out_size=(70, 51)))


def test_when_false_leaves_planes_untouched():
    hm, _ = synth.model_for("ravu-lite-r3")
    x = torch.rand((40, 60), device="cuda")
    y = hm.upscale(x, out_size=(70, 50))  # 0.86x per axis: //!WHEN wants < 0.707
    assert torch.equal(y, x)
    nn, _ = synth.model_for("nnedi3-nns16-win8x4")
    y = nn.upscale(x, out_size=(60, 80))  # rows only
    assert y.shape == (80, 60)


@pytest.mark.parametrize("name", ["ravu-lite-ar-r4", "ravu-lite-r2", "ravu-r3", "ravu-r4-rgb", "ravu-3x-r3-yuv",
                                  "ravu-zoom-ar-r2"])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float16])
def test_tma_staging_gives_identical_pixels(name, dtype):
    """Interior tiles staged by TMA boxes, border tiles by clamped loads: the
    same pixels as clamped loads everywhere."""
    hm, _ = synth.model_for(name)
    x = torch.from_numpy(synth.frame(100, 216, 61, hm.channels)).to("cuda", dtype)
    osz = (400, 180) if hm.family == "zoom" else None
    a = hm.upscale(x, out_size=osz, staging="ldg")
    b = hm.upscale(x, out_size=osz, staging="tma")
    assert torch.equal(a, b)


@pytest.mark.parametrize("name", ["ravu-lite-ar-r4", "ravu-lite-r2", "ravu-r3", "ravu-r4-rgb", "ravu-3x-r3-yuv",
                                  "ravu-zoom-ar-r2-rgb"])
@pytest.mark.parametrize("rows", [4, 8, 16])
@pytest.mark.parametrize("prec,dtype", [("fast", torch.float16), ("fp32", torch.float32)], ids=["fast", "fp32"])
def test_tile_heights_give_identical_pixels(name, rows, prec, dtype):
    """4-, 8- and 16-row tiles (both stagings) give the pixels and keys of the
    default layout; 102 input rows (zoom: 181 output rows) leave a ragged
    last tile row at every height."""
    hm, _ = synth.model_for(name)
    x = torch.from_numpy(synth.frame(102, 216, 63, hm.channels)).to("cuda", dtype)
    osz = (400, 181) if hm.family == "zoom" else None
    want, wkeys = hm.upscale(x, out_size=osz, precision=prec, staging="ldg", return_keys=True)
    for st in ("ldg", "tma"):
        got, keys = hm.upscale(x, out_size=osz, precision=prec, staging=st, tile_rows=rows, return_keys=True)
        assert torch.equal(got, want), st
        assert torch.equal(keys, wkeys), st


def test_tile_rows_are_checked_by_the_library():
    import ctypes
    from mpv_prescalers_gb300 import _ffi
    from mpv_prescalers_gb300 import batch as B
    hm, _ = synth.model_for("ravu-lite-ar-r3")
    x = torch.rand((40, 64), device="cuda")
    y = torch.empty((80, 128), device="cuda")
    pin = (_ffi.Plane * 1)(_ffi.Plane(x.data_ptr(), 64, 40, 64, _ffi.PZ_F32))
    pout = (_ffi.Plane * 1)(_ffi.Plane(y.data_ptr(), 128, 80, 128, _ffi.PZ_F32))
    o = _ffi.Opts()
    L = _ffi.lib()
    for bad in (1, 2, 5, 12, 32, -8):
        o.tile_rows = bad
        assert L.pz_run(hm.device_handle(0), pin, 1, pout, 1, ctypes.byref(o), None) == _ffi.PZ_EINVAL
        assert b"tile_rows" in L.pz_last_error()
    o.tile_rows = 0
    for bad in (-1, 2, 7):
        o.staging = bad
        assert L.pz_run(hm.device_handle(0), pin, 1, pout, 1, ctypes.byref(o), None) == _ffi.PZ_EINVAL
        assert b"staging" in L.pz_last_error()
    assert B.Job.make(hm, x, tile_rows=16).to_c().opts.tile_rows == 16
    assert B.Job.make(hm, x).to_c().opts.tile_rows == 0


def test_tile_autotuner(tmp_path):
    from mpv_prescalers_gb300 import batch as B
    hm, _ = synth.model_for("ravu-r3")
    x = torch.rand((270, 480), device="cuda", dtype=torch.float16)
    cache = B.PlanCache(str(tmp_path / "p.json"))
    (st, rows), times = B.autotune_tiles(hm, x, precision="fast", cache=cache, reps=2)
    assert st in ("ldg", "tma") and rows in (4, 8, 16)
    assert set(times) == {f"{s}/{r}" for s, r in B.tile_layouts(hm)}
    assert B.autotune_tiles(hm, x, precision="fast", cache=cache)[0] == (st, rows)   # cached
    jobs = B.tune_tiles([B.Job.make(hm, x, precision="fast")], cache=cache)
    assert (jobs[0].staging, jobs[0].tile_rows) == (st, rows)


@pytest.mark.parametrize("name", ["ravu-zoom-r2", "ravu-zoom-ar-r2-rgb", "ravu-zoom-r3-yuv", "ravu-zoom-ar-r3"])
@pytest.mark.parametrize("osz", [(218, 101), (241, 131), (324, 150), (500, 101), (801, 367), (218, 370)],
                         ids=["1.0x", "1.1x", "1.5x", "2.3x1x", "3.7x", "1x3.7x"])
@pytest.mark.parametrize("prec,dtype", [("fast", torch.float16), ("fp32", torch.float32)], ids=["fast", "fp32"])
def test_zoom_tma_rectangles_give_identical_pixels(name, osz, prec, dtype):
    """ravu-zoom's input rectangles staged from TMA boxes fitted to the scale
    factor (interior rectangles; the others by clamped loads) give the
    clamped-load pixels at every scale, per axis, at every tile height."""
    hm, _ = synth.model_for(name)
    x = torch.from_numpy(synth.frame(100, 217, 64, hm.channels)).to("cuda", dtype)
    assert hm.enabled(217, 100, osz)
    want = hm.upscale(x, out_size=osz, precision=prec, staging="ldg")
    for rows in (4, 8, 16):
        assert torch.equal(hm.upscale(x, out_size=osz, precision=prec, staging="tma", tile_rows=rows), want), rows


def test_zoom_tma_box_larger_than_the_plane_falls_back():
    hm, _ = synth.model_for("ravu-zoom-ar-r2")
    x = torch.rand((6, 20), device="cuda", dtype=torch.float16)   # smaller than any box
    assert hm.enabled(20, 6, (37, 11))
    assert torch.equal(hm.upscale(x, out_size=(37, 11), staging="tma"), hm.upscale(x, out_size=(37, 11), staging="ldg"))


def test_tma_staging_falls_back_for_unaligned_pitch():
    hm, _ = synth.model_for("ravu-lite-ar-r3")
    big = torch.from_numpy(synth.luma_plane(90, 203, 62)).cuda()   # pitch 203 floats: not 16-byte rows
    view = big[:, :200]
    assert torch.equal(hm.upscale(view, staging="tma"), hm.upscale(view.contiguous(), staging="ldg"))


def test_staging_autotuner(tmp_path):
    from mpv_prescalers_gb300 import batch as B
    hm, _ = synth.model_for("ravu-lite-ar-r3")
    x = torch.rand((270, 480), device="cuda", dtype=torch.float16)
    best, times = B.autotune_staging(hm, x, cache=B.PlanCache(str(tmp_path / "p.json")), reps=2)
    assert best in ("ldg", "tma") and set(times) == {"ldg", "tma"}


@pytest.mark.parametrize("name,osz", [("ravu-lite-ar-r3", None), ("ravu-r3-yuv", None), ("ravu-3x-r2-rgb", None),
                                      ("ravu-zoom-ar-r2", (101, 77)), ("nnedi3-nns16-win8x4", None),
                                      ("nnedi3-nns16-win8x4", (40, 60)), ("nnedi3-nns16-win8x4", (80, 30))])
def test_query_matches_the_python_geometry(name, osz):
    import ctypes
    from mpv_prescalers_gb300 import _ffi
    hm, _ = synth.model_for(name)
    W, H = 40, 30
    o = _ffi.Opts()
    if osz is not None:
        o.out_width, o.out_height = osz
    if hm.family == "nnedi3":
        o.nnedi3_axes = hm.nnedi3_axes(W, H, osz)
    r = _ffi.QueryResult()
    _ffi.check(_ffi.lib().pz_query(hm.device_handle(0), W, H, _ffi.PZ_F16, ctypes.byref(o), ctypes.byref(r)))
    assert (r.out_width, r.out_height) == hm.output_size(W, H, osz)
    assert r.n_planes == hm.n_planes
    want_scratch = 2 * W * H * 2 if hm.family == "nnedi3" and o.nnedi3_axes == 3 else 0
    if hm.family == "ravu":   # the FP32 int11 plane between the two lattice launches
        want_scratch = hm.n_planes * W * H * 4
    assert r.scratch_bytes == want_scratch
