"""Batched persistent execution: mixed models and frame sizes in one launch
give the same pixels as one launch per frame, also when replayed from a
captured CUDA graph after the inputs change in place."""
import numpy as np
import pytest

from mpv_prescalers_gb300 import batch as B
from mpv_prescalers_gb300 import synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    yield


MIX = [  # (model, H, W, dtype, out_size, precision)
    ("ravu-lite-ar-r3", 64, 96, torch.float16, None, "fp32"),
    ("ravu-lite-r2", 17, 29, torch.float32, None, "fp32"),
    ("ravu-r3", 40, 70, torch.float32, None, "fp32"),
    ("ravu-r4-yuv", 21, 33, torch.float16, None, "fp32"),
    ("ravu-r2-rgb", 9, 12, torch.float32, None, "fp32"),
    ("ravu-zoom-ar-r2-rgb", 30, 40, torch.float32, (75, 50), "fp32"),
    ("ravu-zoom-r3", 25, 31, torch.float16, (50, 44), "fp32"),
    ("ravu-3x-r2", 17, 20, torch.float16, None, "fp32"),
    ("ravu-3x-r3-rgb", 11, 13, torch.float32, None, "fp32"),
    ("nnedi3-nns32-win8x4", 40, 48, torch.float32, None, "fast"),
    ("nnedi3-nns16-win8x6", 24, 30, torch.float16, None, "fp32"),
    # the fast form's FP16-texel programs run in their own persistent launch
    ("ravu-lite-ar-r4", 33, 70, torch.float16, None, "fast"),
    ("ravu-3x-r3-yuv", 14, 19, torch.float16, None, "fast"),
    ("ravu-zoom-ar-r2", 22, 35, torch.float32, (60, 41), "fast"),
    ("ravu-r3", 20, 26, torch.float16, None, "fast"),
]


def _jobs(seed=0, staging="tma"):
    jobs = []
    for i, (name, H, W, dt, osz, prec) in enumerate(MIX):
        hm, _ = synth.model_for(name)
        x = torch.from_numpy(synth.frame(H, W, 300 + i + seed, hm.channels)).to("cuda", dt)
        jobs.append(B.Job.make(hm, x, out_size=osz, precision=prec, staging=staging))
    return jobs


def _expected(jobs):
    return [[o.clone() for o in j.model.upscale(torch.stack(j.inputs), out_size=j.out_size,
                                                precision=j.precision).unbind(0)] for j in jobs]


@pytest.mark.parametrize("staging", ["tma", "ldg"])
@pytest.mark.parametrize("ctas", [0, 1, 2])
def test_persistent_batch_matches_per_frame_launches(ctas, staging):
    jobs = _jobs(staging=staging)
    want = _expected(jobs)
    b = B.Batch(jobs, ctas_per_sm=ctas)
    b.launch()
    torch.cuda.synchronize()
    for j, w in zip(jobs, want):
        for o, e in zip(j.outputs, w):
            assert torch.equal(o, e), j.model.name


def test_graph_replay_follows_inputs_changed_in_place():
    jobs = _jobs()
    b = B.Batch(jobs)
    b.launch()
    b.capture()
    for seed in (1, 2):
        fresh = _jobs(seed)
        for j, f in zip(jobs, fresh):
            for p, q in zip(j.inputs, f.inputs):
                p.copy_(q)
        b.replay()
        torch.cuda.synchronize()
        want = _expected(jobs)
        for j, w in zip(jobs, want):
            for o, e in zip(j.outputs, w):
                assert torch.equal(o, e), j.model.name


def test_autotuner_picks_and_caches(tmp_path):
    cache = B.PlanCache(str(tmp_path / "plans.json"))
    jobs = _jobs()
    best, times = B.autotune(jobs, cache, reps=2)
    assert best in B.STRATEGIES and set(times) == set(B.STRATEGIES)
    again, _ = B.autotune(jobs, B.PlanCache(str(tmp_path / "plans.json")), reps=2)
    assert again == best
    ex = B.Executor(jobs, cache=cache)
    # the executor's jobs carry the tuned tile layouts (same tensors)
    assert all(e.tile_rows in (4, 8, 16) and e.outputs[0] is j.outputs[0] for e, j in zip(ex.jobs, jobs))
    ex.run()
    torch.cuda.synchronize()
    want = _expected(jobs)
    for j, w in zip(jobs, want):
        for o, e in zip(j.outputs, w):
            assert torch.equal(o, e)


@pytest.mark.parametrize("use_graph", [False, True])
def test_co_scheduled_streams_match_per_frame_launches(use_graph, tmp_path):
    """The co-scheduled strategy (each model's jobs on their own side stream,
    forked from and joined to the caller's stream; replayed from a CUDA graph
    or launched directly) gives the per-frame pixels bit for bit."""
    jobs = _jobs()
    want = _expected(jobs)
    for j in jobs:
        for o in j.outputs:
            o.zero_()
    cache = B.PlanCache(str(tmp_path / "plans.json"))
    key = B.PlanCache.key(torch.cuda.get_device_name(0), jobs)
    cache.put(key, {"strategy": "streams", "times_ms": {}})
    ex = B.Executor(jobs, cache=cache, use_graph=use_graph, tiles=False)
    assert ex.strategy == "streams" and (ex.graph is not None) == use_graph
    for _ in range(2):
        ex.run()
    torch.cuda.synchronize()
    for j, w in zip(jobs, want):
        for o, e in zip(j.outputs, w):
            assert torch.equal(o, e), j.model.name


def test_ragged_random_batches_match_per_frame_launches():
    """Many small and odd-sized frames of every family in every form: the
    per-program persistent groups give the per-frame pixels bit for bit."""
    rng = np.random.default_rng(7)
    names = ["ravu-lite-r2", "ravu-lite-ar-r3", "ravu-lite-ar-r4", "ravu-r2", "ravu-r3-yuv", "ravu-r4-rgb",
             "ravu-3x-r2-rgb", "ravu-3x-r4", "ravu-zoom-r2", "ravu-zoom-ar-r2-yuv", "ravu-zoom-r3-rgb",
             "nnedi3-nns16-win8x4"]
    jobs = []
    for i in range(40):
        name = names[int(rng.integers(len(names)))]
        hm, _ = synth.model_for(name)
        H, W = int(rng.integers(1, 40)), int(rng.integers(1, 70))
        dt = torch.float16 if rng.random() < 0.5 else torch.float32
        prec = ["fp32", "fast", "mpv"][int(rng.integers(3))]
        if prec == "mpv":
            dt = torch.float16
        osz = (W + int(rng.integers(1, 50)), H + int(rng.integers(1, 30))) if hm.family == "zoom" else None
        x = torch.from_numpy(synth.frame(H, W, 900 + i, hm.channels)).to("cuda", dt)
        jobs.append(B.Job.make(hm, x, out_size=osz, precision=prec, staging=["tma", "ldg"][i % 2]))
    want = _expected(jobs)
    b = B.Batch(jobs)
    b.launch()
    torch.cuda.synchronize()
    for j, w in zip(jobs, want):
        for o, e in zip(j.outputs, w):
            assert torch.equal(o, e), (j.model.name, j.precision, tuple(j.inputs[0].shape))


def test_tma_staged_batches_of_larger_frames():
    """Frames with many interior tiles, TMA-staged and clamped-load jobs
    mixed in one persistent group (the CTAs switch tensor maps between jobs
    and flip their mbarrier phase per TMA tile): per-frame pixels bit for bit."""
    jobs = []
    for i, (name, H, W, dt, prec) in enumerate([
            ("ravu-lite-ar-r3", 120, 260, torch.float16, "fast"), ("ravu-lite-ar-r3", 97, 203, torch.float16, "fast"),
            ("ravu-lite-ar-r3", 64, 150, torch.float16, "fast"), ("ravu-r3", 100, 200, torch.float32, "fp32"),
            ("ravu-r3", 81, 131, torch.float32, "fp32"), ("ravu-3x-r3-rgb", 50, 90, torch.float16, "fast"),
            ("ravu-3x-r3-rgb", 41, 77, torch.float16, "fast")]):
        hm, _ = synth.model_for(name)
        x = torch.from_numpy(synth.frame(H, W, 1200 + i, hm.channels)).to("cuda", dt)
        jobs.append(B.Job.make(hm, x, precision=prec, staging=["tma", "ldg"][i % 2]))
    want = _expected(jobs)
    for ctas in (0, 1):
        for j in jobs:
            for o in j.outputs:
                o.zero_()
        B.Batch(jobs, ctas_per_sm=ctas).launch()
        torch.cuda.synchronize()
        for j, w in zip(jobs, want):
            for o, e in zip(j.outputs, w):
                assert torch.equal(o, e), (j.model.name, j.staging, ctas)
