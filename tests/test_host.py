"""Host-side logic that needs no GPU: the plan cache, request sizing and
admission, serving traces, batch job tables, and the bench's replica timing
(max over ranks, checked with two ``gloo`` ranks on CPU)."""
import json
import os
import socket

import numpy as np
import pytest

from mpv_prescalers_gb300 import batch as B
from mpv_prescalers_gb300 import serve as S
from mpv_prescalers_gb300 import synth

torch = pytest.importorskip("torch")


# ------------------------------------------------------------ plan cache ---

def _jobs(names_shapes, dtype=torch.float16, precision="fast"):
    out = []
    for name, (h, w), osz in names_shapes:
        hm, _ = synth.model_for(name)
        out.append(B.Job.make(hm, torch.zeros((hm.n_planes, h, w), dtype=dtype), out_size=osz, precision=precision))
    return out


def test_plan_cache_roundtrip(tmp_path):
    path = str(tmp_path / "sub" / "plans.json")
    c = B.PlanCache(path)
    assert c.get("x") is None
    c.put("gpu:abc", {"strategy": "batch:2", "times_ms": {"per_job": 1.5}})
    assert json.load(open(path)) == {"gpu:abc": {"strategy": "batch:2", "times_ms": {"per_job": 1.5}}}
    assert B.PlanCache(path).get("gpu:abc")["strategy"] == "batch:2"


def test_plan_cache_tolerates_bad_files(tmp_path):
    bad = tmp_path / "plans.json"
    bad.write_text("{not json")
    c = B.PlanCache(str(bad))
    assert c.entries == {}
    ro = tmp_path / "ro"
    ro.mkdir()
    os.chmod(ro, 0o500)
    try:
        c2 = B.PlanCache(str(ro / "deeper" / "plans.json"))
        c2.put("k", {"strategy": "per_job"})       # no exception: only persistence is lost
        assert c2.get("k") == {"strategy": "per_job"}
    finally:
        os.chmod(ro, 0o700)


def test_plan_cache_key_is_order_free_and_shape_sensitive():
    a = _jobs([("ravu-lite-ar-r3", (40, 60), None), ("nnedi3-nns16-win8x4", (20, 30), None)])
    b = list(reversed(a))
    assert B.PlanCache.key("GB300", a) == B.PlanCache.key("GB300", b)
    c = _jobs([("ravu-lite-ar-r3", (40, 62), None), ("nnedi3-nns16-win8x4", (20, 30), None)])
    assert B.PlanCache.key("GB300", a) != B.PlanCache.key("GB300", c)
    d = _jobs([("ravu-lite-ar-r3", (40, 60), None), ("nnedi3-nns16-win8x4", (20, 30), None)], precision="fp32")
    assert B.PlanCache.key("GB300", a) != B.PlanCache.key("GB300", d)
    assert B.PlanCache.key("GB300", a) != B.PlanCache.key("B200", a)


# ------------------------------------------------------------ batch jobs ---

@pytest.mark.parametrize("name,shape,osz,want,scratch", [
    ("ravu-lite-ar-r3", (36, 52), None, (72, 104), None),
    ("ravu-r4-rgb", (20, 30), None, (40, 60), 3 * 20 * 30 * 4),       # the FP32 int11 plane
    ("ravu-3x-r3-yuv", (20, 30), None, (60, 90), None),
    ("ravu-zoom-ar-r2", (30, 40), (70, 51), (51, 70), None),
    ("nnedi3-nns16-win8x4", (20, 30), None, (40, 60), 2 * 20 * 30 * 2),
    ("nnedi3-nns16-win8x4", (20, 30), (30, 40), (40, 30), None),      # rows only: no intermediate plane
])
def test_job_make_shapes(name, shape, osz, want, scratch):
    hm, _ = synth.model_for(name)
    x = torch.zeros((hm.n_planes,) + shape, dtype=torch.float16)
    j = B.Job.make(hm, x, out_size=osz)
    assert len(j.inputs) == len(j.outputs) == hm.n_planes
    assert all(tuple(o.shape) == want for o in j.outputs)
    # one allocation for all planes of a frame, planes back to back
    if hm.n_planes > 1:
        assert j.outputs[1].data_ptr() - j.outputs[0].data_ptr() == want[0] * want[1] * 2
    assert (j.scratch is None) == (scratch is None)
    if scratch is not None:
        assert j.scratch.numel() == scratch
    assert j.out_size == (want[1], want[0])


def test_stream_lanes_deal_each_models_jobs_unless_scratch_is_shared():
    lite, _ = synth.model_for("ravu-lite-ar-r3")
    ravu, _ = synth.model_for("ravu-r3")
    x = torch.zeros((1, 24, 40), dtype=torch.float16)
    jobs = [B.Job.make(m, x) for m in (lite, ravu) for _ in range(5)]
    lanes = B.stream_lanes(jobs, per_model=2)
    assert [len(l) for l in lanes] == [3, 2, 3, 2]          # per model, dealt in turn
    assert {j.model.name for j in lanes[0] + lanes[1]} == {"ravu-lite-ar-r3"}
    assert sorted(id(j) for l in lanes for j in l) == sorted(id(j) for j in jobs)
    assert [len(l) for l in B.stream_lanes(jobs, per_model=1)] == [5, 5]
    shared = torch.empty(B.scratch_bytes(ravu, 40, 24, 1, 2, (80, 48)), dtype=torch.uint8)
    sj = [B.Job.make(ravu, x, scratch=shared) for _ in range(4)]   # one scratch: one chain, in order
    assert [len(l) for l in B.stream_lanes(sj, per_model=2)] == [4]


def test_zoom_tma_box_covers_every_tile_rectangle():
    """The TMA box of a ravu-zoom launch (tma_box_of in csrc/ravu_tiles.cuh)
    assumes that n consecutive output columns span at most
    floor((n-1) W / OW) + 1 source steps of the exact source position
    floor(((2X+1) W - OW) / (2 OW)); checked here for n = 32 columns and
    4 / 8 / 16 rows over many scale factors."""
    def pos(W, OW):
        X = np.arange(OW, dtype=np.int64)
        return ((2 * X + 1) * W - OW) // (2 * OW)
    rng = np.random.default_rng(3)
    cases = [(W, OW) for W in (7, 30, 217, 1280, 1920) for OW in (W + 1, int(W * 1.5), 2 * W, int(W * 2.25) + 1,
                                                                   int(W * 3.7))]
    cases += [(int(w), int(w * f)) for w, f in zip(rng.integers(2, 4000, 200), rng.uniform(1.001, 6.0, 200))]
    for W, OW in cases:
        if OW <= W:
            continue
        p = pos(W, OW)
        for n in (32, 4, 8, 16):
            if OW < n:   # the tile is clipped to the frame: a shorter span
                continue
            bound = (n - 1) * W // OW + 1
            span = int((p[n - 1:] - p[:OW - n + 1]).max())
            assert span <= bound, (W, OW, n, span, bound)


def test_job_staging_is_checked_and_keyed():
    hm, _ = synth.model_for("ravu-lite-ar-r3")
    x = torch.zeros((1, 36, 52), dtype=torch.float16)
    assert B.Job.make(hm, x).staging == "tma"
    assert B.STAGINGS[B.Job.make(hm, x, staging="ldg").staging] == 0
    with pytest.raises(ValueError):
        B.Job.make(hm, x, staging="texture")
    a, b = B.Job.make(hm, x), B.Job.make(hm, x, staging="ldg")
    assert B.PlanCache.key("GB300", [a]) != B.PlanCache.key("GB300", [b])


def test_job_tile_rows_are_checked_keyed_and_passed():
    hm, _ = synth.model_for("ravu-lite-ar-r3")
    x = torch.zeros((1, 36, 52), dtype=torch.float16)
    for bad in (0, 2, 12, 32, "8"):
        with pytest.raises(ValueError):
            B.Job.make(hm, x, tile_rows=bad)
    a, b, c = B.Job.make(hm, x), B.Job.make(hm, x), B.Job.make(hm, x, tile_rows=16)
    assert B.PlanCache.key("GB300", [a]) == B.PlanCache.key("GB300", [b])
    assert B.PlanCache.key("GB300", [a]) != B.PlanCache.key("GB300", [c])
    assert a.shape_key() == c.shape_key()
    from mpv_prescalers_gb300.prescaler import check_tile_rows
    assert [check_tile_rows(r) for r in (None, 4, 8, 16)] == [0, 4, 8, 16]   # the pz_opts.tile_rows values


def test_tile_layouts_per_family():
    lite, _ = synth.model_for("ravu-lite-ar-r3")
    zoom, _ = synth.model_for("ravu-zoom-ar-r2")
    nn, _ = synth.model_for("nnedi3-nns16-win8x4")
    assert sorted(B.tile_layouts(lite)) == sorted((st, r) for st in ("ldg", "tma") for r in (4, 8, 16))
    assert sorted(B.tile_layouts(zoom)) == sorted(B.tile_layouts(lite))
    assert len(B.tile_layouts(nn)) == 1


# ----------------------------------------------- request sizing / admission --

def test_request_bytes():
    lite, _ = synth.model_for("ravu-lite-ar-r3")
    f = torch.zeros((1, 100, 200), dtype=torch.float16)
    assert S.request_bytes(lite, f, None) == (100 * 200 + 200 * 400) * 2
    rgb, _ = synth.model_for("ravu-r4-rgb")
    f3 = torch.zeros((3, 100, 200), dtype=torch.float32)
    # planes in and out, plus the FP32 int11 plane of the lattice
    assert S.request_bytes(rgb, f3, None) == 3 * (100 * 200 + 200 * 400) * 4 + 3 * 100 * 200 * 4
    nn, _ = synth.model_for("nnedi3-nns64-win8x4")
    assert S.request_bytes(nn, f, None) == (100 * 200 + 200 * 400 + 2 * 100 * 200) * 2
    zoom, _ = synth.model_for("ravu-zoom-ar-r2")
    assert S.request_bytes(zoom, f, (350, 175)) == (100 * 200 + 350 * 175) * 2


def _req(rid, model, h, w, arrival=0.0, osz=None):
    hm, _ = synth.model_for(model)
    return S.Request(rid, 0, model, torch.zeros((hm.n_planes, h, w), dtype=torch.float16), arrival, osz)


def test_admission_respects_budget_and_order():
    models = {n: synth.model_for(n)[0] for n in ("ravu-lite-ar-r3", "nnedi3-nns64-win8x4")}
    one = (100 * 200 + 200 * 400) * 2                         # a lite request's bytes
    q = [_req(i, "ravu-lite-ar-r3", 100, 200) for i in range(5)]
    rejected = []
    g, nb = S.admit_group(q, models, budget=3 * one, in_use=0, max_group=4, rejected=rejected)
    assert [r.rid for r in g] == [0, 1, 2] and nb == 3 * one and [r.rid for r in q] == [3, 4]
    g, nb = S.admit_group(q, models, budget=3 * one, in_use=3 * one, max_group=4, rejected=rejected)
    assert g == [] and nb == 0 and len(q) == 2                # full: nothing admitted, nothing lost
    g, nb = S.admit_group(q, models, budget=3 * one, in_use=2 * one, max_group=1, rejected=rejected)
    assert [r.rid for r in g] == [3] and rejected == []


def test_admission_rejects_requests_larger_than_budget():
    models = {n: synth.model_for(n)[0] for n in ("ravu-lite-ar-r3",)}
    small = (10 * 20 + 20 * 40) * 2
    q = [_req(0, "ravu-lite-ar-r3", 1000, 2000), _req(1, "ravu-lite-ar-r3", 10, 20)]
    rejected = []
    g, nb = S.admit_group(q, models, budget=small, in_use=0, max_group=4, rejected=rejected)
    assert [r.rid for r in rejected] == [0]
    assert [r.rid for r in g] == [1] and nb == small and q == []


# ---------------------------------------------------------------- traces ---

def _trace_models():
    return {n: synth.model_for(n)[0] for n, _ in S.ALGORITHMS}


def test_poisson_trace_is_seeded_and_has_the_mix():
    models = _trace_models()
    res = ((64, 36, 0.5), (96, 54, 0.5))
    a = S.poisson_trace(models, 400, rate=200.0, streams=16, seed=11, resolutions=res)
    b = S.poisson_trace(models, 400, rate=200.0, streams=16, seed=11, resolutions=res)
    assert [(r.arrival, r.model, r.stream_id, r.out_size, tuple(r.frame.shape)) for r in a] == \
           [(r.arrival, r.model, r.stream_id, r.out_size, tuple(r.frame.shape)) for r in b]
    assert all(torch.equal(x.frame, y.frame) for x, y in zip(a, b))
    arr = np.array([r.arrival for r in a])
    assert np.all(np.diff(arr) > 0)
    assert 150 < len(a) / arr[-1] < 260                       # ~200 requests/s
    # a stream keeps its model and resolution
    per_stream = {}
    for r in a:
        per_stream.setdefault(r.stream_id, set()).add((r.model, tuple(r.frame.shape[-2:])))
    assert all(len(v) == 1 for v in per_stream.values())
    for r in a:
        assert r.frame.shape[0] == models[r.model].n_planes and r.frame.dtype == torch.float16
        if r.model == "ravu-zoom-ar-r2":
            h, w = r.frame.shape[-2:]
            assert r.out_size == (int(round(w * 1.75)), int(round(h * 1.75)))
        else:
            assert r.out_size is None
    c = S.poisson_trace(models, 400, rate=200.0, streams=16, seed=12, resolutions=res)
    assert [r.arrival for r in c] != [r.arrival for r in a]


def test_warmup_trace_covers_every_pair():
    models = _trace_models()
    res = ((64, 36, 0.5), (96, 54, 0.5))
    t = S.warmup_trace(models, resolutions=res)
    assert {(r.model, tuple(r.frame.shape[-2:])) for r in t} == \
           {(n, (h, w)) for w, h, _ in res for n, _ in S.ALGORITHMS}


def test_summarize():
    done = []
    for i, lat in enumerate([0.001, 0.002, 0.003, 0.010]):
        r = S.Request(i, 0, "m", None, arrival=0.01 * i)
        r.finish = r.arrival + lat
        r.output = torch.zeros((1, 20, 30))
        done.append(r)
    s = S.summarize(done, peak_bytes=5e9)
    assert s["requests"] == 4 and s["max_ms"] == pytest.approx(10.0)
    assert s["p50_ms"] == pytest.approx(2.5) and s["peak_hbm_gb"] == 5.0
    assert s["out_mpix_s"] == pytest.approx(4 * 600 / 0.04 / 1e6)


# ------------------------------------------------ bench replica timing (gloo) --

def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_bench_replica_timing_is_max_over_ranks(tmp_path):
    import torch.multiprocessing as tmp
    from replica_worker import rank_main
    tmp.spawn(rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    got = [json.load(open(tmp_path / f"r{r}.json")) for r in range(2)]
    for g in got:
        assert g["ms"] == 17.5
        assert g["value"] == pytest.approx(2 * 1000.0 * 4 / 0.0175 / 1e6)


def test_bench_replica_timing_single_process():
    import bench
    assert bench.max_over_ranks(3.25) == 3.25
    assert bench.job_value(2e6, 10, 1000.0, 1) == pytest.approx(20.0)


@pytest.mark.parametrize("kind", ["port", "reference"])
def test_bench_cpu_baseline_kinds(kind):
    """The CPU legs of bench.py on a small sample: the NumPy oracle ("port")
    and the reference's shader text compiled as C++ ("reference", when
    build() made oracle/_ref here)."""
    import bench
    if kind == "reference" and not bench.reference_available():
        pytest.skip("oracle/_ref not built on this machine")
    r = bench.cpu_baseline(16, 2, kind)
    assert r["kind"] == kind and r["cores"] == 2 and r["value"] > 0 and r["unit"] == "Mpix/s"
    assert "16 of 1080 input rows" in r["sample"]


def test_bench_reference_strip_matches_the_oracle():
    """One strip of the compiled reference shaders equals the NumPy oracle on
    the same rows (the two CPU legs compute the same pixels)."""
    import ctypes
    import bench
    if not bench.reference_available():
        pytest.skip("oracle/_ref not built on this machine")
    import oracle
    hm, src = synth.model_for("ravu-lite-ar-r4")
    if src != "parsed":
        pytest.skip("the model cache (the reference's own LUTs) is not present")
    x = synth.luma_plane(20, 48, 77).astype(np.float64)
    lib = bench._ref_lib("ravu-lite-ar-r4")
    out = np.empty(4 * x.size)
    dims = (ctypes.c_int * 2)()
    assert lib.ref_run(x.ctypes.data_as(ctypes.c_void_p), 1, 20, 48, 96, 40,
                       out.ctypes.data_as(ctypes.c_void_p), out.size, dims) == 0
    assert (dims[0], dims[1]) == (40, 96)
    want, _ = oracle.keyed_upscale(hm.model, x[None].astype(np.float32))
    assert np.abs(out.reshape(40, 96) - want[0]).max() < 1e-9


def test_trace_output_rings_are_per_stream_and_shaped():
    models = _trace_models()
    res = ((64, 36, 0.5), (96, 54, 0.5))
    t = S.poisson_trace(models, 200, rate=200.0, streams=8, seed=3, resolutions=res, out_ring=3)
    by_stream = {}
    for r in t:
        m = models[r.model]
        h, w = r.frame.shape[-2:]
        ow, oh = m.output_size(w, h, r.out_size)
        assert tuple(r.output.shape) == (m.n_planes, oh, ow)
        by_stream.setdefault(r.stream_id, []).append(r.output)
    for outs in by_stream.values():
        assert len({o.data_ptr() for o in outs}) == min(3, len(outs))
        for i in range(3, len(outs)):
            assert outs[i] is outs[i - 3]
    # the default is a ring of 3 caller frames per stream; 0 leaves the
    # result frames to the server
    assert all(r.output is not None for r in S.poisson_trace(models, 20, resolutions=res, seed=3))
    assert all(r.output is None for r in S.poisson_trace(models, 20, resolutions=res, seed=3, out_ring=0))
