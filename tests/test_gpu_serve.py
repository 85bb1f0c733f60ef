"""Serving loop: continuous batching under an HBM budget.  Every request's
result is the same served in the mix as computed alone."""
import pytest

from mpv_prescalers_gb300 import serve, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SMALL = ((160, 90, 0.4), (320, 180, 0.4), (480, 270, 0.2))


@pytest.fixture(scope="module")
def models():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return {name: synth.model_for(name)[0] for name, _ in serve.ALGORITHMS}


@pytest.mark.parametrize("mode,ring", [("streams", 0), ("batch", 0), ("streams", 64)])
def test_each_result_same_alone_and_in_the_mix(models, mode, ring):
    """ring > 0: the results land in caller-owned pinned frames (enough per
    stream that none is reused within the trace)."""
    trace = serve.poisson_trace(models, 48, rate=4000.0, streams=12, seed=11, resolutions=SMALL, frame_pool=2,
                                out_ring=ring)
    given = [r.output for r in trace]
    srv = serve.Server(models, hbm_budget=40e9, slots=6, mode=mode)
    if ring:   # arenas sized up front: the run then allocates nothing on the device
        per_slot = srv.reserve(trace)
        assert all(s.arena.numel() == per_slot for s in srv.slots)
    stats = srv.run(trace)
    assert stats["requests"] == len(trace)
    for r in trace:
        alone = models[r.model].upscale(r.frame.cuda(), out_size=r.out_size, precision=r.precision).cpu()
        assert r.output is not None and torch.equal(r.output, alone), (r.rid, r.model)
    if ring:
        assert all(r.output is g for r, g in zip(trace, given))   # written in place
    assert stats["p99_ms"] >= stats["p50_ms"] > 0


def test_hbm_budget_bounds_the_bytes_in_flight(models):
    trace = serve.poisson_trace(models, 24, rate=8000.0, streams=8, seed=12, resolutions=SMALL, frame_pool=1)
    biggest = max(serve.request_bytes(models[r.model], r.frame, r.out_size) for r in trace)
    budget = int(1.5 * biggest)
    srv = serve.Server(models, hbm_budget=budget, slots=8, mode="streams")
    stats = srv.run(trace)
    assert stats["requests"] == len(trace)
    assert srv.peak <= budget
    assert srv.in_use == 0


@pytest.mark.parametrize("real_time", [True, False], ids=["real_time", "back_to_back"])
def test_serial_baseline_runs_the_same_trace(models, real_time):
    trace = serve.poisson_trace(models, 8, rate=500.0, streams=4, seed=13, resolutions=SMALL, frame_pool=1)
    stats = serve.serial_baseline(models, trace, real_time=real_time, passes=2)
    assert stats["requests"] == 8 and stats["p50_ms"] > 0 and stats["p99_ms"] >= stats["p50_ms"]
    if real_time:   # the wall clock covers at least the arrivals
        assert stats["span_s"] >= max(r.arrival for r in trace) - min(r.arrival for r in trace)
    fast = serve.serial_baseline(models, trace, real_time=real_time, precision="fast")
    assert fast["requests"] == 8
