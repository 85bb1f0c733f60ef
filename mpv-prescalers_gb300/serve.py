"""Serving loop: continuous batching of prescaler requests from many streams.

A request is one host frame of one video stream through one model (the
frames a player's render loop would hand to the hook chain).  The server

* keeps every model's LUT / weights resident on the device;
* admits queued requests in arrival order while the device-memory they need
  (input + output planes + scratch) fits the HBM budget and an
  execution slot is free -- requests arriving while others run are admitted
  as soon as memory and slots free up;
* runs each admitted request on its slot's CUDA stream (host->device copy,
  the model's kernels, device->host copy, queued by one call of the
  library's host pipeline, ``pz_run_host``), so the work of different
  requests overlaps on the device; in ``mode="batch"`` the requests admitted
  together are launched as one persistent batch (``batch.Batch``);
* records per-request latency from arrival to the moment the output is back
  in host memory (CUDA event time), and reports p50/p99, throughput and the
  peak device memory in use.

``serial_baseline`` runs the same trace one request at a time with no
overlap (plain FP32 planes, or the trace's own form), the comparison point
for the served numbers.
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _ffi
from . import batch as _batch
from .prescaler import HookModel


def _torch():
    import torch
    return torch


def _pinned(t):
    """Page-locked copy where a CUDA device exists (traces are also built on
    hosts without one, e.g. to check their mix)."""
    return t.pin_memory() if _torch().cuda.is_available() else t


@dataclass
class Request:
    rid: int
    stream_id: int
    model: str
    frame: "torch.Tensor"                 # host [C][H][W] (pinned)
    arrival: float                        # seconds from trace start
    out_size: Optional[Tuple[int, int]] = None
    precision: str = "fast"
    # filled in by the server
    admit: float = -1.0
    finish: float = -1.0
    # the host frame the result lands in: the caller's pinned buffer of the
    # output's shape when given (a player's own frame buffer), else allocated
    output: Optional["torch.Tensor"] = None

    @property
    def latency(self) -> float:
        return self.finish - self.arrival


def request_bytes(model: HookModel, frame, out_size) -> int:
    """Device bytes one request holds while in flight."""
    C, H, W = frame.shape
    OW, OH = model.output_size(W, H, out_size)
    es = frame.element_size()
    nbytes = C * (H * W + OH * OW) * es
    if model.family == "nnedi3" and model.nnedi3_axes(W, H, (OW, OH)) == 3:
        nbytes += 2 * H * W * es
    elif model.family == "ravu":   # the FP32 int11 plane between the lattice launches
        nbytes += C * H * W * 4
    return nbytes


def admit_group(queue: List[Request], models: Dict[str, HookModel], budget: int, in_use: int,
                max_group: int, rejected: List[Request]) -> Tuple[List[Request], int]:
    """Take requests off the head of ``queue`` in arrival order while their
    device bytes fit ``budget - in_use`` (at most ``max_group``).  A request
    larger than the whole budget can never run: it moves to ``rejected``
    instead of stalling the queue.  Returns the group and its bytes."""
    group, nbytes = [], 0
    while queue and len(group) < max_group:
        r = queue[0]
        need = request_bytes(models[r.model], r.frame, r.out_size)
        if need > budget:
            rejected.append(queue.pop(0))
            continue
        if in_use + nbytes + need > budget:
            break
        group.append(queue.pop(0))
        nbytes += need
    return group, nbytes


@dataclass
class _Slot:
    stream: "torch.cuda.Stream"
    reqs: List[Request] = field(default_factory=list)
    done: Optional["torch.cuda.Event"] = None
    nbytes: int = 0
    keep: list = field(default_factory=list)   # objects of the in-flight requests
    # the slot's device arena: every in-flight request's input, output and
    # scratch planes are carved from it; it grows only when an admitted group
    # needs more, so a server in steady state allocates nothing per request
    # (a device allocation mid-trace synchronises the whole device)
    arena: Optional["torch.Tensor"] = None


def _carve(arena, off: int, shape, dtype):
    """A tensor of `shape` / `dtype` at byte offset `off` of `arena`
    (256-byte aligned); returns it and the next offset."""
    torch = _torch()
    n = int(np.prod(shape)) * torch.empty((), dtype=dtype).element_size()
    t = arena[off:off + n].view(dtype).view(tuple(shape))
    return t, off + ((n + 255) & ~255)


class Server:
    def __init__(self, models: Dict[str, HookModel], hbm_budget: float = 40e9, slots: int = 8,
                 mode: str = "streams", device: Optional[int] = None):
        torch = _torch()
        if mode not in ("streams", "batch"):
            raise ValueError(mode)
        self.models = models
        self.budget = int(hbm_budget)
        self.mode = mode
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.slots = [_Slot(torch.cuda.Stream(self.device)) for _ in range(slots)]
        for m in models.values():       # weights / LUTs resident before the first request
            m.device_handle(self.device.index)
        self.in_use = 0
        self.peak = 0
        self.rejected: List[Request] = []

    def _arena_bytes(self, reqs: List[Request]) -> int:
        n = 0
        for r in reqs:
            m = self.models[r.model]
            C, H, W = r.frame.shape
            OW, OH = m.output_size(W, H, r.out_size)
            es = r.frame.element_size()
            for b in (C * H * W * es, C * OH * OW * es,
                      _batch.scratch_bytes(m, W, H, C, es, (OW, OH))):
                n += (b + 255) & ~255
        return n

    def reserve(self, trace: Sequence[Request], max_group: int = 4) -> int:
        """Size every slot's device arena for the largest group of `trace`'s
        requests it could be handed (a server set up for the frame sizes it
        serves), so that serving allocates nothing; returns the bytes per slot."""
        torch = _torch()
        per = sorted((self._arena_bytes([r]) for r in trace), reverse=True)
        need = sum(per[:max_group if self.mode == "batch" else 1])
        for s in self.slots:
            if s.arena is None or s.arena.numel() < need:
                s.arena = None
                s.arena = torch.empty(need, dtype=torch.uint8, device=self.device)
        torch.cuda.synchronize(self.device)
        return need

    # -- one admitted group on one slot ------------------------------------
    def _launch(self, slot: _Slot, reqs: List[Request], now: float):
        torch = _torch()
        jobs = []
        need = self._arena_bytes(reqs)
        if slot.arena is None or slot.arena.numel() < need:
            # the slot is idle here (retired before admission), so the old
            # arena can go; the new one is allocated once for all later groups
            slot.arena = None
            slot.arena = torch.empty(need, dtype=torch.uint8, device=self.device)
        if len(reqs) == 1:
            self._launch_one(slot, reqs[0])
            reqs[0].admit = now
            slot.reqs = reqs
            return
        off = 0
        with torch.cuda.stream(slot.stream):
            for r in reqs:
                m = self.models[r.model]
                C, H, W = r.frame.shape
                OW, OH = m.output_size(W, H, r.out_size)
                xd, off = _carve(slot.arena, off, (C, H, W), r.frame.dtype)
                xd.copy_(r.frame, non_blocking=True)
                out, off = _carve(slot.arena, off, (C, OH, OW), r.frame.dtype)
                sb = _batch.scratch_bytes(m, W, H, C, r.frame.element_size(), (OW, OH))
                scratch = None
                if sb:
                    scratch, off = _carve(slot.arena, off, (sb,), torch.uint8)
                job = _batch.Job.make(m, xd, out_size=r.out_size, precision=r.precision,
                                      out=out if C > 1 else out[0], scratch=scratch)
                jobs.append(job)
            if self.mode == "batch" and len(jobs) > 1:
                b = _batch.Batch(jobs, stream=slot.stream)
                b.launch(stream=slot.stream)
                slot.keep.append(b)
            else:
                _batch.run_per_job(jobs, stream=slot.stream)
            for r, job in zip(reqs, jobs):
                o0 = job.outputs[0]
                out = o0.as_strided((len(job.outputs),) + tuple(o0.shape), (o0.numel(),) + tuple(o0.stride()))
                if not (r.output is not None and tuple(r.output.shape) == tuple(out.shape)
                        and r.output.dtype == out.dtype and r.output.is_pinned()):
                    r.output = torch.empty(out.shape, dtype=out.dtype, pin_memory=True)
                r.output.copy_(out, non_blocking=True)
            slot.done = torch.cuda.Event(enable_timing=True)
            slot.done.record(slot.stream)
        for r in reqs:
            r.admit = now
        slot.reqs = reqs

    def _launch_one(self, slot: _Slot, r: Request):
        """One request through the library's host pipeline (pz_run_host):
        upload, kernels and readback are queued from native code, on the
        slot's stream and a pair of copy streams, with the request's device
        planes in the slot's arena (one frame slot of the pipeline)."""
        torch = _torch()
        m = self.models[r.model]
        C, H, W = r.frame.shape
        if r.frame.is_cuda or not r.frame.is_contiguous():
            raise ValueError("request frames are contiguous host tensors [C][H][W]")
        OW, OH = m.output_size(W, H, r.out_size)
        if not (r.output is not None and tuple(r.output.shape) == (C, OH, OW) and r.output.dtype == r.frame.dtype
                and r.output.is_contiguous() and r.output.is_pinned()):
            r.output = torch.empty((C, OH, OW), dtype=r.frame.dtype, pin_memory=True)
        dt = _ffi.PZ_F32 if r.frame.dtype == torch.float32 else _ffi.PZ_F16
        o = m.host_opts(W, H, r.out_size, r.precision)
        _ffi.check(_ffi.lib().pz_run_host(m.device_handle(self.device.index), r.frame.data_ptr(), r.output.data_ptr(),
                                          1, W, H, dt, ctypes.byref(o), slot.arena.data_ptr(), slot.arena.numel(),
                                          _ffi.PZ_HOST_WORK_IDLE, slot.stream.cuda_stream))
        slot.done = torch.cuda.Event(enable_timing=True)
        slot.done.record(slot.stream)

    def run(self, trace: Sequence[Request], max_group: int = 4) -> Dict[str, float]:
        """Serve a trace in real time; returns latency / throughput stats
        (the HBM peak is this run's)."""
        torch = _torch()
        self.peak = self.in_use
        pending = sorted(trace, key=lambda r: r.arrival)
        queue: List[Request] = []
        t0_event = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(self.device)
        t0_event.record(torch.cuda.current_stream(self.device))
        t0 = time.perf_counter()
        i = 0
        done: List[Request] = []
        while i < len(pending) or queue or any(s.reqs for s in self.slots):
            now = time.perf_counter() - t0
            while i < len(pending) and pending[i].arrival <= now:
                queue.append(pending[i])
                i += 1
            # retire finished slots
            for s in self.slots:
                if s.reqs and s.done.query():
                    fin = t0_event.elapsed_time(s.done) / 1e3
                    for r in s.reqs:
                        r.finish = fin
                        done.append(r)
                    self.in_use -= s.nbytes
                    s.reqs, s.keep, s.nbytes, s.done = [], [], 0, None
            # admit in arrival order while memory and slots allow
            for s in self.slots:
                if s.reqs or not queue:
                    continue
                group, nbytes = admit_group(queue, self.models, self.budget, self.in_use,
                                            max_group if self.mode == "batch" else 1, self.rejected)
                if not group:
                    break
                self.in_use += nbytes
                self.peak = max(self.peak, self.in_use)
                s.nbytes = nbytes
                self._launch(s, group, now)
            if i < len(pending) and not queue and not any(s.reqs for s in self.slots):
                time.sleep(max(0.0, min(pending[i].arrival - (time.perf_counter() - t0), 0.002)))
            else:
                time.sleep(2e-5)
        return summarize(done, self.peak)


def summarize(done: Sequence[Request], peak_bytes: int = 0) -> Dict[str, float]:
    lat = np.array([r.latency for r in done]) * 1e3
    span = max(r.finish for r in done) - min(r.arrival for r in done)
    px = sum(r.output.shape[-1] * r.output.shape[-2] for r in done)
    return {"requests": len(done), "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "max_ms": float(lat.max()), "out_mpix_s": px / span / 1e6,
            "span_s": span, "peak_hbm_gb": peak_bytes / 1e9}


def serial_baseline(models: Dict[str, HookModel], trace: Sequence[Request], real_time: bool = True,
                    passes: int = 1, precision: str = "fp32") -> Dict[str, float]:
    """The same trace, one request at a time, no overlap: each request starts
    when it has arrived and the previous one has finished.  ``precision``
    "fp32": the plain form on FP32 planes (the frames converted once, before
    timing); otherwise that form on the trace's own FP16 frames.
    ``real_time``: requests are taken up at their arrival on the wall clock,
    as a server would (the default); else back to back, each start moved to
    ``max(arrival, previous finish)`` on a virtual clock (no idle time on
    the device).  With ``passes`` > 1 the trace runs that many times and the
    last pass is reported (the earlier ones warm its host frames)."""
    torch = _torch()
    dev = torch.device("cuda", torch.cuda.current_device())
    clock = 0.0
    done = []
    host_out: Dict[Tuple, "torch.Tensor"] = {}   # one pinned result buffer per shape, made before timing
    fp32: Dict[int, "torch.Tensor"] = {}          # one pinned FP32 copy per distinct trace frame

    def as_fp32(f):
        if precision != "fp32":
            return f
        if id(f) not in fp32:
            fp32[id(f)] = _pinned(f.float())
        return fp32[id(f)]
    reqs = [Request(r.rid, r.stream_id, r.model, as_fp32(r.frame), r.arrival, r.out_size, precision)
            for r in sorted(trace, key=lambda q: q.arrival)]
    for q in reqs:
        m = models[q.model]
        C, H, W = q.frame.shape
        OW, OH = m.output_size(W, H, q.out_size)
        key = (C, OH, OW)
        if key not in host_out:
            host_out[key] = _pinned(torch.empty(key, dtype=q.frame.dtype))
    for _ in range(passes):
        done, clock = [], 0.0
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for q in reqs:
            if real_time:
                while time.perf_counter() - t0 < q.arrival:
                    time.sleep(min(2e-4, max(0.0, q.arrival - (time.perf_counter() - t0))))
            start = max(clock, q.arrival)
            t = time.perf_counter()
            xd = q.frame.to(dev, non_blocking=True)
            y = models[q.model].upscale(xd, out_size=q.out_size, precision=precision)
            q.output = host_out[tuple(y.shape)]
            q.output.copy_(y, non_blocking=True)
            torch.cuda.synchronize(dev)
            clock = (time.perf_counter() - t0) if real_time else start + (time.perf_counter() - t)
            q.finish = clock
            done.append(q)
    return summarize(done)


# ------------------------------------------------------------------ traces --

RESOLUTIONS = ((854, 480, 0.3), (1280, 720, 0.3), (1920, 1080, 0.3), (3840, 2160, 0.1))
ALGORITHMS = (("ravu-lite-ar-r3", None), ("ravu-r4-yuv", None), ("nnedi3-nns64-win8x4", None),
              ("ravu-zoom-ar-r2", 1.75))


def warmup_trace(models: Dict[str, HookModel], resolutions=RESOLUTIONS, algorithms=ALGORITHMS,
                 precision: str = "fast") -> List[Request]:
    """One request of every (resolution, algorithm) pair, back to back, so that
    every kernel is loaded and the pinned host buffers of every output size
    are cached before a measured trace."""
    torch = _torch()
    out, rid = [], 0
    for W, H, _ in resolutions:
        for name, zoom in algorithms:
            m = models[name]
            f = _pinned(torch.zeros((m.n_planes, H, W), dtype=torch.float16))
            osz = (int(round(W * zoom)), int(round(H * zoom))) if zoom else None
            out.append(Request(rid, 0, name, f, 0.0, osz, precision))
            rid += 1
    return out


def poisson_trace(models: Dict[str, HookModel], n: int, rate: float = 240.0, streams: int = 64,
                  seed: int = 5000, precision: str = "fast", frame_pool: int = 2,
                  resolutions=RESOLUTIONS, algorithms=ALGORITHMS, out_ring: int = 3) -> List[Request]:
    """Poisson arrivals at `rate` frames/s over `streams` streams; resolution
    and algorithm drawn per stream (the mix of the serving configuration).
    Frames come from a small pool of seeded synthetic frames per resolution.
    ``out_ring`` > 0 (default 3) gives every stream that many pinned output
    frames, reused in turn -- a player's own frame buffers, made before the
    trace runs; 0 lets the server page-lock a new host frame per request,
    which puts tens of MB of page-locking on the request path of every
    2160p result and dominates the latency tail."""
    from . import synth
    torch = _torch()
    rng = np.random.default_rng(seed)
    res_p = np.array([r[2] for r in resolutions])
    stream_res = rng.choice(len(resolutions), size=streams, p=res_p / res_p.sum())
    stream_alg = rng.integers(0, len(algorithms), size=streams)
    pool: Dict[Tuple[int, str], List] = {}

    def frame(ri: int, channels: str, k: int):
        key = (ri, channels)
        if key not in pool:
            W, H, _ = resolutions[ri]
            pool[key] = [_pinned(torch.from_numpy(synth.frame(H, W, seed + 17 * ri + j, channels))
                                 .to(torch.float16)) for j in range(frame_pool)]
        return pool[key][k % frame_pool]

    t = 0.0
    out = []
    rings: Dict[int, list] = {}
    counts: Dict[int, int] = {}
    for rid in range(n):
        t += rng.exponential(1.0 / rate)
        sid = int(rng.integers(0, streams))
        name, zoom = algorithms[stream_alg[sid]]
        W, H, _ = resolutions[stream_res[sid]]
        m = models[name]
        f = frame(int(stream_res[sid]), m.channels, rid)
        osz = (int(round(W * zoom)), int(round(H * zoom))) if zoom else None
        r = Request(rid, sid, name, f, t, osz, precision)
        if out_ring > 0:
            OW, OH = m.output_size(W, H, osz)
            ring = rings.setdefault(sid, [])
            if len(ring) < out_ring:
                ring.append(_pinned(torch.empty((m.n_planes, OH, OW), dtype=torch.float16)))
            r.output = ring[counts.get(sid, 0) % out_ring]
            counts[sid] = counts.get(sid, 0) + 1
        out.append(r)
    return out
