"""Batched execution: many frames of many models per launch.

``Batch`` binds a fixed list of jobs (model, input planes, output planes) to
a ``pz_batch`` plan (``include/prescale.h``): RAVU jobs of every model and
frame size run as one persistent kernel per plane dtype pulling 32x8 tiles
from a device counter (plus a second one for the ravu lattice pass); NNEDI3
jobs run as their own passes.  ``Batch.capture()`` records the whole launch
into a CUDA graph so that a steady-state batch costs one graph replay.

``autotune(jobs)`` times the execution strategies of a batch -- one launch
per frame, each model's frames on its own side stream, or the persistent
kernel with 1, 2 or as many CTAs per SM as fit -- on the live device and
caches the winner per GPU and batch signature in a JSON plan cache;
``autotune_tiles`` does the same for the tile layout of one model and frame
shape (tile height x halo staging of the per-frame launches).
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import threading
from dataclasses import dataclass, field, replace
from typing import Dict, List, Optional, Sequence, Tuple

from . import _ffi
from .prescaler import PRECISIONS, STAGINGS, TILE_ROWS, HookModel, check_tile_rows


def _torch():
    import torch
    return torch


def scratch_bytes(model: HookModel, W: int, H: int, planes: int, elem: int, out_size) -> int:
    """Device scratch of one frame's chain: NNEDI3 doubling both axes, the
    row-doubled plane; ravu (lattice), the FP32 int11 plane; else 0."""
    if model.family == "nnedi3" and model.nnedi3_axes(W, H, out_size) == 3:
        return 2 * H * W * elem
    if model.family == "ravu":
        return planes * H * W * 4
    return 0


@dataclass
class Job:
    """One frame through one model: planes are lists of [H][W] CUDA tensors."""
    model: HookModel
    inputs: List["torch.Tensor"]
    outputs: List["torch.Tensor"]
    out_size: Optional[Tuple[int, int]] = None
    precision: str = "fp32"
    scratch: Optional["torch.Tensor"] = None
    staging: str = "tma"   # RAVU halo staging of interior tiles: "tma" boxes or "ldg" clamped loads
    tile_rows: Optional[int] = None   # RAVU tile height of per-frame launches (4, 8, 16; None: the default)

    @staticmethod
    def make(model: HookModel, frame, out_size=None, precision="fp32", out=None, staging=None,
             scratch=None, tile_rows=None) -> "Job":
        """A job for ``frame`` ([H][W] or [C][H][W] CUDA tensor); allocates
        the outputs unless ``out`` is given, and the scratch the chain needs
        (NNEDI3's row-doubled plane, the ravu lattice's int11 plane) unless
        ``scratch`` (a uint8 tensor of at least ``scratch_bytes``) is given."""
        torch = _torch()
        pl = [frame] if frame.dim() == 2 else list(frame.unbind(0))
        H, W = pl[0].shape
        OW, OH = model.output_size(W, H, out_size)
        if out is None:
            outs = list(torch.empty((len(pl), OH, OW), dtype=pl[0].dtype, device=pl[0].device).unbind(0))
        else:
            outs = [out] if out.dim() == 2 else list(out.unbind(0))
        need = scratch_bytes(model, W, H, len(pl), pl[0].element_size(), (OW, OH))
        if scratch is None and need:
            scratch = torch.empty(need, dtype=torch.uint8, device=pl[0].device)
        elif scratch is not None and scratch.numel() < need:
            raise ValueError(f"scratch of {scratch.numel()} bytes, the chain needs {need}")
        staging = staging or model.default_staging
        if staging not in STAGINGS:
            raise ValueError(f"staging {staging!r}: one of {sorted(STAGINGS)}")
        check_tile_rows(tile_rows)
        return Job(model, pl, outs, (OW, OH), precision, scratch, staging, tile_rows)

    def signature(self) -> Tuple:
        p = self.inputs[0]
        return (self.model.name, p.shape[1], p.shape[0], self.out_size, str(p.dtype), self.precision, self.staging,
                self.tile_rows)

    def shape_key(self) -> Tuple:
        """What the tile layout is tuned for: model, frame shape, dtype, output size, precision."""
        p = self.inputs[0]
        return (self.model.name, len(self.inputs), p.shape[1], p.shape[0], str(p.dtype), self.out_size, self.precision)

    def to_c(self) -> _ffi.Job:
        torch = _torch()
        j = _ffi.Job()
        j.model = self.model.device_handle(self.inputs[0].device.index)
        dt = _ffi.PZ_F32 if self.inputs[0].dtype == torch.float32 else _ffi.PZ_F16
        for i, (p, o) in enumerate(zip(self.inputs, self.outputs)):
            j.inp[i] = _ffi.Plane(p.data_ptr(), p.shape[1], p.shape[0], p.stride(0), dt)
            j.out[i] = _ffi.Plane(o.data_ptr(), o.shape[1], o.shape[0], o.stride(0), dt)
        j.n_planes = len(self.inputs)
        j.opts.precision = PRECISIONS[self.precision]
        j.opts.staging = STAGINGS[self.staging]
        j.opts.tile_rows = check_tile_rows(self.tile_rows)
        j.opts.out_width, j.opts.out_height = self.out_size
        if self.model.family == "nnedi3":
            W, H = self.inputs[0].shape[1], self.inputs[0].shape[0]
            j.opts.nnedi3_axes = self.model.nnedi3_axes(W, H, self.out_size)
        if self.scratch is not None:
            j.opts.scratch = self.scratch.data_ptr()
            j.opts.scratch_bytes = self.scratch.numel()
        return j


class Batch:
    """A persistent-launch plan over fixed jobs (their tensors stay bound)."""

    def __init__(self, jobs: Sequence[Job], ctas_per_sm: int = 0, stream=None):
        torch = _torch()
        if not jobs:
            raise ValueError("empty batch")
        self.jobs = list(jobs)
        self.device = self.jobs[0].inputs[0].device
        self._cjobs = (_ffi.Job * len(self.jobs))(*[j.to_c() for j in self.jobs])
        L = _ffi.lib()
        nbytes = L.pz_batch_work_bytes(self._cjobs, len(self.jobs))
        self.work = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=self.device)
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        h = ctypes.c_void_p()
        _ffi.check(L.pz_batch_create(self._cjobs, len(self.jobs), self.work.data_ptr(), self.work.numel(),
                                     int(ctas_per_sm), s.cuda_stream, ctypes.byref(h)))
        self._plan = h.value
        self.graph = None

    def launch(self, stream=None):
        torch = _torch()
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _ffi.check(_ffi.lib().pz_batch_launch(self._plan, s.cuda_stream))
        if not torch.cuda.is_current_stream_capturing():
            # the job table and counters must outlive this launch even if the
            # plan is dropped first (a no-op on the stream they came from)
            self.work.record_stream(s)

    def capture(self):
        """Record one launch into a CUDA graph (call launch() once first so
        every kernel is loaded and configured)."""
        torch = _torch()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            g.capture_begin()
            self.launch(stream=s)
            g.capture_end()
        torch.cuda.current_stream(self.device).wait_stream(s)
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def close(self):
        if getattr(self, "_plan", None):
            _ffi.lib().pz_batch_destroy(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_per_job(jobs: Sequence[Job], stream=None):
    """The unbatched strategy: one pz_run chain per job."""
    for j in jobs:
        j.model.run_raw(j.inputs, j.outputs, out_size=j.out_size, precision=j.precision, stream=stream,
                        scratch=j.scratch)


_STREAM_POOL: Dict[Tuple[int, int], "torch.cuda.Stream"] = {}


def _pool_stream(device, k: int):
    """Side stream k of `device`, created once and kept for the process."""
    torch = _torch()
    key = (device.index if device.index is not None else torch.cuda.current_device(), k)
    if key not in _STREAM_POOL:
        _STREAM_POOL[key] = torch.cuda.Stream(device)
    return _STREAM_POOL[key]


def stream_lanes(jobs: Sequence[Job], per_model: int = 2) -> List[List[Job]]:
    """The launch chains of the co-scheduled strategy: each model's jobs dealt
    in turn to `per_model` chains (one chain when any two of them share a
    scratch buffer, which must then be used in order)."""
    groups: Dict[str, List[Job]] = {}
    for j in jobs:
        groups.setdefault(j.model.name, []).append(j)
    lanes = []
    for _, g in sorted(groups.items()):
        ptrs = [j.scratch.data_ptr() for j in g if j.scratch is not None]
        k = max(1, min(per_model, len(g))) if len(set(ptrs)) == len(ptrs) else 1
        lanes.extend(g[r::k] for r in range(k))
    return lanes


def run_streams(jobs: Sequence[Job], stream=None, max_streams: int = 8, per_model: int = 2):
    """The co-scheduled strategy: the jobs of each model go on side streams
    of their own (forked from and joined back to `stream`; `per_model`
    streams per model, the model's jobs dealt to them in turn), one pz_run
    chain per job, so that the programs of different models run at the same
    time and fill each other's idle issue slots (e.g. an issue-bound program
    beside a shared-memory-bound one), and the launch boundaries of one
    model's frames overlap.  Capturable in a CUDA graph (fork and join are
    stream waits)."""
    torch = _torch()
    dev = jobs[0].inputs[0].device
    main = stream if stream is not None else torch.cuda.current_stream(dev)
    lanes = stream_lanes(jobs, per_model)
    side = [_pool_stream(dev, k) for k in range(min(max_streams, len(lanes)))]
    for s in side:
        s.wait_stream(main)
    for i, lane in enumerate(lanes):
        run_per_job(lane, stream=side[i % len(side)])
    for s in side:
        main.wait_stream(s)


# ------------------------------------------------------------ autotuner ----

STRATEGIES = ("per_job", "streams", "batch:1", "batch:2", "batch:0")


def _default_cache_path() -> str:
    base = os.environ.get("PRESCALER_PLAN_CACHE")
    if base:
        return base
    return os.path.join(os.path.expanduser("~"), ".cache", "mpv_prescalers_gb300", "plans.json")


class PlanCache:
    """Tuned strategies, keyed by GPU name and batch signature (JSON file)."""

    def __init__(self, path: Optional[str] = None):
        self.path = path or _default_cache_path()
        self._lock = threading.Lock()
        self.entries: Dict[str, dict] = {}
        try:
            with open(self.path) as f:
                self.entries = json.load(f)
        except (OSError, ValueError):
            self.entries = {}

    @staticmethod
    def key(gpu: str, jobs: Sequence[Job]) -> str:
        sig = json.dumps(sorted(str(j.signature()) for j in jobs))
        return gpu + ":" + hashlib.sha1(sig.encode()).hexdigest()[:16]

    def get(self, key: str) -> Optional[dict]:
        return self.entries.get(key)

    def put(self, key: str, value: dict) -> None:
        with self._lock:
            self.entries[key] = value
            try:
                os.makedirs(os.path.dirname(self.path), exist_ok=True)
                tmp = self.path + ".tmp"
                with open(tmp, "w") as f:
                    json.dump(self.entries, f, indent=1, sort_keys=True)
                os.replace(tmp, self.path)
            except OSError:
                pass  # a read-only cache location only loses persistence


def autotune_staging(model: HookModel, frame, out_size=None, precision: str = "fp32",
                     cache: Optional[PlanCache] = None, reps: int = 5) -> Tuple[str, Dict[str, float]]:
    """Time clamped-load vs TMA halo staging for one model and frame shape
    on this GPU; the winner is cached per (GPU, model, shape, dtype)."""
    torch = _torch()
    cache = cache or PlanCache()
    gpu = torch.cuda.get_device_name(frame.device)
    key = f"{gpu}:staging:{model.name}:{tuple(frame.shape)}:{frame.dtype}:{out_size}:{precision}"
    hit = cache.get(key)
    if hit:
        return hit["staging"], hit.get("times_ms", {})
    pl = [frame] if frame.dim() == 2 else list(frame.unbind(0))
    H, W = pl[0].shape
    OW, OH = model.output_size(W, H, out_size)
    outs = [torch.empty((OH, OW), dtype=frame.dtype, device=frame.device) for _ in pl]
    times = {st: _time_ms(lambda st=st: model.run_raw(pl, outs, (OW, OH), precision=precision, staging=st), reps)
             for st in ("ldg", "tma")}
    best = min(times, key=times.get)
    cache.put(key, {"staging": best, "times_ms": times})
    return best, times


def tile_layouts(model: HookModel) -> List[Tuple[str, int]]:
    """The (staging, tile_rows) layouts a model's per-frame launches can run:
    every tile height with both stagings; NNEDI3 has a single layout."""
    if model.family == "nnedi3":
        return [(model.default_staging, 8)]
    return [(st, r) for r in TILE_ROWS for st in ("ldg", "tma")]


def autotune_tiles(model: HookModel, frame, out_size=None, precision: str = "fp32",
                   cache: Optional[PlanCache] = None, reps: int = 5) -> Tuple[Tuple[str, int], Dict[str, float]]:
    """Time every tile layout (tile height x halo staging, ``tile_layouts``)
    of one model and frame shape on this GPU; returns the fastest
    ``(staging, tile_rows)`` and the times by ``"staging/rows"``.  Cached per
    (GPU, model, shape, dtype, output size, precision)."""
    torch = _torch()
    layouts = tile_layouts(model)
    if len(layouts) == 1:   # nothing to choose (NNEDI3)
        return layouts[0], {}
    cache = cache or PlanCache()
    pl = [frame] if frame.dim() == 2 else list(frame.unbind(0))
    H, W = pl[0].shape
    OW, OH = model.output_size(W, H, out_size)
    gpu = torch.cuda.get_device_name(frame.device)
    key = f"{gpu}:tiles:{model.name}:{tuple(frame.shape)}:{frame.dtype}:{(OW, OH)}:{precision}"
    hit = cache.get(key)
    if hit:
        return (hit["staging"], hit["tile_rows"]), hit.get("times_ms", {})
    outs = [torch.empty((OH, OW), dtype=frame.dtype, device=frame.device) for _ in pl]
    need = scratch_bytes(model, W, H, len(pl), pl[0].element_size(), (OW, OH))
    scratch = torch.empty(need, dtype=torch.uint8, device=frame.device) if need else None
    times = {}
    for st, r in layouts:
        times[f"{st}/{r}"] = _time_ms(lambda st=st, r=r: model.run_raw(pl, outs, (OW, OH), precision=precision,
                                                                       scratch=scratch, staging=st, tile_rows=r), reps)
    best = min(times, key=times.get)
    st, r = best.split("/")
    cache.put(key, {"staging": st, "tile_rows": int(r), "times_ms": times})
    return (st, int(r)), times


def tune_tiles(jobs: Sequence[Job], cache: Optional[PlanCache] = None, reps: int = 5) -> List[Job]:
    """The jobs with each one's tile layout set to the fastest for its model
    and frame shape (``autotune_tiles``, once per distinct shape)."""
    best: Dict[Tuple, Tuple[str, int]] = {}
    out = []
    for j in jobs:
        k = j.shape_key()
        if k not in best:
            frame = j.inputs[0] if len(j.inputs) == 1 else _torch().stack(j.inputs)
            best[k] = autotune_tiles(j.model, frame, j.out_size, j.precision, cache, reps)[0]
        st, r = best[k]
        out.append(replace(j, staging=st, tile_rows=r))
    return out


def _time_ms(fn, reps: int) -> float:
    torch = _torch()
    fn()
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def autotune(jobs: Sequence[Job], cache: Optional[PlanCache] = None, reps: int = 5,
             strategies: Sequence[str] = STRATEGIES) -> Tuple[str, Dict[str, float]]:
    """Pick the fastest strategy for this batch on this GPU (cached)."""
    torch = _torch()
    cache = cache or PlanCache()
    gpu = torch.cuda.get_device_name(jobs[0].inputs[0].device)
    key = PlanCache.key(gpu, jobs)
    hit = cache.get(key)
    if hit and hit.get("strategy") in strategies:
        return hit["strategy"], hit.get("times_ms", {})
    times = {}
    for st in strategies:
        if st == "per_job":
            times[st] = _time_ms(lambda: run_per_job(jobs), reps)
        elif st == "streams":
            times[st] = _time_ms(lambda: run_streams(jobs), reps)
        else:
            b = Batch(jobs, ctas_per_sm=int(st.split(":")[1]))
            times[st] = _time_ms(b.launch, reps)
            b.close()
    best = min(times, key=times.get)
    cache.put(key, {"strategy": best, "times_ms": times})
    return best, times


class Executor:
    """Runs a fixed batch with its tuned strategy, replaying a CUDA graph.

    With ``tune`` the jobs first take the fastest tile layout of their model
    and frame shape (``tune_tiles``, unless ``tiles`` is false: the jobs'
    own layouts; the per-frame strategies run it, the persistent kernels
    run 8-row tiles), then the fastest strategy."""

    def __init__(self, jobs: Sequence[Job], cache: Optional[PlanCache] = None, tune: bool = True,
                 use_graph: bool = True, tiles: bool = True):
        torch = _torch()
        self.jobs = tune_tiles(jobs, cache) if tune and tiles else list(jobs)
        # the strategy and the time of every candidate (ms per run; empty untuned)
        self.strategy, self.times = autotune(self.jobs, cache) if tune else ("batch:0", {})
        self.batch = None
        self.graph = None
        if self.strategy.startswith("batch:"):
            self.batch = Batch(self.jobs, ctas_per_sm=int(self.strategy.split(":")[1]))
            if use_graph:
                self.batch.launch()
                self.batch.capture()
        elif self.strategy == "streams" and use_graph:
            # the fork / join of the side streams is recorded into the graph
            dev = self.jobs[0].inputs[0].device
            run_streams(self.jobs)   # every kernel loaded before capture
            cur = torch.cuda.current_stream(dev)
            s = torch.cuda.Stream(dev)
            s.wait_stream(cur)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(s):
                g.capture_begin()
                run_streams(self.jobs, stream=s)
                g.capture_end()
            cur.wait_stream(s)
            self.graph = g

    def run(self):
        if self.graph is not None:
            self.graph.replay()
        elif self.strategy == "streams":
            run_streams(self.jobs)
        elif self.batch is None:
            run_per_job(self.jobs)
        elif self.batch.graph is not None:
            self.batch.replay()
        else:
            self.batch.launch()
