"""Benchmark of the prescaler hot path on one GB300 (or N replicas).

Workload (one *step*): the 1080p -> 2160p batch of the reference's second
benchmark configuration -- 8 synthetic 1920x1080 luma planes stored FP16,
each upscaled 2x by ravu-lite-ar-r4 (anti-ringing 0.8) and by two-pass
ravu-r3, i.e. 16 output frames of 3840x2160 per step.  Planes come from the
seeded generator (seed 2000 + frame); LUTs are the ones parsed from the
``.hook`` files when the model cache is present, otherwise seeded synthetic
LUTs of the same shapes (``config.weights`` says which).

Reported (one JSON line on rank 0):

* ``value``: output Mpix/s of the chosen form (FP16 planes, FP16 LUT texels,
  FP32 math), all ranks together, inputs resident in HBM, the two models
  co-scheduled on side streams (``batch.run_streams``: two per model);
  ``single_stream``: the same with one launch chain after another (the
  roofline's per-launch kernel time comes from that loop); ``fp32_value``:
  the plain FP32 form (FP32 planes), single stream, on the same workload.
* ``e2e``: the same metric through ``HookModel.upscale`` with the frames
  copied host->device (pinned) and the upscaled frames copied back every step.
* ``roofline``: the dominant kernel (ravu-lite-ar-r4, FP16 planes) against
  the FP32 pipe; ``hbm`` against measured copy bandwidth.
* ``cpu_baseline``: the FP64 NumPy oracle on a bounded sample of the same
  workload, on the host's cores.
* ``headline``: chosen vs plain FP32 Mpix/s for ravu-lite-ar-r3 and
  nnedi3-nns128-win8x6 on 1920x1080 -> 3840x2160.
* ``precision``: per configuration, the GPU output against the FP64 oracle
  on the same input (the outputs the ``cpu_baseline`` leg computed): max-abs,
  PSNR and, for RAVU, the LUT-key mismatch and boundary rates (frame 0 of the
  bench batch in the chosen form; ravu-lite-r3 on 960x540 in plain FP32;
  nnedi3-nns128-win8x6 on 1280x720 in both forms).

``--impl reference`` times the reference arm on all host cores, same metric
and workload: the reference's shader text compiled as FP64 C++ and run
through the hook host's pass sequence (``oracle/_ref``, compiled by
``build()``; the shaders themselves need an OpenGL/Vulkan host that this
machine does not have), else the FP64 NumPy restatement of its arithmetic.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)
import __graft_entry__ as _entry  # noqa: E402

H, W, NFRAMES = 1080, 1920, 8
MODELS = ("ravu-lite-ar-r4", "ravu-r3")
SEED0 = 2000
# algorithmic FP32 flops per INPUT pixel (structure tensor 13/point, eigen+key
# 35, filter 8/tap, anti-ringing 48/AR tap + 32; lattice ravu: 3 keyed passes)
FLOPS_PER_IN_PX = {"ravu-lite-ar-r4": 13 * 25 + 35 + 8 * 49 + 48 * 13 + 32,
                   "ravu-lite-ar-r3": 13 * 9 + 35 + 8 * 25 + 48 * 13 + 32,
                   "ravu-r3": 3 * (13 * 16 + 35 + 1.5 * 36 + 2)}


def _pkg():
    return _entry._package()


def _layouts(jobs):
    """The tile layout ("staging/rows") each distinct model and frame shape of
    a job list runs."""
    out = {}
    for j in jobs:
        p = j.inputs[0]
        k = f"{j.model.name} {p.shape[1]}x{p.shape[0]}->{j.out_size[0]}x{j.out_size[1]}"
        out[k] = f"{j.staging}/{j.tile_rows or 'default'}"
    return out


# ------------------------------------------------------------------ CPU ---

_FRAME = {}   # per worker process: the synthetic frame of each seed, made before timing


def _frame(seed: int, h: int = H, w: int = W, fp16: bool = True):
    """The synthetic luma plane of `seed`; fp16: rounded to FP16, the values
    the chosen form's FP16 planes hold (the bench batch is stored FP16)."""
    k = (seed, h, w, fp16)
    if k not in _FRAME:
        from mpv_prescalers_gb300 import synth
        x = synth.luma_plane(h, w, seed)
        _FRAME[k] = x.astype(np.float16).astype(np.float32) if fp16 else x
    return _FRAME[k]


def _worker_init(seed: int, kind: str):
    """Pool initializer: package, frame and (reference) compiled shaders are
    ready before the timed strips start."""
    sys.path.insert(0, REPO)
    _pkg()
    _frame(seed)
    if kind == "reference":
        for n in MODELS:
            _ref_strip((n, 0, 8, seed))       # loads the shader library and its LUT textures
    else:
        import oracle  # noqa: F401


def _cpu_strip(args):
    """Oracle on rows [y0, y1) of one frame (with the window halo); returns
    (output pixels, seconds, payload).  With `keep` the payload holds the
    strip's FP64 outputs (as FP32), and for RAVU its keys, boundary flags
    and key margins, for the precision check of the GPU run."""
    name, y0, y1, seed, h, w, fp16, keep = args
    sys.path.insert(0, REPO)
    _pkg()
    from mpv_prescalers_gb300 import synth
    import oracle
    hm, _ = synth.model_for(name)
    x = _frame(seed, h, w, fp16)
    pad = 6  # covers the windows: lite r4 +-3, ravu r3 int11 (+-3) feeding the lattice (+-3), nnedi3 +-5
    a, b = max(0, y0 - pad), min(h, y1 + pad)
    t = time.perf_counter()
    if hm.family == "nnedi3":
        y, info = oracle.nnedi3_upscale(hm.model, x[a:b])
    else:
        y, info = oracle.keyed_upscale(hm.model, x[a:b][None])
    dt = time.perf_counter() - t
    payload = None
    if keep:
        r0, r1 = y0 - a, y1 - a
        payload = {"y0": y0, "out": np.asarray(y[..., 2 * r0:2 * r1, :], dtype=np.float32)}
        if hm.family != "nnedi3":
            payload.update({k: info[k][..., r0:r1, :] for k in ("key", "boundary")})
            payload["margin"] = np.asarray(info["margin"][..., r0:r1, :], dtype=np.float32)
    return (y1 - y0) * w * 4, dt, payload


_REF_LIBS = {}


def _ref_lib(name: str):
    """The reference's own shader text for `name`, compiled for this machine
    (oracle/_ref, built by build()), or None."""
    import ctypes
    if name not in _REF_LIBS:
        path = os.path.join(REPO, "oracle", "_ref", name + ".so")
        lib = None
        if os.path.exists(path):
            try:
                lib = ctypes.CDLL(path)
                lib.ref_run.restype = ctypes.c_int
            except OSError:
                lib = None
        _REF_LIBS[name] = lib
    return _REF_LIBS[name]


def _ref_strip(args):
    """The compiled reference shaders on rows [y0, y1) of one frame (with the
    window halo): every pass of the file per pixel, as the hook host runs it."""
    import ctypes
    name, y0, y1, seed = args[:4]
    sys.path.insert(0, REPO)
    _pkg()
    from mpv_prescalers_gb300 import synth
    lib = _ref_lib(name)
    x = _frame(seed)
    pad = 6
    a, b = max(0, y0 - pad), min(H, y1 + pad)
    xin = np.ascontiguousarray(x[a:b], dtype=np.float64)
    h = b - a
    out = np.empty(4 * h * W)
    dims = (ctypes.c_int * 2)()
    t = time.perf_counter()
    rc = lib.ref_run(xin.ctypes.data_as(ctypes.c_void_p), 1, h, W, 2 * W, 2 * h,
                     out.ctypes.data_as(ctypes.c_void_p), out.size, dims)
    dt = time.perf_counter() - t
    if rc != 0 or (dims[0], dims[1]) != (2 * h, 2 * W):
        raise RuntimeError(f"reference {name}: ref_run {rc}, dims {dims[0]}x{dims[1]}")
    return (y1 - y0) * W * 4, dt, None


def reference_available() -> bool:
    return all(_ref_lib(n) is not None for n in MODELS)


# The other configurations whose precision the bench line states: (label,
# model, height, width, seed, FP16-rounded input).  Seeds: 1000 * the
# configuration's number + frame.
CHECKS = (("config1 ravu-lite-r3 960x540 fp32", "ravu-lite-r3", 540, 960, 1000, False),
          ("config3 nnedi3-nns128-win8x6 1280x720 fp32", "nnedi3-nns128-win8x6", 720, 1280, 3000, False),
          ("config3 nnedi3-nns128-win8x6 1280x720 fp16", "nnedi3-nns128-win8x6", 720, 1280, 3000, True))


def _assemble(parts):
    """Stack the kept strips of one plane (in row order) into whole arrays."""
    parts = sorted((p for p in parts if p is not None), key=lambda p: p["y0"])
    return {k: np.concatenate([p[k] for p in parts], axis=-2) for k in parts[0] if k != "y0"}


def cpu_baseline(rows_per_model: int, workers: int, kind: str = "port", checks: bool = False):
    """CPU Mpix/s on a bounded sample: `rows_per_model` input rows of frame 0
    of the bench batch (FP16-rounded, the values the chosen form reads) per
    model, split in strips over `workers` spawned processes; `kind` "port"
    runs the FP64 NumPy oracle, "reference" the reference's shader text
    compiled as C++ (oracle/_ref).

    With `checks` (oracle only) it also returns the FP64 outputs it computed
    -- frame 0 of each model, plus untimed oracle runs of the CHECKS
    configurations -- as {label: arrays} for the precision figures of the
    GPU run."""
    ctx = mp.get_context("spawn")
    fn = _ref_strip if kind == "reference" else _cpu_strip
    keep = checks and kind == "port"
    tasks = []
    strip = max(8, rows_per_model // workers)
    for name in MODELS:
        for y0 in range(0, rows_per_model, strip):
            tasks.append((name, y0, min(rows_per_model, y0 + strip), SEED0, H, W, True, keep))
    refs = {}
    with ctx.Pool(workers, initializer=_worker_init, initargs=(SEED0, kind)) as pool:
        pool.map(fn, [(n, 0, 8, SEED0, H, W, True, False) for n in MODELS] * workers)  # warm the workers
        t = time.perf_counter()
        res = pool.map(fn, tasks)
        wall = time.perf_counter() - t
        if keep:
            for name in MODELS:
                refs[name] = _assemble([r[2] for r, tk in zip(res, tasks) if tk[0] == name])
            extra = []
            for label, name, h, w, seed, fp16 in CHECKS:
                st = max(8, h // workers)
                extra += [(label, (name, y0, min(h, y0 + st), seed, h, w, fp16, True)) for y0 in range(0, h, st)]
            out = pool.map(fn, [e[1] for e in extra])
            for label, *_ in CHECKS:
                refs[label] = _assemble([o[2] for o, e in zip(out, extra) if e[0] == label])
    px = sum(r[0] for r in res)
    what = ("the reference's shader text compiled as FP64 C++ (every pass per pixel, as the hook host runs it)"
            if kind == "reference" else "FP64 NumPy oracle")
    cb = {"value": px / wall / 1e6, "unit": "Mpix/s", "cores": workers, "kind": kind,
          "sample": f"{rows_per_model} of {H} input rows of one 1920x1080 frame per model "
                    f"({', '.join(MODELS)}), {what}, {len(tasks)} strips on {workers} processes",
          "seconds": wall}
    return (cb, refs) if checks else cb


# ---------------------------------------------------------------- clocks ---

class Clocks:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [v.strip() for v in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------- GPU ---

def max_over_ranks(ms: float, device=None) -> float:
    """The slowest rank's time (replicas: the job ends with its last rank)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(out_px_per_rank_step: float, steps: int, ms: float, world: int) -> float:
    """Whole-job Mpix/s: the pixels all ranks produced over the slowest rank's time."""
    return world * out_px_per_rank_step * steps / (ms / 1e3) / 1e6


def _key_figures(kg, ref):
    """Key agreement of a GPU run with the oracle's keys (arrays of the same
    shape): mismatch and boundary rates, mismatches off the boundary, and the
    largest margin (units of 2^-24 of the tensor scale) a flipped key had."""
    kg = np.asarray(kg).reshape(ref["key"].shape)
    mism = kg != ref["key"]
    bnd = ref["boundary"]
    marg = ref["margin"][mism] / 2.0 ** -24
    return {"keys": int(mism.size), "key_mismatch_rate": float(mism.mean()), "boundary_rate": float(bnd.mean()),
            "mismatch_off_boundary": int((mism & ~bnd).sum()),
            "max_mismatch_margin_ulp": float(marg.max()) if marg.size else 0.0}


def _value_figures(y, ref_out, flipped=None):
    """max-abs and PSNR (peak 1.0) of GPU output rows against the oracle's;
    with `flipped` (output pixels whose own LUT key differs from the
    oracle's) also the max-abs over the pixels whose keys agree."""
    y = np.asarray(y, dtype=np.float64).reshape(ref_out.shape)
    d = np.abs(y - ref_out.astype(np.float64))
    mse = float(np.mean(d * d))
    f = {"max_abs": float(d.max()), "psnr_db": float("inf") if mse == 0 else 10 * np.log10(1 / mse)}
    if flipped is not None:
        keep = ~flipped
        f["max_abs_key_matched"] = float(d[..., keep].max()) if keep.any() else 0.0
    return f


def _flipped(family, mism, out_hw):
    """Output pixels of flipped keys: the 2x2 block of a lite key, the lattice
    sample of an int11 / int10 / int01 key."""
    if family == "ravu":
        m = np.zeros(out_hw, dtype=bool)
        m[1::2, 1::2], m[0::2, 1::2], m[1::2, 0::2] = mism[0], mism[1], mism[2]
        return m
    return np.repeat(np.repeat(mism, 2, 0), 2, 1)


def precision_figures(models, refs, dev):
    """Per configuration: the GPU's output (and keys) against the FP64
    outputs the CPU leg computed on the same inputs."""
    import torch
    from mpv_prescalers_gb300 import synth
    figs = {}
    for n in MODELS:  # frame 0 of the bench batch, chosen form, FP16 planes
        ref = refs[n]
        rows = ref["out"].shape[-2] // 2
        x = torch.from_numpy(_frame(SEED0)).to(dev, torch.float16)
        y, k = models[n].upscale(x, precision="fast", return_keys=True)
        k = k.cpu().numpy()
        mism = k[..., :rows, :] != ref["key"]
        f = _value_figures(y.float().cpu().numpy()[..., :2 * rows, :], ref["out"],
                           _flipped(models[n].family, mism, ref["out"].shape[-2:]))
        if k.ndim == 3:   # ravu: int11, int10, int01 passes
            for i, pas in enumerate(("int11", "int10", "int01")):
                f[pas] = _key_figures(k[i, :rows], {q: ref[q][i] for q in ("key", "boundary", "margin")})
            f["note"] = ("int10/int01 windows read int11 (the GPU's FP32 plane, the oracle's FP64 one); an int11 "
                         "key that flips on its boundary changes its neighbours' lattice windows, so int10/int01 "
                         "flips off their own boundary follow from int11 flips (the parity tests compare each "
                         "lattice pass on the GPU's own int11 plane)")
        else:
            f.update(_key_figures(k[:rows], ref))
        figs[f"config2 {n} {rows}x{W}->{2 * rows}x{2 * W} fp16 fast"] = f
    for label, name, h, w, seed, fp16 in CHECKS:
        ref = refs[label]
        hm = models.get(name) or synth.model_for(name)[0]
        x = torch.from_numpy(_frame(seed, h, w, fp16)).to(dev, torch.float16 if fp16 else torch.float32)
        prec = "fast" if fp16 else "fp32"
        if hm.family == "nnedi3":
            y = hm.upscale(x, precision=prec)
            f = _value_figures(y.float().cpu().numpy(), ref["out"])
        else:
            y, k = hm.upscale(x, precision=prec, return_keys=True)
            k = k.cpu().numpy()
            f = _value_figures(y.float().cpu().numpy(), ref["out"],
                               _flipped(hm.family, k.reshape(ref["key"].shape) != ref["key"], ref["out"].shape[-2:]))
            f.update(_key_figures(k, ref))
        f["form"] = "fast (FP16 planes, FP16 tensor-core neurons)" if fp16 else "plain FP32"
        figs[label] = f
    figs["oracle"] = "FP64 NumPy restatement on the same inputs (outputs of the cpu_baseline leg)"
    return figs


def run_gpu(args, refs=None):
    import torch
    import torch.distributed as dist
    pkg = _pkg()
    from mpv_prescalers_gb300 import synth

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    def barrier():
        if world > 1:
            dist.barrier()

    models, sources = {}, {}
    for n in MODELS + ("ravu-lite-ar-r3", "nnedi3-nns128-win8x6"):
        models[n], sources[n] = synth.model_for(n)
    frames = np.stack([synth.luma_plane(H, W, SEED0 + f) for f in range(NFRAMES)])
    x16 = torch.from_numpy(frames).to(dev, torch.float16)
    x32 = torch.from_numpy(frames).to(dev, torch.float32)
    outs16 = {n: torch.empty((NFRAMES, 2 * H, 2 * W), dtype=torch.float16, device=dev) for n in MODELS}
    outs32 = {n: torch.empty((NFRAMES, 2 * H, 2 * W), dtype=torch.float32, device=dev) for n in MODELS}
    stream = torch.cuda.current_stream(dev)
    launches_per_step = NFRAMES * (1 + 2)  # lite: 1 kernel/frame, lattice: 2
    # the lattice's FP32 int11 plane, reused by every frame (one stream)
    scratch = torch.empty(H * W * 4, dtype=torch.uint8, device=dev)

    def step(xs, outs, prec, ev=None):
        for n in MODELS:
            hm = models[n]
            for f in range(NFRAMES):
                if ev is not None and n == MODELS[0]:
                    ev.append((torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)))
                    ev[-1][0].record(stream)
                hm.run_raw([xs[f]], [outs[n][f]], out_size=(2 * W, 2 * H), precision=prec, stream=stream,
                           scratch=scratch)
                if ev is not None and n == MODELS[0]:
                    ev[-1][1].record(stream)

    def timed(xs, outs, prec, steps, warmup, kernel_events=None):
        for _ in range(warmup):
            step(xs, outs, prec)
        torch.cuda.synchronize()
        barrier()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(steps):
            step(xs, outs, prec, kernel_events)
        t1.record(stream)
        torch.cuda.synchronize()
        barrier()
        return max_over_ranks(t0.elapsed_time(t1), dev)

    out_px_step = len(MODELS) * NFRAMES * (2 * W) * (2 * H)
    kev = []
    clk = Clocks(local).__enter__()   # sampled over all three timed loops (device, FP32, end to end)
    # chosen form: FP16 planes, FP16 LUT texels (lite), FP32 math; plain form: FP32 everything
    ms16 = timed(x16, outs16, "fast", args.steps, args.warmup, kev)
    ms32 = timed(x32, outs32, "fp32", args.steps, args.warmup)
    value = job_value(out_px_step, args.steps, ms16, world)
    fp32_value = job_value(out_px_step, args.steps, ms32, world)
    kern_ms = statistics.mean(a.elapsed_time(b) for a, b in kev)

    # the same step with the two models co-scheduled: each model's frames
    # dealt to two side streams of its own, forked from and joined back to
    # the timed stream (batch.run_streams), so the two programs share the SMs
    from mpv_prescalers_gb300 import batch as _batch
    co_jobs = [_batch.Job.make(models[n], x16[f], out=outs16[n][f], precision="fast") for n in MODELS
               for f in range(NFRAMES)]
    for _ in range(args.warmup):
        _batch.run_streams(co_jobs, stream=stream)
    torch.cuda.synchronize()
    barrier()
    c0 = torch.cuda.Event(enable_timing=True)
    c1 = torch.cuda.Event(enable_timing=True)
    c0.record(stream)
    for _ in range(args.steps):
        _batch.run_streams(co_jobs, stream=stream)
    c1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms_co = max_over_ranks(c0.elapsed_time(c1), dev)
    co_value = job_value(out_px_step, args.steps, ms_co, world)
    del co_jobs

    # ---- end to end: pinned host frames in, upscaled frames back, per step
    host_in = torch.from_numpy(frames).to(torch.float16).unsqueeze(1).pin_memory()
    host_out = {n: torch.empty((NFRAMES, 1, 2 * H, 2 * W), dtype=torch.float16).pin_memory() for n in MODELS}

    def e2e_step():
        # public API on host frames: H2D copy, upscale and D2H copy of frame i
        # overlap with its neighbours (copy streams and the model's own side
        # stream); both models' calls are queued before waiting, so their
        # kernels share the GPU and their copies the host link, and the step
        # ends when every frame is back
        pending = [models[n].upscale_host(host_in, out=host_out[n], precision="fast", wait=False)[1]
                   for n in MODELS]
        for ev in pending:
            ev.synchronize()

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    barrier()
    # a step returns when the frames are back in host memory; the two events
    # on the (otherwise idle) default stream bracket that wall time
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1), dev)
    clk.__exit__(None, None, None)
    e2e_value = job_value(out_px_step, args.steps, e2e_ms, world)

    # ---- headline pairs at 1080p -> 2160p (single frame, chosen vs FP32)
    headline = {}
    for n in ("ravu-lite-ar-r3", "nnedi3-nns128-win8x6"):
        hm = models[n]
        res = {}
        for prec, dt in (("fast", torch.float16), ("fp32", torch.float32)):
            xi = x32[0].to(dt)
            yo = torch.empty((2 * H, 2 * W), dtype=dt, device=dev)
            scratch = torch.empty(2 * H * W * xi.element_size(), dtype=torch.uint8, device=dev)
            for _ in range(3):
                hm.run_raw([xi], [yo], out_size=(2 * W, 2 * H), precision=prec, scratch=scratch)
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            reps = 10
            a.record(stream)
            for _ in range(reps):
                hm.run_raw([xi], [yo], out_size=(2 * W, 2 * H), precision=prec, scratch=scratch)
            b.record(stream)
            torch.cuda.synchronize()
            res[prec] = 4 * H * W * reps / (a.elapsed_time(b) / 1e3) / 1e6
        # the batched form: all 8 FP16 frames through the batch executor (tile
        # layout and strategy tuned on this GPU, replayed from a CUDA graph
        # unless one launch chain per frame wins),
        # and as one persistent launch (NNEDI3: its stream-ordered passes)
        # captured in a CUDA graph and replayed
        import tempfile
        from mpv_prescalers_gb300 import batch as _batch
        bjobs = [_batch.Job.make(hm, x16[f], precision="fast") for f in range(NFRAMES)]
        ex = _batch.Executor(bjobs, cache=_batch.PlanCache(os.path.join(tempfile.mkdtemp(), "h.json")))
        plan = _batch.Batch(bjobs)
        plan.launch()
        plan.capture()
        reps = 5
        for key, run in (("batched", ex.run), ("persistent", plan.replay)):
            for _ in range(3):
                run()
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                run()
            b.record(stream)
            torch.cuda.synchronize()
            res[key] = NFRAMES * 4 * H * W * reps / (a.elapsed_time(b) / 1e3) / 1e6
        res["strategy"] = ex.strategy
        plan.close()
        del bjobs, ex
        headline[n] = {"chosen_mpix_s": res["fast"], "fp32_mpix_s": res["fp32"],
                       "ratio": res["fast"] / res["fp32"], "chosen": "FP16 planes" + (
                           ", FP16 tensor-core neurons" if n.startswith("nnedi3") else
                           ", FP16 LUT texels, FP32 math"),
                       "batched_mpix_s": res["batched"], "batched_ratio": res["batched"] / res["fp32"],
                       "batched": f"{NFRAMES} FP16 frames through batch.Executor (tile layout and strategy tuned "
                                  f"on this GPU: '{res['strategy']}'; graph replay for the batch and stream strategies)",
                       "persistent_mpix_s": res["persistent"],
                       "persistent": f"{NFRAMES} FP16 frames per persistent launch, CUDA graph replay"}

    # ---- tile layouts of the workload's programs: every tile height x halo
    # staging of one 1080p FP16 frame, fast form (batch.autotune_tiles)
    import tempfile
    from mpv_prescalers_gb300 import batch as _batch
    tile_sweep = {}
    tcache = _batch.PlanCache(os.path.join(tempfile.mkdtemp(), "tiles.json"))
    for n in MODELS:
        (st, rows), t = _batch.autotune_tiles(models[n], x16[0], precision="fast", cache=tcache, reps=10)
        tile_sweep[n] = {"best": f"{st}/{rows}", "us": {k: round(v * 1e3, 1) for k, v in t.items()}}

    # ---- precision of each configuration against the FP64 oracle
    precision = precision_figures(models, refs, dev) if refs else None

    # ---- the other configurations, measured as batches (informational)
    configs = {}
    if args.configs:
        from mpv_prescalers_gb300 import batch as _batch
        # mixed persistent batch: 16 RGB frames through ravu-zoom-ar-r2-rgb at
        # 1.5x and at 2.25x, plus 16 4:4:4 YUV frames through ravu-r4-yuv, FP16,
        # fast form, strategy picked by the autotuner, replayed from a graph
        zm, _ = synth.model_for("ravu-zoom-ar-r2-rgb")
        ym, _ = synth.model_for("ravu-r4-yuv")
        jobs, out_px = [], 0
        for f in range(16):
            rgb = torch.from_numpy(synth.rgb_frame(H, W, 4000 + f)).to(dev, torch.float16)
            yuv = torch.from_numpy(synth.yuv_frame(H, W, 4100 + f)).to(dev, torch.float16)
            for zr in (1.5, 2.25):
                osz = (int(W * zr), int(H * zr))
                jobs.append(_batch.Job.make(zm, rgb, out_size=osz, precision="fast"))
                out_px += osz[0] * osz[1]
            jobs.append(_batch.Job.make(ym, yuv, precision="fast"))
            out_px += 4 * H * W
        import tempfile
        ex = _batch.Executor(jobs, cache=_batch.PlanCache(os.path.join(tempfile.mkdtemp(), "plans.json")))
        for _ in range(2):
            ex.run()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(3):
            ex.run()
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / 3
        configs["zoom_rgb_1.5x_2.25x_plus_ravu_r4_yuv_16_frames_each"] = {
            "jobs": len(jobs), "ms": ms, "out_mpix_s": out_px / (ms / 1e3) / 1e6, "strategy": ex.strategy,
            "times_ms": ex.times, "tile_layouts": _layouts(ex.jobs), "form": "FP16 planes, fast form"}
        del ex, jobs
        # one tick of a 64-stream player: a frame of each stream through the
        # serving mix (resolutions 480p-2160p, ravu-lite-ar-r3 / ravu-r4-yuv /
        # nnedi3-nns64-win8x4 / ravu-zoom-ar-r2 at 1.75x), FP16, fast form:
        # one launch chain per frame against the persistent batch replayed
        # from a CUDA graph, and the strategy the autotuner picks
        from mpv_prescalers_gb300 import serve
        tick_models = {name: synth.model_for(name)[0] for name, _ in serve.ALGORITHMS}
        tick = serve.poisson_trace(tick_models, 64, rate=1e6, streams=64, frame_pool=1, seed=5002, out_ring=0)
        tjobs = [_batch.Job.make(tick_models[r.model], r.frame.to(dev), out_size=r.out_size, precision="fast")
                 for r in tick]
        per_job_ms = _batch._time_ms(lambda: _batch.run_per_job(tjobs), 5)
        tb = _batch.Batch(tjobs)
        tb.launch()
        tb.capture()
        batch_ms = _batch._time_ms(tb.replay, 5)
        tb.close()
        tcache = _batch.PlanCache(os.path.join(tempfile.mkdtemp(), "p.json"))
        strategy, ttimes = _batch.autotune(tjobs, cache=tcache)
        # the same tick with every frame on its tuned tile layout
        tuned = _batch.tune_tiles(tjobs, cache=tcache)
        tstrategy, tttimes = _batch.autotune(tuned, cache=tcache)
        tick_px = sum(j.outputs[0].shape[-1] * j.outputs[0].shape[-2] * len(j.outputs) for j in tjobs)
        configs["serving_tick_64_frames"] = {
            "frames": len(tjobs), "per_job_ms": per_job_ms, "batch_graph_ms": batch_ms,
            "batch_vs_per_job": per_job_ms / batch_ms, "autotuned": strategy, "times_ms": ttimes,
            "out_mpix_s_batch": tick_px / (batch_ms / 1e3) / 1e6,
            "tiles_tuned": {"autotuned": tstrategy, "times_ms": tttimes, "tile_layouts": _layouts(tuned)}}
        del tuned
        del tjobs
        # NNEDI3 nns128-win8x6 on 4 frames of 1280x720, fast vs plain FP32
        nm = models["nnedi3-nns128-win8x6"]
        res = {}
        for prec, dt in (("fast", torch.float16), ("fp32", torch.float32)):
            xs = [torch.from_numpy(synth.luma_plane(720, 1280, 3000 + f)).to(dev, dt) for f in range(4)]
            ys = [torch.empty((1440, 2560), dtype=dt, device=dev) for _ in range(4)]
            sc = torch.empty(2 * 720 * 1280 * xs[0].element_size(), dtype=torch.uint8, device=dev)
            run4 = lambda: [nm.run_raw([x], [y], out_size=(2560, 1440), precision=prec, scratch=sc)
                            for x, y in zip(xs, ys)]
            run4()
            torch.cuda.synchronize()
            a.record()
            for _ in range(3):
                run4()
            b.record()
            torch.cuda.synchronize()
            res[prec] = a.elapsed_time(b) / 3
        configs["nnedi3_nns128_win8x6_4x1280x720"] = {
            "fast_ms": res["fast"], "fp32_ms": res["fp32"], "ratio": res["fp32"] / res["fast"],
            "fast_out_mpix_s": 4 * 2560 * 1440 / (res["fast"] / 1e3) / 1e6}

    # ---- serving: Poisson arrivals over 64 streams, mixed resolutions and
    # algorithms (the serving configuration), against serial plain FP32
    serving = None
    if args.serve_requests > 0:
        from mpv_prescalers_gb300 import serve
        smodels = {name: synth.model_for(name)[0] for name, _ in serve.ALGORITHMS}
        serve.Server(smodels).run(serve.warmup_trace(smodels))
        # each stream's output frames are the caller's (a ring of 3 pinned
        # buffers per stream, the default); the same trace with one host
        # frame page-locked per request is reported beside it.  Each measured
        # trace follows an untimed run of a trace of the same shape, so the
        # device allocator already holds what concurrent requests need (a
        # steady-state server; growing it mid-trace synchronises the device)
        # One server serves every measured trace, set up as a deployment would be:
        # its slot arenas sized for the largest request of the mix (reserve) and
        # one untimed trace served before the measured ones.  Every trace is
        # run twice and its second pass measured, the serial baseline's too:
        # a player's frame buffers in steady state (the first pass of a trace
        # also pays for the first device access to each of its host frames).
        # Both sides run in real time: requests are taken up at their arrival.
        trace = serve.poisson_trace(smodels, args.serve_requests, rate=240.0, streams=64, frame_pool=1)
        srv = serve.Server(smodels, hbm_budget=40e9, slots=8)
        srv.reserve(trace)
        srv.run(serve.poisson_trace(smodels, args.serve_requests, rate=4800.0, streams=64, frame_pool=1))
        srv.run(trace)
        served = srv.run(trace)
        alloc_trace = serve.poisson_trace(smodels, args.serve_requests, rate=240.0, streams=64, frame_pool=1,
                                          out_ring=0)
        srv.run(alloc_trace)
        for r in alloc_trace:   # the measured pass takes a host frame per request again (from the
            r.output = None     # caching host allocator, which holds the warm pass's frames)
        served_alloc = srv.run(alloc_trace)
        serial = serve.serial_baseline(smodels, trace, passes=2)
        serial_fast = serve.serial_baseline(smodels, trace, passes=2, precision="fast")
        # saturating load: the same mix arriving 20x faster (4800 frames/s),
        # beyond what one request at a time can keep up with, so admission
        # by budget and slots and the overlap of requests decide the numbers
        sat = serve.poisson_trace(smodels, args.serve_requests, rate=4800.0, streams=64, frame_pool=1, seed=5001)
        srv.run(sat)
        served_sat = srv.run(sat)
        serial_sat = serve.serial_baseline(smodels, sat, passes=2)
        serving = {"trace": f"{len(trace)} requests, Poisson 240 frames/s over 64 streams, resolutions "
                            "{480p .3, 720p .3, 1080p .3, 2160p .1}, algorithms {ravu-lite-ar-r3, ravu-r4-yuv, "
                            "nnedi3-nns64-win8x4, ravu-zoom-ar-r2 at 1.75x}, FP16 planes, 40 GB budget; "
                            "results into the caller's pinned frames (3 per stream); served and serial both in "
                            "real time, second pass of each trace measured",
                   "served": served, "served_host_frame_per_request": served_alloc, "serial_fp32": serial,
                   "serial_fast": serial_fast,
                   "saturated": {"trace": f"{len(sat)} requests of the same mix at 4800 frames/s",
                                 "served": served_sat, "serial_fp32": serial_sat}}

    props = torch.cuda.get_device_properties(dev)
    clocks = clk.summary()
    sm_mhz = clocks["sm_mhz"] or 0.0
    fl = FLOPS_PER_IN_PX[MODELS[0]] * H * W
    achieved_tf = fl / (kern_ms / 1e3) / 1e12
    max_mhz = clocks.get("sm_max_mhz") or 2070.0
    peak_tf = props.multi_processor_count * 256 * max_mhz * 1e6 / 1e12
    algo_bytes = H * W * 2 + 4 * H * W * 2  # FP16 plane in + 2x2 FP16 out
    peaks = {}
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    line = {
        "metric": "Out Mpix/s 1080p->2160p (ravu-lite-ar-r4 + two-pass ravu-r3, 8 frames each)",
        "value": co_value, "unit": "Mpix/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_co / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp16 planes + fp16 lut texels, fp32 math", "data": "synthetic (seeded sinusoids+polygons+noise)",
        "config": {"workload": "8x 1920x1080 FP16 luma -> 3840x2160 through ravu-lite-ar-r4 and ravu-r3",
                   "frames_per_model": NFRAMES, "weights": {n: sources[n] for n in MODELS},
                   "l2": "per-model working set 166 MB (33 MB in + 133 MB out) > 129 MB L2",
                   "parallelism": f"replicas x{world}"},
        "execution": "chosen form, the two models co-scheduled: each model's 8 frames dealt to two side streams "
                     "of its own, forked from and joined to the timed stream (batch.run_streams)",
        "single_stream": {"value": value, "ms_per_step": ms16 / args.steps,
                          "how": "the same frames one launch chain after another on one stream; the roofline's "
                                 "per-launch kernel time comes from this loop"},
        "fp32_value": fp32_value, "chosen_vs_fp32": value / fp32_value,
        "tile_sweep": tile_sweep,
        "e2e": {"value": e2e_value, "unit": "Mpix/s",
                # each model's call copies the frames in
                "h2d_bytes_per_step": int(len(MODELS) * host_in.numel() * host_in.element_size()),
                "d2h_bytes_per_step": int(sum(t.numel() * t.element_size() for t in host_out.values()))},
        "roofline": {"bound": "fp32", "kernel": "LiteTile<4, AR, half, FP16 texels> (ravu-lite-ar-r4, fast form)",
                     "achieved": achieved_tf, "peak": peak_tf, "unit": "TFLOP/s", "frac": achieved_tf / peak_tf,
                     "peak_source": f"{props.multi_processor_count} SMs x 128 FFMA/clk x 2 x {max_mhz:.0f} MHz "
                                    "(FP32 pipe; not in MEASURED_PEAKS.json)",
                     "flops_per_launch": fl, "launch_ms": kern_ms,
                     "hbm": {"achieved": algo_bytes / (kern_ms / 1e3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                             "frac": algo_bytes / (kern_ms / 1e3) / 1e9 / hbm_peak,
                             "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
                     # dram__bytes_read.sum + dram__bytes_write.sum of this kernel on one 1080p
                     # frame (ncu, profiles/lite_tile_h16_ravu-lite-ar-r4_1080p_fp16.md): the FP16
                     # input plane (4.15 MB) with its tile halos and the LUT; the 16.6 MB output is
                     # still in L2 when the launch ends
                     "traffic": 4997120, "traffic_unit": "bytes per launch",
                     "algorithmic_bytes": algo_bytes},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks,
        "headline": headline,
        "precision": precision,
        "serving": serving,
        "other_configs": configs,
        "device": props.name,
    }
    if world > 1:
        dist.destroy_process_group()
    return line if rank == 0 else None


# ------------------------------------------------------------- reference ---

def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    workers = len(os.sched_getaffinity(0))
    # the reference's own shader text compiled for this machine when build()
    # made it, else the NumPy restatement of its arithmetic
    kind = "reference" if reference_available() else "port"
    # each step is a bounded sample: rows per step are sized from a calibration
    # run so that all steps together take about `ref_budget` seconds
    calib = cpu_baseline(2 * workers, workers, kind)
    rows_per_s = 2 * workers * len(MODELS) / max(calib["seconds"], 1e-3) / len(MODELS)
    rows = int(max(16, min(args.ref_rows, args.ref_budget / max(args.steps, 1) * rows_per_s)))
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_baseline(16, workers, kind)
    vals = []
    for _ in range(args.steps):
        vals.append(cpu_baseline(rows, workers, kind))
    v = statistics.mean(r["value"] for r in vals)
    cb = dict(vals[-1])
    cb["value"] = v
    return {"impl": "reference", "metric": "Out Mpix/s 1080p->2160p (ravu-lite-ar-r4 + two-pass ravu-r3, 8 frames each)",
            "value": v, "unit": "Mpix/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.mean(r["seconds"] for r in vals) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded sinusoids+polygons+noise)",
            "config": {"workload": "8x 1920x1080 FP16 luma -> 3840x2160 through ravu-lite-ar-r4 and ravu-r3",
                       "sample": cb["sample"]},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference's shaders need mpv + OpenGL/Vulkan (unavailable on this box); the reference "
                    "arm runs their GLSL bodies compiled as FP64 C++ (oracle/_ref) through the hook host's pass "
                    "sequence when build() compiled them here, else the FP64 NumPy restatement, all host cores"}


# Single-kernel cases for profilers: (model, channels of the frame, out_size,
# precision); one 1920x1080 FP16 frame, 3 warm-up + 3 measured calls.
CASES = {
    "ravu-lite-ar-r4": ("ravu-lite-ar-r4", None, "fp32"),
    "ravu-lite-ar-r3": ("ravu-lite-ar-r3", None, "fp32"),
    "ravu-r3": ("ravu-r3", None, "fp32"),
    "ravu-r4-yuv": ("ravu-r4-yuv", None, "fp32"),
    "ravu-zoom-ar-r2-rgb": ("ravu-zoom-ar-r2-rgb", (2880, 1620), "fp32"),
    "ravu-3x-r3": ("ravu-3x-r3", None, "fp32"),
    "ravu-lite-ar-r4-fast": ("ravu-lite-ar-r4", None, "fast"),
    "ravu-lite-ar-r3-fast": ("ravu-lite-ar-r3", None, "fast"),
    "ravu-r3-fast": ("ravu-r3", None, "fast"),
    "ravu-3x-r3-fast": ("ravu-3x-r3", None, "fast"),
    "ravu-zoom-ar-r2-rgb-fast": ("ravu-zoom-ar-r2-rgb", (2880, 1620), "fast"),
    # the same through TMA-staged input rectangles (a tile layout the tuner may pick)
    "ravu-zoom-ar-r2-rgb-fast-tma": ("ravu-zoom-ar-r2-rgb", (2880, 1620), "fast", {"staging": "tma"}),
    "nnedi3-nns128-win8x6-fast": ("nnedi3-nns128-win8x6", None, "fast"),
    "nnedi3-nns128-win8x6-fp32": ("nnedi3-nns128-win8x6", None, "fp32"),
    # not a model: the OFFSET correction of a 3840x2160 FP16 plane (pz_resample,
    # Catmull-Rom), and a persistent batch of 8 1080p ravu-lite-ar-r4 frames
    "resample-2160p": (None, None, None),
    "batch-ravu-lite-ar-r4-8x1080p": ("ravu-lite-ar-r4", None, "fast"),
}


def run_case(name: str) -> None:
    """Run one kernel case (for ncu captures; prints per-call ms)."""
    import torch
    _pkg()
    from mpv_prescalers_gb300 import synth
    model, out_size, prec = CASES[name][:3]
    layout = CASES[name][3] if len(CASES[name]) > 3 else {}
    src = "n/a"
    if name == "resample-2160p":
        from mpv_prescalers_gb300 import frame as _frame
        y = torch.from_numpy(synth.luma_plane(2 * H, 2 * W, SEED0)).to("cuda", torch.float16)
        o = torch.empty_like(y)
        call = lambda: _frame.resample_plane(y, 2 * W, 2 * H, 1.0, -0.5, 1.0, -0.5, "catmull_rom", out=o)
    elif name.startswith("batch-"):
        from mpv_prescalers_gb300 import batch as _batch
        hm, src = synth.model_for(model)
        jobs = [_batch.Job.make(hm, torch.from_numpy(synth.luma_plane(H, W, SEED0 + f)).to("cuda", torch.float16),
                                precision=prec) for f in range(NFRAMES)]
        plan = _batch.Batch(jobs)
        call = plan.launch
    else:
        hm, src = synth.model_for(model)
        x = torch.from_numpy(synth.frame(H, W, SEED0, hm.channels)).to("cuda", torch.float16)
        call = lambda: hm.upscale(x, out_size=out_size, precision=prec, **layout)
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(3):
        call()
    b.record()
    torch.cuda.synchronize()
    print(json.dumps({"case": name, "weights": src, "ms_per_call": a.elapsed_time(b) / 3}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", choices=sorted(CASES), help="run one single-kernel case and exit (profiling)")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-rows", type=int, default=1080, help="input rows per model in the CPU sample")
    ap.add_argument("--ref-rows", type=int, default=1080, help="largest CPU sample per reference step (input rows)")
    ap.add_argument("--ref-budget", type=float, default=90.0, help="seconds of CPU work for all reference steps")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=480, help="requests in the serving trace (0: skip)")
    ap.add_argument("--no-configs", dest="configs", action="store_false",
                    help="skip the informational batch / NNEDI3 configuration lines")
    args = ap.parse_args()
    if args.case:
        run_case(args.case)
        return
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.impl == "reference":
        line = run_reference(args)
        if line:
            print(json.dumps(line))
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    cb, refs = None, None
    if rank == 0 and world == 1 and not args.no_cpu:  # the CPU pool starts before any GPU call
        cb, refs = cpu_baseline(args.cpu_rows, len(os.sched_getaffinity(0)), checks=True)
    line = run_gpu(args, refs)
    if line is not None:
        line["cpu_baseline"] = cb
        print(json.dumps(line))


if __name__ == "__main__":
    main()
