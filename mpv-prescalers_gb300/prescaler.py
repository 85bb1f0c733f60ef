"""Host-side mirror of the hook-file interface: ``load_hook`` / ``upscale``.

``load_hook(path)`` reads a reference ``.hook`` file (or a ``.npz`` model
saved by :meth:`HookModel.save`) and returns a :class:`HookModel`.
``HookModel.upscale(planes)`` runs the file's whole pass chain on PyTorch
CUDA tensors through ``libprescale.so``, the way the mpv hook host would run
the shader passes on a frame:

* ravu-lite(-ar) r2-r4: luma, 2x (``ravu-lite-r3.hook:15-131``);
* ravu r2-r4: luma / yuv / rgb, 2x, output shifted by ``OFFSET -0.5 -0.5``
  (``ravu-r3.hook:424``);
* ravu-zoom(-ar) r2/r3: luma / yuv / rgb, any upscale ratio
  (``ravu-zoom-r2.hook:19-21``);
* ravu-3x r2-r4: luma / yuv / rgb, 3x (``compute/ravu-3x-r2.hook:19-21``);
* nnedi3 nns16-256, win8x4/8x6: luma, 2x per enabled axis
  (``nnedi3-nns16-win8x4.hook:19,109-111``).

The ``//!WHEN`` conditions are honoured: a chain whose condition is false
for the requested output size leaves the planes untouched, as mpv would.
"""
from __future__ import annotations

import json
import os
import threading
from typing import Dict, List, Optional, Sequence, Tuple, Union

import numpy as np

from . import _ffi
from . import models as _models
from .hookfile import HookParseError, Pass

PlaneLike = Union["torch.Tensor", Sequence["torch.Tensor"]]

_FAMILY_CODE = {"lite": _ffi.PZ_RAVU_LITE, "ravu": _ffi.PZ_RAVU, "zoom": _ffi.PZ_RAVU_ZOOM,
                "3x": _ffi.PZ_RAVU_3X, "nnedi3": _ffi.PZ_NNEDI3}
_CHANNEL_CODE = {"luma": _ffi.PZ_LUMA, "yuv": _ffi.PZ_YUV, "rgb": _ffi.PZ_RGB}
PRECISIONS = {"fp32": _ffi.PZ_PREC_FP32, "fast": _ffi.PZ_PREC_FAST, "mpv": _ffi.PZ_PREC_MPV}
# RAVU halo staging: clamped loads, or TMA boxes for interior tiles
STAGINGS = {"ldg": 0, "tma": 1}
# RAVU tile heights (rows of 32 pixels, one thread per pixel); None: the
# library's measured default for the model's program
TILE_ROWS = (4, 8, 16)


def check_tile_rows(tile_rows) -> int:
    """The ``pz_opts.tile_rows`` value of ``tile_rows`` (None: 0, the library's default)."""
    if tile_rows is None:
        return 0
    if tile_rows not in TILE_ROWS:
        raise ValueError(f"tile_rows {tile_rows!r}: one of {TILE_ROWS}")
    return int(tile_rows)


def _torch():
    import torch
    return torch


class HookModel:
    """A parsed prescaler with lazily created device copies of its data."""

    def __init__(self, model):
        self.model = model
        self._dev: Dict[int, int] = {}
        self._lock = threading.Lock()
        # device work buffers of host pipelines, per (device, bytes), each
        # with the completion event of its last call: a buffer is handed out
        # again only after that event has passed, and never goes back to the
        # caching allocator meanwhile, so it is idle when a call starts (its
        # copies run on the library's copy streams, which the allocator does
        # not track)
        self._host_work: Dict[Tuple[int, int], List[Tuple["torch.cuda.Event", "torch.Tensor"]]] = {}
        self._side: Dict[int, "torch.cuda.Stream"] = {}   # per device: the host pipeline's default stream
        self._host_opts: Dict[Tuple, "_ffi.Opts"] = {}    # pz_opts of host pipelines, per frame geometry

    # ---- metadata -----------------------------------------------------
    @property
    def name(self) -> str:
        return self.model.name

    @property
    def family(self) -> str:
        return self.model.family

    @property
    def channels(self) -> str:
        return self.model.channels

    @property
    def n_planes(self) -> int:
        return 1 if self.channels == "luma" else 3

    @property
    def passes(self) -> List[Pass]:
        return self.model.passes

    @property
    def default_staging(self) -> str:
        """Halo staging used when none is asked for: TMA boxes for ravu-lite
        (measured faster on GB300: ravu-lite-ar-r3 59 vs 64 us per 1080p
        frame), clamped loads for the other programs (lattice, 3x and zoom
        measured equal or 3-8 % faster with them)."""
        return "tma" if self.family == "lite" else "ldg"

    @property
    def offset(self):
        """``//!OFFSET`` of the chain's final pass (metadata; not resampled)."""
        fam = self.family
        if fam == "nnedi3":
            return (-0.5, -0.5)
        if fam == "ravu":
            return (-0.5, -0.5)
        if fam == "zoom":
            return "ALIGN"
        return (0.0, 0.0)

    @property
    def hook_point(self) -> str:
        """The texture the chain hooks: LUMA (luma files), NATIVE (yuv:
        merged planes before RGB conversion) or MAIN (rgb); e.g.
        ``ravu-lite-r3.hook:16``, ``compute/ravu-r2-yuv.hook:15``,
        ``ravu-r2-rgb.hook:16``."""
        return self.passes[0].hooks[0] if self.passes and self.passes[0].hooks else "LUMA"

    def chain_offset(self, in_w: int, in_h: int, out_size: Optional[Tuple[int, int]] = None,
                     luma_w: Optional[int] = None):
        """Pixel shift of the chain's output that the host would correct in
        its next scaling pass: the sum of the ``//!OFFSET`` of every enabled
        pass that replaces the hooked texture, in output pixels (ravu
        ``(-0.5, -0.5)``; nnedi3 ``(0, -0.5)`` per doubled row axis and
        ``(-0.5, 0)`` per doubled column axis; lite and 3x none).
        ``"ALIGN"`` when the chain aligns centres itself (ravu-zoom)."""
        if not self.enabled(in_w, in_h, out_size, luma_w=luma_w):
            return (0.0, 0.0)
        if self.family == "nnedi3":
            ax = self.nnedi3_axes(in_w, in_h, out_size)
            ox = oy = 0.0
            for p in self.passes:
                if p.save is None and isinstance(p.offset, tuple):
                    y_pass = "_y" in p.desc
                    if (y_pass and ax & 1) or (not y_pass and ax & 2):
                        ox += p.offset[0]
                        oy += p.offset[1]
            return (ox, oy)
        ox = oy = 0.0
        for p in self.passes:
            if p.save is not None or p.offset is None:
                continue
            if p.offset == "ALIGN":
                return "ALIGN"
            ox += p.offset[0]
            oy += p.offset[1]
        return (ox, oy)

    def __repr__(self):
        return f"HookModel({self.name!r}, family={self.family!r}, channels={self.channels!r})"

    # ---- device model -------------------------------------------------
    def _desc(self):
        m = self.model
        d = _ffi.ModelDesc()
        keep = []
        d.family = _FAMILY_CODE[m.family]
        d.channels = _CHANNEL_CODE[m.channels]
        if m.family == "nnedi3":
            arrs = [np.ascontiguousarray(x, dtype=np.float32) for x in
                    (m.weights_a, m.weights_b, m.bias_a, m.bias_b)]
            keep += arrs
            d.nns, d.win_w, d.win_h = m.nns, m.win_w, m.win_h
            d.weights_a, d.weights_b, d.bias_a, d.bias_b = (a.ctypes.data for a in arrs)
            return d, keep
        d.radius = m.radius
        d.ar_strength = float(m.ar)
        lut = np.ascontiguousarray(m.lut, dtype=np.float32)
        keep.append(lut)
        d.lut = lut.ctypes.data
        d.lut_rows, d.lut_cols = lut.shape[0], lut.shape[1]
        if m.lut_ar is not None:
            la = np.ascontiguousarray(m.lut_ar, dtype=np.float32)
            keep.append(la)
            d.lut_ar = la.ctypes.data
        gw = np.ascontiguousarray(m.grad_weights, dtype=np.float64)
        keep.append(gw)
        d.grad_weights = gw.ctypes.data
        d.n_grad = gw.size
        if m.strength[0] == "log2":
            d.strength_log2 = 1
            d.strength_scale = m.strength[1]
            d.strength_max = int(m.strength[2])
        else:
            d.n_strength_thr = len(m.strength[1])
            for i, t in enumerate(m.strength[1]):
                d.strength_thr[i] = t
        d.coherence_thr[0], d.coherence_thr[1] = m.coherence
        return d, keep

    def device_handle(self, device: Optional[int] = None) -> int:
        """The ``pz_model*`` for ``device`` (created on first use)."""
        torch = _torch()
        dev = torch.cuda.current_device() if device is None else int(device)
        with self._lock:
            h = self._dev.get(dev)
            if h is None:
                L = _ffi.lib()
                d, keep = self._desc()
                out = _ffi.ctypes.c_void_p()
                with torch.cuda.device(dev):
                    _ffi.check(L.pz_model_create(_ffi.ctypes.byref(d), _ffi.ctypes.byref(out)))
                h = out.value
                self._dev[dev] = h
                del keep
            return h

    def close(self):
        with self._lock:
            if self._dev:
                L = _ffi.lib()
                for h in self._dev.values():
                    L.pz_model_destroy(h)
                self._dev.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- geometry -----------------------------------------------------
    def output_size(self, in_w: int, in_h: int, out_size: Optional[Tuple[int, int]] = None) -> Tuple[int, int]:
        fam = self.family
        if fam == "zoom":
            if out_size is None:
                raise ValueError("ravu-zoom needs out_size=(width, height)")
            return int(out_size[0]), int(out_size[1])
        if fam == "3x":
            return 3 * in_w, 3 * in_h
        if fam == "nnedi3":
            ax = self.nnedi3_axes(in_w, in_h, out_size)
            return (2 * in_w if ax & 2 else in_w), (2 * in_h if ax & 1 else in_h)
        return 2 * in_w, 2 * in_h

    def nnedi3_axes(self, in_w, in_h, out_size=None) -> int:
        """Axes bitmask enabled by the double_y / double_x ``//!WHEN``."""
        tw, th = out_size if out_size is not None else (2 * in_w, 2 * in_h)
        ax = 0
        for p in self.passes:
            if "double_y" in p.desc and _models.pass_enabled(p, in_w, in_h, tw, th):
                ax |= 1
            if "double_x" in p.desc:
                # double_x runs on the (possibly) row-doubled image
                h2 = 2 * in_h if ax & 1 else in_h
                if _models.pass_enabled(p, in_w, h2, tw, th):
                    ax |= 2
        return ax

    def enabled(self, in_w: int, in_h: int, out_size: Optional[Tuple[int, int]] = None,
                luma_w: Optional[int] = None) -> bool:
        """The chain's ``//!WHEN`` for this size; ``luma_w`` is the width of
        the frame's luma plane (0 for RGB frames, which have none)."""
        if self.family == "nnedi3":
            return self.nnedi3_axes(in_w, in_h, out_size) != 0
        if out_size is None:
            s = {"zoom": None, "3x": 3}.get(self.family, 2)
            if s is None:
                raise ValueError("ravu-zoom needs out_size=(width, height)")
            out_size = (s * in_w, s * in_h)
        return _models.pass_enabled(self.passes[0], in_w, in_h, out_size[0], out_size[1],
                                    luma_w=in_w if luma_w is None else luma_w)

    # ---- execution ----------------------------------------------------
    def upscale(self, planes: PlaneLike, out_size: Optional[Tuple[int, int]] = None, precision: str = "fp32",
                out=None, return_keys: bool = False, stream=None, staging: Optional[str] = None,
                tile_rows: Optional[int] = None):
        """Run the hook chain on ``planes``.

        ``planes``: a CUDA tensor ``[H][W]`` (luma), ``[C][H][W]`` (C = 1
        or 3) or a batch ``[N][C][H][W]``, float32 or float16, or a list of
        ``[H][W]`` tensors.
        ``out_size``: target ``(width, height)``; required for ravu-zoom,
        otherwise it only decides the ``//!WHEN`` conditions.
        ``precision``: "fp32" (plain FP32 arithmetic), "fast" (FP16
        tensor-core NNEDI3 neurons; ravu-lite / 3x / zoom LUTs read as FP16
        texels, all RAVU arithmetic FP32) or "mpv"
        (what the mpv host computes, to measure the distance to it: FP16
        planes only, LUTs rounded to FP16, ravu-zoom LUT bilinear weights
        in 1/256 steps; NNEDI3 as "fp32").
        ``staging``: how RAVU tiles stage their input window: "ldg"
        (clamped loads) or "tma" (TMA boxes for interior tiles), default
        ``default_staging``; the pixels are identical, only the speed
        differs (see ``batch.autotune_staging``).
        ``tile_rows``: RAVU tile height, 4, 8 or 16 rows of 32 pixels (one
        thread per pixel; default: the library's measured choice for the
        model's program, 4 rows but for ravu-lite r2 and ravu-lite-ar r4);
        again only the speed differs (see ``batch.autotune_tiles``).
        Returns the upscaled planes in the input's form (and the raw LUT
        keys as int32 when ``return_keys``).
        """
        torch = _torch()
        if not isinstance(planes, (list, tuple)) and planes.dim() == 4:
            # a batch of frames [N][C][H][W]: one chain per frame, same stream
            # (the results are gathered on that stream, after the kernels)
            with torch.cuda.stream(stream):
                outs = [self.upscale(f, out_size=out_size, precision=precision,
                                     out=None if out is None else out[i], return_keys=return_keys, stream=stream,
                                     staging=staging, tile_rows=tile_rows)
                        for i, f in enumerate(planes.unbind(0))]
                if return_keys:
                    return torch.stack([o[0] for o in outs]), torch.stack([o[1] for o in outs])
                return torch.stack(outs) if out is None else out
        as_list = isinstance(planes, (list, tuple))
        pl = list(planes) if as_list else ([planes] if planes.dim() == 2 else list(planes.unbind(0)))
        if len(pl) != self.n_planes:
            raise ValueError(f"{self.name} takes {self.n_planes} plane(s), got {len(pl)}")
        H, W = pl[0].shape
        if H == 0 or W == 0:
            raise ValueError(f"empty plane {W}x{H}")
        for p in pl:
            if not p.is_cuda:
                raise ValueError("planes must be CUDA tensors")
            if p.dtype not in (torch.float32, torch.float16):
                raise ValueError("planes must be float32 or float16")
            if p.shape != (H, W) or p.dtype != pl[0].dtype or p.stride(1) != 1:
                raise ValueError("planes must share size/dtype and be row-contiguous")
        if not self.enabled(W, H, out_size):
            res = [p.clone() for p in pl]
            return self._pack(res, planes, as_list, None, return_keys)
        OW, OH = self.output_size(W, H, out_size)
        dev = pl[0].device
        # results are allocated (and packed) on the stream that writes them,
        # so the caching allocator orders their reuse after the kernels
        with torch.cuda.device(dev), torch.cuda.stream(stream):
            full = None
            if out is None:
                full = torch.empty((len(pl), OH, OW), dtype=pl[0].dtype, device=dev)
                res = list(full.unbind(0))
            else:
                res = list(out) if isinstance(out, (list, tuple)) else ([out] if out.dim() == 2 else list(out.unbind(0)))
            keys = None
            if return_keys:
                keys = torch.empty(self.key_shape(W, H, OW, OH), dtype=torch.int32, device=dev)
            self.run_raw(pl, res, out_size=(OW, OH), precision=precision, keys=keys, stream=stream,
                         staging=staging, tile_rows=tile_rows)
            return self._pack(res, planes, as_list, keys, return_keys, full)

    def upscale_host(self, frames, out=None, out_size: Optional[Tuple[int, int]] = None, precision: str = "fp32",
                     device=None, wait: bool = True, stream=None):
        """Upscale host frames ``[N][C][H][W]`` (pinned CPU tensor) into host
        memory through ``pz_run_host``: frame i is copied in, run and copied
        back while its neighbours' transfers run under its kernels.
        Returns the host output ``[N][C][OH][OW]`` (``out`` if given; it
        should be pinned).  With ``wait=False`` it returns ``(out, event)``
        as soon as the work is queued: ``out`` is complete once ``event`` (a
        CUDA event on ``stream``) has completed, so calls for several models
        can overlap on the device.  Without ``stream`` the call runs on a
        side stream of this model (ordered after the work queued so far on
        the current stream): the kernels of two models' calls share the GPU
        and their copies share the host link.
        """
        torch = _torch()
        if frames.dim() != 4 or frames.is_cuda:
            raise ValueError("frames must be a host tensor [N][C][H][W]")
        if frames.shape[1] != self.n_planes:
            raise ValueError(f"{self.name} takes {self.n_planes} plane(s), got {frames.shape[1]}")
        if frames.dtype not in (torch.float32, torch.float16):
            raise ValueError("frames must be float32 or float16")
        if not frames.is_contiguous():
            raise ValueError("frames must be contiguous (the copies read them in place)")
        dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        N, C, H, W = frames.shape
        if H == 0 or W == 0:
            raise ValueError(f"empty frames {W}x{H}")
        if not self.enabled(W, H, out_size):   # //!WHEN false: the planes pass through
            out = frames.clone() if out is None else out.copy_(frames)
            return out if wait else (out, None)
        OW, OH = self.output_size(W, H, out_size)
        if out is None:
            out = torch.empty((N, C, OH, OW), dtype=frames.dtype, pin_memory=True)
        elif tuple(out.shape) != (N, C, OH, OW) or out.dtype != frames.dtype or not out.is_contiguous():
            raise ValueError(f"out must be a contiguous {frames.dtype} tensor of shape {(N, C, OH, OW)}")
        dt = _ffi.PZ_F32 if frames.dtype == torch.float32 else _ffi.PZ_F16
        o = self.host_opts(W, H, out_size, precision)
        L = _ffi.lib()
        h = self.device_handle(dev.index)
        with torch.cuda.device(dev):
            if stream is None:
                s = self._side_stream(dev)
                s.wait_stream(torch.cuda.current_stream(dev))
            else:
                s = stream
            nbytes = max(int(L.pz_run_host_work_bytes(h, W, H, dt, _ffi.ctypes.byref(o))), 256)
            work = self._take_host_work(dev, nbytes)   # idle: the copies may start at once
            try:
                _ffi.check(L.pz_run_host(h, frames.data_ptr(), out.data_ptr(), N, W, H, dt,
                                         _ffi.ctypes.byref(o), work.data_ptr(), work.numel(),
                                         _ffi.PZ_HOST_WORK_IDLE, s.cuda_stream))
            finally:
                fin = torch.cuda.Event()
                fin.record(s)
                self._give_host_work(dev, nbytes, fin, work)
            if wait:
                fin.synchronize()
                return out
            return out, fin

    _HOST_WORK_KEEP = 8   # idle buffers kept per (device, size)

    def host_opts(self, W: int, H: int, out_size=None, precision: str = "fp32") -> "_ffi.Opts":
        """The ``pz_opts`` of a host pipeline call on W x H frames (made once
        per geometry and form and kept; the library copies them per call)."""
        key = (W, H, out_size, precision)
        o = self._host_opts.get(key)
        if o is None:
            OW, OH = self.output_size(W, H, out_size)
            o = _ffi.Opts()
            o.precision = PRECISIONS[precision]
            o.out_width, o.out_height = OW, OH
            if self.family == "nnedi3":
                o.nnedi3_axes = self.nnedi3_axes(W, H, out_size)
            o.staging = STAGINGS[self.default_staging]
            with self._lock:
                o = self._host_opts.setdefault(key, o)
        return o

    def _side_stream(self, dev):
        """This model's side stream on ``dev`` (created on first use)."""
        torch = _torch()
        with self._lock:
            s = self._side.get(dev.index)
            if s is None:
                s = self._side[dev.index] = torch.cuda.Stream(dev)
            return s

    def _take_host_work(self, dev, nbytes: int):
        torch = _torch()
        with self._lock:
            pool = self._host_work.setdefault((dev.index, nbytes), [])
            for k, (ev, w) in enumerate(pool):
                if ev.query():
                    del pool[k]
                    return w
        return torch.empty(nbytes, dtype=torch.uint8, device=dev)

    def _give_host_work(self, dev, nbytes: int, ev, work) -> None:
        with self._lock:
            pool = self._host_work.setdefault((dev.index, nbytes), [])
            pool.append((ev, work))
            while len(pool) > self._HOST_WORK_KEEP:   # drop the oldest finished buffer
                k = next((i for i, (e, _) in enumerate(pool) if e.query()), None)
                if k is None:
                    break
                del pool[k]

    def key_shape(self, W, H, OW, OH):
        fam = self.family
        if fam == "ravu":
            return (3, H, W)
        if fam == "zoom":
            return (OH, OW)
        if fam == "nnedi3":
            return (1,)
        return (H, W)

    def run_raw(self, pl, res, out_size, precision="fp32", keys=None, stream=None, scratch=None, staging=None,
                tile_rows=None):
        """Low-level call of ``pz_run`` on prepared tensors (no allocation
        besides the optional NNEDI3 scratch inside the library)."""
        torch = _torch()
        dt = _ffi.PZ_F32 if pl[0].dtype == torch.float32 else _ffi.PZ_F16
        n = len(pl)
        pin = (_ffi.Plane * n)()
        pout = (_ffi.Plane * n)()
        for i, (p, r) in enumerate(zip(pl, res)):
            pin[i] = _ffi.Plane(p.data_ptr(), p.shape[1], p.shape[0], p.stride(0), dt)
            pout[i] = _ffi.Plane(r.data_ptr(), r.shape[1], r.shape[0], r.stride(0), dt)
        o = _ffi.Opts()
        o.precision = PRECISIONS[precision]
        o.out_width, o.out_height = out_size
        if self.family == "nnedi3":
            o.nnedi3_axes = self.nnedi3_axes(pl[0].shape[1], pl[0].shape[0], out_size)
        if keys is not None:
            o.keys = keys.data_ptr()
        if scratch is not None:
            o.scratch = scratch.data_ptr()
            o.scratch_bytes = scratch.numel() * scratch.element_size()
        o.staging = STAGINGS[staging or self.default_staging]
        o.tile_rows = check_tile_rows(tile_rows)
        s = stream if stream is not None else torch.cuda.current_stream(pl[0].device)
        h = self.device_handle(pl[0].device.index)
        _ffi.check(_ffi.lib().pz_run(h, pin, n, pout, n, _ffi.ctypes.byref(o), s.cuda_stream))

    @staticmethod
    def _pack(res, planes, as_list, keys, return_keys, full=None):
        """The results in the input's form; ``full``: the [C][OH][OW] tensor
        whose planes ``res`` are, when the results were allocated here."""
        torch = _torch()
        if as_list:
            r = res
        elif planes.dim() == 2:
            r = res[0]
        elif full is not None:
            r = full
        else:
            r = torch.stack(res) if len(res) > 1 else res[0].unsqueeze(0)
        return (r, keys) if return_keys else r

    # ---- serialisation ------------------------------------------------
    def save(self, path: str) -> None:
        """Store the canonical model (arrays + pass directives) as ``.npz``."""
        m = self.model
        meta = {"name": m.name, "family": m.family, "channels": m.channels, "style": m.style,
                "passes": [_pass_meta(p) for p in m.passes]}
        arrays = {}
        if m.family == "nnedi3":
            meta.update(nns=m.nns, win_w=m.win_w, win_h=m.win_h)
            arrays.update(taps=m.taps, weights_a=m.weights_a, weights_b=m.weights_b,
                          bias_a=m.bias_a, bias_b=m.bias_b)
        else:
            meta.update(radius=m.radius, ar=m.ar, strength=list(m.strength[:1]) + [
                list(m.strength[1]) if m.strength[0] == "thr" else m.strength[1]] + list(m.strength[2:]),
                coherence=list(m.coherence))
            arrays.update(lut=m.lut, grad_weights=m.grad_weights)
            if m.lut_ar is not None:
                arrays["lut_ar"] = m.lut_ar
            if m.ar_taps is not None:
                arrays["ar_taps"] = m.ar_taps
        np.savez_compressed(path, meta=np.array(json.dumps(meta)), **arrays)


def _pass_meta(p: Pass) -> dict:
    return {"desc": p.desc, "hooks": p.hooks, "binds": p.binds, "save": p.save, "width": p.width,
            "height": p.height, "offset": p.offset, "when": p.when, "components": p.components,
            "compute": p.compute, "line": p.line}


def _model_from_npz(path: str):
    z = np.load(path, allow_pickle=False)
    meta = json.loads(str(z["meta"]))
    passes = [Pass(desc=q["desc"], hooks=q["hooks"], binds=q["binds"], save=q["save"], width=q["width"],
                   height=q["height"], offset=tuple(q["offset"]) if isinstance(q["offset"], list) else q["offset"],
                   when=q["when"], components=q["components"],
                   compute=tuple(q["compute"]) if q["compute"] else None, body=[], line=q["line"],
                   body_line=q["line"] + 1) for q in meta["passes"]]
    if meta["family"] == "nnedi3":
        return _models.Nnedi3Model(name=meta["name"], nns=meta["nns"], win_w=meta["win_w"], win_h=meta["win_h"],
                                   taps=z["taps"], weights_a=z["weights_a"], weights_b=z["weights_b"],
                                   bias_a=z["bias_a"], bias_b=z["bias_b"], passes=passes, style=meta["style"],
                                   path=path)
    st = meta["strength"]
    strength = ("thr", tuple(st[1])) if st[0] == "thr" else ("log2", float(st[1]), float(st[2]))
    return _models.RavuModel(name=meta["name"], family=meta["family"], radius=meta["radius"],
                             channels=meta["channels"], ar=meta["ar"], lut=z["lut"],
                             lut_ar=z["lut_ar"] if "lut_ar" in z.files else None,
                             grad_weights=z["grad_weights"], strength=strength,
                             coherence=tuple(meta["coherence"]), passes=passes, style=meta["style"], path=path,
                             ar_taps=z["ar_taps"] if "ar_taps" in z.files else None)


def load_hook(path: str) -> HookModel:
    """Parse a ``.hook`` file (or a saved ``.npz`` model) into a HookModel."""
    path = os.fspath(path)
    if path.endswith(".npz"):
        return HookModel(_model_from_npz(path))
    return HookModel(_models.load_model(path))


MODEL_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_models")


def cached_model(name: str) -> HookModel:
    """A model from the package's cache (``_models/<name>.npz``), which
    :func:`build_model_cache` fills from a directory of ``.hook`` files."""
    p = os.path.join(MODEL_DIR, name + ".npz")
    if not os.path.exists(p):
        raise FileNotFoundError(f"model {name!r} not in {MODEL_DIR}; build the cache from the .hook files first")
    return load_hook(p)


def build_model_cache(hook_dir: str, names: Optional[Sequence[str]] = None) -> List[str]:
    """Parse ``.hook`` files from ``hook_dir`` (root and ``compute/``) into
    ``_models/<name>.npz``.  Returns the cached names."""
    os.makedirs(MODEL_DIR, exist_ok=True)
    found = {}
    for sub in ("", "compute"):
        d = os.path.join(hook_dir, sub)
        if not os.path.isdir(d):
            continue
        for fn in sorted(os.listdir(d)):
            if fn.endswith(".hook") and fn[:-5] not in found:
                found[fn[:-5]] = os.path.join(d, fn)
    out = []
    for name, path in sorted(found.items()):
        if names is not None and name not in names:
            continue
        dst = os.path.join(MODEL_DIR, name + ".npz")
        if os.path.exists(dst) and os.path.getmtime(dst) >= os.path.getmtime(path):
            out.append(name)
            continue
        load_hook(path).save(dst)
        out.append(name)
    return out
