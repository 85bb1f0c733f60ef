"""Whole frames through a hook chain, the way mpv places it.

A prescaler file hooks one texture of the frame (``//!HOOK``):

* ``LUMA`` (ravu, ravu-lite, ravu-zoom, ravu-3x and NNEDI3 luma files,
  e.g. ``ravu-lite-r3.hook:16``): only the luma plane is upscaled; chroma
  planes pass through untouched and the host scales them later with
  ``--cscale`` (``README.md:50-52``).  An RGB frame has no luma plane, so
  the chain does not run.
* ``NATIVE`` (``-yuv`` files, ``compute/ravu-r2-yuv.hook:15``): the planes
  merged at luma size before RGB conversion, i.e. after ``--cscale``
  (``README.md:54-56``).  Subsampled chroma is upsampled first (bilinear or
  Catmull-Rom, at the frame's chroma siting); the ``//!WHEN`` term
  ``LUMA.w 0 >`` (``compute/ravu-r2-yuv.hook:19``) keeps RGB frames out.
* ``MAIN`` (``-rgb`` files, ``ravu-r2-rgb.hook:16``): RGB after conversion;
  the frame must already be RGB.

The chain's ``//!OFFSET`` (ravu ``-0.5 -0.5``, ``ravu-r3.hook:424``; NNEDI3
``0 -0.5`` and ``-0.5 0`` per doubled axis, ``nnedi3-nns16-win8x4.hook:95,
185``) is a shift the host folds into its next scaling pass.  With
``offset_filter`` set, :func:`prescale_frame` applies that correction to the
upscaled planes itself (one ``pz_resample`` per plane), so the result sits
on the centred output grid; with ``None`` the planes are returned as the
chain wrote them and the shift is reported in ``Frame.offset``.

:func:`plan_frame` decides all of this on the host without touching a
device; :func:`prescale_frame` carries the plan out on CUDA tensors.
"""
from __future__ import annotations

import dataclasses
from typing import List, Optional, Sequence, Tuple

from . import _ffi

FILTERS = {"bilinear": _ffi.PZ_FILTER_BILINEAR, "catmull_rom": _ffi.PZ_FILTER_CATMULL_ROM}
KINDS = ("yuv", "rgb", "gray")
# Chroma siting as the luma-grid position of chroma sample 0 per axis:
# MPEG-2 / H.26x 4:2:0 ("left": co-sited horizontally, centred vertically)
# and JPEG / MPEG-1 ("center").
CHROMA_LOCATIONS = {"left": (0.0, 0.5), "center": (0.5, 0.5), "topleft": (0.0, 0.0)}


def _torch():
    import torch
    return torch


@dataclasses.dataclass
class Frame:
    """Planes of one frame (CUDA ``[H][W]`` tensors, FP32 or FP16).

    ``kind``: "yuv" (Y, U, V; chroma may be subsampled), "rgb" (R, G, B) or
    "gray" (Y only).  ``chroma_loc``: siting of subsampled chroma (a key of
    :data:`CHROMA_LOCATIONS` or a luma-grid position per axis).
    ``offset``: shift of plane 0 (and of chroma planes upsampled with it)
    that a later scaler still has to correct, in plane-0 pixels."""
    planes: List["torch.Tensor"]
    kind: str = "yuv"
    chroma_loc: object = "left"
    offset: Tuple[float, float] = (0.0, 0.0)

    @property
    def sizes(self) -> List[Tuple[int, int]]:
        return [(int(p.shape[1]), int(p.shape[0])) for p in self.planes]


@dataclasses.dataclass
class FramePlan:
    """What :func:`prescale_frame` will do (decided on the host)."""
    runs: bool                          # the chain runs on this frame
    reason: str                         # why not, or what it hooks
    upsample_chroma: bool = False       # merge subsampled chroma first (NATIVE)
    chroma_scale: Tuple[float, float] = (1.0, 1.0)   # chroma size / luma size
    chroma_origin: Tuple[float, float] = (0.0, 0.0)  # chroma siting (luma px)
    prescaled: Tuple[int, ...] = ()     # plane indices that go through the chain
    passthrough: Tuple[int, ...] = ()   # plane indices returned untouched
    out_size: Tuple[int, int] = (0, 0)  # size of the prescaled planes
    offset: object = (0.0, 0.0)         # the chain's announced shift (or "ALIGN")


def _siting(loc) -> Tuple[float, float]:
    if isinstance(loc, str):
        if loc not in CHROMA_LOCATIONS:
            raise ValueError(f"unknown chroma location {loc!r}; one of {sorted(CHROMA_LOCATIONS)}")
        return CHROMA_LOCATIONS[loc]
    return float(loc[0]), float(loc[1])


def plan_frame(model, kind: str, sizes: Sequence[Tuple[int, int]], out_size: Optional[Tuple[int, int]] = None,
               chroma_loc="left") -> FramePlan:
    """Decide how ``model`` applies to a frame of ``kind`` with plane
    ``sizes`` [(width, height), ...]; raises ``ValueError`` for frames the
    chain cannot take."""
    if kind not in KINDS:
        raise ValueError(f"frame kind {kind!r} not in {KINDS}")
    want = 1 if kind == "gray" else 3
    if len(sizes) != want:
        raise ValueError(f"a {kind} frame has {want} plane(s), got {len(sizes)}")
    (W, H) = sizes[0]
    if kind == "rgb" and any(s != sizes[0] for s in sizes):
        raise ValueError("RGB planes must share one size")
    hp = model.hook_point
    if hp == "LUMA":
        if kind == "rgb":
            return FramePlan(False, "LUMA hook: an RGB frame has no luma plane")
        if not model.enabled(W, H, out_size):
            return FramePlan(False, "//!WHEN is false for this size", passthrough=tuple(range(want)))
        return FramePlan(True, "LUMA: luma upscaled, chroma passed through", prescaled=(0,),
                         passthrough=tuple(range(1, want)), out_size=model.output_size(W, H, out_size),
                         offset=model.chain_offset(W, H, out_size))
    if hp == "NATIVE":
        if kind == "rgb":
            return FramePlan(False, "NATIVE yuv hook: //!WHEN needs a luma plane (LUMA.w 0 >)")
        if kind == "gray":
            raise ValueError(f"{model.name} hooks NATIVE and needs Y, U and V planes")
        if not model.enabled(W, H, out_size, luma_w=W):
            return FramePlan(False, "//!WHEN is false for this size", passthrough=(0, 1, 2))
        (cw, ch) = sizes[1]
        if sizes[2] != sizes[1]:
            raise ValueError("U and V planes differ in size")
        sub = (cw, ch) != (W, H)
        return FramePlan(True, "NATIVE: planes merged at luma size, then upscaled together",
                         upsample_chroma=sub, chroma_scale=(cw / W, ch / H),
                         chroma_origin=_siting(chroma_loc) if sub else (0.0, 0.0),
                         prescaled=(0, 1, 2), out_size=model.output_size(W, H, out_size),
                         offset=model.chain_offset(W, H, out_size, luma_w=W))
    if hp == "MAIN":
        if kind != "rgb":
            raise ValueError(f"{model.name} hooks MAIN (RGB after conversion); convert the {kind} frame to RGB first")
        if not model.enabled(W, H, out_size, luma_w=0):
            return FramePlan(False, "//!WHEN is false for this size", passthrough=(0, 1, 2))
        return FramePlan(True, "MAIN: RGB planes upscaled together", prescaled=(0, 1, 2),
                         out_size=model.output_size(W, H, out_size), offset=model.chain_offset(W, H, out_size,
                                                                                               luma_w=0))
    raise ValueError(f"unsupported hook point {hp!r}")


def resample_plane(x, out_w: int, out_h: int, sx: float, ox: float, sy: float, oy: float,
                   filt: str = "catmull_rom", out=None, stream=None):
    """``out(x, y) = interp(in, sx*x + ox, sy*y + oy)`` on the device
    (``pz_resample``; texel centres at integers, edges replicated)."""
    torch = _torch()
    if not x.is_cuda or x.dim() != 2 or x.stride(1) != 1:
        raise ValueError("resample_plane takes a row-contiguous CUDA [H][W] tensor")
    if x.dtype not in (torch.float32, torch.float16):
        raise ValueError("planes must be float32 or float16")
    if filt not in FILTERS:
        raise ValueError(f"filter {filt!r} not in {sorted(FILTERS)}")
    if out is None:   # allocated on the stream that writes it
        with torch.cuda.device(x.device), torch.cuda.stream(stream):
            out = torch.empty((out_h, out_w), dtype=x.dtype, device=x.device)
    dt = _ffi.PZ_F32 if x.dtype == torch.float32 else _ffi.PZ_F16
    pin = _ffi.Plane(x.data_ptr(), x.shape[1], x.shape[0], x.stride(0), dt)
    pout = _ffi.Plane(out.data_ptr(), out.shape[1], out.shape[0], out.stride(0), dt)
    s = stream if stream is not None else torch.cuda.current_stream(x.device)
    _ffi.check(_ffi.lib().pz_resample(_ffi.ctypes.byref(pin), _ffi.ctypes.byref(pout), sx, ox, sy, oy,
                                      FILTERS[filt], s.cuda_stream))
    return out


def prescale_frame(model, frame: Frame, out_size: Optional[Tuple[int, int]] = None, precision: str = "fp32",
                   offset_filter: Optional[str] = "catmull_rom", cscale: str = "bilinear", stream=None) -> Frame:
    """Run ``model`` (a :class:`~.prescaler.HookModel`) on ``frame`` per
    its hook point; see the module text.  Returns a new :class:`Frame`
    (untouched planes are the input tensors themselves)."""
    torch = _torch()
    if frame.offset != (0.0, 0.0) and frame.offset != (0, 0):
        raise ValueError("the frame carries an uncorrected offset; correct it before the next prescaler")
    plan = plan_frame(model, frame.kind, frame.sizes, out_size, frame.chroma_loc)
    if not plan.runs:
        return Frame(list(frame.planes), frame.kind, frame.chroma_loc, frame.offset)
    W, H = frame.sizes[0]
    planes = list(frame.planes)
    dev = planes[0].device
    with torch.cuda.device(dev):
        if plan.upsample_chroma:
            (rx, ry), (lx, ly) = plan.chroma_scale, plan.chroma_origin
            planes[1:] = [resample_plane(p, W, H, rx, -lx * rx, ry, -ly * ry, cscale, stream=stream)
                          for p in planes[1:]]
        src = [planes[i] for i in plan.prescaled]
        dt = src[0].dtype
        if any(p.dtype != dt for p in src):
            raise ValueError("prescaled planes must share one dtype")
        up = model.upscale(src, out_size=out_size, precision=precision, stream=stream)
        off = plan.offset
        if isinstance(off, tuple) and off != (0.0, 0.0) and offset_filter is not None:
            OW, OH = plan.out_size
            up = [resample_plane(p, OW, OH, 1.0, off[0], 1.0, off[1], offset_filter, stream=stream) for p in up]
            off = (0.0, 0.0)
        out = list(frame.planes)
        for i, p in zip(plan.prescaled, up):
            out[i] = p
    return Frame(out, frame.kind, frame.chroma_loc if not plan.upsample_chroma else (0.0, 0.0),
                 off if isinstance(off, tuple) else (0.0, 0.0))
