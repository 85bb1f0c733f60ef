"""GB300-native RAVU / NNEDI3 prescalers behind the mpv ``.hook`` interface.

    from mpv_prescalers_gb300 import load_hook
    m = load_hook("ravu-lite-ar-r3.hook")
    out = m.upscale(luma_plane_cuda)          # [H][W] -> [2H][2W]

The arithmetic runs in hand-written sm_103a CUDA kernels inside
``libprescale.so`` (C ABI: ``include/prescale.h``); this package parses the
hook files and drives the library through ctypes.
"""
from .hookfile import HookParseError, parse_hook_file, parse_hook_text, rpn_eval  # noqa: F401
from .hookwriter import format_hook, model_to_hook, write_hook  # noqa: F401
from .frame import Frame, plan_frame, prescale_frame, resample_plane  # noqa: F401
from .models import Nnedi3Model, RavuModel, load_model  # noqa: F401
from .prescaler import (PRECISIONS, HookModel, build_model_cache, cached_model, load_hook,  # noqa: F401
                        MODEL_DIR)
from ._ffi import PrescaleError, PrescaleLibraryError, check_device  # noqa: F401

__all__ = ["load_hook", "HookModel", "cached_model", "build_model_cache", "parse_hook_file",
           "format_hook", "model_to_hook", "write_hook",
           "Frame", "plan_frame", "prescale_frame", "resample_plane",
           "HookParseError", "PrescaleError", "PrescaleLibraryError", "check_device"]
