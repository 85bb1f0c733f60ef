"""ctypes binding of ``libprescale.so`` (the C ABI in ``include/prescale.h``).

The library is loaded from the package's ``_lib/`` directory (built by
:mod:`.build`).  There is no fallback: if it is missing or fails to load,
every device entry point raises :class:`PrescaleLibraryError`.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libprescale.so")

PZ_OK = 0
PZ_EINVAL = -22
PZ_ENOMEM = -12
PZ_EIO = -5
PZ_ENOTSUP = -95
PZ_ETIMEDOUT = -110

PZ_RAVU_LITE, PZ_RAVU, PZ_RAVU_ZOOM, PZ_RAVU_3X, PZ_NNEDI3 = 1, 2, 3, 4, 5
PZ_LUMA, PZ_YUV, PZ_RGB = 0, 1, 2
PZ_F32, PZ_F16 = 0, 1
PZ_PREC_FP32, PZ_PREC_FAST, PZ_PREC_MPV = 0, 1, 2
PZ_FILTER_BILINEAR, PZ_FILTER_CATMULL_ROM = 0, 1
PZ_HOST_WORK_IDLE = 1


class PrescaleLibraryError(RuntimeError):
    pass


class PrescaleError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"prescale error {code}: {msg}")
        self.code = code


class ModelDesc(ctypes.Structure):
    _fields_ = [
        ("family", ctypes.c_int), ("radius", ctypes.c_int), ("channels", ctypes.c_int),
        ("ar_strength", ctypes.c_float),
        ("lut", ctypes.c_void_p), ("lut_rows", ctypes.c_int), ("lut_cols", ctypes.c_int),
        ("lut_ar", ctypes.c_void_p),
        ("grad_weights", ctypes.c_void_p), ("n_grad", ctypes.c_int),
        ("strength_log2", ctypes.c_int), ("strength_thr", ctypes.c_float * 3),
        ("n_strength_thr", ctypes.c_int), ("strength_scale", ctypes.c_float), ("strength_max", ctypes.c_int),
        ("coherence_thr", ctypes.c_float * 2),
        ("nns", ctypes.c_int), ("win_w", ctypes.c_int), ("win_h", ctypes.c_int),
        ("weights_a", ctypes.c_void_p), ("weights_b", ctypes.c_void_p),
        ("bias_a", ctypes.c_void_p), ("bias_b", ctypes.c_void_p),
    ]


class Plane(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("width", ctypes.c_int), ("height", ctypes.c_int),
                ("pitch", ctypes.c_int), ("dtype", ctypes.c_int)]


class Opts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("out_width", ctypes.c_int), ("out_height", ctypes.c_int),
                ("nnedi3_axes", ctypes.c_int), ("keys", ctypes.c_void_p),
                ("scratch", ctypes.c_void_p), ("scratch_bytes", ctypes.c_size_t), ("staging", ctypes.c_int),
                ("tile_rows", ctypes.c_int)]


class QueryResult(ctypes.Structure):
    _fields_ = [("out_width", ctypes.c_int), ("out_height", ctypes.c_int), ("n_planes", ctypes.c_int),
                ("family", ctypes.c_int), ("scratch_bytes", ctypes.c_size_t)]


class Job(ctypes.Structure):
    _fields_ = [("model", ctypes.c_void_p), ("inp", Plane * 3), ("out", Plane * 3),
                ("n_planes", ctypes.c_int), ("opts", Opts)]


EXPORTS = {
    "pz_version": (ctypes.c_int, []),
    "pz_last_error": (ctypes.c_char_p, []),
    "pz_model_create": (ctypes.c_int, [ctypes.POINTER(ModelDesc), ctypes.POINTER(ctypes.c_void_p)]),
    "pz_model_destroy": (None, [ctypes.c_void_p]),
    "pz_scratch_bytes": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.POINTER(Plane), ctypes.POINTER(Opts)]),
    "pz_query": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(Opts),
                                ctypes.POINTER(QueryResult)]),
    "pz_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Plane), ctypes.c_int, ctypes.POINTER(Plane),
                              ctypes.c_int, ctypes.POINTER(Opts), ctypes.c_void_p]),
    "pz_batch_work_bytes": (ctypes.c_size_t, [ctypes.POINTER(Job), ctypes.c_int]),
    "pz_batch_create": (ctypes.c_int, [ctypes.POINTER(Job), ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t,
                                       ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "pz_batch_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "pz_batch_destroy": (None, [ctypes.c_void_p]),
    "pz_batch_run": (ctypes.c_int, [ctypes.POINTER(Job), ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t,
                                    ctypes.c_void_p]),
    "pz_nnedi3_run_static": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Plane), ctypes.POINTER(Plane),
                                            ctypes.POINTER(Opts), ctypes.c_void_p]),
    "pz_run_host_work_bytes": (ctypes.c_size_t, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                 ctypes.POINTER(Opts)]),
    "pz_run_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int, ctypes.POINTER(Opts), ctypes.c_void_p,
                                   ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p]),
    "pz_resample": (ctypes.c_int, [ctypes.POINTER(Plane), ctypes.POINTER(Plane), ctypes.c_float, ctypes.c_float,
                                   ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_void_p]),
    "pz_check_device_error": (ctypes.c_int, [ctypes.c_void_p]),
    "pz_selftest_wait": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_void_p]),
}

# Size of the static intermediate-plane array behind pz_nnedi3_run_static.
PZ_STATIC_SCRATCH_BYTES = 16 * 1024 * 1024

_lib = None
_lock = threading.Lock()


def lib():
    """The loaded library (raises if it was not built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise PrescaleLibraryError(
                    f"{LIB_PATH} not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
            try:
                L = ctypes.CDLL(LIB_PATH)
            except OSError as e:
                raise PrescaleLibraryError(f"cannot load {LIB_PATH}: {e}") from e
            for name, (res, args) in EXPORTS.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
        return _lib


def check(rc: int) -> None:
    if rc != PZ_OK:
        msg = lib().pz_last_error()
        raise PrescaleError(rc, msg.decode() if msg else "")


def check_device(stream=None) -> None:
    """Wait for `stream` (default: the current torch stream), read and clear
    the device error word; raises :class:`PrescaleError` (code
    ``PZ_ETIMEDOUT`` when a bounded device-side wait ran out)."""
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    check(lib().pz_check_device_error(s.cuda_stream))
