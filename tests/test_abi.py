"""The C-ABI library builds, loads and exports every declared entry point
(no device calls: this runs without a GPU)."""
import os
import re

import pytest

from mpv_prescalers_gb300 import _ffi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "prescale.h")


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_ffi.LIB_PATH):
        from mpv_prescalers_gb300 import build
        build.build()
    return _ffi.lib()


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(pz_[a-z_]+)\s*\(", text)))


def test_header_declares_the_entry_points():
    names = declared()
    for n in ("pz_model_create", "pz_model_destroy", "pz_run", "pz_last_error", "pz_version",
              "pz_scratch_bytes", "pz_batch_run", "pz_batch_work_bytes"):
        assert n in names


def test_every_declared_symbol_is_exported(lib):
    for n in declared():
        assert hasattr(lib, n), n
    assert set(_ffi.EXPORTS) >= set(declared()) - set()


def test_version_and_error_without_device(lib):
    assert lib.pz_version() == 2
    assert isinstance(lib.pz_last_error(), bytes)


def test_null_arguments_are_rejected_on_the_host(lib):
    assert lib.pz_model_create(None, None) == _ffi.PZ_EINVAL
    assert b"null" in lib.pz_last_error()
    assert lib.pz_run(None, None, 0, None, 0, None, None) == _ffi.PZ_EINVAL


# ctypes mirror -> (C struct, {ctypes field: C field} where the names differ)
_STRUCTS = {"ModelDesc": ("pz_model_desc", {}), "Plane": ("pz_plane", {}), "Opts": ("pz_opts", {}),
            "QueryResult": ("pz_query_result", {}), "Job": ("pz_job", {"inp": "in"})}


def test_struct_layouts_match_the_header(tmp_path):
    """Every ctypes mirror has the header struct's size and field offsets
    (a C program compiled against include/prescale.h prints them)."""
    import ctypes
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines, want = [], []
    for py, (cs, rename) in _STRUCTS.items():
        cls = getattr(_ffi, py)
        lines.append(f'printf("%zu\\n", sizeof({cs}));')
        want.append(ctypes.sizeof(cls))
        for f, *_ in cls._fields_:
            lines.append(f'printf("%zu\\n", offsetof({cs}, {rename.get(f, f)}));')
            want.append(getattr(cls, f).offset)
    src = tmp_path / "layout.c"
    src.write_text("#include <stdio.h>\n#include <stddef.h>\n#include \"prescale.h\"\nint main(void) {\n" +
                   "\n".join(lines) + "\nreturn 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == want


def test_resample_arguments_are_checked_on_the_host(lib):
    import ctypes
    fake = 4096   # never dereferenced: every call below is refused before a launch
    a = _ffi.Plane(fake, 8, 8, 8, _ffi.PZ_F32)
    b = _ffi.Plane(fake, 8, 8, 8, _ffi.PZ_F16)
    assert lib.pz_resample(None, ctypes.byref(a), 1, 0, 1, 0, 0, None) == _ffi.PZ_EINVAL
    assert lib.pz_resample(ctypes.byref(a), ctypes.byref(b), 1, 0, 1, 0, 0, None) == _ffi.PZ_EINVAL
    assert b"dtype" in lib.pz_last_error()
    assert lib.pz_resample(ctypes.byref(a), ctypes.byref(a), 1, 0, 1, 0, 7, None) == _ffi.PZ_EINVAL
    assert b"filter" in lib.pz_last_error()
    assert lib.pz_resample(ctypes.byref(a), ctypes.byref(a), float("nan"), 0, 1, 0, 1, None) == _ffi.PZ_EINVAL
    assert lib.pz_resample(ctypes.byref(a), ctypes.byref(a), 1, 0, 1, 3e9, 1, None) == _ffi.PZ_EINVAL
    assert b"out of range" in lib.pz_last_error()


def test_query_arguments_are_checked_on_the_host(lib):
    import ctypes
    r = _ffi.QueryResult()
    assert lib.pz_query(None, 8, 8, _ffi.PZ_F16, None, ctypes.byref(r)) == _ffi.PZ_EINVAL
    assert b"null" in lib.pz_last_error()


def test_host_pipeline_arguments_are_checked_on_the_host(lib):
    assert lib.pz_run_host(None, None, None, 1, 8, 8, _ffi.PZ_F16, None, None, 0, 0, None) == _ffi.PZ_EINVAL
    assert b"null" in lib.pz_last_error()
    assert lib.pz_run_host_work_bytes(None, 8, 8, _ffi.PZ_F16, None) == 0
