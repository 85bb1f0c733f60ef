"""Shared pytest setup: the ``gpu`` marker and the package import.

The package directory is ``mpv-prescalers_gb300/`` (not a valid module
name), so it is registered under the import name ``mpv_prescalers_gb300``.
"""
import importlib.util
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def _load_package():
    if "mpv_prescalers_gb300" in sys.modules:
        return sys.modules["mpv_prescalers_gb300"]
    root = os.path.join(REPO, "mpv-prescalers_gb300")
    spec = importlib.util.spec_from_file_location(
        "mpv_prescalers_gb300", os.path.join(root, "__init__.py"), submodule_search_locations=[root])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["mpv_prescalers_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


_load_package()

# the reference checkout: $PRESCALER_REFERENCE, else a sibling directory
# named "reference" next to this repository
REFERENCE = os.environ.get("PRESCALER_REFERENCE", os.path.join(os.path.dirname(REPO), "reference"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(autouse=True)
def _no_silent_device_errors(request):
    """After every GPU test: no bounded device-side wait ran out unnoticed
    (the kernels record that in the device error word instead of hanging)."""
    yield
    if request.node.get_closest_marker("gpu") is None:
        return
    try:
        import torch
    except ImportError:
        return
    if not torch.cuda.is_available():
        return
    from mpv_prescalers_gb300 import _ffi
    if _ffi._lib is None:   # the test never loaded the library
        return
    lib = _ffi.lib()
    rc = lib.pz_check_device_error(torch.cuda.current_stream().cuda_stream)
    assert rc == _ffi.PZ_OK, f"device error after the test: {lib.pz_last_error().decode()}"


@pytest.fixture(scope="session")
def reference_dir():
    if not os.path.isdir(REFERENCE):
        pytest.skip("reference .hook files not present on this machine")
    return REFERENCE
