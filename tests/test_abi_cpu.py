"""CPU-only checks of the boundary: the engine library loads, exports every entry
point the header declares, and reports errors without touching a GPU."""
import ctypes
import os
import re
import shutil

import numpy as np
import pytest

from qibojit_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "qibojit_gb300.h")


def _declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sv_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
            pytest.skip("engine library not built and nvcc unavailable")
        from qibojit_gb300 import build

        build.build()
    return _lib.load()


def test_header_and_binding_agree():
    assert _declared_symbols() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in _declared_symbols():
        assert hasattr(lib, name), name


def test_version_and_error_string(lib):
    assert lib.sv_version() >= 100
    assert isinstance(_lib.last_error(), str)


def test_no_device_maps_to_import_error(lib):
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = lib.sv_context_create(0, ctypes.byref(h))
    assert rc == _lib.SV_ERR_NO_DEVICE
    with pytest.raises(ImportError):
        _lib.check(rc, "sv_context_create")


def test_null_context_is_rejected(lib):
    rc = lib.sv_apply_one_qubit(None, None, 0, 4, 0, None, 0, None, 0)
    assert rc == _lib.SV_ERR_ARG
    assert "context" in _lib.last_error()
    with pytest.raises(ValueError):
        _lib.check(rc)


@pytest.mark.parametrize("rc,exc", [(_lib.SV_ERR_ARG, ValueError), (_lib.SV_ERR_OOM, RuntimeError),
                                    (_lib.SV_ERR_UNSUPPORTED, NotImplementedError),
                                    (_lib.SV_ERR_TIMEOUT, TimeoutError), (_lib.SV_ERR_CUDA, RuntimeError)])
def test_status_to_exception(lib, rc, exc):
    with pytest.raises(exc):
        _lib.check(rc, "x")


def test_int32_array():
    a, n = _lib.int32_array([3, 1, 2])
    assert n == 3 and list(a) == [3, 1, 2]
    assert _lib.int32_array([]) == (None, 0)
