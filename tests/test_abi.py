"""The C ABI library: it builds for sm_103a, loads, exports every entry point
declared in include/miogpu.h, and reports a missing GPU as a status code."""
import ctypes
import os
import re

import pytest

from memilio_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_entry_points():
    names = []
    for h in ("miogpu.h",):
        src = open(os.path.join(ROOT, "include", h)).read()
        names += re.findall(r"^\s*(?:const\s+)?[\w\*\s]+?\b(mgpu_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    path = B.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared_entry_points()
    assert "mgpu_batch_advance" in names and "mgpu_simulate" in names and len(names) >= 15


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_entry_points() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_lists_every_symbol():
    from memilio_gb300 import _native
    assert sorted(_native.EXPORTED) == declared_entry_points()


def test_create_without_gpu_returns_status(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = ctypes.c_void_p()
    lib.mgpu_create.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    rc = lib.mgpu_create(0, ctypes.byref(h))
    assert rc == 100 and not h.value  # MGPU_CUDA_ERROR, no context


def test_status_codes_mirror_reference_statuscode():
    # cpp/memilio/io/io.h:49-59: OK, UnknownError, OutOfRange, InvalidValue, InvalidFileFormat,
    # KeyNotFound, InvalidType, FileNotFound
    src = open(os.path.join(ROOT, "include", "miogpu.h")).read()
    order = ["MGPU_OK", "MGPU_UNKNOWN_ERROR", "MGPU_OUT_OF_RANGE", "MGPU_INVALID_VALUE", "MGPU_INVALID_FILE_FORMAT",
             "MGPU_KEY_NOT_FOUND", "MGPU_INVALID_TYPE", "MGPU_FILE_NOT_FOUND"]
    for i, name in enumerate(order):
        assert re.search(rf"{name}\s*=\s*{i}\b", src), name
