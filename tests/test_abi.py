"""The C ABI library: it builds for sm_103a, loads, exports every entry point
declared in include/miogpu.h, reports a missing GPU as a status code, and the
Python mirror lays out the ABI's structs as a C compiler does from the headers."""
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


def test_struct_layouts_match_the_python_mirror(tmp_path):
    # sizes and field offsets of the ABI's structs, as a C compiler lays them
    # out from the headers, against the ctypes mirror the Python entry uses
    import subprocess
    from memilio_gb300 import _native as N
    from memilio_gb300 import layout as L
    mirrors = {"mgpu_solver_opts": N.MgpuSolverOpts, "mgpu_server_opts": N.MgpuServerOpts,
               "mgpu_timing": N.MgpuTiming, "mgpu_stats": N.MgpuStats, "mgpu_graph": L.MgpuGraph,
               "mgpu_integrator_opts": L.MgpuIntegratorOpts}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "miogpu.h"', 'int main(void) {']
    for cname, py in mirrors.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append('return 0; }')
    src = tmp_path / "layout.c"
    exe = tmp_path / "layout"
    src.write_text("\n".join(lines))
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    c = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in mirrors.items():
        assert c[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert c[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
