"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/nlgpu.h (no compute calls: these run without a GPU)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "nlgpu.h")


@pytest.fixture(scope="module")
def built():
    from nonlocal_gb300 import build
    return build.build()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nlgpu_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "nlgpu_stationary_2d" in names and "nlgpu_cg_solve" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(built):
    out = subprocess.run(["nm", "-D", "--defined-only", built], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (nlgpu_\w+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_python_signatures_cover_header(built):
    from nonlocal_gb300 import _lib
    lib = _lib.load(built)
    for name in declared_functions():
        assert name in _lib.SIGNATURES, name
        assert getattr(lib, name) is not None


def test_build_targets_sm103a_only():
    from nonlocal_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_no_device_is_reported_cleanly(built):
    from nonlocal_gb300 import _lib
    lib = _lib.load(built)
    if _lib.device_count() > 0:
        pytest.skip("a GPU is visible")
    import ctypes
    h = ctypes.c_void_p()
    assert lib.nlgpu_create(ctypes.byref(h), None) == 2   # NLGPU_ERR_CUDA
    assert lib.nlgpu_status_string(2) == b"CUDA error"
    assert lib.nlgpu_mesh_2d(None, 2, 0, None, 0, None) == 1   # NLGPU_ERR_ARG


def test_batched_solve_checks_its_arguments(built):
    """nlgpu_solve_assembled_batch rejects a negative count and missing arrays
    before touching a device, and an empty batch is a no-op."""
    import ctypes
    from nonlocal_gb300 import _lib
    lib = _lib.load(built)
    opts = _lib.SolveOptions()
    opts.tolerance, opts.max_iterations = 1e-10, 100
    assert lib.nlgpu_solve_assembled_batch(-1, None, ctypes.byref(opts), None, None) == 1   # NLGPU_ERR_ARG
    assert lib.nlgpu_solve_assembled_batch(2, None, ctypes.byref(opts), None, None) == 1
    handles = (ctypes.c_void_p * 1)(None)
    outs = (ctypes.c_void_p * 1)(None)
    assert lib.nlgpu_solve_assembled_batch(1, handles, ctypes.byref(opts), outs, None) == 1   # null context
    assert lib.nlgpu_solve_assembled_batch(0, None, ctypes.byref(opts), None, None) == 0
    assert lib.nlgpu_solve_assembled_batch(0, None, None, None, None) == 1   # options are required
