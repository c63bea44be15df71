"""The C-ABI library loads and exports every entry point include/skewgpu.h
declares (CPU only: no compute calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "skewgpu.h")


def header_functions():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"SKEW_API\s+(?:const\s+)?\w+\*?\s+\*?(skew_\w+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    import build_lib  # skewlinearalgebra.jl_gb300/build_lib.py

    path = build_lib.build()
    return ctypes.CDLL(path)


def test_header_parses():
    names = header_functions()
    assert "skew_logabspf_d" in names and "skew_batch_logabspf_d" in names
    assert len(names) >= 15


def test_exports_match_header(lib):
    for name in header_functions():
        assert hasattr(lib, name), f"{name} declared in skewgpu.h but not exported"


def test_python_binding_covers_header():
    from skewgpu import _lib as L

    assert sorted(L.SIGNATURES) == header_functions()


def test_status_strings_without_gpu(lib):
    lib.skew_status_string.restype = ctypes.c_char_p
    assert lib.skew_status_string(0) == b"ok"
    assert b"skew" in lib.skew_status_string(1)
    assert b"converge" in lib.skew_status_string(2)
    assert lib.skew_version() >= 100


def test_bad_args_rejected_on_host(lib):
    # argument validation happens before any CUDA call
    assert lib.skew_create(None) == 3  # SKEW_BAD_ARG
    assert lib.skew_batch_plan_destroy(None) == 3


def test_no_gpu_is_an_error_not_a_crash(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("GPU present")
    h = ctypes.c_void_p()
    st = lib.skew_create(ctypes.byref(h))
    assert st == 4  # SKEW_CUDA_ERROR
