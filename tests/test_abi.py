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


def header_param_types():
    """name -> list of parameter type strings, from the header's declarations."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", " ", txt, flags=re.S)
    out = {}
    for m in re.finditer(r"SKEW_API\s+[^;(]*?\b(skew_\w+)\s*\(([^)]*)\)\s*;", txt, flags=re.S):
        params = " ".join(m.group(2).split())
        if params in ("", "void"):
            out[m.group(1)] = []
        else:
            out[m.group(1)] = [p.strip() for p in params.split(",")]
    return out


def _ctype_kind(t):
    import ctypes as C

    if t in (C.c_int64,):
        return "int64"
    if t in (C.c_int,):
        return "int"
    if t in (C.c_double,):
        return "double"
    return "ptr"


def _decl_kind(p):
    p = p.strip()
    if "*" in p or p.split()[0] in ("skew_handle_t", "skew_batch_plan_t", "skew_stream_t"):
        return "ptr"
    if p.startswith("int64_t"):
        return "int64"
    if p.startswith("int"):
        return "int"
    if p.startswith("double"):
        return "double"
    return "?"


def test_python_signatures_match_header():
    """Every ctypes signature has the header's arity and argument kinds (pointer,
    int, int64, double), so a call through the binding passes what the C side reads."""
    from skewgpu import _lib as L

    decl = header_param_types()
    assert sorted(decl) == header_functions()
    for name, (_, args) in L.SIGNATURES.items():
        want = [_decl_kind(p) for p in decl[name]]
        got = [_ctype_kind(a) for a in args]
        assert "?" not in want, (name, decl[name])
        assert got == want, (name, decl[name], got)


def test_plain_c_caller(lib, tmp_path):
    """include/skewgpu.h compiles as C99 (-Wall -Wextra -pedantic -Werror) and a C
    program links against libskewgpu.so and runs: without a GPU skew_create returns a
    status instead of crashing; with one, a bad argument is rejected on the host."""
    import shutil
    import subprocess

    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no gcc")
    libdir = os.path.dirname(lib._name)
    exe = str(tmp_path / "caller")
    src = os.path.join(ROOT, "tests", "c_caller", "caller.c")
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                    src, "-L", libdir, "-lskewgpu", "-Wl,-rpath," + libdir, "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "skew_create ->" in r.stdout
