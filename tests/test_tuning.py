"""The tuning table (CPU only: the library reads table files without a GPU).

A handle starts from compiled-in defaults and loads its device's entry from a JSON
table; skew_tuning_file_get shows what a file holds for a device name.  Checked
here: defaults when a file has no entry for the device, an entry's values, list
keys, range and syntax errors (the whole load is refused), members that are not
keys (measurement records) being skipped, and the committed GB300 table.
"""
import ctypes
import json
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TABLE = os.path.join(ROOT, "skewlinearalgebra.jl_gb300", "skewgpu", "skew_tuning.json")

OK, BAD_ARG, UNSUPPORTED = 0, 3, 6


@pytest.fixture(scope="module")
def lib():
    import build_lib  # skewlinearalgebra.jl_gb300/build_lib.py

    L = ctypes.CDLL(build_lib.build())
    L.skew_tuning_file_get.restype = ctypes.c_int
    L.skew_tuning_file_get.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                       ctypes.POINTER(ctypes.c_int64), ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.skew_tuning_key.restype = ctypes.c_char_p
    L.skew_tuning_key.argtypes = [ctypes.c_int]
    return L


def get(lib, path, device, key):
    vals = (ctypes.c_int64 * 16)()
    cnt = ctypes.c_int(0)
    st = lib.skew_tuning_file_get(str(path).encode(), device.encode(), key.encode(), vals, 16, ctypes.byref(cnt))
    return st, list(vals[: cnt.value])


def write(tmp_path, obj, name="t.json"):
    p = tmp_path / name
    p.write_text(obj if isinstance(obj, str) else json.dumps(obj))
    return p


def test_keys_listed(lib):
    keys = []
    while (k := lib.skew_tuning_key(len(keys))) is not None:
        keys.append(k.decode())
    for k in ("bucket_edges", "batch_smem_nmax", "blocked_min_n", "persist_items", "wait_polls", "qr_max_iter"):
        assert k in keys


def test_defaults_without_entry(lib, tmp_path):
    p = write(tmp_path, {"devices": {"Some Other GPU": {"batch_smem_nmax": 64}}})
    st, v = get(lib, p, "NVIDIA GB300", "batch_smem_nmax")
    assert st == UNSUPPORTED and v == [96]
    st, v = get(lib, p, "NVIDIA GB300", "bucket_edges")
    assert st == UNSUPPORTED and v == [32, 64, 96, 128, 152]


def test_entry_values_and_lists(lib, tmp_path):
    p = write(tmp_path, {"tool": "x", "devices": {"GPU A": {"batch_smem_nmax": 128, "bucket_edges": [48, 96, 160],
                                                            "measurements": {"batch_smem_nmax": [[96, 1.0]]},
                                                            "wait_polls": 1 << 33},
                                                  "GPU B": {"batch_smem_nmax": 64}}})
    assert get(lib, p, "GPU A", "batch_smem_nmax") == (OK, [128])
    assert get(lib, p, "GPU A", "bucket_edges") == (OK, [48, 96, 160])
    assert get(lib, p, "GPU A", "wait_polls") == (OK, [1 << 33])
    assert get(lib, p, "GPU A", "persist_items") == (OK, [8])  # not in the entry: the default
    assert get(lib, p, "GPU B", "batch_smem_nmax") == (OK, [64])


@pytest.mark.parametrize("entry", [{"batch_smem_nmax": 400}, {"batch_global_nt": 384}, {"bucket_edges": [64, 32]},
                                   {"bucket_edges": list(range(10, 100, 10))}, {"persist_items": 1.5}])
def test_out_of_range_refused(lib, tmp_path, entry):
    p = write(tmp_path, {"devices": {"G": entry}})
    assert get(lib, p, "G", "batch_smem_nmax")[0] == BAD_ARG


@pytest.mark.parametrize("text", ["{", '{"devices": {"G": {"batch_smem_nmax": }}}', "[1, 2]", ""])
def test_syntax_errors_refused(lib, tmp_path, text):
    assert get(lib, write(tmp_path, text), "G", "batch_smem_nmax")[0] == BAD_ARG


def test_unknown_key_and_missing_file(lib, tmp_path):
    p = write(tmp_path, {"devices": {}})
    assert get(lib, p, "G", "no_such_key")[0] == BAD_ARG
    assert get(lib, tmp_path / "missing.json", "G", "batch_smem_nmax")[0] == BAD_ARG


def test_committed_table(lib):
    """The table beside the library holds a GB300 entry that loads."""
    with open(TABLE) as f:
        t = json.load(f)
    assert "NVIDIA GB300" in t["devices"]
    assert get(lib, TABLE, "NVIDIA GB300", "bucket_edges")[0] == OK
