"""skew_eigvals_noalloc_d: eigvals for callers that cannot allocate device memory.

Such callers (a host that owns every device byte through its own pool, or a
path where an allocation's synchronisation or failure is not acceptable) get
the eigenvalues of skew_eigvals_d, sorted descending, from an entry point whose
scratch is a fixed array inside the library.  The test calls both entry points
through the C ABI on the same matrix and compares them (within the 1e-11
normwise eigenvalue tolerance of the parity tests), and compares both with the
binary128 oracle at the same tolerance (its FP64 restatement at n = 1024).  The sizes run twice in a row on
different matrices, so a call that reused stale scratch contents would show up;
they include n = 1 (no scratch), an odd size and n = 1024, the largest size,
which uses every entry of the array.  This file is named so pytest collects it
last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-11  # eigenvalue tolerance used by the parity tests (normwise)


def _skew(n, seed):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n)) / np.sqrt(n)
    return (B - B.T) / 2


def _run_both(skewgpu, A):
    import torch

    L = skewgpu._lib.load()
    n = A.shape[0]
    d1 = skewgpu.to_device(A)
    d2 = skewgpu.to_device(A)
    v1 = torch.zeros(n, dtype=torch.float64, device="cuda")
    v2 = torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
    i1 = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    i2 = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    h = skewgpu.handle().bind()
    st = L.skew_eigvals_d(h, ctypes.c_void_p(d1.data_ptr()), n, n, ctypes.c_void_p(v1.data_ptr()),
                          ctypes.c_void_p(i1.data_ptr()))
    assert st == 0
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = L.skew_eigvals_noalloc_d(ctypes.c_void_p(d2.data_ptr()), n, n, ctypes.c_void_p(v2.data_ptr()),
                                  ctypes.c_void_p(i2.data_ptr()), stream)
    assert st == 0
    torch.cuda.synchronize()
    assert int(i1.item()) in (0, 8) and int(i2.item()) == 0
    return v1.cpu().numpy(), v2.cpu().numpy()


@pytest.mark.parametrize("sizes", [[200, 64], [1024, 129], [1, 2]])
def test_noalloc_matches_eigvals_twice(skewgpu, oracle, sizes):
    for call, n in enumerate(sizes):
        A = _skew(n, 31 * n + call)
        ref, got = _run_both(skewgpu, A)
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.all(np.diff(got) <= 0), "values come out sorted descending"
        np.testing.assert_allclose(got, np.sort(ref)[::-1], atol=RTOL * scale, err_msg=f"call {call}, n={n}")
        # binary128 oracle; at n = 1024 its FP64 restatement (about 1e-13 from binary128 there)
        vq, _ = oracle.eigvals(A, quad=(n <= 512))
        np.testing.assert_allclose(got, np.sort(vq)[::-1], atol=RTOL * max(np.abs(vq).max(), 1e-300),
                                   err_msg=f"call {call}, n={n} vs the oracle")


def test_noalloc_rejects_oversize(skewgpu):
    L = skewgpu._lib.load()
    # rejected on the host before any launch: no buffers are touched
    st = L.skew_eigvals_noalloc_d(ctypes.c_void_p(16), 1025, 1025, ctypes.c_void_p(16), None, None)
    assert st == 6  # SKEW_UNSUPPORTED
