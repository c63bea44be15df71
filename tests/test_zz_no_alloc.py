"""skew_eigvals_noalloc_d: eigvals for callers that cannot allocate device memory.

Such callers (a host that owns every device byte through its own pool, or a
path where an allocation's synchronisation or failure is not acceptable) get
the same eigenvalues as skew_eigvals_d from an entry point whose scratch is a
fixed array inside the library.  The test calls both entry points through the
C ABI and compares them, twice in a row on different matrices, so a second call
that reused stale scratch contents wrongly would show up.  This file is named
so pytest collects it last.
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
    v2 = torch.zeros(n, dtype=torch.float64, device="cuda")
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
    assert int(i2.item()) == 0
    return v1.cpu().numpy(), v2.cpu().numpy()


def test_noalloc_matches_eigvals_twice(skewgpu):
    for call, (n, seed) in enumerate([(200, 1), (64, 2)]):
        A = _skew(n, seed)
        ref, got = _run_both(skewgpu, A)
        scale = np.abs(ref).max()
        np.testing.assert_allclose(got, ref, atol=RTOL * scale, err_msg=f"call {call}")
        np.testing.assert_allclose(np.sort(got), np.sort(np.linalg.eigvals(A).imag), atol=1e-12 * scale * n)


def test_noalloc_rejects_oversize(skewgpu):
    L = skewgpu._lib.load()
    # rejected on the host before any launch: no buffers are touched
    st = L.skew_eigvals_noalloc_d(ctypes.c_void_p(16), 1025, 1025, ctypes.c_void_p(16), None, None)
    assert st == 6  # SKEW_UNSUPPORTED
