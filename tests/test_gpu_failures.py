"""Failure paths, made to happen without faulting or hanging the GPU.

* Bounded waits: the three cooperative kernels (the persistent real reduction, the
  persistent complex reduction and the complex Pfaffian's grid) synchronise their
  CTAs with grid barriers whose polls are bounded.  The tuning keys wait_polls
  (a short limit) and wait_skip_cta (one CTA never arrives) make a barrier's wait
  run out on purpose: every CTA must return, the call must report SKEW_TIMEOUT
  (and NaN outputs where it has them), and the next call on the same handle must
  be correct again.
* Non-convergence: the reference raises error("Maximum number of iterations
  reached ...") when its QR exceeds max_iter sweeps (skeweigen.jl:154).  The
  tuning key qr_max_iter = 1 makes the GPU's QR chains stop after one sweep:
  SKEW_NO_CONVERGENCE from the single-matrix, batched and eigen paths.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SKEW_TIMEOUT = 9
SKEW_NO_CONVERGENCE = 2


def _skew(n, seed, complex_=False):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n))
    if complex_:
        B = B + 1j * rng.standard_normal((n, n))
        return (B - B.conj().T) / 2
    return (B - B.T) / 2


def _P(t):
    return ctypes.c_void_p(t.data_ptr())


def test_timeout_real_persistent_reduction(skewgpu, oracle):
    import torch

    n = 512
    A = _skew(n, 1)
    L = skewgpu._lib.load()
    h = skewgpu.handle().bind()
    tau = torch.zeros(n, dtype=torch.float64, device="cuda")
    ev = torch.zeros(n, dtype=torch.float64, device="cuda")
    info = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    work = skewgpu.to_device(A)
    # n = 512 is in the cluster reduction's range (hardware cluster barriers, no
    # polls of ours): cluster_max_n = 0 sends it to the persistent grid-wide kernel
    with skewgpu.tuned(wait_polls=20000, wait_skip_cta=3, cluster_max_n=0):
        assert L.skew_hessenberg_d(h, _P(work), n, n, _P(tau), _P(ev), _P(info)) == 0
        torch.cuda.synchronize()
    assert int(info.item()) == SKEW_TIMEOUT
    # the handle and the context stay usable: the same call is right again
    work = skewgpu.to_device(A)
    info.fill_(-1)
    assert L.skew_hessenberg_d(h, _P(work), n, n, _P(tau), _P(ev), _P(info)) == 0
    torch.cuda.synchronize()
    assert int(info.item()) == 0
    _, _, evq = oracle.hessenberg(A)
    np.testing.assert_allclose(ev.cpu().numpy()[: n - 1], evq, atol=1e-11 * np.abs(evq).max())


def test_timeout_complex_persistent_reduction(skewgpu):
    import torch

    n = 512
    A = _skew(n, 2, complex_=True)
    L = skewgpu._lib.load()
    h = skewgpu.handle().bind()
    W = skewgpu.to_device_complex(A)
    tau = torch.zeros(n, dtype=torch.complex128, device="cuda")
    ev = torch.zeros(n, dtype=torch.float64, device="cuda")
    dv = torch.zeros(n, dtype=torch.float64, device="cuda")
    info = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    with skewgpu.tuned(wait_polls=20000, wait_skip_cta=5):
        assert L.skew_hessenberg_z(h, _P(W), n, n, _P(tau), _P(ev), _P(dv), _P(info)) == 0
        torch.cuda.synchronize()
    assert int(info.item()) == SKEW_TIMEOUT
    H = skewgpu.hessenberg_complex(A)
    e = H.ev.cpu().numpy()
    d = H.dvim.cpu().numpy()
    fa = np.linalg.norm(A)
    assert abs(np.sqrt(2.0 * np.sum(e * e) + np.sum(d * d)) - fa) <= 1e-12 * fa


def test_timeout_complex_pfaffian_grid(skewgpu, oracle):
    import torch

    n = 400  # above one CTA's size: the cooperative grid kernel
    rng = np.random.default_rng(3)
    C = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
    A = (C - C.T) / 2
    L = skewgpu._lib.load()
    h = skewgpu.handle().bind()
    W = skewgpu.to_device_complex(A)
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    info = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    with skewgpu.tuned(wait_polls=20000, wait_skip_cta=0):
        assert L.skew_logabspf_z(h, _P(W), n, n, _P(out), ctypes.c_void_p(out.data_ptr() + 8), 0, _P(info)) == 0
        torch.cuda.synchronize()
    assert int(info.item()) == SKEW_TIMEOUT
    assert np.isnan(out.cpu().numpy()[:3]).all()
    lp, ph = skewgpu.logabspfaffian_complex(A)
    rl, rp, _ = oracle.pfaffian_complex(A)
    assert abs(lp - rl) <= 1e-11 * max(1.0, abs(rl))


def test_qr_iteration_limit_single_and_batched(skewgpu):
    import torch

    A = _skew(64, 4)
    with skewgpu.tuned(qr_max_iter=1):
        with pytest.raises(RuntimeError, match="Maximum number of iterations"):
            skewgpu.eigvals(A)
        with pytest.raises(RuntimeError, match="Maximum number of iterations"):
            skewgpu.eigen(A)
        sizes = [64, 40, 2]
        mats = [_skew(n, 10 + n) for n in sizes]
        plan = skewgpu.BatchPlan(sizes)
        devs = [skewgpu.to_device(M) for M in mats]
        vals = [torch.zeros(n, dtype=torch.float64, device="cuda") for n in sizes]
        st = plan.eigvals(plan.pointer_array(devs), plan.pointer_array(vals)).cpu().numpy()
        plan.close()
        assert st[0] == SKEW_NO_CONVERGENCE and st[1] == SKEW_NO_CONVERGENCE and st[2] == 0
    # the default limit again: converges, and agrees with the oracle's order
    v = skewgpu.eigvals(A).imag
    assert np.all(np.isfinite(v)) and abs(np.sort(v)[-1] - np.abs(np.linalg.eigvals(A)).max()) < 1e-12 * 64
