"""Batched entry points replayed as CUDA graphs.

The first batched call with a given set of argument pointers captures the
plan's launches into a graph; later calls with the same pointers replay it.
These tests change the matrices behind unchanged pointer arrays between calls
(the replay must see the new contents), swap output arrays (a new capture),
and run a batched call inside a stream that the caller is itself capturing.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-11
GTOL = 1e-8


def skew_random(n, seed):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n)) / np.sqrt(n)
    return (B - B.T) / 2


def _check_logpf(oracle, mats, lp, sg, grads=None):
    for b, A in enumerate(mats):
        rl, rs = oracle.logabspfaffian(A, quad=True)
        assert sg[b] == rs
        assert abs(lp[b] - rl) <= RTOL * max(1.0, abs(rl))
        if grads is not None:
            Gq = oracle.logabspfaffian_grad(A)
            assert np.abs(grads[b] - Gq).max() <= GTOL * np.abs(Gq).max()


def test_replay_sees_new_contents(skewgpu, oracle):
    import torch

    sizes = [16, 40, 64, 100, 130, 200, 256, 18]
    plan = skewgpu.BatchPlan(sizes)
    devs = [torch.empty((n, n), dtype=torch.float64, device="cuda") for n in sizes]
    grads = [torch.empty((n, n), dtype=torch.float64, device="cuda") for n in sizes]
    a_ptrs, g_ptrs = plan.pointer_array(devs), plan.pointer_array(grads)
    lp = torch.empty(len(sizes), dtype=torch.float64, device="cuda")
    sg = torch.empty_like(lp)
    st = torch.empty(len(sizes), dtype=torch.int32, device="cuda")
    for rnd in range(3):
        mats = [skew_random(n, 100 * rnd + k) for k, n in enumerate(sizes)]
        for d, A in zip(devs, mats):
            d.copy_(skewgpu.to_device(A))
        plan.logabspfaffian(a_ptrs, g_ptrs, lp, sg, st)
        torch.cuda.synchronize()
        assert (st.cpu().numpy() == 0).all()
        _check_logpf(oracle, mats, lp.cpu().numpy(), sg.cpu().numpy(), [skewgpu.from_device(g) for g in grads])
    plan.close()


def test_new_outputs_recapture(skewgpu, oracle):
    import torch

    sizes = [32, 64, 96]
    mats = [skew_random(n, 7 + k) for k, n in enumerate(sizes)]
    plan = skewgpu.BatchPlan(sizes)
    devs = [skewgpu.to_device(A) for A in mats]
    a_ptrs = plan.pointer_array(devs)
    outs = []
    for _ in range(3):  # fresh output tensors each time (kept alive so addresses differ)
        lp, sg, st = plan.logabspfaffian(a_ptrs)
        outs.append((lp, sg, st))
    torch.cuda.synchronize()
    for lp, sg, st in outs:
        _check_logpf(oracle, mats, lp.cpu().numpy(), sg.cpu().numpy())
    plan.close()


def test_eigvals_replay(skewgpu, oracle):
    import torch

    sizes = [8, 30, 64, 128]
    plan = skewgpu.BatchPlan(sizes)
    devs = [torch.empty((n, n), dtype=torch.float64, device="cuda") for n in sizes]
    vals = [torch.zeros(n, dtype=torch.float64, device="cuda") for n in sizes]
    a_ptrs, v_ptrs = plan.pointer_array(devs), plan.pointer_array(vals)
    st = torch.empty(len(sizes), dtype=torch.int32, device="cuda")
    for rnd in range(2):
        mats = [skew_random(n, 500 + 10 * rnd + k) for k, n in enumerate(sizes)]
        for d, A in zip(devs, mats):
            d.copy_(skewgpu.to_device(A))
        plan.eigvals(a_ptrs, v_ptrs, st)
        torch.cuda.synchronize()
        for b, A in enumerate(mats):
            vd, _ = oracle.eigvals(A)
            np.testing.assert_allclose(vals[b].cpu().numpy(), vd, atol=RTOL * np.abs(vd).max())
    plan.close()


def test_exp_replay(skewgpu, oracle):
    import torch

    sizes = [6, 33, 64]
    plan = skewgpu.BatchPlan(sizes)
    devs = [torch.empty((n, n), dtype=torch.float64, device="cuda") for n in sizes]
    outs = [torch.empty((n, n), dtype=torch.float64, device="cuda") for n in sizes]
    a_ptrs, o_ptrs = plan.pointer_array(devs), plan.pointer_array(outs)
    st = torch.empty(len(sizes), dtype=torch.int32, device="cuda")
    for rnd in range(2):
        mats = [skew_random(n, 900 + 10 * rnd + k) * 3.0 for k, n in enumerate(sizes)]
        for d, A in zip(devs, mats):
            d.copy_(skewgpu.to_device(A))
        plan.exp(a_ptrs, o_ptrs, st)
        torch.cuda.synchronize()
        for b, A in enumerate(mats):
            Eq = oracle.expm(A, quad=True)
            np.testing.assert_allclose(skewgpu.from_device(outs[b]), Eq, atol=1e-11 * np.sqrt(A.shape[0]))
    plan.close()


def test_inside_caller_capture(skewgpu, oracle):
    """A caller capturing its own graph gets the plan's kernels in it (no nested capture)."""
    import torch

    sizes = [24, 50, 120]
    mats = [skew_random(n, 300 + k) for k, n in enumerate(sizes)]
    plan = skewgpu.BatchPlan(sizes)
    devs = [skewgpu.to_device(A) for A in mats]
    a_ptrs = plan.pointer_array(devs)
    lp = torch.empty(len(sizes), dtype=torch.float64, device="cuda")
    sg = torch.empty_like(lp)
    st = torch.empty(len(sizes), dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        plan.logabspfaffian(a_ptrs, None, lp, sg, st)  # warm-up on s: binds the handle to s
        torch.cuda.synchronize()
        with torch.cuda.graph(g, stream=s, capture_error_mode="relaxed"):
            plan.logabspfaffian(a_ptrs, None, lp, sg, st)
    torch.cuda.synchronize()
    lp.fill_(0.0)
    g.replay()
    torch.cuda.synchronize()
    _check_logpf(oracle, mats, lp.cpu().numpy(), sg.cpu().numpy())
    plan.close()
