"""Batched logabspfaffian + gradient on host buffers (skew_batch_logabspf_host_d):
the kernels read every matrix from page-locked host memory and write every
gradient back there themselves.

Checks, with the tolerances written in each test:
* against the device-resident batched call on the same plan and inputs:
  log|Pf| within 1e-13 relative, sign and status equal, gradients within 1e-13
  relative to the largest entry (the same kernels' arithmetic, another
  instantiation);
* against the oracle on a sample: log|Pf| within 1e-11 relative (floor 1), sign
  equal, gradient within 1e-8 relative (normwise);
* odd sizes and a zero Pfaffian give status SKEW_SINGULAR with NaN gradients, as
  the device path;
* without a gradient buffer only (log|Pf|, sign) are written;
* pageable (not page-locked) buffers are refused with ValueError by the Python
  layer and with SKEW_BAD_ARG by the C ABI itself, before any launch.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _batch(sizes, seed):
    rng = np.random.default_rng(seed)
    mats = []
    for n in sizes:
        B = rng.standard_normal((n, n)) / np.sqrt(max(n, 1))
        mats.append((B - B.T) / 2)
    return mats


def _packed(mats):
    return np.concatenate([m.T.reshape(-1) for m in mats]) if mats else np.zeros(0)


def _device_run(skewgpu, plan, mats, sizes):
    buf = torch.from_numpy(_packed(mats)).cuda()
    grad = torch.empty_like(buf)
    offs = np.concatenate([[0], np.cumsum(np.asarray(sizes, dtype=np.int64) ** 2)[:-1]])
    a_ptrs = torch.tensor((buf.data_ptr() + 8 * offs).tolist(), dtype=torch.int64, device="cuda")
    g_ptrs = torch.tensor((grad.data_ptr() + 8 * offs).tolist(), dtype=torch.int64, device="cuda")
    lp, sg, st = plan.logabspfaffian(a_ptrs, g_ptrs)
    torch.cuda.synchronize()
    return lp.cpu().numpy(), sg.cpu().numpy(), st.cpu().numpy(), grad.cpu().numpy(), offs


SIZES = [2, 16, 3, 40, 64, 96, 97, 100, 128, 150, 170, 200, 256, 1, 8, 250, 30, 64]


def test_host_matches_device(skewgpu):
    sizes = SIZES * 6
    mats = _batch(sizes, 1)
    plan = skewgpu.BatchPlan(sizes)
    lp_d, sg_d, st_d, g_d, offs = _device_run(skewgpu, plan, mats, sizes)
    h_in = torch.from_numpy(_packed(mats)).pin_memory()
    h_g = torch.empty(plan.packed_size(), dtype=torch.float64).pin_memory()
    lp, sg, st = plan.logabspfaffian_host(h_in, h_g)
    lp, sg, st, g = lp.numpy(), sg.numpy(), st.numpy(), h_g.numpy()
    np.testing.assert_array_equal(st, st_d)
    np.testing.assert_array_equal(sg, sg_d)
    ok = st == 0
    assert ok.sum() > 0
    np.testing.assert_allclose(lp[ok], lp_d[ok], rtol=1e-13, atol=0)
    assert np.all(lp[~ok] == lp_d[~ok])
    for b, n in enumerate(sizes):
        gb = g[offs[b]:offs[b] + n * n]
        gd = g_d[offs[b]:offs[b] + n * n]
        if st[b] == 0:
            scale = max(np.abs(gd).max(), 1e-300)
            assert np.abs(gb - gd).max() <= 1e-13 * scale, (b, n)
        else:
            assert np.all(np.isnan(gb)) and np.all(np.isnan(gd))
    plan.close()


def test_host_vs_oracle(skewgpu, oracle):
    sizes = [2, 6, 33, 64, 90, 120, 180, 256]
    mats = _batch(sizes, 2)
    plan = skewgpu.BatchPlan(sizes)
    h_in = torch.from_numpy(_packed(mats)).pin_memory()
    h_g = torch.empty(plan.packed_size(), dtype=torch.float64).pin_memory()
    lp, sg, st = plan.logabspfaffian_host(h_in, h_g)
    offs = np.concatenate([[0], np.cumsum(np.asarray(sizes) ** 2)[:-1]])
    for b, n in enumerate(sizes):
        if n % 2:
            assert st[b] == 5 and lp[b] == -np.inf and sg[b] == 0
            continue
        lq, sq = oracle.logabspfaffian(mats[b], quad=True)
        assert st[b] == 0
        assert abs(lp[b].item() - lq) <= 1e-11 * max(1.0, abs(lq))
        assert sg[b].item() == sq
        G = h_g.numpy()[offs[b]:offs[b] + n * n].reshape(n, n).T
        Gref = oracle.logabspfaffian_grad(mats[b])
        assert np.linalg.norm(G - Gref) <= 1e-8 * np.linalg.norm(Gref)
    plan.close()


def test_host_zero_pfaffian_and_no_gradient(skewgpu):
    sizes = [6, 140, 200]
    mats = _batch(sizes, 3)
    z = mats[1]  # zero first row and column: the first subdiagonal entry is exactly 0
    z[0, :] = 0
    z[:, 0] = 0
    plan = skewgpu.BatchPlan(sizes)
    h_in = torch.from_numpy(_packed(mats)).pin_memory()
    h_g = torch.full((plan.packed_size(),), 7.0, dtype=torch.float64).pin_memory()
    lp, sg, st = plan.logabspfaffian_host(h_in, h_g)
    assert st[1] == 5 and lp[1] == -np.inf and sg[1] == 0
    assert np.all(np.isnan(h_g.numpy()[36:36 + 140 * 140]))
    lp2, sg2, st2 = plan.logabspfaffian_host(h_in)
    np.testing.assert_array_equal(lp2.numpy(), lp.numpy())
    np.testing.assert_array_equal(sg2.numpy(), sg.numpy())
    plan.close()


def test_pageable_buffers_refused(skewgpu):
    from skewgpu import _lib

    sizes = [4, 8]
    mats = _batch(sizes, 4)
    plan = skewgpu.BatchPlan(sizes)
    pageable = torch.from_numpy(_packed(mats))
    with pytest.raises(ValueError):
        plan.logabspfaffian_host(pageable)
    pinned = pageable.pin_memory()
    with pytest.raises(ValueError):
        plan.logabspfaffian_host(pinned, torch.empty(plan.packed_size(), dtype=torch.float64))
    # the C ABI checks the mapping itself
    a = np.ascontiguousarray(_packed(mats))
    lp = np.zeros(2)
    sg = np.zeros(2)
    st = np.zeros(2, dtype=np.int32)
    vp = lambda x: ctypes.c_void_p(x.ctypes.data)
    rc = _lib.load().skew_batch_logabspf_host_d(plan.plan, vp(a), None, vp(lp), vp(sg), vp(st))
    assert rc == _lib.SKEW_BAD_ARG
    plan.close()
