"""GPU parity: libskewgpu (through its C ABI) against the oracle.

Tolerances: log|Pf| and eigenvalues within 1e-11 relative of the
binary128 oracle (eigenvalues normwise: max |lambda - lambda*| / max |lambda*|),
Pfaffian sign exactly equal, gradients within 1e-8 relative (normwise).
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_known_answers.json")))["cases"]
RTOL = 1e-11
GTOL = 1e-8


def skew_random(n, seed, scale=None):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n)) * (1 / np.sqrt(max(n, 1)) if scale is None else scale)
    return (B - B.T) / 2


def tridiag_dense(ev):
    n = len(ev) + 1
    T = np.zeros((n, n))
    T[np.arange(1, n), np.arange(n - 1)] = ev
    T[np.arange(n - 1), np.arange(1, n)] = -np.asarray(ev)
    return T


def assert_logpf(got, ref, n):
    (lp, sg), (rl, rs) = got, ref
    assert sg == rs, f"sign mismatch n={n}: {sg} vs {rs}"
    if np.isfinite(rl):
        assert abs(lp - rl) <= RTOL * max(1.0, abs(rl)), f"n={n}: {lp} vs {rl}"
    else:
        assert lp == rl


# --- goldens of the reference test-suite -----------------------------------------
def test_readme_hessenberg_golden(skewgpu, oracle):
    A = np.array(GOLD["readme_A"]["A"])
    H = skewgpu.hessenberg(A)
    ev = H.ev.cpu().numpy()
    np.testing.assert_allclose(ev, GOLD["readme_hessenberg_v"]["v"], rtol=1e-14)
    F = skewgpu.from_device(H.factors)
    Q = oracle.formq(F, H.tau.cpu().numpy())
    np.testing.assert_allclose(Q, np.array(GOLD["readme_Q"]["Q"]), atol=1e-14)


def test_readme_pfaffian_and_eigvals(skewgpu):
    A = np.array(GOLD["readme_A"]["A"])
    lp, sg = skewgpu.logabspfaffian(A)
    assert sg == -1.0 and abs(lp - np.log(9.0)) < 1e-14
    l1, l2 = GOLD["readme_eigs"]["ilambda"]
    vals = skewgpu.eigvals(A).imag
    np.testing.assert_allclose(np.sort(vals), np.sort([l1, l2, -l2, -l1]), rtol=1e-13)


def test_known_pfaffians(skewgpu):
    lp, sg = skewgpu.logabspfaffian(np.array(GOLD["issue49"]["A"]))
    assert sg * np.exp(lp) == pytest.approx(GOLD["issue49"]["pfaffian"], rel=1e-13)
    lp, sg = skewgpu.logabspfaffian(np.array(GOLD["issue121"]["A"]))
    assert sg * np.exp(lp) == pytest.approx(1.0, rel=1e-14)
    rng = np.random.default_rng(1)
    for _ in range(10):
        a, b, c, d, e, f = (float(x) for x in rng.integers(-10, 11, 6))
        A = np.array([[0, a, b, c], [-a, 0, d, e], [-b, -d, 0, f], [-c, -e, -f, 0]])
        assert skewgpu.pfaffian(A) == pytest.approx(c * d - b * e + a * f, rel=1e-12, abs=1e-12)


def test_not_skew_raises(skewgpu):
    A = skew_random(6, 0)
    A[1, 0] += 1.0
    with pytest.raises(ValueError):
        skewgpu.logabspfaffian(A)


# --- single-matrix path ----------------------------------------------------------
@pytest.mark.parametrize("n", list(range(0, 21)) + [31, 64, 65, 128, 200, 256])
def test_single_logabspf_vs_quad(skewgpu, oracle, n):
    A = skew_random(n, 100 + n)
    assert_logpf(skewgpu.logabspfaffian(A), oracle.logabspfaffian(A, quad=True), n)


@pytest.mark.parametrize("n", [2, 3, 4, 9, 16, 33, 100, 256])
def test_single_hessenberg_structure(skewgpu, oracle, n):
    A = skew_random(n, 200 + n)
    H = skewgpu.hessenberg(A)
    ev = H.ev.cpu().numpy()
    tau = H.tau.cpu().numpy()
    F = skewgpu.from_device(H.factors)
    Q = oracle.formq(F, tau)
    T = tridiag_dense(ev)
    np.testing.assert_allclose(Q @ T @ Q.T, A, atol=1e-13 * max(1.0, np.abs(A).max()) * n)
    _, tq, evq = oracle.hessenberg(A, quad=True)
    # same reflector convention: ev agree entrywise (signs included)
    np.testing.assert_allclose(ev, evq, atol=1e-12 * np.abs(evq).max())
    assert np.array_equal(tau != 0, tq != 0)


@pytest.mark.parametrize("n", [2, 4, 6, 10, 32, 64, 128])
def test_single_gradient(skewgpu, oracle, n):
    A = skew_random(n, 300 + n) + 0.5 * np.kron(np.eye(n // 2), np.array([[0, 1], [-1, 0]]))
    (lp, sg), pb = skewgpu.logabspfaffian_rrule(A)
    assert_logpf((lp, sg), oracle.logabspfaffian(A, quad=True), n)
    G = skewgpu.from_device(pb(1.0))
    Gq = oracle.logabspfaffian_grad(A)
    assert np.abs(G - Gq).max() <= GTOL * np.abs(Gq).max()
    # central finite differences on skew pairs (h = 1e-6)
    rng = np.random.default_rng(n)
    h = 1e-6
    for _ in range(4):
        i, j = rng.choice(n, 2, replace=False)
        Ap, Am = A.copy(), A.copy()
        Ap[i, j] += h
        Ap[j, i] -= h
        Am[i, j] -= h
        Am[j, i] += h
        fd = (oracle.logabspfaffian(Ap, quad=True)[0] - oracle.logabspfaffian(Am, quad=True)[0]) / (2 * h)
        assert fd == pytest.approx(G[i, j] - G[j, i], rel=1e-6, abs=1e-7)


@pytest.mark.parametrize("n", [2, 3, 4, 7, 16, 33, 64, 128, 191, 192, 255, 256, 512, 1024])
def test_single_eigvals_vs_quad(skewgpu, oracle, n):
    """Values against the binary128 oracle, and the order against the FP64
    restatement of skewtrieigvals! (the reference's deflation order), through the
    one-CTA (n < 192) and the blocked (n >= 192) reductions."""
    A = skew_random(n, 400 + n)
    vq, _ = oracle.eigvals(A, quad=(n <= 512))
    vals = skewgpu.eigvals(A).imag
    scale = max(np.abs(vq).max(), 1e-300)
    np.testing.assert_allclose(np.sort(vals), np.sort(vq), atol=RTOL * scale)
    vd, st = oracle.eigvals(A)
    assert st == 0
    np.testing.assert_allclose(vals, vd, atol=RTOL * scale)  # the reference's order


def test_odd_sizes(skewgpu):
    for n in (1, 3, 7):
        lp, sg = skewgpu.logabspfaffian(skew_random(n, n))
        assert lp == -np.inf and sg == 0.0


def test_determinism(skewgpu):
    A = skew_random(96, 5)
    r1 = skewgpu.logabspfaffian(A)
    r2 = skewgpu.logabspfaffian(A)
    assert r1 == r2
    (l1, _), p1 = skewgpu.logabspfaffian_rrule(A)
    (l2, _), p2 = skewgpu.logabspfaffian_rrule(A)
    assert np.array_equal(skewgpu.from_device(p1()), skewgpu.from_device(p2()))


# --- batched path ----------------------------------------------------------------
def _batch(skewgpu, mats, grad=True):
    import torch

    plan = skewgpu.BatchPlan([m.shape[0] for m in mats])
    devs = [skewgpu.to_device(A) for A in mats]
    grads = [torch.full_like(d, np.nan) for d in devs] if grad else None
    lp, sg, st = plan.logabspfaffian(plan.pointer_array(devs), plan.pointer_array(grads) if grad else None)
    torch.cuda.synchronize()
    out = (lp.cpu().numpy(), sg.cpu().numpy(), st.cpu().numpy(),
           [skewgpu.from_device(g) for g in grads] if grad else None)
    plan.close()
    return out


def test_batch_mixed_sizes(skewgpu, oracle):
    rng = np.random.default_rng(7)
    sizes = [int(x) for x in rng.choice(np.arange(2, 257, 2), 48)] + [16, 160, 162, 256, 2, 4, 130]
    mats = [skew_random(n, 1000 + k) for k, n in enumerate(sizes)]
    lp, sg, st, grads = _batch(skewgpu, mats)
    for b, A in enumerate(mats):
        assert st[b] == 0
        assert_logpf((lp[b], sg[b]), oracle.logabspfaffian(A, quad=True), A.shape[0])
        Gq = oracle.logabspfaffian_grad(A)
        assert np.abs(grads[b] - Gq).max() <= GTOL * np.abs(Gq).max(), f"grad n={A.shape[0]}"


def test_batch_pfaffian_adjoint_config(skewgpu, oracle):
    # the batched adjoint workload's matrices: (B - B^T)/2 with B ~ N(0, 1/n), plus 0.5 J
    n = 128
    J = np.kron(np.eye(n // 2), np.array([[0.0, 1.0], [-1.0, 0.0]]))
    mats = [skew_random(n, 5000 + k) + 0.5 * J for k in range(16)]
    lp, sg, st, grads = _batch(skewgpu, mats)
    for b, A in enumerate(mats[:8]):
        assert_logpf((lp[b], sg[b]), oracle.logabspfaffian(A, quad=True), n)
        Gq = oracle.logabspfaffian_grad(A)
        assert np.abs(grads[b] - Gq).max() <= GTOL * np.abs(Gq).max()


def test_batch_odd_and_edge(skewgpu, oracle):
    mats = [skew_random(n, n) for n in (1, 2, 3, 5, 8)] + [np.zeros((4, 4))]
    lp, sg, st, grads = _batch(skewgpu, mats)
    for b, A in enumerate(mats):
        n = A.shape[0]
        if n % 2 == 1 or not A.any():
            assert lp[b] == -np.inf and sg[b] == 0.0
            assert st[b] == 5  # SKEW_SINGULAR
            assert np.isnan(grads[b]).all()
        else:
            assert_logpf((lp[b], sg[b]), oracle.logabspfaffian(A, quad=True), n)


def test_batch_eigvals_reference_order(skewgpu, oracle):
    import torch

    rng = np.random.default_rng(11)
    sizes = [int(x) for x in rng.choice(np.arange(2, 257, 2), 40)] + [3, 5, 17]
    mats = [skew_random(n, 2000 + k) for k, n in enumerate(sizes)]
    plan = skewgpu.BatchPlan(sizes)
    devs = [skewgpu.to_device(A) for A in mats]
    vals = [torch.zeros(n, dtype=torch.float64, device="cuda") for n in sizes]
    st = plan.eigvals(plan.pointer_array(devs), plan.pointer_array(vals))
    torch.cuda.synchronize()
    st = st.cpu().numpy()
    for b, A in enumerate(mats):
        assert st[b] in (0, 8)
        v = vals[b].cpu().numpy()
        vd, _ = oracle.eigvals(A)  # FP64 restatement: same algorithm, same order
        vq, _ = oracle.eigvals(A, quad=True)
        scale = np.abs(vq).max()
        np.testing.assert_allclose(np.sort(v), np.sort(vq), atol=RTOL * scale)
        np.testing.assert_allclose(v, vd, atol=1e-11 * scale)  # reference order
    plan.close()


def test_batch_eigvals_tridiagonal_cases(skewgpu, oracle):
    """issue #116 / #118 lists, as dense skew matrices through the batched path."""
    import torch

    lists = GOLD["issue116"]["ev_lists"] + GOLD["issue118"]["ev_lists"]
    mats = [tridiag_dense(ev) for ev in lists]
    sizes = [m.shape[0] for m in mats]
    plan = skewgpu.BatchPlan(sizes)
    devs = [skewgpu.to_device(A) for A in mats]
    vals = [torch.zeros(n, dtype=torch.float64, device="cuda") for n in sizes]
    st = plan.eigvals(plan.pointer_array(devs), plan.pointer_array(vals))
    torch.cuda.synchronize()
    for b, A in enumerate(mats):
        v = vals[b].cpu().numpy()
        ref = np.sort(np.linalg.eigvals(A).imag)
        np.testing.assert_allclose(np.sort(v), ref, atol=1e-12)
    plan.close()


def test_batch_eigvals_stagnation_fallback(skewgpu, oracle):
    """Matrix 274 (n = 200) of the seeded 4096-matrix workload makes the Wilkinson
    shifts stagnate in the reference algorithm (the oracle's FP64 restatement
    takes the fallback there too).  The batched eigvals must report
    SKEW_FALLBACK_USED and return the fallback's descending values."""
    import torch

    import bench

    sizes = bench.workload_sizes()[:275]
    buf, offs = bench.packed_inputs(sizes)
    pick = [274, 0, 1, 273]
    mats = [buf[offs[b]:offs[b] + sizes[b] ** 2].reshape(sizes[b], sizes[b], order="F") for b in pick]
    assert oracle.eigvals(mats[0])[1] != 0  # the oracle stagnates on it as well
    ns = [m.shape[0] for m in mats]
    plan = skewgpu.BatchPlan(ns)
    devs = [skewgpu.to_device(A) for A in mats]
    vals = [torch.zeros(n, dtype=torch.float64, device="cuda") for n in ns]
    st = plan.eigvals(plan.pointer_array(devs), plan.pointer_array(vals))
    torch.cuda.synchronize()
    st = st.cpu().numpy()
    assert st[0] == 8 and (st[1:] == 0).all()
    for b, A in enumerate(mats):
        v = vals[b].cpu().numpy()
        vq, _ = oracle.eigvals(A, quad=True)
        vd, _ = oracle.eigvals(A)
        scale = np.abs(vq).max()
        np.testing.assert_allclose(np.sort(v), np.sort(vq), atol=RTOL * scale)
        np.testing.assert_allclose(v, vd, atol=1e-11 * scale)  # same order as the reference
    plan.close()


def test_batch_schedule_invariance(skewgpu, oracle):
    """Every matrix of a batch is reduced, and its gradient formed, by one CTA with the
    same arithmetic whichever CTA takes it.  So the launch shape (global-memory size
    buckets merged into one launch or not, the two regions split at different shares
    of the work or not at all) must not change a single bit of log|Pf|, sign or
    gradient; the default is also checked against the oracle on a sample."""
    rng = np.random.default_rng(404)
    sizes = [int(2 * rng.integers(8, 129)) for _ in range(700)] + [256, 255, 97, 96, 2, 1, 0]
    mats = [skew_random(n, 5000 + k) / max(1.0, np.sqrt(n)) for k, n in enumerate(sizes)]
    ref = _batch(skewgpu, mats)
    for keys in ({"batch_merge_global": 0}, {"batch_split_pct": 0}, {"batch_split_pct": 30},
                 {"batch_merge_global": 0, "batch_split_pct": 0}):
        with skewgpu.tuned(**keys):
            out = _batch(skewgpu, mats)
        assert np.array_equal(out[0], ref[0], equal_nan=True), keys
        assert np.array_equal(out[1], ref[1], equal_nan=True), keys
        assert np.array_equal(out[2], ref[2]), keys
        for g, h in zip(out[3], ref[3]):
            assert np.array_equal(g, h, equal_nan=True), keys
    for k in list(range(0, 700, 97)) + [700, 701]:
        lp, sg = oracle.logabspfaffian(mats[k])
        assert ref[1][k] == sg
        if np.isfinite(lp):
            assert abs(ref[0][k] - lp) <= 1e-11 * max(1.0, abs(lp))
        else:
            assert ref[0][k] == lp
