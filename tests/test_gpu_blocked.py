"""GPU parity of the multi-CTA blocked reduction used for single large matrices.

Moderate sizes are checked against the oracle (binary128 for n <= 384, the FP64
restatement above).  Large sizes use size-independent properties: orthogonal
similarity keeps the Frobenius norm (|T|_F = |A|_F), and log|Pf(A)| equals
1/2 log|det A| (LU on the host).  Tolerances as in test_gpu_parity.py.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-11


def skew_random(n, seed):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n))
    return (B - B.T) / 2


def tridiag_dense(ev):
    n = len(ev) + 1
    T = np.zeros((n, n))
    T[np.arange(1, n), np.arange(n - 1)] = ev
    T[np.arange(n - 1), np.arange(1, n)] = -np.asarray(ev)
    return T


@pytest.mark.parametrize("n", [192, 193, 200, 255, 256, 300, 384])
def test_blocked_hessenberg_vs_quad(skewgpu, oracle, n):
    A = skew_random(n, 700 + n)
    H = skewgpu.hessenberg(A)
    ev = H.ev.cpu().numpy()
    tau = H.tau.cpu().numpy()
    _, tq, evq = oracle.hessenberg(A, quad=True)
    scale = np.abs(evq).max()
    np.testing.assert_allclose(ev, evq, atol=1e-12 * scale)  # same reflector convention, entrywise
    assert np.array_equal(tau != 0, tq != 0)
    Q = oracle.formq(skewgpu.from_device(H.factors), tau)
    np.testing.assert_allclose(Q @ tridiag_dense(ev) @ Q.T, A, atol=1e-12 * np.abs(A).max() * np.sqrt(n))
    np.testing.assert_allclose(Q.T @ Q, np.eye(n), atol=1e-13 * np.sqrt(n))


@pytest.mark.parametrize("n", [192, 256, 512, 1000, 1024])
def test_blocked_logabspf(skewgpu, oracle, n):
    A = skew_random(n, 800 + n) / np.sqrt(n)
    ref = oracle.logabspfaffian(A, quad=(n <= 384))
    lp, sg = skewgpu.logabspfaffian_(skewgpu.SkewHermitian(A))
    assert sg == ref[1]
    assert abs(lp - ref[0]) <= RTOL * max(1.0, abs(ref[0]))


@pytest.mark.parametrize("n", [200, 512, 1024])
def test_blocked_eigvals(skewgpu, oracle, n):
    A = skew_random(n, 900 + n)
    vd, _ = oracle.eigvals(A, quad=(n <= 256))
    vals = skewgpu.eigvals(A).imag
    np.testing.assert_allclose(np.sort(vals), np.sort(vd), atol=RTOL * np.abs(vd).max())


def test_blocked_large_properties(skewgpu):
    n = 4096
    A = skew_random(n, 4096) / np.sqrt(n)
    H = skewgpu.hessenberg(A)
    ev = H.ev.cpu().numpy()
    fro_T = np.sqrt(2.0 * np.sum(ev.astype(np.float64) ** 2))
    fro_A = np.linalg.norm(A)
    assert abs(fro_T - fro_A) <= 1e-13 * fro_A * np.sqrt(n)
    lp, sg = skewgpu.logabspfaffian_(skewgpu.SkewHermitian(A))
    s, ld = np.linalg.slogdet(A)
    assert s > 0
    assert abs(lp - 0.5 * ld) <= 1e-11 * abs(ld) + 1e-9


def test_blocked_determinism(skewgpu):
    A = skew_random(640, 3)
    r1 = skewgpu.logabspfaffian(A)
    r2 = skewgpu.logabspfaffian(A)
    assert r1 == r2
    h1 = skewgpu.hessenberg(A).ev.cpu().numpy()
    h2 = skewgpu.hessenberg(A).ev.cpu().numpy()
    assert np.array_equal(h1, h2)


@pytest.mark.parametrize("n", [16, 17, 31, 64, 97, 160, 255, 320, 511, 513, 640])
def test_cluster_reduction_vs_oracle(skewgpu, oracle, n):
    """The 16-CTA cluster reduction (the matrix in distributed shared memory), forced
    down to n = 16 through the tuning key blocked_min_n: ev entrywise against the
    oracle (binary128 up to n = 384, its FP64 restatement above), the same reflector
    pattern, Q T Q^T = A and log|Pf|; and the same values as the grid-wide reduction
    (cluster_max_n = 0) to rounding."""
    A = skew_random(n, 1300 + n) / np.sqrt(n)
    with skewgpu.tuned(blocked_min_n=16):
        H = skewgpu.hessenberg(A)
        lp, sg = skewgpu.logabspfaffian(A)
        with skewgpu.tuned(cluster_max_n=0):
            H2 = skewgpu.hessenberg(A)
    ev = H.ev.cpu().numpy()
    tau = H.tau.cpu().numpy()
    _, tq, evq = oracle.hessenberg(A, quad=(n <= 384))
    scale = np.abs(evq).max()
    np.testing.assert_allclose(ev, evq, atol=RTOL * scale)
    assert np.array_equal(tau != 0, tq != 0)
    np.testing.assert_allclose(ev, H2.ev.cpu().numpy(), atol=1e-13 * scale)
    Q = oracle.formq(skewgpu.from_device(H.factors), tau)
    np.testing.assert_allclose(Q @ tridiag_dense(ev) @ Q.T, A, atol=1e-12 * np.abs(A).max() * np.sqrt(n))
    rl, rs = oracle.logabspfaffian(A, quad=(n <= 384))
    assert sg == rs
    if np.isfinite(rl):
        assert abs(lp - rl) <= RTOL * max(1.0, abs(rl))
    else:
        assert lp == rl


_PANEL_REF = {}


def _panel_ref(oracle, n):
    """Oracle reduction of the panel-width test matrix (binary128 up to n = 384)."""
    if n not in _PANEL_REF:
        A = skew_random(n, 1700 + n) / np.sqrt(n)
        _, tq, evq = oracle.hessenberg(A, quad=(n <= 384))
        _PANEL_REF[n] = (A, tq, evq, oracle.logabspfaffian(A, quad=(n <= 384)))
    return _PANEL_REF[n]


@pytest.mark.parametrize("n,path,nb", [
    (300, "persistent", 8), (300, "persistent", 24), (300, "persistent", 64), (300, "persistent", 72),
    (300, "persistent", 128), (300, "multilaunch", 8), (300, "multilaunch", 40), (300, "multilaunch", 128),
    (1000, "persistent", 40), (1000, "persistent", 96), (1000, "persistent", 128)])
def test_blocked_panel_width_vs_oracle(skewgpu, oracle, n, path, nb):
    """The panel width of the blocked reduction (the tuning key persist_nb, the role of
    setnb in hessenberg.jl:133-142) changes the order of the arithmetic, not the
    result: for widths 8 .. 128 on the persistent kernel (the 64- and 128-entry
    instantiations) and on the multi-launch path (which caps the width at 64), ev
    entrywise against the oracle, the same reflector pattern, Q T Q^T = A and
    log|Pf|.  The cluster reduction is switched off so these sizes reach the grid-wide
    kernels."""
    A, tq, evq, (rl, rs) = _panel_ref(oracle, n)
    keys = dict(blocked_min_n=16, cluster_max_n=0, persist_nb=nb,
                blocked_persistent=1 if path == "persistent" else 0)
    with skewgpu.tuned(**keys):
        H = skewgpu.hessenberg(A)
        lp, sg = skewgpu.logabspfaffian(A)
    ev = H.ev.cpu().numpy()
    tau = H.tau.cpu().numpy()
    scale = np.abs(evq).max()
    np.testing.assert_allclose(ev, evq, atol=RTOL * scale)
    assert np.array_equal(tau != 0, tq != 0)
    Q = oracle.formq(skewgpu.from_device(H.factors), tau)
    np.testing.assert_allclose(Q @ tridiag_dense(ev) @ Q.T, A, atol=1e-12 * np.abs(A).max() * np.sqrt(n))
    assert sg == rs
    assert abs(lp - rl) <= RTOL * max(1.0, abs(rl))
