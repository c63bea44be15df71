"""GPU parity of eigen / exp / cis / exp adjoint (skew_eigen.cu) against the oracle.

Tolerances: eigenvalues 1e-11 normwise against binary128; exp and cis 1e-11
normwise against the binary128 restatement of skewexp!/skewcis!; the exp
adjoint 1e-8 normwise against the binary128 block-matrix exp (independent of
eigen).  Eigenvectors are compared through reconstruction, orthonormality and
against the FP64 restatement's vectors (same algorithm, same deflation order).
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_known_answers.json")))["cases"]


def skew_random(n, seed, scale=None):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n)) * (1 / np.sqrt(n) if scale is None else scale)
    return (B - B.T) / 2


def tridiag_dense(ev):
    n = len(ev) + 1
    T = np.zeros((n, n))
    T[np.arange(1, n), np.arange(n - 1)] = ev
    T[np.arange(n - 1), np.arange(1, n)] = -np.asarray(ev)
    return T


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 8, 17, 32, 64, 100, 129, 256])
def test_eigen_vs_oracle(skewgpu, oracle, n):
    A = skew_random(n, 3000 + n)
    vals, V = skewgpu.eigen(A)
    vd, Vrd, Vid, std = oracle.eigen(A)
    vq, _, _, _ = oracle.eigen(A, quad=(n <= 129))
    scale = max(np.abs(vq).max(), 1e-300)
    np.testing.assert_allclose(vals.imag, vd, atol=1e-11 * scale)  # reference order
    np.testing.assert_allclose(np.sort(vals.imag), np.sort(vq), atol=1e-11 * scale)
    np.testing.assert_allclose(V @ np.diag(vals) @ V.conj().T, A, atol=1e-12 * max(1, np.abs(A).max()) * np.sqrt(n))
    np.testing.assert_allclose(V.conj().T @ V, np.eye(n), atol=1e-12 * np.sqrt(n))
    Vd = Vrd + 1j * Vid
    np.testing.assert_allclose(V, Vd, atol=1e-8)


@pytest.mark.parametrize("key", ["issue130_10x10", "issue130_66x66"])
def test_eigen_reference_hard_cases(skewgpu, key):
    A = np.array(GOLD[key]["A"])
    vals, V = skewgpu.eigen(A)
    np.testing.assert_allclose(V @ np.diag(vals) @ V.conj().T, A, atol=1e-11 * np.abs(A).max())
    np.testing.assert_allclose(V.conj().T @ V, np.eye(A.shape[0]), atol=1e-11)


@pytest.mark.parametrize("k", [0, 1])
def test_eigen_issue118(skewgpu, k):
    T = tridiag_dense(GOLD["issue118"]["ev_lists"][k])
    vals, V = skewgpu.eigen(T)
    np.testing.assert_allclose(V @ np.diag(vals) @ V.conj().T, T, atol=2e-11)


@pytest.mark.parametrize("n", [1, 2, 3, 6, 10, 31, 64, 128, 200])
def test_exp_cis_vs_oracle(skewgpu, oracle, n):
    A = skew_random(n, 4000 + n, scale=1.0)
    E = skewgpu.exp(A)
    Eq = oracle.expm(A, quad=(n <= 128))
    np.testing.assert_allclose(E, Eq, atol=1e-11 * max(1.0, np.abs(Eq).max()) * np.sqrt(n))
    np.testing.assert_allclose(E @ E.T, np.eye(n), atol=1e-12 * np.sqrt(n))
    C = skewgpu.cis(A)
    Cq = oracle.cis(A, quad=(n <= 128))
    np.testing.assert_allclose(C, Cq, atol=1e-11 * np.abs(Cq).max() * np.sqrt(n))


@pytest.mark.parametrize("n", [2, 4, 7, 16, 48])
def test_exp_vjp_vs_oracle(skewgpu, oracle, n):
    rng = np.random.default_rng(n)
    A = skew_random(n, 5000 + n, scale=1.0)
    Cb = rng.standard_normal((n, n))
    _, pb = skewgpu.exp_rrule(A)
    G = pb(Cb)
    Gq = oracle.exp_vjp(A, Cb)
    assert np.abs(G - Gq).max() <= 1e-8 * np.abs(Gq).max()
    # central differences on a few entries
    h = 1e-6
    for i, j in [(0, 1), (n - 1, 0)]:
        Ap, Am = A.copy(), A.copy()
        Ap[i, j] += h
        Am[i, j] -= h
        fd = (np.sum(Cb * oracle.expm_dense(Ap)) - np.sum(Cb * oracle.expm_dense(Am))) / (2 * h)
        assert fd == pytest.approx(G[i, j], rel=1e-6, abs=1e-8)


def test_batch_eigen_exp_vjp_mixed(skewgpu, oracle):
    import torch

    sizes = [32, 64, 96, 128, 160, 3, 2, 33]
    rng = np.random.default_rng(77)
    mats = []
    for k, n in enumerate(sizes):
        A = skew_random(n, 6000 + k, scale=1.0)
        # spectral radius ~ U(0.5, 8) as in the exp-adjoint workload
        rho = np.abs(np.linalg.eigvals(A)).max() if n > 1 else 1.0
        mats.append(A * (rng.uniform(0.5, 8.0) / max(rho, 1e-12)))
    cots = [rng.standard_normal((n, n)) for n in sizes]
    plan = skewgpu.BatchPlan(sizes)
    devs = [skewgpu.to_device(A) for A in mats]
    Eo = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in sizes]
    st = plan.exp(plan.pointer_array(devs), plan.pointer_array(Eo))
    torch.cuda.synchronize()
    assert (st.cpu().numpy() >= 0).all()
    for b, A in enumerate(mats):
        Eq = oracle.expm(A)
        np.testing.assert_allclose(skewgpu.from_device(Eo[b]), Eq, atol=1e-11 * np.sqrt(A.shape[0]) * max(1, np.abs(Eq).max()))
    cd = [skewgpu.to_device(C) for C in cots]
    Go = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in sizes]
    plan.exp_vjp(plan.pointer_array(devs), plan.pointer_array(cd), plan.pointer_array(Go))
    torch.cuda.synchronize()
    for b, A in enumerate(mats):
        Gq = oracle.exp_vjp(A, cots[b])
        G = skewgpu.from_device(Go[b])
        assert np.abs(G - Gq).max() <= 1e-8 * np.abs(Gq).max(), f"n={A.shape[0]}"
    vals = [torch.zeros(n, dtype=torch.float64, device="cuda") for n in sizes]
    Vr = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in sizes]
    Vi = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in sizes]
    plan.eigen(plan.pointer_array(devs), plan.pointer_array(vals), plan.pointer_array(Vr), plan.pointer_array(Vi))
    torch.cuda.synchronize()
    for b, A in enumerate(mats):
        V = skewgpu.from_device(Vr[b]) + 1j * skewgpu.from_device(Vi[b])
        lam = 1j * vals[b].cpu().numpy()
        np.testing.assert_allclose(V @ np.diag(lam) @ V.conj().T, A, atol=1e-11 * max(1, np.abs(A).max()) * np.sqrt(A.shape[0]))
    plan.close()


def test_eigen_stagnation_fallback(skewgpu, oracle):
    """Matrix 274 (n = 200) of the seeded 4096-matrix workload makes the shifts of
    skewtrieigen_divided! stagnate (the oracle takes the fallback too); the
    batched eigen must take the reference's fallback (skewtrieigen_backup!:
    values descending, fallback eigenvector layout) and still reconstruct A."""
    import torch

    import bench

    sizes = bench.workload_sizes()[:275]
    buf, offs = bench.packed_inputs(sizes)
    A = buf[offs[274]:offs[274] + 200 * 200].reshape(200, 200, order="F")
    assert oracle.eigen(A)[3] != 0
    mats = [A, skew_random(31, 3), skew_random(200, 4)]
    ns = [m.shape[0] for m in mats]
    plan = skewgpu.BatchPlan(ns)
    devs = [skewgpu.to_device(M) for M in mats]
    vals = [torch.zeros(n, dtype=torch.float64, device="cuda") for n in ns]
    Vr = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in ns]
    Vi = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in ns]
    st = plan.eigen(plan.pointer_array(devs), plan.pointer_array(vals), plan.pointer_array(Vr),
                    plan.pointer_array(Vi))
    torch.cuda.synchronize()
    st = st.cpu().numpy()
    assert st[0] == 8 and st[1] == 0 and st[2] == 0
    for b, M in enumerate(mats):
        v = vals[b].cpu().numpy()
        V = skewgpu.from_device(Vr[b]) + 1j * skewgpu.from_device(Vi[b])
        rho = np.abs(v).max()
        if b == 0:
            assert np.all(np.diff(v) <= 0.0)  # the fallback's order
            vq, _ = oracle.eigvals(M, quad=True)
            np.testing.assert_allclose(v, np.sort(vq)[::-1], atol=1e-11 * rho)
        np.testing.assert_allclose(V.conj().T @ V, np.eye(ns[b]), atol=1e-11)
        np.testing.assert_allclose(V @ np.diag(1j * v) @ V.conj().T, M, atol=1e-11 * rho)
    plan.close()


def test_batch_exp_vjp_twisted_path(skewgpu, oracle):
    """Above n = 64 the batched function paths take bisection and twisted vectors
    instead of the QR chain (the order of the eigenpairs does not matter there).
    Odd and even sizes, repeated sizes (groups of several problems): exp against the
    oracle, the adjoint against the oracle's binary128 block exponential for one
    matrix and against the QR-chain path (the tuning key func_chain_nmax) for all."""
    import torch

    sizes = [161, 200, 200, 257, 301, 64]
    rng = np.random.default_rng(91)
    mats = []
    for k, n in enumerate(sizes):
        A = skew_random(n, 7000 + k, scale=1.0)
        rho = np.abs(np.linalg.eigvals(A)).max()
        mats.append(A * (rng.uniform(0.5, 8.0) / rho))
    cots = [rng.standard_normal((n, n)) for n in sizes]

    def run():
        plan = skewgpu.BatchPlan(sizes)
        devs = [skewgpu.to_device(A) for A in mats]
        cd = [skewgpu.to_device(C) for C in cots]
        Eo = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in sizes]
        Go = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in sizes]
        st = plan.exp(plan.pointer_array(devs), plan.pointer_array(Eo))
        st2 = plan.exp_vjp(plan.pointer_array(devs), plan.pointer_array(cd), plan.pointer_array(Go))
        torch.cuda.synchronize()
        assert (st.cpu().numpy() == 0).all() and (st2.cpu().numpy() == 0).all()
        out = [skewgpu.from_device(E) for E in Eo], [skewgpu.from_device(G) for G in Go]
        plan.close()
        return out

    E1, G1 = run()
    for b, A in enumerate(mats):
        Eq = oracle.expm(A)
        np.testing.assert_allclose(E1[b], Eq, atol=1e-11 * np.sqrt(A.shape[0]) * max(1, np.abs(Eq).max()))
    Gq = oracle.exp_vjp(mats[0], cots[0])
    assert np.abs(G1[0] - Gq).max() <= 1e-8 * np.abs(Gq).max()
    with skewgpu.tuned(func_chain_nmax=100000):
        E2, G2 = run()
    for b in range(len(sizes)):
        np.testing.assert_allclose(E1[b], E2[b], atol=1e-11 * np.sqrt(sizes[b]) * max(1, np.abs(E2[b]).max()))
        assert np.abs(G1[b] - G2[b]).max() <= 1e-9 * np.abs(G2[b]).max(), f"n={sizes[b]}"


def test_functions_several_odd_blocks(skewgpu):
    """exp and the exp adjoint of singular block-diagonal inputs whose tridiagonal
    splits exactly into several odd blocks (one zero eigenvalue each), through the
    batched function path above n = 64 (bisection and twisted vectors) and the
    single-matrix call, against scipy's expm and expm_frechet."""
    import scipy.linalg as sl
    import torch

    def blockdiag(sizes, seed):
        n = sum(sizes)
        A = np.zeros((n, n))
        o = 0
        for k, m in enumerate(sizes):
            A[o:o + m, o:o + m] = skew_random(m, seed + k, scale=2.0 / np.sqrt(m))
            o += m
        return A

    mats = [blockdiag((67, 67, 66), 10), blockdiag((101, 99, 101), 20), blockdiag((33, 31, 35, 29, 2), 30)]
    sizes = [m.shape[0] for m in mats]
    rng = np.random.default_rng(8)
    cots = [rng.standard_normal((n, n)) for n in sizes]
    plan = skewgpu.BatchPlan(sizes)
    devs = [skewgpu.to_device(A) for A in mats]
    cd = [skewgpu.to_device(C) for C in cots]
    Eo = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in sizes]
    Go = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in sizes]
    st = plan.exp(plan.pointer_array(devs), plan.pointer_array(Eo)).cpu().numpy()
    st2 = plan.exp_vjp(plan.pointer_array(devs), plan.pointer_array(cd), plan.pointer_array(Go)).cpu().numpy()
    torch.cuda.synchronize()
    plan.close()
    assert (st == 0).all() and (st2 == 0).all()
    for b, A in enumerate(mats):
        n = sizes[b]
        np.testing.assert_allclose(skewgpu.from_device(Eo[b]), sl.expm(A), atol=1e-11 * np.sqrt(n))
        _, Lf = sl.expm_frechet(A.T, cots[b])
        assert np.abs(skewgpu.from_device(Go[b]) - Lf).max() <= 1e-8 * np.abs(Lf).max(), n
        np.testing.assert_allclose(skewgpu.exp(A), sl.expm(A), atol=1e-11 * np.sqrt(n))


def test_function_forms_agree(skewgpu, oracle):
    """exp, cis and the exp adjoint in the real Schur basis (the default) and in the
    complex form Re(V f V^H) (tuning key func_real_schur = 0, the form a matrix takes
    when its spectrum does not split into exact +- pairs): both against the oracle,
    on the QR-chain sizes and the bisection sizes, odd and even."""
    import torch

    sizes = [5, 16, 33, 64, 97, 130]
    rng = np.random.default_rng(31)
    mats, cots = [], []
    for k, n in enumerate(sizes):
        A = skew_random(n, 9100 + k, scale=1.0)
        rho = np.abs(np.linalg.eigvals(A)).max()
        mats.append(A * (rng.uniform(0.5, 8.0) / rho))
        cots.append(rng.standard_normal((n, n)))

    def run():
        plan = skewgpu.BatchPlan(sizes)
        devs = [skewgpu.to_device(A) for A in mats]
        cd = [skewgpu.to_device(C) for C in cots]
        Eo = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in sizes]
        Co = [torch.zeros((n, n), dtype=torch.complex128, device="cuda") for n in sizes]
        Go = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in sizes]
        st = [plan.exp(plan.pointer_array(devs), plan.pointer_array(Eo)),
              plan.cis(plan.pointer_array(devs), plan.pointer_array(Co)),
              plan.exp_vjp(plan.pointer_array(devs), plan.pointer_array(cd), plan.pointer_array(Go))]
        torch.cuda.synchronize()
        assert all((s.cpu().numpy() == 0).all() for s in st)
        out = ([skewgpu.from_device(E) for E in Eo], [skewgpu.from_device_complex(C) for C in Co],
               [skewgpu.from_device(G) for G in Go])
        plan.close()
        return out

    forms = [run()]
    with skewgpu.tuned(func_real_schur=0):
        forms.append(run())
    for E, C, G in forms:
        for b, A in enumerate(mats):
            n = sizes[b]
            Eq = oracle.expm(A)
            np.testing.assert_allclose(E[b], Eq, atol=1e-11 * np.sqrt(n) * max(1, np.abs(Eq).max()))
            Cq = oracle.cis(A)
            np.testing.assert_allclose(C[b], Cq, atol=1e-11 * np.sqrt(n) * max(1, np.abs(Cq).max()))
            Gq = oracle.exp_vjp(A, cots[b])
            assert np.abs(G[b] - Gq).max() <= 1e-8 * np.abs(Gq).max(), n
