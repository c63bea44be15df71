"""Pins the oracle (CPU restatement) against SkewLinearAlgebra.jl's own known
answers (tests/golden/reference_known_answers.json, extracted from
test/runtests.jl) and cross-checks the FP64 restatement against the binary128
run and against independent dense methods.  CPU only."""
import json
import os

import numpy as np
import pytest

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_known_answers.json")))["cases"]


def skew_random(n, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n)) * scale
    return (B - B.T) / 2


def tridiag_dense(ev):
    n = len(ev) + 1
    T = np.zeros((n, n))
    T[np.arange(1, n), np.arange(n - 1)] = ev
    T[np.arange(n - 1), np.arange(1, n)] = -np.asarray(ev)
    return T


# --- README testset (runtests.jl:9-30) -------------------------------------
def test_readme_hessenberg(oracle):
    A = np.array(GOLD["readme_A"]["A"])
    for quad in (False, True):
        F, tau, ev = oracle.hessenberg(A, quad=quad)
        np.testing.assert_allclose(ev, GOLD["readme_hessenberg_v"]["v"], rtol=1e-14)
        Q = oracle.formq(F, tau)
        np.testing.assert_allclose(Q, np.array(GOLD["readme_Q"]["Q"]), atol=1e-15)
        np.testing.assert_allclose(Q @ tridiag_dense(ev) @ Q.T, A, atol=1e-13)


def test_readme_eigvals_and_pfaffian(oracle):
    A = np.array(GOLD["readme_A"]["A"])
    l1, l2 = GOLD["readme_eigs"]["ilambda"]
    for quad in (False, True):
        vals, st = oracle.eigvals(A, quad=quad)
        assert st == 0
        np.testing.assert_allclose(np.sort(vals), np.sort([l1, l2, -l2, -l1]), rtol=1e-14)
        lp, sg = oracle.logabspfaffian(A, quad=quad)
        assert sg == -1.0  # Pf = -9 (docs/src/pfaffian.md:56-57)
        assert abs(lp - np.log(9.0)) < 1e-14
    assert oracle.exact_pfaffian(A.astype(int).tolist()) == -9
    assert (-9) ** 2 == GOLD["readme_det"]["det"]


def test_readme_inverse_via_gradient(oracle):
    A = np.array(GOLD["readme_A"]["A"])
    G = oracle.logabspfaffian_grad(A)  # 1/2 A^{-T} = -1/2 A^{-1}
    np.testing.assert_allclose(-2 * G, np.array(GOLD["readme_inv_times9"]["Ainv9"]) / 9, atol=1e-15)


# --- pfaffian testset (runtests.jl:388-434) --------------------------------
def test_issue49(oracle):
    A = GOLD["issue49"]["A"]
    assert oracle.exact_pfaffian([[int(x) for x in r] for r in A]) == GOLD["issue49"]["pfaffian"]
    for quad in (False, True):
        lp, sg = oracle.logabspfaffian(np.array(A), quad=quad)
        assert sg == -1.0
        assert abs(lp - np.log(119000.0)) < 1e-13


def test_issue121(oracle):
    A = np.array(GOLD["issue121"]["A"])
    lp, sg = oracle.logabspfaffian(A)
    assert sg * np.exp(lp) == pytest.approx(GOLD["issue121"]["pfaffian"], rel=1e-15)


def test_4x4_formula(oracle):
    rng = np.random.default_rng(314159)
    for _ in range(10):
        a, b, c, d, e, f = (int(x) for x in rng.integers(-10, 11, 6))
        A = [[0, a, b, c], [-a, 0, d, e], [-b, -d, 0, f], [-c, -e, -f, 0]]
        ex = oracle.exact_pfaffian(A)
        assert ex == c * d - b * e + a * f
        lp, sg = oracle.logabspfaffian(np.array(A, float))
        assert sg * np.exp(lp) == pytest.approx(float(ex), rel=1e-12, abs=1e-12)


@pytest.mark.parametrize("n", [1, 2, 3, 10, 11])
def test_integer_pfaffian_exact(oracle, n):
    rng = np.random.default_rng(n)
    R = rng.integers(-10, 11, (n, n)) * 2
    A = (R - R.T) // 2
    ex = oracle.exact_pfaffian(A.tolist())
    lp, sg = oracle.logabspfaffian(A.astype(float))
    val = 0.0 if sg == 0 else sg * np.exp(lp)
    assert val == pytest.approx(float(ex), rel=1e-11, abs=1e-9)
    if n % 2 == 0:
        assert float(ex) ** 2 == pytest.approx(np.linalg.det(A.astype(float)), rel=1e-9)


# --- issue #116 / #118 / #130 (runtests.jl:488-529) ------------------------
@pytest.mark.parametrize("k", range(14))
def test_issue116_tridiagonal(oracle, k):
    # runtests.jl:490-507 checks eigvals (skewtrieigvals!) against the dense solver
    ev = GOLD["issue116"]["ev_lists"][k]
    T = tridiag_dense(ev)
    vals, st = oracle.skewtrieigvals(ev)
    assert st >= 0
    ref = np.sort(np.linalg.eigvals(T).imag)
    np.testing.assert_allclose(np.sort(vals), ref, atol=1e-13)
    vq, _ = oracle.skewtrieigvals(ev, quad=True)
    np.testing.assert_allclose(np.sort(vq), ref, atol=1e-13)


def test_divided_reconstruction_generic(oracle):
    for ev in ([1.0, 2.0, 3.0, 2.0, 1.0], [0.3, 1.7, -0.2, 2.5, 0.9, 1.1]):
        T = tridiag_dense(ev)
        v2, Qr, Qi, st = oracle.skewtrieigen(ev)
        assert st >= 0
        V = Qr + 1j * Qi
        np.testing.assert_allclose(V @ np.diag(1j * v2) @ V.conj().T, T, atol=1e-12)


def test_divided_mem_quirk(oracle):
    """skewtrieigen_divided! (skeweigen.jl:355-358) deflates when |ev[n-1] - mem| < tol
    with mem initialised to 1 (:343), so an exact ev[n-1] == 1 after the first sweep
    deflates a wrong pair.  The restatement reproduces the reference: for
    ev = [0, 1, 1] the values come out {0, 0, +-1} where the true spectrum (and
    skewtrieigvals!) gives {0, 0, +-sqrt(2)}."""
    v2, Qr, Qi, st = oracle.skewtrieigen([0.0, 1.0, 1.0])
    np.testing.assert_allclose(np.sort(v2), [-1.0, 0.0, 0.0, 1.0], atol=1e-15)
    vals, _ = oracle.skewtrieigvals([0.0, 1.0, 1.0])
    np.testing.assert_allclose(np.sort(vals), [-np.sqrt(2), 0.0, 0.0, np.sqrt(2)], atol=1e-15)


@pytest.mark.parametrize("key", ["issue130_10x10", "issue130_66x66"])
def test_issue130_reconstruction(oracle, key):
    A = np.array(GOLD[key]["A"])
    for quad in (False, True):
        vals, Vr, Vi, st = oracle.eigen(A, quad=quad)
        assert st >= 0
        V = Vr + 1j * Vi
        np.testing.assert_allclose(V @ np.diag(1j * vals) @ V.conj().T, A, atol=1e-11 * np.abs(A).max())


@pytest.mark.parametrize("k", [0, 1])
def test_issue118(oracle, k):
    # The reference checks these with the default rtol sqrt(eps) (runtests.jl:521-528).
    # For [2, 1e-11, 2, 1e-11, 2] its absolute stagnation deflation
    # (|ev[n-1] - mem| < 10 eps, skeweigen.jl:355) drops the 1e-11 couplings, so
    # the reconstruction is good to ~1e-11 absolute, not to rounding.
    ev = GOLD["issue118"]["ev_lists"][k]
    T = tridiag_dense(ev)
    v2, Qr, Qi, st = oracle.skewtrieigen(ev)
    V = Qr + 1j * Qi
    np.testing.assert_allclose(V @ np.diag(1j * v2) @ V.conj().T, T, atol=2e-11)
    vals, Vr, Vi, st = oracle.eigen(T)
    V = Vr + 1j * Vi
    np.testing.assert_allclose(V @ np.diag(1j * vals) @ V.conj().T, T, atol=2e-11)


# --- FP64 restatement vs binary128 and independent methods ------------------
@pytest.mark.parametrize("n", [2, 5, 8, 13, 32, 61, 100, 128])
def test_double_vs_quad(oracle, n):
    A = skew_random(n, 1000 + n, 1 / np.sqrt(n))
    lpd, sgd = oracle.logabspfaffian(A)
    lpq, sgq = oracle.logabspfaffian(A, quad=True)
    assert sgd == sgq
    if n % 2 == 0:
        assert abs(lpd - lpq) <= 1e-12 * max(1.0, abs(lpq))
    vd, _ = oracle.eigvals(A)
    vq, _ = oracle.eigvals(A, quad=True)
    scale = np.abs(vq).max()
    np.testing.assert_allclose(np.sort(vd), np.sort(vq), atol=1e-13 * scale)
    # quad hessenberg reproduces A
    F, tau, ev = oracle.hessenberg(A, quad=True)
    Q = oracle.formq(F, tau)
    np.testing.assert_allclose(Q @ tridiag_dense(ev) @ Q.T, A, atol=1e-13)


def test_eigvals_vs_numpy(oracle):
    A = skew_random(40, 7)
    vals, st = oracle.eigvals(A)
    np.testing.assert_allclose(np.sort(vals), np.sort(np.linalg.eigvals(A).imag), atol=1e-12)


def test_gradient_fd(oracle):
    n = 10
    A = skew_random(n, 3) + 0.5 * np.kron(np.eye(n // 2), np.array([[0, 1], [-1, 0]]))
    G = oracle.logabspfaffian_grad(A)
    np.testing.assert_allclose(G, 0.5 * np.linalg.inv(A).T, atol=1e-13)
    h = 1e-6
    rng = np.random.default_rng(0)
    for _ in range(8):
        i, j = rng.choice(n, 2, replace=False)
        Ap, Am = A.copy(), A.copy()
        Ap[i, j] += h
        Ap[j, i] -= h
        Am[i, j] -= h
        Am[j, i] += h
        fd = (oracle.logabspfaffian(Ap)[0] - oracle.logabspfaffian(Am)[0]) / (2 * h)
        assert fd == pytest.approx(G[i, j] - G[j, i], rel=1e-6, abs=1e-8)


def test_exp_and_cis(oracle):
    for n in (1, 2, 7, 10, 31):
        A = skew_random(n, 50 + n)
        E = oracle.expm(A)
        np.testing.assert_allclose(E, oracle.expm_dense(A), atol=1e-13)
        np.testing.assert_allclose(E @ E.T, np.eye(n), atol=1e-13)
        Eq = oracle.expm(A, quad=True)
        np.testing.assert_allclose(E, Eq, atol=1e-13)
        C = oracle.cis(A)
        w, V = np.linalg.eigh(1j * A)  # cis(A) = exp(iA), iA Hermitian
        np.testing.assert_allclose(C, (V * np.exp(w)) @ V.conj().T, atol=1e-12 * np.exp(np.abs(w).max()))


def test_exp_vjp_fd(oracle):
    n = 6
    A = skew_random(n, 11)
    C = np.random.default_rng(2).standard_normal((n, n))
    G = oracle.exp_vjp(A, C)
    h = 1e-6
    for i, j in [(0, 1), (2, 5), (4, 3)]:
        Ap, Am = A.copy(), A.copy()
        Ap[i, j] += h
        Am[i, j] -= h
        fd = (np.sum(C * oracle.expm_dense(Ap)) - np.sum(C * oracle.expm_dense(Am))) / (2 * h)
        assert fd == pytest.approx(G[i, j], rel=1e-7, abs=1e-9)


def test_odd_and_tiny_sizes(oracle):
    for n in (1, 3, 5):
        lp, sg = oracle.logabspfaffian(skew_random(n, n))
        assert lp == -np.inf and sg == 0.0
    A = np.array([[0.0, 3.0], [-3.0, 0.0]])
    assert oracle.logabspfaffian(A) == (pytest.approx(np.log(3.0)), 1.0)


def test_complex_hessenberg(oracle):
    n = 9
    rng = np.random.default_rng(5)
    Cm = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A = (Cm - Cm.conj().T) / 2
    for quad in (False, True):
        F, tau, ev, dvim = oracle.hessenberg_complex(A, quad=quad)
        T = np.diag(1j * dvim) + np.diag(ev.astype(complex), -1) - np.diag(ev.astype(complex), 1)
        # eigenvalues of T equal those of A (unitary similarity)
        np.testing.assert_allclose(np.sort(np.linalg.eigvals(T).imag), np.sort(np.linalg.eigvals(A).imag), atol=1e-12)


# --- complex skew-symmetric Pfaffian (pfaffian.jl:98-137, :193-233) ---------
def complex_int_skew(n, seed):
    """The reference's recipe (runtests.jl:408-409): R with entries in
    (-10:10) + i(-10:10), A = (R - transpose(R)) / 2."""
    rng = np.random.default_rng(seed)
    R = rng.integers(-10, 11, (n, n)) + 1j * rng.integers(-10, 11, (n, n))
    return (R - R.T) / 2


@pytest.mark.parametrize("n", [1, 2, 3, 10, 20])
def test_complex_pfaffian_exact(oracle, n):
    """runtests.jl:406-420: Pf(A) ~ exactpfaffian(Complex{Rational{BigInt}}), Pf^2 ~ det(A)
    (atol sqrt(eps) max(1, |det A|)), Pf ~ sign * exp(logpf); the FP64 restatement is
    held to 1e-13 here, binary128 is exact to FP64 rounding."""
    for seed in range(3):
        A = complex_int_skew(n, 1000 * n + seed)
        exact = complex(oracle.exact_pfaffian_complex(A.tolist()))
        for quad, tol in ((False, 1e-13), (True, 1e-16)):
            lp, ph, pf = oracle.pfaffian_complex(A, quad=quad)
            assert abs(pf - exact) <= tol * max(1.0, abs(exact))
            if exact != 0:
                assert abs(ph * np.exp(lp) - exact) <= 1e-13 * abs(exact)
            else:
                assert lp == -np.inf and ph == 0
        d = np.linalg.det(A)
        assert abs(exact**2 - d) <= np.sqrt(np.finfo(float).eps) * max(1.0, abs(d))


def test_complex_pfaffian_known_answers(oracle):
    """The real known answers (runtests.jl:423, :426-430, :433) through the complex path."""
    A = np.array(GOLD["issue49"]["A"], dtype=np.complex128)
    _, _, pf = oracle.pfaffian_complex(A, quad=True)
    assert abs(pf - GOLD["issue49"]["pfaffian"]) <= 1e-9
    A = np.array(GOLD["issue121"]["A"], dtype=np.complex128)
    lp, ph, pf = oracle.pfaffian_complex(A)
    assert pf == 1 and lp == 0 and ph == 1
    rng = np.random.default_rng(5)
    for _ in range(10):
        a, b, c, d, e, f = rng.integers(-10, 11, 6)
        M = np.array([[0, a, b, c], [-a, 0, d, e], [-b, -d, 0, f], [-c, -e, -f, 0]], dtype=np.complex128)
        _, _, pf = oracle.pfaffian_complex(M * (1 + 2j))  # Pf(s M) = s^2 Pf(M)
        assert abs(pf - (c * d - b * e + a * f) * (1 + 2j) ** 2) <= 1e-12 * max(1, abs(pf))


def test_complex_pfaffian_random_double_vs_quad(oracle):
    rng = np.random.default_rng(3)
    for n in (6, 31, 64):
        R = rng.standard_normal((n + n % 2, n + n % 2)) + 1j * rng.standard_normal((n + n % 2, n + n % 2))
        A = (R - R.T) / 2
        lp, ph, _ = oracle.pfaffian_complex(A)
        lq, pq, _ = oracle.pfaffian_complex(A, quad=True)
        assert abs(lp - lq) <= 1e-12 * max(1.0, abs(lq))
        assert abs(ph - pq) <= 1e-12
        sign, logdet = np.linalg.slogdet(A)
        assert abs(2 * lq - logdet) <= 1e-11 * max(1.0, abs(logdet))
        assert abs(pq**2 - sign) <= 1e-11
