"""ComplexF64 skew-Hermitian matrices on the GPU.

The reduction follows the reference's complex householder!/skewlatrd!/
skewblockedhess! (hessenberg.jl), checked against the oracle's restatement
(binary128 for the subdiagonal and diagonal, FP64 for tau and the reflectors)
and by Q^H A Q = H.  The reference computes complex eigenvalues and eigenvectors
with LAPACK on Hermitian(i A) (eigen.jl:18-27, 101-106); numpy's eigvalsh/eigh is
that LAPACK, so it is the check for eigvals, next to reconstruction and
orthonormality for eigen.  exp (exp.jl:37-46) is checked against scipy's expm and
its adjoint against the block exponential exp([[A^H, C], [0, A^H]]) (whose upper
right block is the adjoint of the Frechet derivative) and central finite
differences.  Tolerances are written in each test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def skewh_random(n, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    C = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * scale
    return (C - C.conj().T) / 2


def formq_complex(F, tau):
    n = F.shape[0]
    Q = np.eye(n, dtype=np.complex128)
    for c in range(n - 1):
        if tau[c] == 0:
            continue
        v = np.zeros(n, dtype=np.complex128)
        v[c + 1] = 1.0
        v[c + 2:] = F[c + 2:, c]
        Q = Q @ (np.eye(n) - tau[c] * np.outer(v, v.conj()))
    return Q


@pytest.mark.parametrize("n", [1, 2, 3, 5, 16, 64, 128, 129, 300])
def test_hessenberg_complex_vs_oracle(skewgpu, oracle, n):
    A = skewh_random(n, 600 + n)
    Hc = skewgpu.hessenberg_complex(A)
    ev = Hc.ev.cpu().numpy()
    dvim = Hc.dvim.cpu().numpy()
    tau = Hc.tau.cpu().numpy()
    F = skewgpu.from_device_complex(Hc.factors)
    scale = max(1.0, np.abs(A).max())
    _, tq, eq, dq = oracle.hessenberg_complex(A, quad=(n <= 129))
    np.testing.assert_allclose(ev, eq, atol=1e-11 * scale * np.sqrt(n))
    np.testing.assert_allclose(dvim, dq, atol=1e-11 * scale * np.sqrt(n))
    np.testing.assert_allclose(tau, tq, atol=1e-10)
    if n > 1:
        Q = formq_complex(F, tau)
        np.testing.assert_allclose(Q.conj().T @ Q, np.eye(n), atol=1e-13 * n)
        np.testing.assert_allclose(Q.conj().T @ A @ Q, Hc.H(), atol=1e-13 * scale * n)


@pytest.mark.parametrize("n", [131, 160, 257, 300, 520, 777])
def test_hessenberg_complex_persistent_vs_oracle(skewgpu, oracle, n):
    """The blocked persistent reduction (panels of 32 columns, the complex latrd with
    the alpha correction, rank-64 trailing updates), forced down to n = 131 with
    the tuning key zpersist_min_n; checked like the per-column path."""
    A = skewh_random(n, 1600 + n)
    with skewgpu.tuned(zpersist_min_n=130):
        Hc = skewgpu.hessenberg_complex(A)
    ev = Hc.ev.cpu().numpy()
    dvim = Hc.dvim.cpu().numpy()
    tau = Hc.tau.cpu().numpy()
    F = skewgpu.from_device_complex(Hc.factors)
    scale = max(1.0, np.abs(A).max())
    _, tq, eq, dq = oracle.hessenberg_complex(A, quad=False)
    np.testing.assert_allclose(ev, eq, atol=1e-11 * scale * np.sqrt(n))
    np.testing.assert_allclose(dvim, dq, atol=1e-11 * scale * np.sqrt(n))
    np.testing.assert_allclose(tau, tq, atol=1e-10)
    Q = formq_complex(F, tau)
    np.testing.assert_allclose(Q.conj().T @ Q, np.eye(n), atol=1e-13 * n)
    np.testing.assert_allclose(Q.conj().T @ A @ Q, Hc.H(), atol=1e-13 * scale * n)


@pytest.mark.parametrize("nb", [4, 12, 32])
def test_hessenberg_complex_panel_width(skewgpu, oracle, nb):
    """The complex persistent reduction at panel widths 4, 12 and 32 (the tuning key
    zpersist_nb): the same checks as at the default width."""
    n = 300
    A = skewh_random(n, 1900 + n)
    with skewgpu.tuned(zpersist_min_n=130, zpersist_nb=nb):
        Hc = skewgpu.hessenberg_complex(A)
    ev = Hc.ev.cpu().numpy()
    dvim = Hc.dvim.cpu().numpy()
    tau = Hc.tau.cpu().numpy()
    F = skewgpu.from_device_complex(Hc.factors)
    scale = max(1.0, np.abs(A).max())
    _, tq, eq, dq = oracle.hessenberg_complex(A, quad=False)
    np.testing.assert_allclose(ev, eq, atol=1e-11 * scale * np.sqrt(n))
    np.testing.assert_allclose(dvim, dq, atol=1e-11 * scale * np.sqrt(n))
    np.testing.assert_allclose(tau, tq, atol=1e-10)
    Q = formq_complex(F, tau)
    np.testing.assert_allclose(Q.conj().T @ A @ Q, Hc.H(), atol=1e-13 * scale * n)


def test_hessenberg_complex_not_skew(skewgpu):
    A = skewh_random(8, 1)
    A[0, 0] += 0.5  # a real diagonal part: not skew-Hermitian
    with pytest.raises(ValueError):
        skewgpu.hessenberg_complex(A)


@pytest.mark.parametrize("n", [1, 2, 7, 64, 200, 513])
def test_eigvals_eigen_complex(skewgpu, n):
    A = skewh_random(n, 700 + n)
    rho = max(np.abs(np.linalg.eigvalsh(1j * A)).max(), 1e-300)
    v = skewgpu.eigvals_complex(A)
    ref = -np.linalg.eigvalsh(1j * A)  # the reference's values: -eigvals(Hermitian(iA)), LAPACK
    assert np.all(np.diff(v.imag) <= 0.0)
    np.testing.assert_allclose(v.imag, ref, atol=1e-11 * rho)
    lam, V = skewgpu.eigen_complex(A)
    np.testing.assert_array_equal(lam, v)
    np.testing.assert_allclose(V.conj().T @ V, np.eye(n), atol=1e-11)
    np.testing.assert_allclose(V @ np.diag(lam) @ V.conj().T, A, atol=1e-11 * rho)


def test_eigen_complex_large(skewgpu):
    n = 1100
    A = skewh_random(n, 9)
    lam, V = skewgpu.eigen_complex(A)
    rho = np.abs(lam).max()
    np.testing.assert_allclose(lam.imag, -np.linalg.eigvalsh(1j * A), atol=1e-11 * rho)
    np.testing.assert_allclose(V.conj().T @ V, np.eye(n), atol=1e-11)
    assert np.abs(A @ V - V * lam).max() <= 1e-11 * rho


def test_eigen_complex_real_input(skewgpu):
    """A real skew matrix through the complex path: same spectrum as the real path."""
    rng = np.random.default_rng(4)
    B = rng.standard_normal((40, 40))
    A = (B - B.T) / 2
    lam_c = skewgpu.eigvals_complex(A.astype(np.complex128))
    lam_r = skewgpu.eigvals(A)
    np.testing.assert_allclose(np.sort(lam_c.imag), np.sort(lam_r.imag), atol=1e-12 * np.abs(lam_r).max())


@pytest.mark.parametrize("n", [1, 3, 16, 100, 256])
def test_exp_complex(skewgpu, n):
    import scipy.linalg as sl

    A = skewh_random(n, 800 + n, scale=2.0 / np.sqrt(max(n, 1)))
    E = skewgpu.exp_complex(A)
    Er = sl.expm(A)
    np.testing.assert_allclose(E, Er, atol=1e-11 * np.sqrt(n))
    np.testing.assert_allclose(E @ E.conj().T, np.eye(n), atol=1e-12 * np.sqrt(n))


@pytest.mark.parametrize("n", [2, 8, 33, 96])
def test_exp_complex_adjoint(skewgpu, n):
    import scipy.linalg as sl

    rng = np.random.default_rng(900 + n)
    A = skewh_random(n, 900 + n, scale=3.0 / np.sqrt(n))
    C = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    _, pullback = skewgpu.exp_complex_rrule(A)
    G = pullback(C)
    # block exponential: the upper right block of exp([[A^H, C], [0, A^H]])
    Z = np.zeros((n, n), dtype=np.complex128)
    M = np.block([[A.conj().T, C], [Z, A.conj().T]])
    Gref = sl.expm(M)[:n, n:]
    np.testing.assert_allclose(G, Gref, atol=1e-10 * np.abs(Gref).max())
    # central finite differences along a skew-Hermitian direction
    Ed = skewh_random(n, 1000 + n)
    h = 1e-6
    L = lambda X: np.real(np.trace(C.conj().T @ sl.expm(X)))  # noqa: E731
    fd = (L(A + h * Ed) - L(A - h * Ed)) / (2 * h)
    an = np.real(np.trace(G.conj().T @ Ed))
    assert abs(fd - an) <= 1e-6 * max(1.0, abs(an))


@pytest.mark.parametrize("n", [1, 5, 40, 200])
def test_batch_complex_eigen_exp_vjp(skewgpu, n):
    """Strided batches of one size (skew_batch_*_z) against the single-matrix calls,
    LAPACK, expm and the block exponential."""
    import scipy.linalg as sl

    count = 6
    mats = [skewh_random(n, 1100 + 17 * n + b, scale=2.0 / np.sqrt(n)) for b in range(count)]
    rng = np.random.default_rng(n)
    cots = [rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) for _ in range(count)]
    vals, vecs = skewgpu.batch_eigen_complex(mats)
    Es = skewgpu.batch_exp_complex(mats)
    Gs = skewgpu.batch_exp_vjp_complex(mats, cots)
    for b, A in enumerate(mats):
        rho = max(np.abs(vals[b]).max(), 1e-300)
        np.testing.assert_allclose(vals[b].imag, -np.linalg.eigvalsh(1j * A), atol=1e-11 * rho)
        np.testing.assert_allclose(vals[b], skewgpu.eigvals_complex(A), atol=1e-12 * rho)
        V = vecs[b]
        np.testing.assert_allclose(V.conj().T @ V, np.eye(n), atol=1e-11)
        np.testing.assert_allclose(V @ np.diag(vals[b]) @ V.conj().T, A, atol=1e-11 * rho)
        np.testing.assert_allclose(Es[b], sl.expm(A), atol=1e-11 * np.sqrt(n))
        Z = np.zeros((n, n), dtype=np.complex128)
        Gref = sl.expm(np.block([[A.conj().T, cots[b]], [Z, A.conj().T]]))[:n, n:]
        np.testing.assert_allclose(Gs[b], Gref, atol=1e-10 * np.abs(Gref).max())


def test_eigen_complex_repeated_eigenvalues(skewgpu):
    """Exact splits with repeated eigenvalues: i*diag(1, 1, 2, 1), a direct sum of
    two equal blocks, and the same at n > 1024 (the reference's LAPACK handles
    these; each copy of an eigenvalue must get its own block's vector)."""
    cases = [np.diag(1j * np.array([1.0, 1.0, 2.0, 1.0])), np.diag(1j * np.zeros(5))]
    Bk = skewh_random(40, 2)
    D = np.zeros((80, 80), dtype=np.complex128)
    D[:40, :40] = Bk
    D[40:, 40:] = Bk
    cases.append(D)
    Bl = skewh_random(600, 3)
    Dl = np.zeros((1200, 1200), dtype=np.complex128)
    Dl[:600, :600] = Bl
    Dl[600:, 600:] = Bl
    cases.append(Dl)
    for A in cases:
        n = A.shape[0]
        lam, V = skewgpu.eigen_complex(A)
        rho = max(np.abs(lam).max(), 1.0)
        np.testing.assert_allclose(lam.imag, -np.linalg.eigvalsh(1j * A), atol=1e-11 * rho)
        np.testing.assert_allclose(V.conj().T @ V, np.eye(n), atol=1e-11)
        np.testing.assert_allclose(V @ np.diag(lam) @ V.conj().T, A, atol=1e-11 * rho)
