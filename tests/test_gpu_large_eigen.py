"""eigen of one large real skew matrix (n > 1024): blocked reduction, bisection,
twisted-factorisation eigenvectors with a banded orthogonal correction, and
blocked back-transformation (the reference's fallback formulation,
skewtrieigen_backup!, skeweigen.jl:470-489, through skeweigen!, eigen.jl:75-91).

Checks, with the tolerances written here: eigenvalues within 1e-11 of the
oracle's (sorted; relative to the spectral radius), reconstruction
V diag(i*vals) V^H = A within 1e-11 relative to the spectral radius,
orthonormality |V^H V - I| within 1e-11, per-pair residuals, and the output
order: descending values with the -sigma vector the conjugate of the +sigma one.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def skew_random(n, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n)) * scale
    return (B - B.T) / 2


def _check(skewgpu, oracle, A, tol=1e-11, ref_vals=None):
    n = A.shape[0]
    lam, V = skewgpu.eigen(A)
    vals = lam.imag
    assert np.all(lam.real == 0.0)
    assert np.all(np.diff(vals) <= 0.0), "values must be sorted descending"
    h = n // 2
    np.testing.assert_allclose(vals[:h], -vals[::-1][:h], rtol=0, atol=0)
    if n % 2:
        assert vals[h] == 0.0
    rho = np.abs(vals).max()
    if ref_vals is None:
        vd, _ = oracle.eigvals(A)
        ref_vals = np.sort(vd)[::-1]
    np.testing.assert_allclose(vals, ref_vals, atol=tol * rho)
    # conjugate pairing of the +sigma / -sigma columns
    np.testing.assert_array_equal(V[:, :h], np.conj(V[:, ::-1][:, :h]))
    G = V.conj().T @ V
    assert np.abs(G - np.eye(n)).max() <= tol, f"orthonormality {np.abs(G - np.eye(n)).max()}"
    R = V @ np.diag(lam) @ V.conj().T - A
    assert np.abs(R).max() <= tol * rho, f"reconstruction {np.abs(R).max() / rho}"
    res = np.abs(A @ V - V * lam).max()
    assert res <= tol * rho, f"residual {res / rho}"


@pytest.mark.parametrize("n", [1025, 1100, 1101])
def test_large_eigen_random(skewgpu, oracle, n):
    _check(skewgpu, oracle, skew_random(n, 31 + n))


def test_large_eigen_split_blocks(skewgpu, oracle):
    """Block-diagonal input: the tridiagonal splits exactly and eigenvalues of the
    two blocks interleave; each vector must stay within its block."""
    A = np.zeros((1200, 1200))
    A[:700, :700] = skew_random(700, 5)
    A[700:, 700:] = skew_random(500, 6, scale=1.3)
    _check(skewgpu, oracle, A)


def test_large_eigen_scaled(skewgpu, oracle):
    """Entries of size 1e-150 and 1e+150: the twisted recurrences and the pivot
    guard must not under- or overflow.  The reference's QR deflates at an absolute
    10 eps and returns zeros for the tiny scale, so the values are checked by
    scale invariance against the unscaled matrix instead of the oracle."""
    base = skew_random(1030, 77)
    vals1 = skewgpu.eigen(base)[0].imag
    for s in (1e-150, 1e150):
        _check(skewgpu, oracle, base * s, ref_vals=vals1 * s)


def test_large_eigvals_agree(skewgpu):
    """The values of eigen equal those of eigvals (same reduction and bisection)."""
    A = skew_random(1500, 12)
    lam, _ = skewgpu.eigen(A)
    v = skewgpu.eigvals(A)
    np.testing.assert_array_equal(lam.imag, v.imag)


def test_large_eigen_identical_blocks(skewgpu, oracle):
    """A direct sum of two identical blocks: the tridiagonal splits exactly and
    every eigenvalue is double; each copy must get its own block's vector."""
    B = skew_random(560, 21)
    A = np.zeros((1120, 1120))
    A[:560, :560] = B
    A[560:, 560:] = B
    _check(skewgpu, oracle, A)


def _check_full_mode(skewgpu, A, tol=1e-11, otol=1e-12):
    """Several zero eigenvalues (the fallback's layout): values against LAPACK
    (sorted descending), reconstruction, orthonormality and residuals."""
    n = A.shape[0]
    lam, V = skewgpu.eigen(A)
    vals = lam.imag
    assert np.all(np.diff(vals) <= 0.0), "values must be sorted descending"
    rho = np.abs(vals).max()
    ref = np.sort(-np.linalg.eigvalsh(1j * A))[::-1]
    np.testing.assert_allclose(vals, ref, atol=tol * rho)
    G = V.conj().T @ V
    assert np.abs(G - np.eye(n)).max() <= otol, f"orthonormality {np.abs(G - np.eye(n)).max()}"
    R = V @ np.diag(lam) @ V.conj().T - A
    assert np.abs(R).max() <= tol * rho, f"reconstruction {np.abs(R).max() / rho}"
    assert np.abs(A @ V - V * lam).max() <= tol * rho
    return lam, V


@pytest.mark.parametrize("sizes", [(367, 401, 333), (501, 299, 301, 8), (551, 551)])
def test_large_eigen_several_odd_blocks(skewgpu, sizes):
    """A block-diagonal input whose tridiagonal splits exactly into several blocks of
    odd size: one zero eigenvalue per odd block.  More zero eigenvalues than n mod 2
    do not come in +-sigma pairs, so the path solves the whole tridiagonal in full
    mode, as the reference's fallback does (skeweigen.jl:470-489); every zero
    eigenvalue must get its own null vector."""
    n = sum(sizes)
    A = np.zeros((n, n))
    o = 0
    for k, m in enumerate(sizes):
        A[o:o + m, o:o + m] = skew_random(m, 400 + k)
        o += m
    zeros = sum(m % 2 for m in sizes)
    lam, V = _check_full_mode(skewgpu, A)
    assert np.sum(np.abs(lam.imag) <= 1e-12 * np.abs(lam).max()) == zeros


def test_large_tridiagonal_several_odd_blocks(skewgpu):
    """The same through the SkewHermTridiagonal entry point (no reduction, Q = I):
    ev with exact zeros leaving three odd blocks."""
    rng = np.random.default_rng(9)
    n = 1203
    ev = rng.standard_normal(n - 1)
    # exact zeros split the rows into blocks of 11, 2, 388, 400, 1, 299, 50 and 52:
    # three odd blocks, three zero eigenvalues
    for i in (10, 12, 400, 800, 801, 1100, 1150):
        ev[i] = 0.0
    T = skewgpu.SkewHermTridiagonal(ev)
    lam, V = T.eigen()
    Td = np.zeros((n, n))
    Td[np.arange(1, n), np.arange(n - 1)] = ev
    Td[np.arange(n - 1), np.arange(1, n)] = -ev
    rho = np.abs(lam).max()
    ref = np.sort(-np.linalg.eigvalsh(1j * Td))[::-1]
    np.testing.assert_allclose(lam.imag, ref, atol=1e-11 * rho)
    assert np.abs(V.conj().T @ V - np.eye(n)).max() <= 1e-12
    assert np.abs(V @ np.diag(lam) @ V.conj().T - Td).max() <= 1e-11 * rho
    assert np.sum(np.abs(lam.imag) <= 1e-12 * rho) == 3


def test_large_exp_several_odd_blocks(skewgpu):
    """exp of a singular block-diagonal input with three odd blocks above n = 1024
    (its eigenpairs come from the same path) against scipy's expm."""
    import scipy.linalg as sl

    sizes = (401, 333, 367)
    n = sum(sizes)
    A = np.zeros((n, n))
    o = 0
    for k, m in enumerate(sizes):
        A[o:o + m, o:o + m] = skew_random(m, 500 + k, scale=1.0 / np.sqrt(m))
        o += m
    E = skewgpu.exp(A)
    np.testing.assert_allclose(E, sl.expm(A), atol=1e-11 * np.sqrt(n))
