"""Selected eigenvalues: eigvals(A, irange) and eigvals(A, vl, vh) (eigen.jl:8-16,
:29-41, :57-73).  The reference negates the selected ascending eigenvalues of
SymTridiagonal(0, ev) (real) or of Hermitian(iA) (complex, LAPACK): selection by
index counts from the largest imaginary part; by interval returns the imaginary
parts in [vl, vh), descending.  Checked against the full spectrum (the oracle's
for real, LAPACK's for complex) at 1e-11 relative to the spectral radius.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-11


def skew(n, seed, complex_=False):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n))
    if complex_:
        B = B + 1j * rng.standard_normal((n, n))
        return (B - B.conj().T) / 2
    return (B - B.T) / 2


@pytest.mark.parametrize("n", [1, 2, 7, 50, 300, 1100])
def test_irange_real(skewgpu, oracle, n):
    A = skew(n, 70 + n)
    full = np.sort(oracle.eigvals(A)[0])[::-1]
    rho = max(np.abs(full).max(), 1.0)
    for il, iu in {(1, 1), (1, min(3, n)), (max(1, n // 2), n), (n, n), (1, n)}:
        v = skewgpu.eigvals_irange(A, il, iu).imag
        assert len(v) == iu - il + 1
        np.testing.assert_allclose(v, full[il - 1:iu], atol=TOL * rho)


@pytest.mark.parametrize("n", [1, 9, 64, 300, 1100])
def test_interval_real(skewgpu, oracle, n):
    A = skew(n, 90 + n)
    full = np.sort(oracle.eigvals(A)[0])[::-1]
    rho = max(np.abs(full).max(), 1.0)
    for vl, vh in ((-1e300, 1e300), (0.1 * rho, 0.6 * rho), (-0.3 * rho, 0.25 * rho), (2 * rho, 3 * rho)):
        v = skewgpu.eigvals_interval(A, vl, vh).imag
        ref = full[(full >= vl) & (full < vh)]
        assert len(v) == len(ref), (vl, vh, len(v), len(ref))
        np.testing.assert_allclose(v, ref, atol=TOL * rho)


@pytest.mark.parametrize("n", [1, 6, 100, 257])
def test_interval_complex(skewgpu, n):
    A = skew(n, 110 + n, complex_=True)
    full = -np.linalg.eigvalsh(1j * A)  # descending
    rho = max(np.abs(full).max(), 1.0)
    for vl, vh in ((-1e300, 1e300), (0.0, 0.5 * rho), (-0.7 * rho, -0.1 * rho)):
        v = skewgpu.eigvals_interval(A, vl, vh).imag
        ref = full[(full >= vl) & (full < vh)]
        assert len(v) == len(ref)
        np.testing.assert_allclose(v, ref, atol=TOL * rho)
