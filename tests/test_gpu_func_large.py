"""exp, cis, the other matrix functions and the exp adjoint of one large real skew
matrix (n > 1024; exp.jl:3-283), and the functions of a large SkewHermTridiagonal
(tridiag.jl:558-583 via exp.jl).  The eigenpairs come from the blocked reduction,
bisection and twisted vectors; the assembly is the batched path's.

Checks, with the tolerances written in each test:
* exp(A) against scipy.linalg.expm(A) within 1e-11 (Frobenius, relative to
  ||exp(A)||_F), and exp(A)^T exp(A) = I within 1e-11 (max entry);
* cis(A) against expm(iA) within 1e-11 (Frobenius, relative);
* cos, sin and sinh against scipy's cosm / sinm / sinhm within 1e-10 (Frobenius,
  relative to the reference result);
* the exp adjoint: <G, E> against the central difference of <Cbar, exp(A + hE)>
  along a skew direction E (h = 1e-5) within 1e-6 relative;
* log of an odd-size matrix raises ValueError (exact zero eigenvalue), as in the
  small-matrix path (exp.jl:252-283);
* SkewHermTridiagonal(ev).function("exp") against expm of the dense tridiagonal.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

scipy_linalg = pytest.importorskip("scipy.linalg")


def skew_random(n, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n)) * scale / np.sqrt(n)
    return (B - B.T) / 2


def _rel(X, Y):
    return np.linalg.norm(X - Y) / np.linalg.norm(Y)


def test_exp_large(skewgpu):
    n = 1100
    A = skew_random(n, 1, scale=4.0)
    E = skewgpu.exp(A)
    Eref = scipy_linalg.expm(A)
    assert _rel(E, Eref) <= 1e-11
    assert np.abs(E.T @ E - np.eye(n)).max() <= 1e-11


def test_cis_large(skewgpu):
    n = 1030
    A = skew_random(n, 2, scale=2.0)
    C = skewgpu.cis(A)
    Cref = scipy_linalg.expm(1j * A)
    assert _rel(C, Cref) <= 1e-11


@pytest.mark.parametrize("name,ref", [("cos", "cosm"), ("sin", "sinm"), ("sinh", "sinhm")])
def test_functions_large(skewgpu, name, ref):
    n = 1040
    A = skew_random(n, 3, scale=2.0)
    F = skewgpu.matrix_function(A, name)
    Fref = np.real(getattr(scipy_linalg, ref)(A))
    assert _rel(F, Fref) <= 1e-10


def test_exp_adjoint_large(skewgpu):
    n = 1060
    A = skew_random(n, 4, scale=2.0)
    rng = np.random.default_rng(5)
    Cbar = rng.standard_normal((n, n))
    E = skew_random(n, 6)
    _, pullback = skewgpu.exp_rrule(A)
    G = pullback(Cbar)
    h = 1e-5
    fp = np.sum(Cbar * skewgpu.exp(A + h * E))
    fm = np.sum(Cbar * skewgpu.exp(A - h * E))
    fd = (fp - fm) / (2 * h)
    an = np.sum(G * E)
    assert abs(an - fd) <= 1e-6 * abs(fd)


def test_log_odd_large_is_singular(skewgpu):
    A = skew_random(1025, 7)
    with pytest.raises(ValueError):
        skewgpu.matrix_function(A, "log")


def test_tridiagonal_exp_large(skewgpu):
    n = 1200
    rng = np.random.default_rng(8)
    ev = rng.standard_normal(n - 1)
    T = np.zeros((n, n))
    T[np.arange(1, n), np.arange(n - 1)] = ev
    T[np.arange(n - 1), np.arange(1, n)] = -ev
    F = skewgpu.SkewHermTridiagonal(ev).function("exp")
    assert _rel(F, scipy_linalg.expm(T)) <= 1e-11
