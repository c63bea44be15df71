"""svdvals / svd / schur from the eigenpairs (eigen.jl:110-144,
skewhermitian.jl:238-243, tridiag.jl:526-555).

Checks, with the tolerances written in each test:
* singular values against numpy's (LAPACK) within 1e-11 of the largest,
  descending;
* A = U diag(S) Vt within 1e-11 relative to the largest singular value, U and Vt
  unitary within 1e-11;
* the reference's construction: U is the eigenvectors stably sorted by |lambda|
  descending and V = -i U with the columns of negative lambda negated.  For real
  input (n <= 256) this is compared with the same construction applied to the
  oracle's eigenpairs, which follow the reference's eigenvalue order (1e-8, the
  eigenvector tolerance of the eigen tests);
* the README known answer svdvals(A) = [|l1|, |l1|, |l2|, |l2|] (runtests.jl:27);
* schur: A = Z T Z^H with T = Diagonal(values) (runtests.jl:133-136).
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_known_answers.json")))["cases"]


def skew_random(n, seed):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n))
    return (B - B.T) / 2


def skewh_random(n, seed):
    rng = np.random.default_rng(seed)
    C = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return (C - C.conj().T) / 2


def reference_svd(vals_im, W):
    """eigen.jl:119-136 applied to eigenpairs (vals_im, W): stable sort by |lambda|
    descending, V = -i U, columns of negative lambda negated."""
    order = np.argsort(-np.abs(vals_im), kind="stable")
    lam = vals_im[order]
    U = W[:, order]
    V = -1j * U
    V[:, lam < 0] *= -1
    return U, np.abs(lam), V.conj().T


def _check_svd(A, U, S, Vt, tol=1e-11):
    n = A.shape[0]
    smax = max(S.max() if n else 0.0, 1e-300)
    assert np.all(np.diff(S) <= 0.0)
    np.testing.assert_allclose(S, np.linalg.svd(A, compute_uv=False), atol=tol * smax)
    np.testing.assert_allclose(U @ np.diag(S) @ Vt, A, atol=tol * smax)
    np.testing.assert_allclose(U.conj().T @ U, np.eye(n), atol=tol)
    np.testing.assert_allclose(Vt @ Vt.conj().T, np.eye(n), atol=tol)


@pytest.mark.parametrize("n", [1, 2, 3, 7, 16, 64, 129, 256])
def test_svd_real_vs_reference_construction(skewgpu, oracle, n):
    A = skew_random(n, 70 + n)
    U, S, Vt = skewgpu.svd(A)
    _check_svd(A, U, S, Vt)
    vd, Vrd, Vid, st = oracle.eigen(A)
    Ur, Sr, Vtr = reference_svd(vd, Vrd + 1j * Vid)
    np.testing.assert_allclose(S, Sr, atol=1e-11 * max(Sr.max(), 1e-300))
    np.testing.assert_allclose(U, Ur, atol=1e-8)
    np.testing.assert_allclose(Vt, Vtr, atol=1e-8)
    np.testing.assert_allclose(skewgpu.svdvals(A), S, atol=1e-12 * max(S.max(), 1e-300))


def test_svd_real_large(skewgpu):
    """n > 1024: the bisection / twisted-vector eigen path underneath."""
    A = skew_random(1100, 5)
    U, S, Vt = skewgpu.svd(A)
    _check_svd(A, U, S, Vt)
    np.testing.assert_allclose(skewgpu.svdvals(A), S, atol=1e-12 * S.max())


def test_svdvals_readme(skewgpu):
    """runtests.jl:27: svdvals(A) ~ [i l1, i l1, i l2, i l2] for the README matrix."""
    A = np.array(GOLD["readme_A"]["A"])
    il = np.abs(np.array(GOLD["readme_eigs"]["ilambda"]))
    S = skewgpu.svdvals(A)
    np.testing.assert_allclose(S, np.sort(np.repeat(il, 2))[::-1], rtol=1e-13)


@pytest.mark.parametrize("n", [1, 5, 64, 200])
def test_svd_complex(skewgpu, n):
    A = skewh_random(n, 90 + n)
    U, S, Vt = skewgpu.svd(A)
    _check_svd(A, U, S, Vt)
    np.testing.assert_allclose(skewgpu.svdvals(A), S, atol=1e-12 * max(S.max(), 1e-300))
    # the construction: V = -i sign(lambda) U with A U = U diag(i lambda)
    lam = np.real(np.diag(U.conj().T @ A @ U) / 1j)
    V = Vt.conj().T
    sg = np.where(lam < 0, -1.0, 1.0)
    np.testing.assert_allclose(V, -1j * U * sg, atol=1e-12)


@pytest.mark.parametrize("n", [2, 9, 40])
def test_svd_tridiagonal(skewgpu, n):
    rng = np.random.default_rng(n)
    ev = rng.standard_normal(n - 1)
    T = np.zeros((n, n))
    T[np.arange(1, n), np.arange(n - 1)] = ev
    T[np.arange(n - 1), np.arange(1, n)] = -ev
    Tr = skewgpu.SkewHermTridiagonal(ev)
    U, S, Vt = Tr.svd()
    _check_svd(T, U, S, Vt)
    np.testing.assert_allclose(Tr.svdvals(), S, atol=1e-12 * S.max())
    evc = rng.standard_normal(n - 1) + 1j * rng.standard_normal(n - 1)
    dvim = rng.standard_normal(n)
    Tc = np.diag(1j * dvim).astype(np.complex128)
    Tc[np.arange(1, n), np.arange(n - 1)] = evc
    Tc[np.arange(n - 1), np.arange(1, n)] = -evc.conj()
    Tz = skewgpu.SkewHermTridiagonal(evc, dvim)
    U, S, Vt = Tz.svd()
    _check_svd(Tc, U, S, Vt)
    np.testing.assert_allclose(Tz.svdvals(), S, atol=1e-12 * S.max())


@pytest.mark.parametrize("n", [1, 4, 33, 200])
def test_schur(skewgpu, n):
    A = skew_random(n, 11 + n)
    T, Z, lam = skewgpu.schur(A)
    np.testing.assert_allclose(Z @ T @ Z.conj().T, A, atol=1e-11 * max(1.0, np.abs(lam).max()))
    np.testing.assert_array_equal(np.diag(T), lam)
    np.testing.assert_allclose(Z.conj().T @ Z, np.eye(n), atol=1e-11)
