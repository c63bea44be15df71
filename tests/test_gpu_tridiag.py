"""SkewHermTridiagonal inputs (tridiag.jl): eigvals in the reference's QR order
(skewtrieigvals!), eigen through skewtrieigen_merged! (which, unlike the dense path's
skewtrieigen_divided!, has no mem deflation), exp.jl functions, and the complex
tridiagonal through to_symtridiagonal.  Reference lists from runtests.jl (#116,
#118) and seeded random subdiagonals; tolerances: eigenvalues 1e-11 of the oracle,
reconstructions 1e-11 relative.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_known_answers.json")))["cases"]


def dense(ev, dvim=None):
    ev = np.asarray(ev)
    n = len(ev) + 1
    T = np.zeros((n, n), dtype=np.complex128 if (np.iscomplexobj(ev) or dvim is not None) else np.float64)
    T[np.arange(1, n), np.arange(n - 1)] = ev
    T[np.arange(n - 1), np.arange(1, n)] = -np.conj(ev)
    if dvim is not None:
        T[np.arange(n), np.arange(n)] = 1j * np.asarray(dvim)
    return T


def lists():
    rng = np.random.default_rng(5)
    out = [np.array(v, dtype=float) for v in GOLD["issue116"]["ev_lists"] + GOLD["issue118"]["ev_lists"]]
    out += [rng.standard_normal(n - 1) for n in (2, 3, 10, 31, 64, 257)]
    return out


@pytest.mark.parametrize("k", range(len(lists())))
def test_tridiag_eigvals_reference_order(skewgpu, oracle, k):
    ev = lists()[k]
    T = skewgpu.SkewHermTridiagonal(ev)
    v = T.eigvals().imag
    vd, st = oracle.skewtrieigvals(ev)
    scale = max(np.abs(vd).max(), 1.0)
    np.testing.assert_allclose(v, vd, atol=1e-11 * scale)  # same QR order


@pytest.mark.parametrize("k", range(len(lists())))
def test_tridiag_eigen_merged(skewgpu, k):
    ev = lists()[k]
    T = skewgpu.SkewHermTridiagonal(ev)
    lam, V = T.eigen()
    D = dense(ev)
    n = D.shape[0]
    rho = max(np.abs(lam).max(), 1.0)
    np.testing.assert_allclose(V @ np.diag(lam) @ V.conj().T, D, atol=2e-11 * rho)
    np.testing.assert_allclose(V.conj().T @ V, np.eye(n), atol=1e-11)


def test_merged_has_no_mem_deflation(skewgpu):
    """[0, 1, 1]: skewtrieigen_merged! has no mem check, so the values are the true
    +-i sqrt(2) (the dense path's skewtrieigen_divided! deflates at ev = 1)."""
    lam, V = skewgpu.SkewHermTridiagonal([0.0, 1.0, 1.0]).eigen()
    np.testing.assert_allclose(np.sort(np.abs(lam.imag)), [0, 0, np.sqrt(2), np.sqrt(2)], atol=1e-14)


def test_tridiag_large(skewgpu):
    rng = np.random.default_rng(8)
    ev = rng.standard_normal(1199)
    T = skewgpu.SkewHermTridiagonal(ev)
    lam, V = T.eigen()
    D = dense(ev)
    rho = np.abs(lam).max()
    assert np.all(np.diff(lam.imag) <= 0)
    np.testing.assert_allclose(np.abs(D @ V - V * lam).max(), 0.0, atol=1e-11 * rho)
    np.testing.assert_allclose(V.conj().T @ V, np.eye(1200), atol=1e-11)
    np.testing.assert_allclose(T.eigvals(), lam)


@pytest.mark.parametrize("name", ["exp", "cos", "sin", "sinh"])
def test_tridiag_functions(skewgpu, name):
    import scipy.linalg as sl

    rng = np.random.default_rng(9)
    ev = rng.standard_normal(40) * 0.5
    ref = {"exp": sl.expm, "cos": sl.cosm, "sin": sl.sinm, "sinh": sl.sinhm}[name](dense(ev))
    F = skewgpu.SkewHermTridiagonal(ev).function(name)
    np.testing.assert_allclose(F, ref, atol=1e-11 * np.abs(ref).max())


@pytest.mark.parametrize("n", [1, 2, 9, 100, 1100])
def test_tridiag_complex(skewgpu, n):
    rng = np.random.default_rng(10 + n)
    ev = rng.standard_normal(n - 1) + 1j * rng.standard_normal(n - 1)
    dvim = rng.standard_normal(n)
    T = skewgpu.SkewHermTridiagonal(ev, dvim)
    D = dense(ev, dvim)
    lam, V = T.eigen()
    rho = max(np.abs(lam).max(), 1.0)
    np.testing.assert_allclose(lam.imag, -np.linalg.eigvalsh(1j * D), atol=1e-11 * rho)
    np.testing.assert_allclose(T.eigvals(), lam)
    np.testing.assert_allclose(V.conj().T @ V, np.eye(n), atol=1e-11)
    assert np.abs(D @ V - V * lam).max() <= 1e-11 * rho
