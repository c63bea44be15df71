"""ORACLE -- test infrastructure only (never imported by the product path).

ctypes front end for ``libskew_oracle.so``, the CPU restatement of the
SkewLinearAlgebra.jl skew-Householder pipeline (see ``skew_oracle.cpp``), plus
two pure-Python exact checks:

* :func:`exact_pfaffian` -- Pfaffian over the rationals by the Galbiati-Maffioli
  elimination that the reference uses for exact types (src/pfaffian.jl:17-56);
* :func:`exact_pfaffian_gm` is the same routine kept under the reference's name.

Every array is a float64 numpy array in Fortran (column-major) order, the layout
the Julia reference uses.  Functions with ``quad=True`` run the same algorithm
in IEEE binary128 (the stand-in for the reference's BigFloat runs) and round
the result to float64.
"""
from __future__ import annotations

import ctypes
import os
from fractions import Fraction

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libskew_oracle.so")
_lib = None

_D = ctypes.POINTER(ctypes.c_double)
_I64 = ctypes.c_int64


def build(force: bool = False) -> str:
    """Compile the oracle shared library next to its source (gcc, no GPU)."""
    from oracle.build_oracle import build_oracle  # local import keeps ctypes light

    return build_oracle(force=force)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = ctypes.CDLL(_LIB_PATH)
        for name in ("orc_hessenberg_d", "orc_hessenberg_q"):
            getattr(_lib, name).argtypes = [_D, _I64, _D, _D]
        for name in ("orc_hessenberg_z", "orc_hessenberg_zq"):
            getattr(_lib, name).argtypes = [_D, _I64, _D, _D, _D]
        _lib.orc_formq_d.argtypes = [_D, _I64, _D, _D]
        for name in ("orc_logabspf_d", "orc_logabspf_q"):
            getattr(_lib, name).argtypes = [_D, _I64, _D, _D]
        for name in ("orc_skewtrieigvals_d", "orc_skewtrieigvals_q", "orc_eigvals_d", "orc_eigvals_q"):
            getattr(_lib, name).argtypes = [_D, _I64, _D]
            getattr(_lib, name).restype = ctypes.c_int
        _lib.orc_skewtrieigen_d.argtypes = [_D, _I64, _D, _D, _D]
        _lib.orc_skewtrieigen_d.restype = ctypes.c_int
        for name in ("orc_eigen_d", "orc_eigen_q"):
            getattr(_lib, name).argtypes = [_D, _I64, _D, _D, _D]
            getattr(_lib, name).restype = ctypes.c_int
        for name in ("orc_exp_d", "orc_exp_q"):
            getattr(_lib, name).argtypes = [_D, _I64, _D]
            getattr(_lib, name).restype = ctypes.c_int
        for name in ("orc_cis_d", "orc_cis_q"):
            getattr(_lib, name).argtypes = [_D, _I64, _D, _D]
            getattr(_lib, name).restype = ctypes.c_int
        _lib.orc_logabspf_grad_q.argtypes = [_D, _I64, _D]
        _lib.orc_logabspf_grad_q.restype = ctypes.c_int
        _lib.orc_exp_vjp_q.argtypes = [_D, _D, _I64, _D]
        _lib.orc_expm_dense_q.argtypes = [_D, _I64, _D]
        _lib.orc_symtri_eigvals_q.argtypes = [_D, _D, _I64, _D]
        for name in ("orc_pfaffian_z", "orc_pfaffian_zq"):
            getattr(_lib, name).argtypes = [_D, _I64, _D, _D, _D]
        _lib.orc_batch_logabspf_d.argtypes = [_D, ctypes.POINTER(_I64), ctypes.POINTER(_I64), _I64, _D, _D,
                                              ctypes.c_int]
        _lib.orc_batch_logabspf_grad_d.argtypes = [_D, ctypes.POINTER(_I64), ctypes.POINTER(_I64), _I64, _D, _D,
                                                   _D, ctypes.c_int]
        _lib.orc_batch_logabspf_fd.argtypes = [_D, ctypes.POINTER(_I64), ctypes.POINTER(_I64), _I64,
                                               ctypes.POINTER(_I64), _I64, ctypes.c_double, ctypes.c_int, _D,
                                               ctypes.c_int]
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _fmat(A) -> np.ndarray:
    A = np.asarray(A, dtype=np.float64)
    return np.array(A, dtype=np.float64, order="F", copy=True)


def hessenberg(A, quad: bool = False):
    """skewblockedhess! (hessenberg.jl:144-173).  Returns (factors, tau, ev):
    factors holds the reflectors below the subdiagonal (v[0] = 1 on it), tau and
    ev (the subdiagonal of H = SkewHermTridiagonal(ev)) have n-1 entries."""
    F = _fmat(A)
    n = F.shape[0]
    tau = np.zeros(max(n - 1, 1))
    ev = np.zeros(max(n - 1, 1))
    fn = lib().orc_hessenberg_q if quad else lib().orc_hessenberg_d
    fn(_p(F), n, _p(tau), _p(ev))
    return F, tau[: max(n - 1, 0)], ev[: max(n - 1, 0)]


def hessenberg_complex(A, quad: bool = False):
    """Complex skew-Hermitian hessenberg (hessenberg.jl:5-13, complex branches).
    Returns (factors complex, tau complex, ev real, dvim real)."""
    A = np.asarray(A, dtype=np.complex128)
    n = A.shape[0]
    flat = np.ascontiguousarray(np.asarray(A, dtype=np.complex128).ravel(order="F"))
    buf = flat.view(np.float64)  # interleaved re/im, column-major
    tau = np.zeros(2 * max(n - 1, 1))
    ev = np.zeros(max(n - 1, 1))
    dvim = np.zeros(max(n, 1))
    fn = lib().orc_hessenberg_zq if quad else lib().orc_hessenberg_z
    fn(buf.ctypes.data_as(_D), n, _p(tau), _p(ev), _p(dvim))
    t = tau.view(np.complex128)[: max(n - 1, 0)]
    F = flat.reshape((n, n), order="F")
    return F, t.copy(), ev[: max(n - 1, 0)], dvim[:n]


def formq(factors, tau) -> np.ndarray:
    """Matrix(H.Q): the product of the stored reflectors."""
    F = _fmat(factors)
    n = F.shape[0]
    t = np.zeros(max(n, 1))
    t[: len(tau)] = tau
    Q = np.zeros((n, n), order="F")
    lib().orc_formq_d(_p(F), n, _p(t), _p(Q))
    return Q


def logabspfaffian(A, quad: bool = False):
    """_logabspfaffian! (pfaffian.jl:167-179): returns (log|Pf A|, sign)."""
    F = _fmat(A)
    n = F.shape[0]
    lp = np.zeros(1)
    sg = np.zeros(1)
    fn = lib().orc_logabspf_q if quad else lib().orc_logabspf_d
    fn(_p(F), n, _p(lp), _p(sg))
    return float(lp[0]), float(sg[0])


def pfaffian_complex(A, quad: bool = False):
    """Parlett-Reid elimination with pivoting for complex skew-symmetric A
    (pfaffian.jl:98-137 and :193-233).  Returns (log|Pf A|, cis(phase), Pf A):
    the two outputs of _logabspfaffian! and the product of _pfaffian!."""
    A = np.asarray(A, dtype=np.complex128)
    n = A.shape[0]
    buf = np.ascontiguousarray(A.ravel(order="F")).view(np.float64)
    lp = np.zeros(1)
    ph = np.zeros(2)
    pf = np.zeros(2)
    fn = lib().orc_pfaffian_zq if quad else lib().orc_pfaffian_z
    fn(_p(buf), n, _p(lp), _p(ph), _p(pf))
    return float(lp[0]), complex(ph[0], ph[1]), complex(pf[0], pf[1])


def skewtrieigvals(ev, quad: bool = False):
    """skewtrieigvals! (skeweigen.jl:105-156) on the skew tridiagonal with
    subdiagonal ev.  Returns (imag parts of the eigenvalues, status) where status
    is 0 (converged), 1 (fallback used) or -1 (no convergence)."""
    e = np.array(ev, dtype=np.float64, copy=True)
    N = len(e) + 1
    e2 = np.zeros(max(N, 1))
    e2[: len(e)] = e
    vals = np.zeros(N)
    fn = lib().orc_skewtrieigvals_q if quad else lib().orc_skewtrieigvals_d
    st = fn(_p(e2), N, _p(vals))
    return vals, st


def eigvals(A, quad: bool = False):
    """eigvals(::SkewHermitian{Float64}) (eigen.jl:2-6, 312-318): imaginary parts
    in the reference's (deflation) order, and the status."""
    F = _fmat(A)
    n = F.shape[0]
    vals = np.zeros(n)
    fn = lib().orc_eigvals_q if quad else lib().orc_eigvals_d
    st = fn(_p(F), n, _p(vals))
    return vals, st


def skewtrieigen(ev):
    """skewtrieigen_divided! (skeweigen.jl:322-457): (vals_im, Qr, Qim, status)."""
    e = np.array(ev, dtype=np.float64, copy=True)
    N = len(e) + 1
    e2 = np.zeros(max(N, 1))
    e2[: len(e)] = e
    vals = np.zeros(N)
    Qr = np.zeros((N, N), order="F")
    Qi = np.zeros((N, N), order="F")
    st = lib().orc_skewtrieigen_d(_p(e2), N, _p(vals), _p(Qr), _p(Qi))
    return vals, Qr, Qi, st


def eigen(A, quad: bool = False):
    """eigen(::SkewHermitian{Float64}) (eigen.jl:75-97): (vals_im, Vr, Vi, status);
    eigenvectors are Vr + i Vi."""
    F = _fmat(A)
    n = F.shape[0]
    vals = np.zeros(n)
    Vr = np.zeros((n, n), order="F")
    Vi = np.zeros((n, n), order="F")
    fn = lib().orc_eigen_q if quad else lib().orc_eigen_d
    st = fn(_p(F), n, _p(vals), _p(Vr), _p(Vi))
    return vals, Vr, Vi, st


def expm(A, quad: bool = False):
    """skewexp! (exp.jl:3-35), real input."""
    F = _fmat(A)
    n = F.shape[0]
    out = np.zeros((n, n), order="F")
    fn = lib().orc_exp_q if quad else lib().orc_exp_d
    st = fn(_p(F), n, _p(out))
    if st < 0:
        raise RuntimeError("oracle exp: no convergence")
    return out


def cis(A, quad: bool = False):
    """skewcis! (exp.jl:99-110), real input: complex Hermitian n x n."""
    F = _fmat(A)
    n = F.shape[0]
    re = np.zeros((n, n), order="F")
    im = np.zeros((n, n), order="F")
    fn = lib().orc_cis_q if quad else lib().orc_cis_d
    st = fn(_p(F), n, _p(re), _p(im))
    if st < 0:
        raise RuntimeError("oracle cis: no convergence")
    return re + 1j * im


def logabspfaffian_grad(A) -> np.ndarray:
    """1/2 A^{-T} by a quad Gauss-Jordan inverse (independent of Householder)."""
    F = _fmat(A)
    n = F.shape[0]
    G = np.zeros((n, n), order="F")
    if lib().orc_logabspf_grad_q(_p(F), n, _p(G)) != 0:
        raise ZeroDivisionError("singular matrix")
    return G


def exp_vjp(A, C) -> np.ndarray:
    """Gradient of <C, exp(A)> w.r.t. A (quad block-triangular exp)."""
    F = _fmat(A)
    Cf = _fmat(C)
    n = F.shape[0]
    G = np.zeros((n, n), order="F")
    lib().orc_exp_vjp_q(_p(F), _p(Cf), n, _p(G))
    return G


def expm_dense(A) -> np.ndarray:
    """Dense Taylor/scaling-squaring exp in quad (independent of eigen)."""
    F = _fmat(A)
    n = F.shape[0]
    out = np.zeros((n, n), order="F")
    lib().orc_expm_dense_q(_p(F), n, _p(out))
    return out


def symtri_eigvals(d, e) -> np.ndarray:
    n = len(e) + 1
    dd = np.zeros(n) if d is None else np.array(d, dtype=np.float64)
    ee = np.zeros(max(n, 1))
    ee[: len(e)] = e
    w = np.zeros(n)
    lib().orc_symtri_eigvals_q(_p(dd), _p(ee), n, _p(w))
    return w


def batch_logabspfaffian(mats, nthreads: int = 1):
    """FP64 logabspfaffian over a list of matrices (OpenMP across matrices)."""
    ns = np.array([m.shape[0] for m in mats], dtype=np.int64)
    offs = np.zeros(len(mats), dtype=np.int64)
    offs[1:] = np.cumsum(ns[:-1] ** 2)
    buf = np.concatenate([np.asarray(m, dtype=np.float64).ravel(order="F") for m in mats])
    return batch_logabspfaffian_packed(buf, offs, ns, nthreads)


def batch_logabspfaffian_packed(buf, offs, ns, nthreads: int = 1):
    count = len(ns)
    lp = np.zeros(count)
    sg = np.zeros(count)
    lib().orc_batch_logabspf_d(_p(buf), offs.ctypes.data_as(ctypes.POINTER(_I64)),
                               ns.ctypes.data_as(ctypes.POINTER(_I64)), count, _p(lp), _p(sg), int(nthreads))
    return lp, sg


def batch_logabspfaffian_grad_packed(buf, offs, ns, nthreads: int = 1):
    """FP64 log|Pf| + 1/2 A^{-T} over a packed batch (OpenMP across matrices)."""
    count = len(ns)
    lp = np.zeros(count)
    sg = np.zeros(count)
    grad = np.zeros_like(buf)
    lib().orc_batch_logabspf_grad_d(_p(buf), offs.ctypes.data_as(ctypes.POINTER(_I64)),
                                    ns.ctypes.data_as(ctypes.POINTER(_I64)), count, _p(lp), _p(sg), _p(grad),
                                    int(nthreads))
    return lp, sg, grad


def batch_logabspfaffian_fd(buf, offs, ns, pairs, h: float = 1e-6, quad: bool = True, nthreads: int = 1):
    """Central differences of log|Pf| along skew pairs for a packed batch:
    (f(A + hE) - f(A - hE)) / 2h with E = e_i e_j^T - e_j e_i^T, which equals
    G_ij - G_ji for the gradient G = 1/2 A^{-T}.  pairs is (count, k, 2), 0-based.
    quad=True evaluates f and the difference in binary128."""
    pairs = np.ascontiguousarray(pairs, dtype=np.int64)
    count, k = pairs.shape[0], pairs.shape[1]
    buf = np.ascontiguousarray(buf, dtype=np.float64)
    offs = np.ascontiguousarray(offs, dtype=np.int64)
    ns = np.ascontiguousarray(ns, dtype=np.int64)
    fd = np.zeros(count * k)
    lib().orc_batch_logabspf_fd(_p(buf), offs.ctypes.data_as(ctypes.POINTER(_I64)),
                                ns.ctypes.data_as(ctypes.POINTER(_I64)), count,
                                pairs.ctypes.data_as(ctypes.POINTER(_I64)), k, float(h), int(bool(quad)), _p(fd),
                                int(nthreads))
    return fd.reshape(count, k)


# ---------------------------------------------------------------------------
# Exact Pfaffian (pure Python, Fractions): Galbiati & Maffioli elimination,
# restating the algorithm the reference documents at src/pfaffian.jl:17-56.
# ---------------------------------------------------------------------------
def exact_pfaffian(A) -> Fraction:
    """Exact Pfaffian of a skew-symmetric matrix with integer/rational entries."""
    n = len(A)
    if n % 2 == 1:
        return Fraction(0)
    B = [[Fraction(A[i][j]) for j in range(n)] for i in range(n)]
    c = Fraction(1)
    flip = False
    h = n // 2
    while h > 1:
        m = 2 * h  # active size; pivot row is m-2 (0-based)
        k = m
        while k > 0 and B[m - 2][k - 1] == 0:
            k -= 1
        if k == 0:
            return Fraction(0)
        if k != m:  # swap rows/cols k-1 and m-1
            B[k - 1], B[m - 1] = B[m - 1], B[k - 1]
            for row in B:
                row[k - 1], row[m - 1] = row[m - 1], row[k - 1]
            flip = not flip
        for j in range(m - 2):
            for i in range(j):
                d = B[m - 2][m - 1] * B[i][j] - B[i][m - 2] * B[j][m - 1] + B[j][m - 2] * B[i][m - 1]
                B[i][j] = d / c
                B[j][i] = -B[i][j]
        c = B[m - 2][m - 1]
        h -= 1
    return -B[0][1] if flip else B[0][1]


exact_pfaffian_gm = exact_pfaffian


class GaussQ:
    """Gaussian rational a + b i with Fraction parts: the field the reference's
    Complex{Rational{BigInt}} exact Pfaffians are taken in (runtests.jl:410-416)."""

    __slots__ = ("re", "im")

    def __init__(self, re, im=0):
        self.re = Fraction(re)
        self.im = Fraction(im)

    @staticmethod
    def of(z) -> "GaussQ":
        if isinstance(z, GaussQ):
            return z
        z = complex(z)
        return GaussQ(Fraction(z.real), Fraction(z.imag))

    def __add__(self, o):
        o = GaussQ.of(o)
        return GaussQ(self.re + o.re, self.im + o.im)

    def __sub__(self, o):
        o = GaussQ.of(o)
        return GaussQ(self.re - o.re, self.im - o.im)

    def __neg__(self):
        return GaussQ(-self.re, -self.im)

    def __mul__(self, o):
        o = GaussQ.of(o)
        return GaussQ(self.re * o.re - self.im * o.im, self.re * o.im + self.im * o.re)

    def __truediv__(self, o):
        o = GaussQ.of(o)
        d = o.re * o.re + o.im * o.im
        return GaussQ((self.re * o.re + self.im * o.im) / d, (self.im * o.re - self.re * o.im) / d)

    def __eq__(self, o):
        o = GaussQ.of(o)
        return self.re == o.re and self.im == o.im

    def __complex__(self):
        return complex(float(self.re), float(self.im))


def exact_pfaffian_complex(A) -> GaussQ:
    """Exact Pfaffian of a complex skew-symmetric matrix whose entries are exact
    binary fractions (integers, halves, ...), by the same Galbiati-Maffioli
    elimination as exact_pfaffian, over the Gaussian rationals."""
    n = len(A)
    if n == 0:
        return GaussQ(1)
    if n % 2 == 1:
        return GaussQ(0)
    B = [[GaussQ.of(A[i][j]) for j in range(n)] for i in range(n)]
    c = GaussQ(1)
    flip = False
    h = n // 2
    while h > 1:
        m = 2 * h
        k = m
        while k > 0 and B[m - 2][k - 1] == 0:
            k -= 1
        if k == 0:
            return GaussQ(0)
        if k != m:
            B[k - 1], B[m - 1] = B[m - 1], B[k - 1]
            for row in B:
                row[k - 1], row[m - 1] = row[m - 1], row[k - 1]
            flip = not flip
        for j in range(m - 2):
            for i in range(j):
                d = B[m - 2][m - 1] * B[i][j] - B[i][m - 2] * B[j][m - 1] + B[j][m - 2] * B[i][m - 1]
                B[i][j] = d / c
                B[j][i] = -B[i][j]
        c = B[m - 2][m - 1]
        h -= 1
    return -B[0][1] if flip else B[0][1]
