"""skewgpu -- host-side mirror of SkewLinearAlgebra.jl's skew-Householder API over
the GB300 C ABI (libskewgpu.so).

Names, argument meaning and error behaviour follow the Julia package:

==========================  =====================================================
Julia (SkewLinearAlgebra)   here
==========================  =====================================================
``SkewHermitian(A)``        :class:`SkewHermitian` (checks A == -A^T, skewhermitian.jl:23-26)
``hessenberg(A)``           :func:`hessenberg` -> :class:`Hessenberg` (hessenberg.jl:5-15)
``logabspfaffian(A)``       :func:`logabspfaffian` (pfaffian.jl:235-263)
``logabspfaffian!(A)``      :func:`logabspfaffian_` (in place)
``pfaffian(A)``             :func:`pfaffian` (real inputs: sign * exp(log|Pf|))
``eigvals(A)``              :func:`eigvals` (eigen.jl:2-6)
``rrule(logabspfaffian,A)`` :func:`logabspfaffian_rrule` (no reference counterpart)
==========================  =====================================================

Batched work goes through :class:`BatchPlan` (skew_batch_* in the C ABI).

Matrices live on the GPU in Julia's column-major layout.  A torch tensor ``T``
of shape (n, n) holds matrix ``A`` when ``T = A^T`` in torch's row-major sense
(``T[j, i] == A[i, j]``); :func:`to_device` and :func:`from_device` convert.
PyTorch is used only for device memory and streams; every computation runs in
libskewgpu's kernels, and there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from ._lib import SkewError, check

__all__ = [
    "SkewHermitian", "Hessenberg", "BatchPlan", "SkewError", "to_device", "from_device", "hessenberg",
    "logabspfaffian", "logabspfaffian_", "pfaffian", "eigvals", "logabspfaffian_rrule", "handle",
    "measure_fp64_peak", "eigen", "exp", "cis", "exp_rrule",
]

_lib.load()  # fail loudly at import if the CUDA library is missing


class _Handle:
    def __init__(self):
        h = ctypes.c_void_p()
        check(_lib.load().skew_create(ctypes.byref(h)), "skew_create")
        self.h = h
        self.stream = None

    def bind(self, stream: Optional[torch.cuda.Stream] = None) -> ctypes.c_void_p:
        s = stream if stream is not None else torch.cuda.current_stream()
        if self.stream != s.cuda_stream:
            check(_lib.load().skew_set_stream(self.h, ctypes.c_void_p(s.cuda_stream)), "skew_set_stream")
            self.stream = s.cuda_stream
        return self.h


_handles = {}


def handle(device: Optional[int] = None) -> _Handle:
    d = torch.cuda.current_device() if device is None else device
    if d not in _handles:
        with torch.cuda.device(d):
            _handles[d] = _Handle()
    return _handles[d]


# ---------------------------------------------------------------------------
# Tuning table of the current device's handle (skew_tuning_* in skewgpu.h)
# ---------------------------------------------------------------------------
def tuning_keys() -> list:
    """Names of the tuning keys."""
    out, i = [], 0
    while True:
        k = _lib.load().skew_tuning_key(i)
        if not k:
            return out
        out.append(k.decode())
        i += 1


def tuning_get(key: str):
    """The key's value (a list for bucket_edges)."""
    vals = (ctypes.c_int64 * 16)()
    cnt = ctypes.c_int(0)
    check(_lib.load().skew_tuning_get(handle().h, key.encode(), vals, 16, ctypes.byref(cnt)), f"tuning_get {key}")
    return list(vals[: cnt.value]) if key == "bucket_edges" else int(vals[0])


def tuning_set(key: str, value) -> None:
    """Set one key (an int, or a list for bucket_edges); raises SkewError if out of range."""
    if isinstance(value, (list, tuple)):
        arr = (ctypes.c_int64 * len(value))(*[int(v) for v in value])
        check(_lib.load().skew_tuning_set_list(handle().h, key.encode(), arr, len(value)), f"tuning_set {key}")
    else:
        check(_lib.load().skew_tuning_set(handle().h, key.encode(), int(value)), f"tuning_set {key}")


def tuning_reset() -> None:
    check(_lib.load().skew_tuning_reset(handle().h), "tuning_reset")


def tuning_load(path: str) -> None:
    check(_lib.load().skew_tuning_load(handle().h, os.fspath(path).encode()), "tuning_load")


def tuning_source() -> str:
    return _lib.load().skew_tuning_source(handle().h).decode()


class tuned:
    """Context manager: set tuning keys on the current device's handle, restore them on exit."""

    def __init__(self, **keys):
        self.keys = keys
        self.saved = {}

    def __enter__(self):
        for k, v in self.keys.items():
            self.saved[k] = tuning_get(k)
            tuning_set(k, v)
        return self

    def __exit__(self, *exc):
        for k, v in self.saved.items():
            tuning_set(k, v)
        return False


def _ptr(t: Optional[torch.Tensor]) -> ctypes.c_void_p:
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def to_device(A, device="cuda") -> torch.Tensor:
    """Host matrix -> device tensor holding it column-major (T = A^T row-major)."""
    A = np.asarray(A, dtype=np.float64)
    return torch.from_numpy(np.ascontiguousarray(A.T)).to(device)


def from_device(T: torch.Tensor) -> np.ndarray:
    return T.detach().cpu().numpy().T.copy()


class SkewHermitian:
    """A real skew-symmetric Float64 matrix on the GPU (column-major storage).

    ``SkewHermitian(A)`` verifies A == -A^T exactly like the reference
    constructor (skewhermitian.jl:23-26) and raises ``ValueError`` otherwise.
    """

    def __init__(self, data, check_skew: bool = True):
        if not isinstance(data, torch.Tensor):
            data = to_device(data)
        if data.dtype != torch.float64 or data.dim() != 2 or data.shape[0] != data.shape[1]:
            raise ValueError("SkewHermitian expects a square float64 matrix")
        if not data.is_cuda:
            data = data.cuda()
        self.data = data.contiguous()
        if check_skew and not bool(torch.equal(self.data, -self.data.T)):
            raise ValueError("Matrix is not skew-hermitian")

    @property
    def n(self) -> int:
        return self.data.shape[0]

    def copy(self) -> "SkewHermitian":
        return SkewHermitian(self.data.clone(), check_skew=False)

    def numpy(self) -> np.ndarray:
        return from_device(self.data)


def _as_skew(A) -> SkewHermitian:
    return A if isinstance(A, SkewHermitian) else SkewHermitian(A)


@dataclass
class Hessenberg:
    """Result of hessenberg(A): factors (reflectors below the subdiagonal, column
    major as in ``F.factors``), tau and the subdiagonal ``ev`` of H."""

    factors: torch.Tensor
    tau: torch.Tensor
    ev: torch.Tensor

    def H(self) -> np.ndarray:
        """Dense SkewHermTridiagonal(ev) on the host."""
        e = self.ev.cpu().numpy()
        n = len(e) + 1
        T = np.zeros((n, n))
        T[np.arange(1, n), np.arange(n - 1)] = e
        T[np.arange(n - 1), np.arange(1, n)] = -e
        return T


def _info_tensor(k: int = 1) -> torch.Tensor:
    return torch.zeros(k, dtype=torch.int32, device="cuda")


def hessenberg(A) -> Hessenberg:
    """LA.hessenberg(A::SkewHermitian) -- copy, then reduce in place on the GPU."""
    S = _as_skew(A).copy()
    n = S.n
    tau = torch.zeros(max(n - 1, 0), dtype=torch.float64, device="cuda")
    ev = torch.zeros(max(n - 1, 0), dtype=torch.float64, device="cuda")
    info = _info_tensor()
    h = handle().bind()
    check(_lib.load().skew_hessenberg_d(h, _ptr(S.data), n, n, _ptr(tau), _ptr(ev), _ptr(info)), "hessenberg")
    return Hessenberg(S.data, tau, ev)


def logabspfaffian_(A, check_skew: bool = False) -> Tuple[float, float]:
    """logabspfaffian!(A): in place, returns (log|Pf(A)|, sign)."""
    S = _as_skew(A) if not isinstance(A, torch.Tensor) else SkewHermitian(A, check_skew=False)
    n = S.n
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    info = _info_tensor()
    h = handle().bind()
    check(_lib.load().skew_logabspf_d(h, _ptr(S.data), n, n, ctypes.c_void_p(out.data_ptr()),
                                      ctypes.c_void_p(out.data_ptr() + 8), int(check_skew), _ptr(info)),
          "logabspfaffian")
    st = int(info.item())
    if st == _lib.SKEW_NOT_SKEW:
        raise ValueError("Pfaffian requires a skew-Hermitian matrix")
    lp, sg = out.tolist()
    return lp, sg


def _is_complex(A) -> bool:
    if isinstance(A, SkewHermitian):
        return False
    if isinstance(A, torch.Tensor):
        return A.is_complex()
    return np.iscomplexobj(A)


def logabspfaffian(A):
    """logabspfaffian(A) (pfaffian.jl:236, :246): (log|Pf(A)|, sign); A is not modified.
    Plain matrices are checked for exact skew-symmetry first (pfaffian.jl:255).
    Complex matrices must be skew-symmetric (A == -transpose(A)); they take the
    Parlett-Reid path and return (log|Pf(A)|, cis(phase)) (pfaffian.jl:193-233)."""
    if _is_complex(A):
        return logabspfaffian_complex(A)
    if isinstance(A, SkewHermitian):
        return logabspfaffian_(A.copy())
    S = SkewHermitian(A, check_skew=False)
    return logabspfaffian_(S.copy(), check_skew=True)


def pfaffian(A):
    """pfaffian(A) for real A, returned as sign * exp(log|Pf|) (pfaffian.jl:74-84);
    for complex skew-symmetric A the product of the Parlett-Reid pivots
    (pfaffian.jl:98-137)."""
    if _is_complex(A):
        return pfaffian_complex(A)
    lp, sg = logabspfaffian(A)
    return float(sg * np.exp(lp))


def logabspfaffian_rrule(A):
    """Forward (log|Pf|, sign) and a pullback: pullback(dlogpf) -> dA = dlogpf * 1/2 A^{-T}.

    Gradient convention: entries are treated as independent, so G = 1/2 A^{-T}; for a
    skew-constrained perturbation (A_ij += h, A_ji -= h) the derivative is
    G_ij - G_ji = (A^{-T})_ij.
    """
    S = _as_skew(A).copy()
    n = S.n
    G = torch.empty((n, n), dtype=torch.float64, device="cuda")
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    info = _info_tensor()
    h = handle().bind()
    check(_lib.load().skew_logabspf_grad_d(h, _ptr(S.data), n, n, ctypes.c_void_p(out.data_ptr()),
                                           ctypes.c_void_p(out.data_ptr() + 8), _ptr(G), n, _ptr(info)),
          "logabspfaffian_rrule")
    lp, sg = out.tolist()

    def pullback(dy: float = 1.0) -> torch.Tensor:
        return G * dy  # column-major storage, like every device matrix here

    return (lp, sg), pullback


def eigvals(A) -> np.ndarray:
    """eigvals(A::SkewHermitian{Float64}) (eigen.jl:2-6) -> complex numpy vector
    (0 + i*vals): for n <= 1024 in the reference's QR deflation order, above that
    sorted descending.  Raises where the reference's QR raises (skeweigen.jl:154)."""
    S = _as_skew(A).copy()
    n = S.n
    vals = torch.zeros(n, dtype=torch.float64, device="cuda")
    info = _info_tensor()
    h = handle().bind()
    check(_lib.load().skew_eigvals_d(h, _ptr(S.data), n, n, _ptr(vals), _ptr(info)), "eigvals")
    _info_ok(info, "eigvals")
    return 1j * vals.cpu().numpy()


def eigvals_irange(A, il: int, iu: int) -> np.ndarray:
    """eigvals(A::SkewHermitian{Float64}, il:iu) (eigen.jl:8-11, :57-64): the
    eigenvalues il..iu counted from the largest imaginary part, as 0 + i*vals."""
    S = _as_skew(A).copy()
    n = S.n
    vals = torch.zeros(max(iu - il + 1, 1), dtype=torch.float64, device="cuda")
    info = _info_tensor()
    h = handle().bind()
    check(_lib.load().skew_eigvals_irange_d(h, _ptr(S.data), n, n, il, iu, _ptr(vals), _ptr(info)), "eigvals_irange")
    return 1j * vals.cpu().numpy()[: iu - il + 1]


def eigvals_interval(A, vl: float, vh: float) -> np.ndarray:
    """eigvals(A::SkewHermitian, vl, vh) (eigen.jl:13-16, :36-41, :66-73): the
    eigenvalues with imaginary part in [vl, vh), descending; real or complex A."""
    h = handle().bind()
    info = _info_tensor()
    count = _info_tensor()
    if np.iscomplexobj(A):
        W = _skew_hermitian_complex(A)
        n = W.shape[0]
        vals = torch.zeros(max(n, 1), dtype=torch.float64, device="cuda")
        check(_lib.load().skew_eigvals_interval_z(h, _ptr(W), n, n, float(vl), float(vh), _ptr(vals), _ptr(count),
                                                  _ptr(info)), "eigvals_interval")
    else:
        S = _as_skew(A).copy()
        n = S.n
        vals = torch.zeros(max(n, 1), dtype=torch.float64, device="cuda")
        check(_lib.load().skew_eigvals_interval_d(h, _ptr(S.data), n, n, float(vl), float(vh), _ptr(vals),
                                                  _ptr(count), _ptr(info)), "eigvals_interval")
    m = int(count.item())
    return 1j * vals.cpu().numpy()[:m]


def _info_ok(info: torch.Tensor, where: str) -> int:
    st = int(info.item())
    if st == _lib.SKEW_NO_CONVERGENCE:
        raise RuntimeError("Maximum number of iterations reached, the algorithm didn't converge")
    return st


def eigen(A):
    """eigen(A::SkewHermitian{Float64}) (eigen.jl:75-97): (values, vectors) as numpy
    complex arrays; values in the reference's order, vectors = Vr + i Vi."""
    S = _as_skew(A).copy()
    n = S.n
    vals = torch.zeros(n, dtype=torch.float64, device="cuda")
    Vr = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    Vi = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    info = _info_tensor()
    h = handle().bind()
    check(_lib.load().skew_eigen_d(h, _ptr(S.data), n, n, _ptr(vals), _ptr(Vr), _ptr(Vi), n, _ptr(info)), "eigen")
    _info_ok(info, "eigen")
    return 1j * vals.cpu().numpy(), from_device(Vr) + 1j * from_device(Vi)


def svdvals(A) -> np.ndarray:
    """svdvals(A::SkewHermitian) (eigen.jl:110-117): singular values, descending.
    Real input: |imag(eigvals)|; complex skew-Hermitian: svdvals(Hermitian(i A))."""
    n = _square_n(A)
    S = torch.zeros(max(n, 1), dtype=torch.float64, device="cuda")
    info = _info_tensor()
    h = handle().bind()
    if _is_complex(A):
        W = _skew_hermitian_complex(A)
        check(_lib.load().skew_svdvals_z(h, _ptr(W), n, n, _ptr(S), _ptr(info)), "svdvals")
    else:
        X = _as_skew(A).copy()
        check(_lib.load().skew_svdvals_d(h, _ptr(X.data), n, n, _ptr(S), _ptr(info)), "svdvals")
    _info_ok(info, "svdvals")
    return S.cpu().numpy()[:n]


def svd(A):
    """svd(A::SkewHermitian) (eigen.jl:119-144): (U, S, Vt) with A = U diag(S) Vt, as
    LinearAlgebra.SVD(U, S, Vt); U and Vt complex.  The eigenvectors are sorted stably
    by |lambda| descending, S = |lambda| and V = -i U with the columns of negative
    lambda negated (complex input: the same rule on Hermitian(i A), as LinearAlgebra's
    svd of a Hermitian matrix)."""
    n = _square_n(A)
    S = torch.zeros(max(n, 1), dtype=torch.float64, device="cuda")
    info = _info_tensor()
    h = handle().bind()
    if _is_complex(A):
        W = _skew_hermitian_complex(A)
        U = torch.zeros((n, n), dtype=torch.complex128, device="cuda")
        V = torch.zeros((n, n), dtype=torch.complex128, device="cuda")
        check(_lib.load().skew_svd_z(h, _ptr(W), n, n, _ptr(S), _ptr(U), _ptr(V), n, _ptr(info)), "svd")
        _info_ok(info, "svd")
        Uh, Vh = from_device_complex(U), from_device_complex(V)
    else:
        X = _as_skew(A).copy()
        planes = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for _ in range(4)]
        check(_lib.load().skew_svd_d(h, _ptr(X.data), n, n, _ptr(S), *[_ptr(t) for t in planes], n, _ptr(info)),
              "svd")
        _info_ok(info, "svd")
        Ur, Ui, Vr, Vi = (from_device(t) for t in planes)
        Uh, Vh = Ur + 1j * Ui, Vr + 1j * Vi
    return Uh, S.cpu().numpy()[:n], Vh.conj().T


def schur(A):
    """schur(A::SkewHermitian{Float64}) (skewhermitian.jl:238-243): (T, Z, values) with
    T = Diagonal(values) as a dense complex matrix and Z the eigenvectors, A = Z T Z^H."""
    lam, Z = eigen(A)
    return np.diag(lam), Z, lam


def _square_n(A) -> int:
    if isinstance(A, SkewHermitian):
        return A.n
    shape = tuple(A.shape)
    if len(shape) != 2 or shape[0] != shape[1]:
        raise ValueError("a square matrix is required")
    return int(shape[0])


def exp(A) -> np.ndarray:
    """exp(A::SkewHermitian{Float64}) (exp.jl:3-35, :48), real n x n."""
    S = _as_skew(A).copy()
    n = S.n
    E = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    info = _info_tensor()
    h = handle().bind()
    check(_lib.load().skew_exp_d(h, _ptr(S.data), n, n, _ptr(E), n, _ptr(info)), "exp")
    _info_ok(info, "exp")
    return from_device(E)


def cis(A) -> np.ndarray:
    """cis(A::SkewHermitian{Float64}) = exp(iA) (exp.jl:99-110, :204), complex Hermitian."""
    S = _as_skew(A).copy()
    n = S.n
    C = torch.zeros((n, n, 2), dtype=torch.float64, device="cuda")  # column-major complex: C[j, i, :]
    info = _info_tensor()
    h = handle().bind()
    check(_lib.load().skew_cis_d(h, _ptr(S.data), n, n, _ptr(C), n, _ptr(info)), "cis")
    _info_ok(info, "cis")
    c = C.cpu().numpy()
    return (c[..., 0] + 1j * c[..., 1]).T.copy()


def exp_rrule(A):
    """Forward exp(A) and a pullback Cbar -> d<Cbar, exp(A)>/dA (Daleckii-Krein)."""
    Anp = _as_skew(A).numpy()
    E = exp(Anp)

    def pullback(Cbar) -> np.ndarray:
        S = SkewHermitian(Anp)
        n = S.n
        Cd = to_device(np.asarray(Cbar, dtype=np.float64))
        G = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        info = _info_tensor()
        h = handle().bind()
        check(_lib.load().skew_exp_vjp_d(h, _ptr(S.data), n, n, _ptr(Cd), _ptr(G), n, _ptr(info)), "exp_vjp")
        _info_ok(info, "exp_vjp")
        return from_device(G)

    return E, pullback


# matrix functions of exp.jl (skew_func_t)
FUNCS = {"exp": 0, "cos": 1, "sin": 2, "cosh": 3, "sinh": 4, "tan": 5, "tanh": 6, "cot": 7, "coth": 8, "log": 9}


def matrix_function(A, name: str):
    """Base.<name>(A::SkewHermitian) for name in exp, cos, sin, cosh, sinh, tan, tanh,
    cot, coth, log (exp.jl:3-283): real n x n for a real skew matrix, ComplexF64 for a
    complex skew-Hermitian one.  Raises ValueError where the reference throws
    (log / cot / coth of a matrix with a zero eigenvalue)."""
    f = FUNCS[name]
    h = handle().bind()
    info = _info_tensor()
    if np.iscomplexobj(A) or (isinstance(A, torch.Tensor) and A.is_complex()):
        W = _skew_hermitian_complex(A)
        n = W.shape[0]
        F = torch.zeros((n, n), dtype=torch.complex128, device="cuda")
        check(_lib.load().skew_func_z(h, _ptr(W), n, n, f, _ptr(F), n, _ptr(info)), name)
        out = from_device_complex(F)
    else:
        S = _as_skew(A).copy()
        n = S.n
        F = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        check(_lib.load().skew_func_d(h, _ptr(S.data), n, n, f, _ptr(F), n, _ptr(info)), name)
        out = from_device(F)
    if int(info.item()) == _lib.SKEW_SINGULAR:
        raise ValueError(f"{name} of a singular matrix doesn't exist")
    return out


def sincos(A):
    """sincos(A::SkewHermitian) (exp.jl:206-245): (sin(A), cos(A))."""
    return matrix_function(A, "sin"), matrix_function(A, "cos")


class SkewHermTridiagonal:
    """SkewHermTridiagonal(ev) / SkewHermTridiagonal(ev, dvim) (tridiag.jl): the
    subdiagonal ev (real, or complex with the imaginary diagonal dvim) on the device."""

    def __init__(self, ev, dvim=None):
        ev = np.asarray(ev)
        self.complex = np.iscomplexobj(ev) or dvim is not None
        self.n = len(ev) + 1
        dt = torch.complex128 if self.complex else torch.float64
        self.ev = torch.from_numpy(np.ascontiguousarray(ev.astype(np.complex128 if self.complex else np.float64))).to(
            "cuda") if len(ev) else torch.zeros(1, dtype=dt, device="cuda")
        self.dvim = None if dvim is None else torch.from_numpy(np.asarray(dvim, dtype=np.float64)).cuda()

    def eigvals(self) -> np.ndarray:
        n = self.n
        vals = torch.zeros(n, dtype=torch.float64, device="cuda")
        info = _info_tensor()
        h = handle().bind()
        if self.complex:
            check(_lib.load().skew_tridiag_eigvals_z(h, _ptr(self.ev), _ptr(self.dvim), n, _ptr(vals), _ptr(info)),
                  "tridiag eigvals")
        else:
            check(_lib.load().skew_tridiag_eigvals_d(h, _ptr(self.ev), n, _ptr(vals), _ptr(info)), "tridiag eigvals")
        _info_ok(info, "tridiag eigvals")
        return 1j * vals.cpu().numpy()

    def eigen(self):
        n = self.n
        vals = torch.zeros(n, dtype=torch.float64, device="cuda")
        info = _info_tensor()
        h = handle().bind()
        if self.complex:
            V = torch.zeros((n, n), dtype=torch.complex128, device="cuda")
            check(_lib.load().skew_tridiag_eigen_z(h, _ptr(self.ev), _ptr(self.dvim), n, _ptr(vals), _ptr(V), n,
                                                   _ptr(info)), "tridiag eigen")
            return 1j * vals.cpu().numpy(), from_device_complex(V)
        Vr = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        Vi = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        check(_lib.load().skew_tridiag_eigen_d(h, _ptr(self.ev), n, _ptr(vals), _ptr(Vr), _ptr(Vi), n, _ptr(info)),
              "tridiag eigen")
        _info_ok(info, "tridiag eigen")
        return 1j * vals.cpu().numpy(), from_device(Vr) + 1j * from_device(Vi)

    def svdvals(self) -> np.ndarray:
        """svdvals!(::SkewHermTridiagonal) (tridiag.jl:526-530): descending."""
        n = self.n
        S = torch.zeros(n, dtype=torch.float64, device="cuda")
        info = _info_tensor()
        h = handle().bind()
        if self.complex:
            check(_lib.load().skew_tridiag_svdvals_z(h, _ptr(self.ev), _ptr(self.dvim), n, _ptr(S), _ptr(info)),
                  "tridiag svdvals")
        else:
            check(_lib.load().skew_tridiag_svdvals_d(h, _ptr(self.ev), n, _ptr(S), _ptr(info)), "tridiag svdvals")
        _info_ok(info, "tridiag svdvals")
        return S.cpu().numpy()

    def svd(self):
        """svd!(::SkewHermTridiagonal) (tridiag.jl:534-555): (U, S, Vt), A = U diag(S) Vt."""
        n = self.n
        S = torch.zeros(n, dtype=torch.float64, device="cuda")
        info = _info_tensor()
        h = handle().bind()
        if self.complex:
            U = torch.zeros((n, n), dtype=torch.complex128, device="cuda")
            V = torch.zeros((n, n), dtype=torch.complex128, device="cuda")
            check(_lib.load().skew_tridiag_svd_z(h, _ptr(self.ev), _ptr(self.dvim), n, _ptr(S), _ptr(U), _ptr(V), n,
                                                 _ptr(info)), "tridiag svd")
            _info_ok(info, "tridiag svd")
            Uh, Vh = from_device_complex(U), from_device_complex(V)
        else:
            planes = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for _ in range(4)]
            check(_lib.load().skew_tridiag_svd_d(h, _ptr(self.ev), n, _ptr(S), *[_ptr(t) for t in planes], n,
                                                 _ptr(info)), "tridiag svd")
            _info_ok(info, "tridiag svd")
            Ur, Ui, Vr, Vi = (from_device(t) for t in planes)
            Uh, Vh = Ur + 1j * Ui, Vr + 1j * Vi
        return Uh, S.cpu().numpy(), Vh.conj().T

    def function(self, name: str) -> np.ndarray:
        n = self.n
        F = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        info = _info_tensor()
        h = handle().bind()
        check(_lib.load().skew_tridiag_func_d(h, _ptr(self.ev), n, FUNCS[name], _ptr(F), n, _ptr(info)), name)
        if int(info.item()) == _lib.SKEW_SINGULAR:
            raise ValueError(f"{name} of a singular matrix doesn't exist")
        return from_device(F)


# ---------------------------------------------------------------------------
# ComplexF64 skew-Hermitian matrices
# ---------------------------------------------------------------------------
def to_device_complex(A, device="cuda") -> torch.Tensor:
    """Host complex matrix -> device complex128 tensor holding it column-major."""
    A = np.asarray(A, dtype=np.complex128)
    return torch.from_numpy(np.ascontiguousarray(A.T)).to(device)


def from_device_complex(T: torch.Tensor) -> np.ndarray:
    return T.detach().cpu().numpy().T.copy()


def _skew_hermitian_complex(A) -> torch.Tensor:
    """A copy of A on the device after the reference constructor's check
    A == -A^H (skewhermitian.jl:23-26)."""
    if isinstance(A, torch.Tensor):
        T = A.to(torch.complex128).cuda().clone()
        if not bool(torch.equal(T, -T.conj().T)):
            raise ValueError("Matrix is not skew-hermitian")
        return T
    A = np.asarray(A, dtype=np.complex128)
    if A.ndim != 2 or A.shape[0] != A.shape[1] or not np.array_equal(A, -A.conj().T):
        raise ValueError("Matrix is not skew-hermitian")
    return to_device_complex(A)


@dataclass
class HessenbergComplex:
    """hessenberg(A::SkewHermitian{ComplexF64}): factors (reflectors, column major,
    complex128), tau (complex), the real subdiagonal ev and dvim = imag(diag(H))."""

    factors: torch.Tensor
    tau: torch.Tensor
    ev: torch.Tensor
    dvim: torch.Tensor

    def H(self) -> np.ndarray:
        e = self.ev.cpu().numpy()
        d = self.dvim.cpu().numpy()
        n = len(d)
        T = np.diag(1j * d).astype(np.complex128)
        T[np.arange(1, n), np.arange(n - 1)] = e
        T[np.arange(n - 1), np.arange(1, n)] = -e
        return T


def hessenberg_complex(A) -> HessenbergComplex:
    """LA.hessenberg(A::SkewHermitian{ComplexF64}) on the GPU (copy, reduce in place)."""
    W = _skew_hermitian_complex(A)
    n = W.shape[0]
    tau = torch.zeros(max(n - 1, 0), dtype=torch.complex128, device="cuda")
    ev = torch.zeros(max(n - 1, 0), dtype=torch.float64, device="cuda")
    dvim = torch.zeros(n, dtype=torch.float64, device="cuda")
    info = _info_tensor()
    h = handle().bind()
    check(_lib.load().skew_hessenberg_z(h, _ptr(W), n, n, _ptr(tau), _ptr(ev), _ptr(dvim), _ptr(info)),
          "hessenberg_complex")
    return HessenbergComplex(W, tau, ev, dvim)


def eigvals_complex(A) -> np.ndarray:
    """eigvals(A::SkewHermitian{ComplexF64}) (eigen.jl:18-27): 0 + i*vals, vals descending."""
    W = _skew_hermitian_complex(A)
    n = W.shape[0]
    vals = torch.zeros(n, dtype=torch.float64, device="cuda")
    info = _info_tensor()
    h = handle().bind()
    check(_lib.load().skew_eigvals_z(h, _ptr(W), n, n, _ptr(vals), _ptr(info)), "eigvals_complex")
    return 1j * vals.cpu().numpy()


def eigen_complex(A):
    """eigen(A::SkewHermitian{ComplexF64}) (eigen.jl:101-106): (values, vectors)."""
    W = _skew_hermitian_complex(A)
    n = W.shape[0]
    vals = torch.zeros(n, dtype=torch.float64, device="cuda")
    V = torch.zeros((n, n), dtype=torch.complex128, device="cuda")
    info = _info_tensor()
    h = handle().bind()
    check(_lib.load().skew_eigen_z(h, _ptr(W), n, n, _ptr(vals), _ptr(V), n, _ptr(info)), "eigen_complex")
    return 1j * vals.cpu().numpy(), from_device_complex(V)


def exp_complex(A) -> np.ndarray:
    """exp(A::SkewHermitian{ComplexF64}) (exp.jl:37-46)."""
    W = _skew_hermitian_complex(A)
    n = W.shape[0]
    E = torch.zeros((n, n), dtype=torch.complex128, device="cuda")
    info = _info_tensor()
    h = handle().bind()
    check(_lib.load().skew_exp_z(h, _ptr(W), n, n, _ptr(E), n, _ptr(info)), "exp_complex")
    return from_device_complex(E)


def exp_complex_rrule(A):
    """Forward exp(A) and a pullback Cbar -> G with dL = Re tr(G^H dA) for
    L = Re tr(Cbar^H exp(A)) (Daleckii-Krein divided differences)."""
    E = exp_complex(A)
    Ah = np.asarray(A, dtype=np.complex128)

    def pullback(Cbar) -> np.ndarray:
        W = _skew_hermitian_complex(Ah)
        n = W.shape[0]
        Cd = to_device_complex(Cbar)
        G = torch.zeros((n, n), dtype=torch.complex128, device="cuda")
        info = _info_tensor()
        h = handle().bind()
        check(_lib.load().skew_exp_vjp_z(h, _ptr(W), n, n, _ptr(Cd), _ptr(G), n, _ptr(info)), "exp_vjp_complex")
        return from_device_complex(G)

    return E, pullback


def _stack_complex(mats) -> torch.Tensor:
    """count x n x n host complex matrices -> one device buffer, each matrix column-major."""
    arr = np.stack([np.asarray(M, dtype=np.complex128).T for M in mats])  # row-major of A^T = column-major A
    return torch.from_numpy(np.ascontiguousarray(arr)).cuda()


def _unstack_complex(T: torch.Tensor):
    return [m.T.copy() for m in T.cpu().numpy()]


def batch_eigen_complex(mats):
    """eigen for many ComplexF64 skew-Hermitian matrices of one size (skew_batch_eigen_z)."""
    for M in mats:
        M = np.asarray(M, dtype=np.complex128)
        if not np.array_equal(M, -M.conj().T):
            raise ValueError("Matrix is not skew-hermitian")
    A = _stack_complex(mats)
    count, n = A.shape[0], A.shape[1]
    vals = torch.zeros((count, n), dtype=torch.float64, device="cuda")
    V = torch.zeros((count, n, n), dtype=torch.complex128, device="cuda")
    st = torch.zeros(count, dtype=torch.int32, device="cuda")
    h = handle().bind()
    check(_lib.load().skew_batch_eigen_z(h, _ptr(A), n, count, _ptr(vals), _ptr(V), _ptr(st)), "batch_eigen_complex")
    return [1j * v for v in vals.cpu().numpy()], _unstack_complex(V)


def batch_exp_complex(mats):
    A = _stack_complex(mats)
    count, n = A.shape[0], A.shape[1]
    E = torch.zeros_like(A)
    h = handle().bind()
    check(_lib.load().skew_batch_exp_z(h, _ptr(A), n, count, _ptr(E), None), "batch_exp_complex")
    return _unstack_complex(E)


def batch_exp_vjp_complex(mats, cots):
    A = _stack_complex(mats)
    C = _stack_complex(cots)
    count, n = A.shape[0], A.shape[1]
    G = torch.zeros_like(A)
    h = handle().bind()
    check(_lib.load().skew_batch_exp_vjp_z(h, _ptr(A), n, count, _ptr(C), _ptr(G), None), "batch_exp_vjp_complex")
    return _unstack_complex(G)


# ---------------------------------------------------------------------------
# Complex skew-symmetric Pfaffian (pfaffian.jl:98-137, :193-233)
# ---------------------------------------------------------------------------
def _complex_work(A) -> torch.Tensor:
    """A device copy of A (complex128, column-major storage)."""
    if isinstance(A, torch.Tensor):
        if A.dim() != 2 or A.shape[0] != A.shape[1]:
            raise ValueError("a square matrix is required")
        return A.to(torch.complex128).cuda().contiguous().clone()
    A = np.asarray(A, dtype=np.complex128)
    if A.ndim != 2 or A.shape[0] != A.shape[1]:
        raise ValueError("a square matrix is required")
    return to_device_complex(A)


def _pfz_info(info: torch.Tensor, where: str):
    st = int(info.item())
    if st == _lib.SKEW_NOT_SKEW:
        raise ValueError("Pfaffian requires a skew-symmetric matrix")
    if st not in (_lib.SKEW_OK, _lib.SKEW_SINGULAR):
        raise RuntimeError(f"{where}: {_lib.load().skew_status_string(st).decode()}")


def logabspfaffian_complex_(T: torch.Tensor, check_skew: bool = True):
    """logabspfaffian!(A) for a complex skew-symmetric device matrix (column-major
    storage), in place: (log|Pf(A)|, cis(phase)) with Pf(A) = cis(phase) exp(log|Pf|)."""
    n = T.shape[0]
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    info = _info_tensor()
    h = handle().bind()
    check(_lib.load().skew_logabspf_z(h, _ptr(T), n, n, _ptr(out), ctypes.c_void_p(out.data_ptr() + 8),
                                      int(check_skew), _ptr(info)), "logabspfaffian")
    _pfz_info(info, "logabspfaffian")
    lp, c, s_ = out.tolist()
    return lp, complex(c, s_)


def logabspfaffian_complex(A):
    """logabspfaffian(A::AbstractMatrix{ComplexF64}) (pfaffian.jl:193-233, :259-263)."""
    return logabspfaffian_complex_(_complex_work(A), check_skew=True)


def pfaffian_complex(A) -> complex:
    """pfaffian(A::AbstractMatrix{ComplexF64}) (pfaffian.jl:98-137, :160-164): the
    running product of the Parlett-Reid pivots."""
    T = _complex_work(A)
    n = T.shape[0]
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    info = _info_tensor()
    h = handle().bind()
    check(_lib.load().skew_pfaffian_z(h, _ptr(T), n, n, _ptr(out), 1, _ptr(info)), "pfaffian")
    _pfz_info(info, "pfaffian")
    re, im = out.tolist()
    return complex(re, im)


def batch_logabspfaffian_complex(mats, check_skew: bool = True):
    """logabspfaffian and pfaffian of many complex skew-symmetric matrices of one
    size (skew_batch_logabspf_z).  ``mats``: a list of host matrices, or a device
    tensor count x n x n holding each matrix column-major.  Returns numpy arrays
    (log|Pf|, cis(phase), Pf, status)."""
    A = mats if isinstance(mats, torch.Tensor) else _stack_complex(mats)
    count, n = A.shape[0], A.shape[1]
    lp = torch.zeros(count, dtype=torch.float64, device="cuda")
    ph = torch.zeros(count, dtype=torch.complex128, device="cuda")
    pf = torch.zeros(count, dtype=torch.complex128, device="cuda")
    st = torch.zeros(count, dtype=torch.int32, device="cuda")
    h = handle().bind()
    check(_lib.load().skew_batch_logabspf_z(h, _ptr(A), n, count, _ptr(lp), _ptr(ph), _ptr(pf), int(check_skew),
                                            _ptr(st)), "batch_logabspfaffian_complex")
    return lp.cpu().numpy(), ph.cpu().numpy(), pf.cpu().numpy(), st.cpu().numpy()


def batch_logabspfaffian_complex_host(A_host: torch.Tensor, check_skew: bool = True):
    """batch_logabspfaffian_complex on host memory (skew_batch_logabspf_host_z): ``A_host``
    is a page-locked complex128 CPU tensor count x n x n holding each matrix column-major;
    the kernels read it directly.  Returns numpy arrays (log|Pf|, cis(phase), Pf, status)."""
    if A_host.device.type != "cpu" or A_host.dtype != torch.complex128 or A_host.dim() != 3 \
            or not A_host.is_contiguous():
        raise ValueError("A_host must be a contiguous complex128 CPU tensor count x n x n")
    if not A_host.is_pinned():
        raise ValueError("A_host must be page-locked (pin_memory())")
    count, n = A_host.shape[0], A_host.shape[1]
    lp = torch.zeros(count, dtype=torch.float64)
    ph = torch.zeros(count, dtype=torch.complex128)
    pf = torch.zeros(count, dtype=torch.complex128)
    st = torch.zeros(count, dtype=torch.int32)
    h = handle().bind()
    check(_lib.load().skew_batch_logabspf_host_z(h, _ptr(A_host), n, count, _ptr(lp), _ptr(ph), _ptr(pf),
                                                 int(check_skew), _ptr(st)), "batch_logabspfaffian_complex_host")
    return lp.numpy(), ph.numpy(), pf.numpy(), st.numpy()


def measure_fp64_peak() -> float:
    t = ctypes.c_double()
    check(_lib.load().skew_measure_fp64_peak(handle().bind(), ctypes.byref(t)), "measure_fp64_peak")
    return t.value


def measure_fp64_pipes() -> dict:
    """DFMA against the FP64 tensor instruction (mma.sync f64), alone and with half the
    warps of one kernel on each (skew_measure_fp64_pipes), in TFLOP/s."""
    t = (ctypes.c_double * 5)()
    check(_lib.load().skew_measure_fp64_pipes(handle().bind(), t), "measure_fp64_pipes")
    return {"dfma": t[0], "mma_m8n8k4": t[1], "mma_m16n8k16": t[2], "half_dfma_half_m8n8k4": t[3],
            "half_dfma_half_m16n8k16": t[4]}


class BatchPlan:
    """A batch of real skew matrices of sizes ``sizes`` (skew_batch_plan_create).

    Inputs are passed as device tensors (column-major storage, one per matrix)."""

    def __init__(self, sizes: Sequence[int]):
        self.sizes = np.asarray(sizes, dtype=np.int64)
        self.count = len(self.sizes)
        arr = (ctypes.c_int64 * max(self.count, 1))(*self.sizes.tolist())
        p = ctypes.c_void_p()
        self._h = handle()
        check(_lib.load().skew_batch_plan_create(self._h.bind(), arr, self.count, ctypes.byref(p)),
              "skew_batch_plan_create")
        self.plan = p

    def close(self):
        if getattr(self, "plan", None) is not None and self.plan.value:
            _lib.load().skew_batch_plan_destroy(self.plan)
            self.plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def pointer_array(tensors: Sequence[torch.Tensor]) -> torch.Tensor:
        return torch.tensor([t.data_ptr() for t in tensors], dtype=torch.int64, device="cuda")

    def logabspfaffian(self, A_ptrs: torch.Tensor, grad_ptrs: Optional[torch.Tensor] = None,
                       logpf: Optional[torch.Tensor] = None, sign: Optional[torch.Tensor] = None,
                       status: Optional[torch.Tensor] = None):
        """Launch the batched log|Pf| (+ gradient) on the current stream.  A_ptrs /
        grad_ptrs are device int64 tensors of device pointers (see pointer_array)."""
        dev = "cuda"
        logpf = torch.empty(self.count, dtype=torch.float64, device=dev) if logpf is None else logpf
        sign = torch.empty(self.count, dtype=torch.float64, device=dev) if sign is None else sign
        status = torch.empty(self.count, dtype=torch.int32, device=dev) if status is None else status
        self._h.bind()
        check(_lib.load().skew_batch_logabspf_d(self.plan, _ptr(A_ptrs), _ptr(logpf), _ptr(sign), _ptr(grad_ptrs),
                                                _ptr(status)), "skew_batch_logabspf_d")
        return logpf, sign, status

    def packed_size(self) -> int:
        """Doubles in the packed layout of the batch (sum of n^2)."""
        return int((self.sizes * self.sizes).sum())

    def logabspfaffian_host(self, A_host: torch.Tensor, grad_host: Optional[torch.Tensor] = None,
                            logpf: Optional[torch.Tensor] = None, sign: Optional[torch.Tensor] = None,
                            status: Optional[torch.Tensor] = None):
        """log|Pf| (+ gradient) on host buffers (skew_batch_logabspf_host_d).  A_host and
        grad_host are page-locked float64 CPU tensors holding the matrices back to back
        (column-major, in plan order); the kernels read and write them directly.
        Returns host tensors (logpf, sign, status) once the results are in host memory."""
        total = self.packed_size()
        for name, t in (("A_host", A_host), ("grad_host", grad_host)):
            if t is None:
                continue
            if t.device.type != "cpu" or t.dtype != torch.float64 or not t.is_contiguous() or t.numel() != total:
                raise ValueError(f"{name} must be a contiguous float64 CPU tensor of {total} elements")
            if not t.is_pinned():
                raise ValueError(f"{name} must be page-locked (pin_memory())")
        logpf = torch.empty(self.count, dtype=torch.float64) if logpf is None else logpf
        sign = torch.empty(self.count, dtype=torch.float64) if sign is None else sign
        status = torch.empty(self.count, dtype=torch.int32) if status is None else status
        for name, t, dt in (("logpf", logpf, torch.float64), ("sign", sign, torch.float64),
                            ("status", status, torch.int32)):
            if t.device.type != "cpu" or t.dtype != dt or not t.is_contiguous() or t.numel() != self.count:
                raise ValueError(f"{name} must be a contiguous {dt} CPU tensor of {self.count} elements")
        self._h.bind()
        check(_lib.load().skew_batch_logabspf_host_d(self.plan, _ptr(A_host), _ptr(grad_host), _ptr(logpf),
                                                     _ptr(sign), _ptr(status)), "skew_batch_logabspf_host_d")
        return logpf, sign, status

    def eigen(self, A_ptrs, val_ptrs, vr_ptrs, vi_ptrs, status=None):
        status = torch.empty(self.count, dtype=torch.int32, device="cuda") if status is None else status
        self._h.bind()
        check(_lib.load().skew_batch_eigen_d(self.plan, _ptr(A_ptrs), _ptr(val_ptrs), _ptr(vr_ptrs), _ptr(vi_ptrs),
                                             _ptr(status)), "skew_batch_eigen_d")
        return status

    def exp(self, A_ptrs, out_ptrs, status=None):
        status = torch.empty(self.count, dtype=torch.int32, device="cuda") if status is None else status
        self._h.bind()
        check(_lib.load().skew_batch_exp_d(self.plan, _ptr(A_ptrs), _ptr(out_ptrs), _ptr(status)), "skew_batch_exp_d")
        return status

    def cis(self, A_ptrs, out_ptrs, status=None):
        status = torch.empty(self.count, dtype=torch.int32, device="cuda") if status is None else status
        self._h.bind()
        check(_lib.load().skew_batch_cis_d(self.plan, _ptr(A_ptrs), _ptr(out_ptrs), _ptr(status)), "skew_batch_cis_d")
        return status

    def func(self, A_ptrs, out_ptrs, name: str, status=None):
        """A matrix function (FUNCS: exp, cos, sin, ...) of every matrix (skew_batch_func_d)."""
        status = torch.empty(self.count, dtype=torch.int32, device="cuda") if status is None else status
        self._h.bind()
        check(_lib.load().skew_batch_func_d(self.plan, _ptr(A_ptrs), FUNCS[name], _ptr(out_ptrs), _ptr(status)),
              "skew_batch_func_d")
        return status

    def exp_vjp(self, A_ptrs, cot_ptrs, out_ptrs, status=None):
        status = torch.empty(self.count, dtype=torch.int32, device="cuda") if status is None else status
        self._h.bind()
        check(_lib.load().skew_batch_exp_vjp_d(self.plan, _ptr(A_ptrs), _ptr(cot_ptrs), _ptr(out_ptrs), _ptr(status)),
              "skew_batch_exp_vjp_d")
        return status

    def eigvals(self, A_ptrs: torch.Tensor, val_ptrs: torch.Tensor, status: Optional[torch.Tensor] = None):
        status = torch.empty(self.count, dtype=torch.int32, device="cuda") if status is None else status
        self._h.bind()
        check(_lib.load().skew_batch_eigvals_d(self.plan, _ptr(A_ptrs), _ptr(val_ptrs), _ptr(status)),
              "skew_batch_eigvals_d")
        return status
