"""Pfaffian of complex skew-symmetric matrices (A == -transpose(A)) on the GPU:
Parlett-Reid elimination with pivoting, pfaffian.jl:98-137 (pfaffian) and
:193-233 (logabspfaffian), through skew_logabspf_z / skew_pfaffian_z /
skew_batch_logabspf_z.

Checks, with the tolerances written in each test:
* the reference's own recipe (runtests.jl:406-420): integer complex entries,
  Pf against the exact Gaussian-rational Pfaffian, Pf^2 against det(A);
* log|Pf| within 1e-11 (relative, floor 1) and cis(phase) within 1e-11 of the
  oracle's restatement in binary128 (n <= 300), and of the FP64 restatement
  above that with the phase tolerance widened by 2e-14 n (the reference's own
  running-sum rounding); Pf(A)^2 = det(A) (slogdet) within 1e-11;
* both single-matrix paths (one CTA up to n = 128, the cooperative grid above),
  the batched kernel in shared memory and in global slots, and the per-matrix
  grid path for a few large matrices;
* zero Pfaffians (odd n, a zero row/column) -> (-Inf, 0), non-skew input ->
  ValueError / SKEW_NOT_SKEW, the reference's known answers.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def complex_int_skew(n, seed):
    rng = np.random.default_rng(seed)
    R = rng.integers(-10, 11, (n, n)) + 1j * rng.integers(-10, 11, (n, n))
    return (R - R.T) / 2


def complex_skew(n, seed, scale=None):
    rng = np.random.default_rng(seed)
    s = 1.0 / np.sqrt(max(n, 1)) if scale is None else scale
    R = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * s
    return (R - R.T) / 2


def _close(lp, ph, lq, pq, tol=1e-11, n=0):
    """log|Pf| relative (floor 1) and cis(phase) absolute.  Against the FP64
    restatement (n > 0) the phase tolerance grows by 2e-14 n: the reference sums
    the n/2 pivot angles and n/2 multiples of pi in one FP64 running sum, whose
    rounding grows with n (the library sums them compensated)."""
    assert abs(lp - lq) <= tol * max(1.0, abs(lq)), (lp, lq)
    assert abs(ph - pq) <= tol + 2e-14 * n, (ph, pq)


@pytest.mark.parametrize("n", [0, 1, 2, 3, 10, 20])
def test_reference_recipe_exact(skewgpu, oracle, n):
    """runtests.jl:406-420 with the same tolerances (and tighter ones on the exact value)."""
    for seed in range(3):
        A = complex_int_skew(n, 50 * n + seed)
        exact = complex(oracle.exact_pfaffian_complex(A.tolist()))
        pf = skewgpu.pfaffian(A)
        assert abs(pf - exact) <= 1e-13 * max(1.0, abs(exact))
        d = np.linalg.det(A) if n else 1.0
        assert abs(pf**2 - d) <= np.sqrt(np.finfo(float).eps) * max(1.0, abs(d))
        lp, ph = skewgpu.logabspfaffian(A)
        if exact == 0:
            assert lp == -np.inf and ph == 0
        else:
            assert abs(ph * np.exp(lp) - pf) <= 1e-13 * abs(pf)


@pytest.mark.parametrize("n", [2, 4, 16, 64, 96, 128, 130, 200, 256, 300, 601, 640])
def test_single_vs_oracle(skewgpu, oracle, n):
    A = complex_skew(n, 7 + n)
    lp, ph = skewgpu.logabspfaffian(A)
    quad = n <= 300
    lq, pq, pfq = oracle.pfaffian_complex(A, quad=quad)
    if n % 2:
        assert lp == -np.inf and ph == 0
        return
    _close(lp, ph, lq, pq, n=0 if quad else n)
    pf = skewgpu.pfaffian(A)
    assert abs(pf - pfq) <= 1e-11 * abs(pfq)
    sign, logdet = np.linalg.slogdet(A)
    assert abs(2 * lp - logdet) <= 1e-11 * max(1.0, abs(logdet))
    assert abs(ph**2 - sign) <= 1e-11


def test_single_large(skewgpu, oracle):
    """The cooperative-grid path at n = 1500 against the FP64 restatement and det."""
    n = 1500
    A = complex_skew(n, 99)
    lp, ph = skewgpu.logabspfaffian(A)
    lq, pq, _ = oracle.pfaffian_complex(A)
    _close(lp, ph, lq, pq, n=n)
    sign, logdet = np.linalg.slogdet(A)
    assert abs(2 * lp - logdet) <= 1e-11 * max(1.0, abs(logdet))
    assert abs(ph**2 - sign) <= 1e-11


def test_integer_pivot_ties_large(skewgpu, oracle):
    """Integer entries give many equal moduli in the pivot column (first maximum wins)."""
    for n in (64, 300):
        A = complex_int_skew(n, n)
        lp, ph = skewgpu.logabspfaffian(A)
        lq, pq, _ = oracle.pfaffian_complex(A, quad=(n <= 64))
        _close(lp, ph, lq, pq, n=0 if n <= 64 else n)


@pytest.mark.parametrize("n,count", [(8, 300), (64, 40), (150, 20), (170, 160), (200, 5), (33, 7)])
def test_batch(skewgpu, oracle, n, count):
    """Shared-memory (n <= ~164), global-slot (n = 170 x 160) and per-matrix grid
    (n = 200 x 5) batches against the FP64 restatement and the single call."""
    mats = [complex_skew(n, 1000 * n + b) for b in range(count)]
    lp, ph, pf, st = skewgpu.batch_logabspfaffian_complex(mats)
    for b in (range(count) if count <= 40 else range(0, count, 7)):
        lq, pq, pfq = oracle.pfaffian_complex(mats[b], quad=(n <= 64))
        if n % 2:
            assert lp[b] == -np.inf and ph[b] == 0 and pf[b] == 0 and st[b] == 5
            continue
        assert st[b] == 0
        _close(lp[b], ph[b], lq, pq, n=0 if n <= 64 else n)
        assert abs(pf[b] - pfq) <= 1e-11 * abs(pfq)
    if n % 2 == 0:
        l1, p1 = skewgpu.logabspfaffian(mats[0])
        _close(l1, p1, lp[0], ph[0], tol=1e-13)


def test_zero_pfaffian(skewgpu):
    """A zero row/column gives an exactly zero pivot column: (-Inf, 0), Pf = 0
    (pfaffian.jl:127-129, :226-228), in every path."""
    for n in (6, 64, 140, 400):
        A = complex_skew(n, n)
        z = n // 3
        A[z, :] = 0
        A[:, z] = 0
        lp, ph = skewgpu.logabspfaffian(A)
        assert lp == -np.inf and ph == 0
        assert skewgpu.pfaffian(A) == 0
        lpb, phb, pfb, st = skewgpu.batch_logabspfaffian_complex([A, A])
        assert np.all(lpb == -np.inf) and np.all(phb == 0) and np.all(pfb == 0) and np.all(st == 5)


def test_not_skew_symmetric(skewgpu):
    """isskewsymmetric (skewhermitian.jl:101-110) is checked first: a skew-Hermitian
    (not skew-symmetric) matrix, or a nonzero diagonal, is rejected."""
    for n in (4, 140, 300):
        R = complex_skew(n, 3)
        rng = np.random.default_rng(n)
        C = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        H = (C - C.conj().T) / 2  # skew-Hermitian, not skew-symmetric
        with pytest.raises(ValueError):
            skewgpu.logabspfaffian(H)
        B = R.copy()
        B[1, 1] = 1e-300j
        with pytest.raises(ValueError):
            skewgpu.pfaffian(B)
        lp, ph, pf, st = skewgpu.batch_logabspfaffian_complex([R, B])
        assert st[0] == 0 and st[1] == 1 and np.isnan(lp[1])


def test_known_answers(skewgpu):
    """runtests.jl:423 (Pf = -119000), :433 (Pf = 1), :426-430 (4x4 formula) as complex input."""
    import json
    import os

    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_known_answers.json")))["cases"]
    A = np.array(gold["issue49"]["A"], dtype=np.complex128)
    assert abs(skewgpu.pfaffian(A) - gold["issue49"]["pfaffian"]) <= 1e-9
    A = np.array(gold["issue121"]["A"], dtype=np.complex128)
    assert skewgpu.pfaffian(A) == 1
    lp, ph = skewgpu.logabspfaffian(A)
    assert lp == 0 and ph == 1
    rng = np.random.default_rng(8)
    for _ in range(10):
        a, b, c, d, e, f = rng.integers(-10, 11, 6)
        M = np.array([[0, a, b, c], [-a, 0, d, e], [-b, -d, 0, f], [-c, -e, -f, 0]], dtype=np.complex128)
        s = 2 - 1j
        assert abs(skewgpu.pfaffian(M * s) - (c * d - b * e + a * f) * s**2) <= 1e-12 * max(1, abs(c * d - b * e + a * f))


def test_real_input_agrees_with_real_path(skewgpu):
    """A real skew matrix through the complex path: |Pf| and the sign of the real path."""
    for n in (10, 100, 300):
        rng = np.random.default_rng(n)
        B = rng.standard_normal((n, n))
        A = (B - B.T) / 2
        lr, sr = skewgpu.logabspfaffian(A)
        lc, pc = skewgpu.logabspfaffian(A.astype(np.complex128))
        assert abs(lr - lc) <= 1e-11 * max(1.0, abs(lr))
        assert abs(pc - sr) <= 1e-11


def test_scaled_entries(skewgpu, oracle):
    """Entries of 1e-150 and 1e+150: log|Pf| shifts by (n/2) log(s), the phase not."""
    n = 80
    A = complex_skew(n, 5)
    l0, p0 = skewgpu.logabspfaffian(A)
    for s in (1e-150, 1e150):
        ls, ps = skewgpu.logabspfaffian(A * s)
        assert abs(ls - (l0 + n / 2 * np.log(s))) <= 1e-11 * abs(ls)
        assert abs(ps - p0) <= 1e-12


@pytest.mark.parametrize("n,count", [(8, 50), (64, 40), (170, 12), (33, 7), (200, 5)])
def test_batch_host_buffers(skewgpu, n, count):
    """skew_batch_logabspf_host_z: the same kernels reading page-locked host memory
    (shared-memory, global-slot and per-matrix grid paths, odd n) give bit-identical
    results to the device-resident call; a non-skew-symmetric matrix is reported in
    both (status SKEW_NOT_SKEW); pageable input is refused before any launch."""
    import ctypes

    import torch
    from skewgpu import _lib

    mats = [complex_skew(n, 3000 * n + b) for b in range(count)]
    if count > 3:
        mats[2] = mats[2].copy()
        mats[2][0, 1] += 1e-3  # no longer skew-symmetric
    lp, ph, pf, st = skewgpu.batch_logabspfaffian_complex(mats)
    host = np.ascontiguousarray(np.stack([m.T for m in mats]))  # column-major storage
    pinned = torch.from_numpy(host).pin_memory()
    lph, phh, pfh, sth = skewgpu.batch_logabspfaffian_complex_host(pinned)
    np.testing.assert_array_equal(sth, st)
    np.testing.assert_array_equal(lph, lp)
    np.testing.assert_array_equal(phh, ph)
    np.testing.assert_array_equal(pfh, pf)
    if count > 3:
        assert st[2] == 1
    with pytest.raises(ValueError):
        skewgpu.batch_logabspfaffian_complex_host(torch.from_numpy(host))
    out = np.zeros(count)
    rc = _lib.load().skew_batch_logabspf_host_z(skewgpu.handle().bind(), ctypes.c_void_p(host.ctypes.data), n,
                                                count, ctypes.c_void_p(out.ctypes.data), None, None, 1, None)
    assert rc == _lib.SKEW_BAD_ARG
