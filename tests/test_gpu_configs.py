"""GPU parity on the five benchmark configurations, at their exact sizes and
seeded inputs (the generators are the ones bench.py times).

* plain method, n = 512: hessenberg, eigvals and logabspfaffian against the
  binary128 oracle (and the eigenvalue order against the FP64 restatement);
* single large dense, n = 8192 real and n = 4096 ComplexF64: every output on the
  leading 256 x 256 principal submatrix against the binary128 oracle, and the
  full-size outputs through size-independent checks computed on the device by
  cuSOLVER/cuBLAS (log|Pf| = 1/2 log|det A|, eigenvalues of Hermitian(iA),
  A V = V Lambda and V^H V = I for every eigenpair, |T|_F = |A|_F);
* batched uneven (4096 matrices, even n in [16, 256]): log|Pf|, sign and the
  gradient of every matrix against the FP64 restatement, a sample against
  binary128, eigenvalues in the reference's order;
* batched Pfaffian adjoint (1024 x n = 128): the gradient against the binary128
  Gauss-Jordan inverse on 8 matrices, central differences (h = 1e-6) on 32 skew
  pairs of every matrix (FP64) and of 16 matrices (binary128), each allowed its
  O(h^2) truncation error on top of the stated tolerance;
* exp adjoint (512 real matrices, n in {32, ..., 512}; 64 ComplexF64 n = 256): the
  gradient against the Frechet derivative L(A^H, C) (scipy's expm_frechet,
  Al-Mohy-Higham, independent of the eigendecomposition), exp against the oracle's
  FP64 restatement of skewexp!, and central differences.

Tolerances (stated per check): eigenvalues and log|Pf| 1e-11 relative (normwise for
eigenvalues), signs exactly equal, gradients 1e-8 relative normwise against the
binary128 / Frechet references and binary128 central differences; FP64 central
differences carry about 1e-9 of rounding noise and are held to 1e-6.
"""
import os

import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu

RTOL = 1e-11
GTOL = 1e-8
NTHREADS = os.cpu_count() or 1


def tridiag_dense(ev):
    n = len(ev) + 1
    T = np.zeros((n, n))
    T[np.arange(1, n), np.arange(n - 1)] = ev
    T[np.arange(n - 1), np.arange(1, n)] = -np.asarray(ev)
    return T


def check_real_against_quad(skewgpu, oracle, A):
    """hessenberg (ev entrywise, same reflector convention), eigvals and log|Pf| of
    a real skew matrix against the binary128 oracle."""
    n = A.shape[0]
    H = skewgpu.hessenberg(A)
    ev = H.ev.cpu().numpy()
    _, tq, evq = oracle.hessenberg(A, quad=True)
    np.testing.assert_allclose(ev, evq, atol=RTOL * np.abs(evq).max())
    assert np.array_equal(H.tau.cpu().numpy() != 0, tq != 0)
    vals = skewgpu.eigvals(A).imag
    vq, _ = oracle.eigvals(A, quad=True)
    np.testing.assert_allclose(np.sort(vals), np.sort(vq), atol=RTOL * np.abs(vq).max())
    lp, sg = skewgpu.logabspfaffian(A)
    rl, rs = oracle.logabspfaffian(A, quad=True)
    assert sg == rs
    assert abs(lp - rl) <= RTOL * max(1.0, abs(rl)), (n, lp, rl)
    return vals


# --- plain method, n = 512 ---------------------------------------------------------
def test_plain_n512(skewgpu, oracle):
    A = bench.dense_skew_input(512)
    vals = check_real_against_quad(skewgpu, oracle, A)
    vd, st = oracle.eigvals(A)  # FP64 restatement of skewtrieigvals!: the reference's order
    assert st == 0
    np.testing.assert_allclose(vals, vd, atol=RTOL * np.abs(vd).max())


# --- single large dense ------------------------------------------------------------
@pytest.fixture(scope="module")
def large_real():
    return bench.dense_skew_input(8192)


def test_large_real_leading_256(skewgpu, oracle, large_real):
    check_real_against_quad(skewgpu, oracle, np.ascontiguousarray(large_real[:256, :256]))


def test_large_real_n8192(skewgpu, large_real):
    import torch

    A = large_real
    n = A.shape[0]
    dA = torch.from_numpy(A).cuda()
    # log|Pf| and sign: Pf^2 = det, so log|Pf| = 1/2 log|det A| (cuSOLVER LU on the device)
    lp, sg = skewgpu.logabspfaffian(A)
    s, ld = torch.linalg.slogdet(dA)
    assert s.item() > 0 and sg in (-1.0, 1.0)
    assert abs(lp - 0.5 * ld.item()) <= RTOL * abs(ld.item())
    # hessenberg: orthogonal similarity keeps the Frobenius norm
    H = skewgpu.hessenberg(A)
    ev = H.ev.cpu().numpy()
    fa = np.linalg.norm(A)
    assert abs(np.sqrt(2.0 * np.sum(ev * ev)) - fa) <= 1e-13 * fa * np.sqrt(n)
    # eigenvalues against cuSOLVER's Hermitian solver on i A (eigvalsh ascending = -imag, descending)
    vals = np.sort(skewgpu.eigvals(A).imag)
    ref = np.sort(-torch.linalg.eigvalsh(1j * dA.to(torch.complex128)).cpu().numpy())
    np.testing.assert_allclose(vals, ref, atol=RTOL * np.abs(ref).max())


def test_large_real_eigen_n8192(skewgpu, large_real):
    """Every eigenpair of the n = 8192 matrix: residual and orthonormality."""
    import ctypes

    import torch

    n = large_real.shape[0]
    dA = skewgpu.to_device(large_real)
    work = dA.clone()
    vals = torch.empty(n, dtype=torch.float64, device="cuda")
    Vr = torch.empty((n, n), dtype=torch.float64, device="cuda")
    Vi = torch.empty_like(Vr)
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    L = skewgpu._lib.load()
    assert L.skew_eigen_d(skewgpu.handle().bind(), P(work), n, n, P(vals), P(Vr), P(Vi), n, P(info)) == 0
    torch.cuda.synchronize()
    assert info.item() == 0
    del work
    # device buffers are row-major views of the column-major matrices: A = dA.T, V = (Vr + i Vi).T
    At, Xr, Xi = dA.T, Vr.T, Vi.T
    lam = vals
    scale = lam.abs().max().item()
    # A (Xr + i Xi) = (Xr + i Xi) diag(i lam):  A Xr = -Xi lam,  A Xi = Xr lam
    r1 = (At @ Xr + Xi * lam).abs().max().item()
    r2 = (At @ Xi - Xr * lam).abs().max().item()
    assert max(r1, r2) <= 1e-12 * scale * np.sqrt(n), (r1, r2)
    G = Xr.T @ Xr + Xi.T @ Xi
    G.diagonal().sub_(1.0)
    o_re = G.abs().max().item()
    del G
    o_im = (Xr.T @ Xi - Xi.T @ Xr).abs().max().item()
    assert max(o_re, o_im) <= 1e-12 * np.sqrt(n), (o_re, o_im)


@pytest.fixture(scope="module")
def large_complex():
    A, _ = bench.dense_skewh_input(4096)
    return A


def test_large_complex_leading_256(skewgpu, oracle, large_complex):
    A = np.ascontiguousarray(large_complex[:256, :256])
    H = skewgpu.hessenberg_complex(A)
    _, _, evq, dvq = oracle.hessenberg_complex(A, quad=True)
    ev = H.ev.cpu().numpy()
    np.testing.assert_allclose(ev, evq, atol=RTOL * np.abs(evq).max())
    np.testing.assert_allclose(H.dvim.cpu().numpy(), dvq, atol=RTOL * np.abs(evq).max())
    vals = skewgpu.eigvals_complex(A).imag
    ref = np.sort(-np.linalg.eigvalsh(1j * A))[::-1]
    np.testing.assert_allclose(vals, ref, atol=RTOL * np.abs(ref).max())


def test_large_complex_n4096(skewgpu, large_complex):
    import torch

    A = large_complex
    n = A.shape[0]
    H = skewgpu.hessenberg_complex(A)
    ev = H.ev.cpu().numpy()
    dv = H.dvim.cpu().numpy()
    fa = np.linalg.norm(A)
    assert abs(np.sqrt(2.0 * np.sum(ev * ev) + np.sum(dv * dv)) - fa) <= 1e-13 * fa * np.sqrt(n)
    vals = skewgpu.eigvals_complex(A).imag
    ref = np.sort(-torch.linalg.eigvalsh(1j * torch.from_numpy(A).cuda()).cpu().numpy())[::-1]
    np.testing.assert_allclose(vals, ref, atol=RTOL * np.abs(ref).max())


# --- batched uneven: 4096 matrices, even n in [16, 256] ------------------------------
def test_batched_uneven_4096(skewgpu, oracle):
    import torch

    sizes = bench.workload_sizes()
    buf, offs = bench.packed_inputs(sizes)
    count = len(sizes)
    d_in = torch.from_numpy(buf).cuda()
    d_g = torch.full_like(d_in, np.nan)
    a_ptrs = torch.tensor((d_in.data_ptr() + 8 * offs).tolist(), dtype=torch.int64, device="cuda")
    g_ptrs = torch.tensor((d_g.data_ptr() + 8 * offs).tolist(), dtype=torch.int64, device="cuda")
    plan = skewgpu.BatchPlan(sizes)
    lp, sg, st = plan.logabspfaffian(a_ptrs, g_ptrs)
    torch.cuda.synchronize()
    lp, sg, st = lp.cpu().numpy(), sg.cpu().numpy(), st.cpu().numpy()
    G = d_g.cpu().numpy()
    assert (st == 0).all()
    rl, rs, rg = oracle.batch_logabspfaffian_grad_packed(buf, offs, sizes, NTHREADS)
    assert np.array_equal(sg, rs)
    assert (np.abs(lp - rl) <= RTOL * np.maximum(1.0, np.abs(rl))).all()
    for b in range(count):
        a, e = int(offs[b]), int(offs[b] + sizes[b] ** 2)
        assert np.abs(G[a:e] - rg[a:e]).max() <= GTOL * np.abs(rg[a:e]).max(), b
    # binary128 on a sample spread over every size bucket
    for b in np.linspace(0, count - 1, 16).astype(int):
        n = int(sizes[b])
        A = buf[offs[b]:offs[b] + n * n].reshape(n, n, order="F")
        ql, qs = oracle.logabspfaffian(A, quad=True)
        assert qs == sg[b] and abs(lp[b] - ql) <= RTOL * max(1.0, abs(ql))
        Gq = oracle.logabspfaffian_grad(A)
        Gb = G[offs[b]:offs[b] + n * n].reshape(n, n, order="F")
        assert np.abs(Gb - Gq).max() <= GTOL * np.abs(Gq).max()
    # eigenvalues of every matrix through the batched eigvals, in the reference's order
    voff = np.zeros(count, dtype=np.int64)
    voff[1:] = np.cumsum(sizes[:-1])
    vals = torch.zeros(int(sizes.sum()), dtype=torch.float64, device="cuda")
    v_ptrs = torch.tensor((vals.data_ptr() + 8 * voff).tolist(), dtype=torch.int64, device="cuda")
    est = plan.eigvals(a_ptrs, v_ptrs).cpu().numpy()
    V = vals.cpu().numpy()
    plan.close()
    assert set(np.unique(est)) <= {0, 8}
    for b in range(0, count, 8):
        n = int(sizes[b])
        A = buf[offs[b]:offs[b] + n * n].reshape(n, n, order="F")
        vd, ost = oracle.eigvals(A)
        v = V[voff[b]:voff[b] + n]
        assert (ost != 0) == (est[b] == 8), b
        np.testing.assert_allclose(v, vd, atol=RTOL * np.abs(vd).max())


# --- batched Pfaffian adjoint: 1024 x n = 128 ---------------------------------------
def test_pfaffian_adjoint_1024x128(skewgpu, oracle):
    import torch

    count, n = 1024, 128
    buf, w = bench.pfaffian_adjoint_inputs(count, n)
    offs = np.arange(count, dtype=np.int64) * n * n
    d_in = torch.from_numpy(buf).cuda()
    d_g = torch.empty_like(d_in)
    a_ptrs = torch.tensor((d_in.data_ptr() + 8 * offs).tolist(), dtype=torch.int64, device="cuda")
    g_ptrs = torch.tensor((d_g.data_ptr() + 8 * offs).tolist(), dtype=torch.int64, device="cuda")
    plan = skewgpu.BatchPlan([n] * count)
    lp, sg, st = plan.logabspfaffian(a_ptrs, g_ptrs)
    torch.cuda.synchronize()
    plan.close()
    lp, sg, st = lp.cpu().numpy(), sg.cpu().numpy(), st.cpu().numpy()
    G = d_g.cpu().numpy().reshape(count, n, n)  # row-major view of column-major G: G[b].T
    assert (st == 0).all()
    # the loss sum_i w_i log|Pf(A_i)| against the FP64 restatement
    rl, rs = oracle.batch_logabspfaffian_packed(buf, offs, np.full(count, n, dtype=np.int64), NTHREADS)
    assert np.array_equal(sg, rs)
    assert abs(np.dot(w, lp) - np.dot(w, rl)) <= RTOL * np.abs(w * rl).sum()
    # binary128 Gauss-Jordan gradient on 8 matrices
    for b in range(0, count, count // 8):
        A = buf[offs[b]:offs[b] + n * n].reshape(n, n, order="F")
        Gq = oracle.logabspfaffian_grad(A)
        assert np.abs(G[b].T - Gq).max() <= GTOL * np.abs(Gq).max(), b
    # central differences on 32 random skew pairs per matrix: d/dh log|Pf(A + h E_ij)| = G_ij - G_ji
    rng = np.random.default_rng(4)
    pairs = np.empty((count, 32, 2), dtype=np.int64)
    for b in range(count):
        i = rng.choice(n, 32)
        j = (i + rng.integers(1, n, 32)) % n  # j != i
        pairs[b, :, 0], pairs[b, :, 1] = i, j
    raw = G.reshape(count, n * n)  # raw[b, i + n j] = G_b(i, j) (column-major storage)
    an = np.take_along_axis(raw, pairs[:, :, 0] + n * pairs[:, :, 1], 1) - \
        np.take_along_axis(raw, pairs[:, :, 1] + n * pairs[:, :, 0], 1)
    # A central difference carries the truncation error h^2/6 |f'''(xi)|, and the third
    # derivative of log|Pf| along E is bounded by |A^{-1}|^3 |E|^3 ~ (2 S)^3 with S the
    # matrix's largest gradient entry (|1/2 A^{-T}|); for the rare ill-conditioned matrix
    # of the batch (S in the thousands) that term, not the gradient, dominates.
    h = 1e-6
    ns = np.full(count, n, dtype=np.int64)
    S = np.abs(an).max(axis=1)
    trunc = h * h * (2.0 * S) ** 3
    fd = oracle.batch_logabspfaffian_fd(buf, offs, ns, pairs, h=h, quad=False, nthreads=NTHREADS)
    err = np.abs(fd - an).max(axis=1)
    assert (err <= 1e-6 * S + trunc).all(), np.argmax(err / (1e-6 * S + trunc))
    pick = np.linspace(0, count - 1, 16).astype(int)
    sub = np.concatenate([buf[offs[b]:offs[b] + n * n] for b in pick])
    fq = oracle.batch_logabspfaffian_fd(sub, np.arange(16, dtype=np.int64) * n * n, ns[:16], pairs[pick], h=h,
                                        quad=True, nthreads=NTHREADS)
    for k, b in enumerate(pick):
        assert np.abs(fq[k] - an[b]).max() <= GTOL * S[b] + trunc[b], b


# --- exp adjoint: 512 real matrices n in {32, ..., 512}; 64 ComplexF64 n = 256 -------
def test_exp_adjoint_512_mixed(skewgpu, oracle):
    import scipy.linalg as sl
    import torch

    sizes, offs, buf, cot = bench.exp_adjoint_inputs(512)
    count = len(sizes)
    d_in = torch.from_numpy(buf).cuda()
    d_c = torch.from_numpy(cot).cuda()
    d_g = torch.full_like(d_in, np.nan)
    d_e = torch.full_like(d_in, np.nan)
    ptr = lambda t: torch.tensor((t.data_ptr() + 8 * offs).tolist(), dtype=torch.int64, device="cuda")  # noqa: E731
    plan = skewgpu.BatchPlan(sizes)
    st = plan.exp_vjp(ptr(d_in), ptr(d_c), ptr(d_g)).cpu().numpy()
    st2 = plan.exp(ptr(d_in), ptr(d_e)).cpu().numpy()
    torch.cuda.synchronize()
    plan.close()
    assert (st == 0).all() and (st2 == 0).all()
    G, E = d_g.cpu().numpy(), d_e.cpu().numpy()
    mat = lambda x, b: x[offs[b]:offs[b] + sizes[b] ** 2].reshape(sizes[b], sizes[b], order="F")  # noqa: E731
    # every n = 512 matrix, and two of every other size
    pick = [b for b in range(count) if sizes[b] == 512]
    for m in range(32, 512, 32):
        pick += [b for b in range(count) if sizes[b] == m][:2]
    assert len([b for b in pick if sizes[b] == 512]) >= 8
    for b in pick:
        A, C = mat(buf, b), mat(cot, b)
        _, Lf = sl.expm_frechet(A.T, C)  # gradient of <C, exp(A)> = L(A^T, C)
        assert np.abs(mat(G, b) - Lf).max() <= GTOL * np.abs(Lf).max(), (b, sizes[b])
    # exp against the oracle's FP64 restatement of skewexp! (the reference's algorithm)
    for b in [b for b in pick if sizes[b] <= 256][::3] + pick[:1]:
        Eo = oracle.expm(mat(buf, b))
        np.testing.assert_allclose(mat(E, b), Eo, atol=RTOL * np.sqrt(sizes[b]) * max(1.0, np.abs(Eo).max()))
    # central differences along skew pairs of one n = 512 matrix (FP64 expm; rounding ~1e-9)
    b = pick[0]
    A, C = mat(buf, b), mat(cot, b)
    Gb = mat(G, b)
    rng = np.random.default_rng(5)
    h = 1e-6
    for _ in range(4):
        i, j = rng.choice(sizes[b], 2, replace=False)
        Ap, Am = A.copy(), A.copy()
        Ap[i, j] += h
        Ap[j, i] -= h
        Am[i, j] -= h
        Am[j, i] += h
        fd = (np.sum(C * sl.expm(Ap)) - np.sum(C * sl.expm(Am))) / (2 * h)
        assert fd == pytest.approx(Gb[i, j] - Gb[j, i], rel=1e-6, abs=1e-6 * np.abs(Gb).max())


def test_exp_adjoint_complex_64x256(skewgpu):
    import scipy.linalg as sl

    mats, cots = bench.complex_exp_adjoint_inputs(64, 256)
    Gs = skewgpu.batch_exp_vjp_complex(mats, cots)
    Es = skewgpu.batch_exp_complex(mats)
    for b in range(0, 64, 4):
        A, C = mats[b], cots[b]
        Eref, Lf = sl.expm_frechet(A.conj().T, C)
        assert np.abs(Gs[b] - Lf).max() <= GTOL * np.abs(Lf).max(), b
        np.testing.assert_allclose(Es[b], Eref.conj().T, atol=RTOL * 16)
    # central differences along a skew-Hermitian direction of one matrix
    A, C = mats[0], cots[0]
    rng = np.random.default_rng(6)
    D = rng.standard_normal((256, 256)) + 1j * rng.standard_normal((256, 256))
    D = (D - D.conj().T) / 2
    h = 1e-6
    f = lambda X: np.real(np.sum(C.conj() * sl.expm(X)))  # noqa: E731
    fd = (f(A + h * D) - f(A - h * D)) / (2 * h)
    an = np.real(np.sum(Gs[0].conj() * D))
    assert abs(fd - an) <= 1e-6 * max(1.0, abs(an))
