"""Matrix functions of exp.jl (cos, sin, sincos, cosh, sinh, tan, tanh, cot, coth,
log, exp) for real skew and complex skew-Hermitian matrices, in the manner of the
reference's own exp.jl testset (runtests.jl:207-243): n in {1, 2, 10, 11}, dense
results of the standard matrix functions as the check (scipy here), log checked by
exp(log(A)) = A for even n or complex, tan/tanh/cot/coth where defined.
Tolerance: 1e-10 relative to the largest entry of the reference result; cos and
cosh must come out exactly Hermitian, sin/sinh/tan/tanh/cot/coth exactly skew.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-10


def skew(n, seed, complex_=False):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((n, n))
    if complex_:
        B = B + 1j * rng.standard_normal((n, n))
        return (B - B.conj().T) / 2
    return (B - B.T) / 2


def close(F, R):
    np.testing.assert_allclose(F, R, atol=TOL * max(1.0, np.abs(R).max()))


@pytest.mark.parametrize("complex_", [False, True])
@pytest.mark.parametrize("n", [1, 2, 10, 11])
def test_functions_vs_dense(skewgpu, n, complex_):
    import scipy.linalg as sl

    A = skew(n, 40 + n + 100 * complex_, complex_)
    F = lambda name: skewgpu.matrix_function(A, name)  # noqa: E731
    close(F("exp"), sl.expm(A))
    C, S = F("cos"), F("sin")
    close(C, sl.cosm(A))
    close(S, sl.sinm(A))
    np.testing.assert_array_equal(C, C.conj().T)  # Hermitian
    np.testing.assert_array_equal(S, -S.conj().T)  # skew
    s2, c2 = skewgpu.sincos(A)
    np.testing.assert_array_equal(s2, S)
    np.testing.assert_array_equal(c2, C)
    Sh, Ch = F("sinh"), F("cosh")
    close(Sh, sl.sinhm(A))
    close(Ch, sl.coshm(A))
    np.testing.assert_array_equal(Sh, -Sh.conj().T)
    np.testing.assert_array_equal(Ch, Ch.conj().T)
    if np.abs(np.linalg.det(sl.cosm(A))) > 1e-6:
        close(F("tan"), np.linalg.solve(sl.cosm(A), sl.sinm(A)))
    E2 = sl.expm(2 * A)
    I = np.eye(n)
    if np.abs(np.linalg.det(E2 + I)) > 1e-6:
        close(F("tanh"), np.linalg.solve(E2 + I, E2 - I))
    if complex_ or n % 2 == 0:
        L = F("log")
        close(sl.expm(L), A)
        if np.abs(np.linalg.det(sl.sinm(A))) > 1e-6:
            close(F("cot"), np.linalg.solve(sl.sinm(A), sl.cosm(A)))
        if np.abs(np.linalg.det(E2 - I)) > 1e-6:
            close(F("coth"), np.linalg.solve(E2 - I, E2 + I))


@pytest.mark.parametrize("name", ["log", "cot", "coth"])
def test_singular_raises(skewgpu, name):
    """Odd n has a zero eigenvalue: the reference throws DomainError (log) or a
    singular solve (cot, coth)."""
    with pytest.raises(ValueError):
        skewgpu.matrix_function(skew(5, 1), name)


def test_batch_functions(skewgpu):
    import scipy.linalg as sl
    import torch

    sizes = [4, 9, 40, 130, 200]
    mats = [skew(n, 500 + n) / np.sqrt(n) for n in sizes]
    plan = skewgpu.BatchPlan(sizes)
    devs = [skewgpu.to_device(A) for A in mats]
    for name, ref in (("cos", sl.cosm), ("sin", sl.sinm), ("sinh", sl.sinhm), ("exp", sl.expm)):
        outs = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for n in sizes]
        st = plan.func(plan.pointer_array(devs), plan.pointer_array(outs), name)
        torch.cuda.synchronize()
        assert (st.cpu().numpy() == 0).all()
        for b, A in enumerate(mats):
            close(skewgpu.from_device(outs[b]), ref(A))
    plan.close()
