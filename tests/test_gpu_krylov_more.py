"""Conjugate residuals (both drivers), MINRES and the diagonally preconditioned Chebyshev
iteration on the GPU (solver/sparsesolver.cpp:1687-2590) through the C ABI, against the
oracle (pinned bit-exact to the reference on every golden fixture; the fixture comparison
runs in test_gpu_parity.py). Bar: iteration count within 2 % (at least +-1), solution
within max(1e-9, 2 x the oracle's own error against a dense solve) of the oracle's."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close_K(K, K_o):
    return abs(K - K_o) <= max(1, int(np.ceil(0.02 * K_o)))


def _bounds(A, C, V):
    """[0.99 lambda_min, 1.01 lambda_max] of D^-1 A by a dense eigensolve (small cases)."""
    n = len(A) - 1
    M = np.zeros((n, n))
    np.add.at(M, (np.repeat(np.arange(n), np.diff(A)), C), V)
    d = 1.0 / np.sqrt(np.diag(M))
    ev = np.linalg.eigvalsh(d[:, None] * M * d[None, :])
    return 0.99 * ev[0], 1.01 * ev[-1]


@pytest.mark.parametrize("dim,r,L", [(2, 1, 5), (3, 1, 3), (2, 2, 4), (3, 2, 2)])
def test_cr_minres_chebyshev_match_oracle(cuda, dim, r, L):
    import simplefem_gb300 as S
    from oracle import oracle
    from simplefem_gb300 import workloads
    A, C, V = workloads.lattice_matrix(dim, r, L, 5)
    n = len(A) - 1
    b = workloads.uniform_vector(91, n)
    diag = oracle.csr_diagonal(A, C, V)
    precon = 1.0 / diag
    lo, hi = _bounds(A, C, V)
    M = np.zeros((n, n))
    np.add.at(M, (np.repeat(np.arange(n), np.diff(A)), C), V)
    xs = np.linalg.solve(M, b)
    runs = {
        "cr": (lambda x, res: S.ConjugateResidualSolverCSR(n, x, b, A, C, V, res, 1e-10, -3),
               lambda: oracle.cr(A, C, V, b, precision=1e-10)),
        "crt": (lambda x, res: S.ConjugateResidualSolverCSR_textbook(n, x, b, A, C, V, res, 1e-10, -3),
                lambda: oracle.cr(A, C, V, b, precision=1e-10)),
        "minres": (lambda x, res: S.MINRESCSR(n, x, b, A, C, V, res, 1e-10, -3),
                   lambda: oracle.minres(A, C, V, b, precision=1e-10)),
        "cheb": (lambda x, res: S.ChebyshevIteration_DiagonalPreconditioner(n, x, b, A, C, V, res, 1e-10, -3,
                                                                            precon, lo, hi),
                 lambda: oracle.chebyshev(A, C, V, b, precon, lo, hi, precision=1e-10)),
    }
    for key, (gpu, ora) in runs.items():
        x = np.zeros(n); res = np.zeros(n)
        K = gpu(x, res)
        info = S.last_info()
        K_o, x_o, res_o = ora()
        assert info["status"] == 0, (key, info)
        assert _close_K(K, K_o), (key, K, K_o)
        own = np.linalg.norm(x_o - xs) / np.linalg.norm(xs)
        assert np.linalg.norm(x - x_o) / np.linalg.norm(x_o) <= max(1e-9, 2.0 * own), (key, own)
        assert np.linalg.norm(res - res_o) <= 1e-6 * np.linalg.norm(b), key


def test_minres_on_indefinite_operator(cuda):
    """MINRES's use case: a symmetric indefinite operator (the lattice operator shifted past
    its four lowest eigenvalues), where CG-type energies lose their sign."""
    import simplefem_gb300 as S
    from oracle import oracle
    from simplefem_gb300 import workloads
    A, C, V = workloads.lattice_matrix(2, 1, 4, 0)
    n = len(A) - 1
    M = np.zeros((n, n))
    np.add.at(M, (np.repeat(np.arange(n), np.diff(A)), C), V)
    ev = np.linalg.eigvalsh(M)
    shift = 0.5 * (ev[3] + ev[4])
    V2 = V.copy()
    for i in range(n):
        for k in range(A[i], A[i + 1]):
            if C[k] == i:
                V2[k] -= shift
    b = workloads.uniform_vector(3, n)
    x = np.zeros(n); res = np.zeros(n)
    K = S.MINRESCSR(n, x, b, A, C, V2, res, 1e-8, -3)
    K_o, x_o, _ = oracle.minres(A, C, V2, b, precision=1e-8)
    M2 = M - shift * np.eye(n)
    # an indefinite, ill-conditioned case: rounding differences grow, so the bar is looser;
    # like the reference, the solve may use all N iterations
    assert abs(K - K_o) <= max(2, int(np.ceil(0.05 * K_o))), (K, K_o)
    assert S.last_info()["status"] == (3 if K == n else 0)
    rel = np.linalg.norm(b - M2 @ x) / np.linalg.norm(b)
    rel_o = np.linalg.norm(b - M2 @ x_o) / np.linalg.norm(b)
    assert rel <= max(2e-8, 10.0 * rel_o), (rel, rel_o)
    assert np.allclose(res, b - M2 @ x, atol=1e-12 * np.linalg.norm(b) + 1e-14)
    assert K < n and rel <= 2e-8
    # CR meets a negative residual energy and stops with a breakdown, as the reference does
    x = np.zeros(n); res = np.zeros(n)
    Kc = S.ConjugateResidualSolverCSR(n, x, b, A, C, V2, res, 1e-8, -3)
    Kc_o, _, _ = oracle.cr(A, C, V2, b, precision=1e-8)
    assert S.last_info()["status"] == 1
    assert abs(Kc - Kc_o) <= 1, (Kc, Kc_o)


def test_zero_rhs_and_bad_csr(cuda):
    import simplefem_gb300 as S
    from simplefem_gb300 import _native, workloads
    A, C, V = workloads.lattice_matrix(2, 1, 3, 0)
    n = len(A) - 1
    for fn in (S.ConjugateResidualSolverCSR, S.MINRESCSR):
        x = np.zeros(n); res = np.zeros(n)
        assert fn(n, x, np.zeros(n), A, C, V, res, 1e-10, -3) == 0
        assert S.last_info()["status"] == 0 and np.all(x == 0)
    x = np.zeros(n); res = np.zeros(n)
    assert S.ChebyshevIteration_DiagonalPreconditioner(n, x, np.zeros(n), A, C, V, res, 1e-10, -3, np.ones(n),
                                                       0.1, 2.0) == 0
    Cb = C.copy(); Cb[5] = n + 7                        # column out of range: refused before any product
    info = _native.FeecSolveInfo()
    st = _native.gpu().feec_cr_csr(n, np.zeros(n), np.ones(n), A, Cb, V, np.zeros(n), 1e-10, -3, ctypes.byref(info))
    assert st == _native.FEEC_BADARG
