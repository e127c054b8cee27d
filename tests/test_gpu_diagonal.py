"""CG with a diagonal preconditioner on the GPU (ConjugateGradientSolverCSR_DiagonalPreconditioner,
solver/sparsesolver.cpp:221-416), through the C ABI, against the oracle (pinned bit-exact to
the reference on every golden fixture; the fixture comparison runs in test_gpu_parity.py).
Bar: iteration count within 2% (at least +-1), solution within 1e-9 relative."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _inv(d):
    return np.where(d != 0, 1.0 / np.where(d != 0, d, 1.0), 0.0)


def _close_K(K, K_o):
    return abs(K - K_o) <= max(1, int(np.ceil(0.02 * K_o)))


@pytest.mark.parametrize("dim,r,L", [(3, 2, 3), (2, 1, 7), (3, 3, 2), (2, 2, 6)])
def test_diagonal_precon_matches_oracle_on_lattice(cuda, dim, r, L):
    import simplefem_gb300 as S
    from oracle import oracle
    from simplefem_gb300 import workloads
    A, C, V = workloads.lattice_matrix(dim, r, L, 2)
    n = len(A) - 1
    b = workloads.uniform_vector(55, n)
    precon = _inv(oracle.csr_diagonal(A, C, V))
    K_o, x_o, _ = oracle.cg_diag(A, C, V, b, precon, precision=1e-10)
    x = np.zeros(n); res = np.zeros(n)
    K = S.ConjugateGradientSolverCSR_DiagonalPreconditioner(n, x, b, A, C, V, res, 1e-10, -3, precon)
    assert S.last_info()["status"] == 0
    assert _close_K(K, K_o), (K, K_o)
    assert np.linalg.norm(x - x_o) / np.linalg.norm(x_o) < 1e-9


def test_diagonal_precon_zero_entries_like_reference(cuda):
    """precon == 0 rows are skipped; as in the reference, their never-written (NaN)
    directions then enter the products of other rows and the solve breaks down at once."""
    import simplefem_gb300 as S
    from oracle import oracle
    g = load_golden("lap5_n16")
    n = len(g["A"]) - 1
    precon = _inv(g["diag"]); precon[[3, 40]] = 0.0
    K_o, _, _ = oracle.cg_diag(g["A"], g["C"], g["V"], g["b"], precon)
    x = np.zeros(n); res = np.array(g["b"])
    K = S.ConjugateGradientSolverCSR_DiagonalPreconditioner(n, x, g["b"], g["A"], g["C"], g["V"], res, 1e-10, -3,
                                                            precon)
    assert K == K_o == 0
    assert S.last_info()["status"] == 1          # FEEC_BREAKDOWN


def test_resident_system_diagonal_and_nonzero_guess(cuda):
    torch = cuda
    import simplefem_gb300 as S
    from oracle import oracle
    from simplefem_gb300 import workloads
    from simplefem_gb300.system import System
    A, C, V = workloads.lattice_matrix(3, 2, 3)
    n = len(A) - 1
    b = workloads.uniform_vector(8, n)
    x0 = np.sin(np.arange(n))
    precon = _inv(oracle.csr_diagonal(A, C, V))
    K_o, x_o, _ = oracle.cg_diag(A, C, V, b, precon, x0=x0, precision=1e-10)
    sysm = System(A, C, V)
    sysm.set_diagonal_precon(precon)
    x = torch.from_numpy(x0.copy()).cuda()
    info = sysm.solve(torch.from_numpy(b).cuda(), x, method="diagonal", mode="reference", precision=1e-10)
    assert info["status"] == 0 and _close_K(info["iterations"], K_o)
    assert np.linalg.norm(x.cpu().numpy() - x_o) / np.linalg.norm(x_o) < 1e-9
    with pytest.raises(S.FeecError):
        sysm.solve(torch.from_numpy(b).cuda(), x, method="diagonal", mode="fp64", precision=1e-10)
    sysm.close()
