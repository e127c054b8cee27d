"""SSOR-PCG with Eisenstat's trick on the GPU (ConjugateGradientSolverCSR_SSOR_Eisenstat,
solver/sparsesolver.cpp:726-995, and _Eisenstat_Rainbow, :1338-1645), through the C ABI,
against the oracle (itself pinned bit-exact to the reference on every golden fixture;
the fixture comparison runs in test_gpu_parity.py). Bar: iteration count within 2% of
the oracle's (at least +-1), solution within 1e-9 relative."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _close_K(K, K_o):
    return abs(K - K_o) <= max(1, int(np.ceil(0.02 * K_o)))


@pytest.mark.parametrize("dim,r,L", [(3, 2, 3), (2, 1, 7), (3, 1, 4), (2, 3, 4)])
def test_eisenstat_variants_match_oracle_on_lattice(cuda, dim, r, L):
    import simplefem_gb300 as S
    from oracle import oracle
    from simplefem_gb300 import workloads
    A, C, V = workloads.lattice_matrix(dim, r, L, 1)
    n = len(A) - 1
    b = workloads.uniform_vector(4321, n)
    diag = oracle.csr_diagonal(A, C, V)
    rb = oracle.rainbow(A, C)
    for om in (1.0, 1.4):
        K_o, x_o, _ = oracle.cg_eisenstat_rainbow(A, C, V, b, diag, rb, om, precision=1e-10)
        x = np.zeros(n); res = np.zeros(n)
        K = S.ConjugateGradientSolverCSR_Eisenstat_Rainbow(n, x, b, A, C, V, res, 1e-10, -3, diag, om, *rb)
        assert S.last_info()["status"] == 0
        assert _close_K(K, K_o), (om, K, K_o)
        assert np.linalg.norm(x - x_o) / np.linalg.norm(x_o) < 1e-9
        K_o, x_o, _ = oracle.cg_ssor_eisenstat(A, C, V, b, diag, om, precision=1e-10)
        x = np.zeros(n); res = np.zeros(n)
        K = S.ConjugateGradientSolverCSR_SSOR_Eisenstat(n, x, b, A, C, V, res, 1e-10, -3, diag, om)
        assert S.last_info()["status"] == 0
        assert _close_K(K, K_o), (om, K, K_o)
        assert np.linalg.norm(x - x_o) / np.linalg.norm(x_o) < 1e-9


def test_eisenstat_nonzero_initial_guess(cuda):
    import simplefem_gb300 as S
    from oracle import oracle
    g = load_golden("fem3d_p2_l3")
    n = len(g["A"]) - 1
    x0 = np.cos(np.arange(n))
    rb = (int(g["rb_nc"]), g["rb_F"], g["rb_B"], g["rb_R"])
    K_o, x_o, _ = oracle.cg_eisenstat_rainbow(g["A"], g["C"], g["V"], g["b"], g["diag"], rb, 1.0, x0=x0)
    x = x0.copy(); res = np.zeros(n)
    K = S.ConjugateGradientSolverCSR_Eisenstat_Rainbow(n, x, g["b"], g["A"], g["C"], g["V"], res, 1e-10, -3,
                                                       g["diag"], 1.0, *rb)
    assert _close_K(K, K_o)
    assert np.linalg.norm(x - x_o) / np.linalg.norm(x_o) < 1e-9


def test_zero_diagonal_rows_like_reference(cuda):
    """Rows whose given diagonal is 0 are skipped. The index-order variant also skips
    their columns everywhere and converges like the oracle; the Rainbow variant, as the
    reference, reads their never-written (NaN) technical values in its iteration sweeps
    and stops at once with a breakdown."""
    import simplefem_gb300 as S
    from oracle import oracle
    g = load_golden("lap5_n16")
    n = len(g["A"]) - 1
    diag = np.array(g["diag"]); diag[[5, 17, 100]] = 0.0
    K_o, x_o, _ = oracle.cg_ssor_eisenstat(g["A"], g["C"], g["V"], g["b"], diag, 1.0)
    x = np.zeros(n); res = np.array(g["b"])
    K = S.ConjugateGradientSolverCSR_SSOR_Eisenstat(n, x, g["b"], g["A"], g["C"], g["V"], res, 1e-10, -3, diag, 1.0)
    assert _close_K(K, K_o)
    assert np.linalg.norm(x - x_o) <= 1e-8 * np.linalg.norm(x_o)
    rb = oracle.rainbow(g["A"], g["C"])
    K_o, _, _ = oracle.cg_eisenstat_rainbow(g["A"], g["C"], g["V"], g["b"], diag, rb, 1.0)
    x = np.zeros(n); res = np.array(g["b"])
    K = S.ConjugateGradientSolverCSR_Eisenstat_Rainbow(n, x, g["b"], g["A"], g["C"], g["V"], res, 1e-10, -3, diag,
                                                       1.0, *rb)
    assert K == K_o == 0
    assert S.last_info()["status"] == 1          # FEEC_BREAKDOWN


def test_full_size_eisenstat_rainbow_cfg2_matches_oracle(cuda):
    """3D P2 refined 5 times (N = 274,625)."""
    import simplefem_gb300 as S
    from oracle import oracle
    from simplefem_gb300 import workloads
    A, C, V = workloads.lattice_matrix(3, 2, 5)
    n = len(A) - 1
    b = workloads.uniform_vector(2026, n)
    diag = oracle.csr_diagonal(A, C, V)
    rb = oracle.rainbow(A, C)
    oracle.set_threads(oracle.max_threads())
    K_o, x_o, _ = oracle.cg_eisenstat_rainbow(A, C, V, b, diag, rb, 1.0, precision=1e-10)
    x = np.zeros(n); res = np.zeros(n)
    K = S.ConjugateGradientSolverCSR_Eisenstat_Rainbow(n, x, b, A, C, V, res, 1e-10, -3, diag, 1.0, *rb)
    assert _close_K(K, K_o), (K, K_o)
    assert np.linalg.norm(x - x_o) / np.linalg.norm(x_o) < 1e-9


def test_resident_system_eisenstat_and_mode_check(cuda):
    """feec_system_solve runs both variants on a resident system in REFERENCE mode (same
    iterations and solution as the drop-in); other modes are rejected."""
    torch = cuda
    import simplefem_gb300 as S
    from oracle import oracle
    from simplefem_gb300 import workloads
    from simplefem_gb300.system import System
    A, C, V = workloads.lattice_matrix(3, 2, 3)
    n = len(A) - 1
    b = workloads.uniform_vector(7, n)
    diag = oracle.csr_diagonal(A, C, V)
    rb = oracle.rainbow(A, C)
    for method, layout in (("rainbow_eisenstat", "rainbow"), ("ssor_eisenstat", "ssor")):
        sysm = System(A, C, V)
        if layout == "rainbow":
            sysm.set_rainbow(diag, 1.0, *rb)
        else:
            sysm.set_ssor(diag, 1.0)
        x = torch.zeros(n, dtype=torch.float64, device="cuda")
        info = sysm.solve(torch.from_numpy(b).cuda(), x, method=method, mode="reference", precision=1e-10)
        xh = np.zeros(n); res = np.zeros(n)
        if layout == "rainbow":
            K = S.ConjugateGradientSolverCSR_Eisenstat_Rainbow(n, xh, b, A, C, V, res, 1e-10, -3, diag, 1.0, *rb)
        else:
            K = S.ConjugateGradientSolverCSR_SSOR_Eisenstat(n, xh, b, A, C, V, res, 1e-10, -3, diag, 1.0)
        assert info["status"] == 0 and info["iterations"] == K
        assert np.linalg.norm(x.cpu().numpy() - xh) <= 1e-12 * np.linalg.norm(xh)
        with pytest.raises(S.FeecError):
            sysm.solve(torch.from_numpy(b).cuda(), x, method=method, mode="fp64", precision=1e-10)
        sysm.close()
