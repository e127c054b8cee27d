"""GPU parity of the CUDA path against the reference's own outputs (golden fixtures)
and against the oracle at larger sizes. Every call goes through the C ABI.

Parity bar (FP64):
* SpMV: max |y_gpu - y_ref| <= 1e-13 * max |y_ref| (summation order differs);
* diagonal: identical bits;
* drop-in solvers (reference stopping rule): iteration count within 2% of the
  reference's (at least +-1 for short solves), and the solution as close to the
  reference's solution as the reference's own solution is to the exact one
  (never looser than 1e-9 relative);
* FP64 / mixed product modes: true relative residual <= the requested 1e-10 and
  solution error below 1e-9 against an exact solve.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu
NAMES = golden_names()


def exact_solution(g):
    n = len(g["A"]) - 1
    M = sp.csr_matrix((g["V"], g["C"], g["A"]), shape=(n, n))
    return sla.spsolve(M.tocsc(), g["b"]), M


@pytest.mark.parametrize("name", NAMES)
def test_spmv_matches_reference(cuda, name):
    from simplefem_gb300 import MatrixCSR
    g = load_golden(name)
    n = len(g["A"]) - 1
    y = np.empty(n)
    MatrixCSR(n, n, g["A"], g["C"], g["V"]).apply(y, g["b"], 0.7)
    ref = g["apply_out"]
    assert np.max(np.abs(y - ref)) <= 1e-13 * np.max(np.abs(ref))


@pytest.mark.parametrize("name", NAMES)
def test_diagonal_matches_reference(cuda, name):
    from simplefem_gb300 import MatrixCSR
    g = load_golden(name)
    n = len(g["A"]) - 1
    d = MatrixCSR(n, n, g["A"], g["C"], g["V"]).getDiagonal().raw()
    assert np.array_equal(d, g["diag"])


def _run_dropin(g, key):
    import simplefem_gb300 as S
    n = len(g["A"]) - 1
    x = np.zeros(n)
    res = np.array(g["b"], np.float64)
    prec = float(g["precision"])
    om = float(g[key + "_omega"])
    if key == "cg":
        K = S.ConjugateGradientSolverCSR(n, x, g["b"], g["A"], g["C"], g["V"], res, prec, -3)
    elif key == "cr":
        K = S.ConjugateResidualSolverCSR(n, x, g["b"], g["A"], g["C"], g["V"], res, prec, -3)
    elif key == "crt":
        K = S.ConjugateResidualSolverCSR_textbook(n, x, g["b"], g["A"], g["C"], g["V"], res, prec, -3)
    elif key == "minres":
        K = S.MINRESCSR(n, x, g["b"], g["A"], g["C"], g["V"], res, prec, -3)
    elif key == "cheb":
        d = g["diag"]
        precon = np.where(d != 0, 1.0 / np.where(d != 0, d, 1.0), 0.0)
        K = S.ChebyshevIteration_DiagonalPreconditioner(n, x, g["b"], g["A"], g["C"], g["V"], res, prec, -3, precon,
                                                        float(g["cheb_lower"]), float(g["cheb_upper"]))
    elif key == "jac":
        d = g["diag"]
        precon = np.where(d != 0, 1.0 / np.where(d != 0, d, 1.0), 0.0)
        K = S.ConjugateGradientSolverCSR_DiagonalPreconditioner(n, x, g["b"], g["A"], g["C"], g["V"], res, prec, -3,
                                                               precon)
    elif key.startswith("ssor"):
        K = S.ConjugateGradientSolverCSR_SSOR(n, x, g["b"], g["A"], g["C"], g["V"], res, prec, -3, g["diag"], om)
    elif key.startswith("eisrb"):
        K = S.ConjugateGradientSolverCSR_Eisenstat_Rainbow(n, x, g["b"], g["A"], g["C"], g["V"], res, prec, -3,
                                                           g["diag"], om, int(g["rb_nc"]), g["rb_F"], g["rb_B"],
                                                           g["rb_R"])
    elif key.startswith("eis"):
        K = S.ConjugateGradientSolverCSR_SSOR_Eisenstat(n, x, g["b"], g["A"], g["C"], g["V"], res, prec, -3,
                                                        g["diag"], om)
    else:
        K = S.ConjugateGradientSolverCSR_Rainbow(n, x, g["b"], g["A"], g["C"], g["V"], res, prec, -3, g["diag"], om,
                                                 int(g["rb_nc"]), g["rb_F"], g["rb_B"], g["rb_R"])
    return K, x, res, S.last_info()


@pytest.mark.parametrize("name", NAMES)
def test_dropin_solvers_match_reference(cuda, name):
    g = load_golden(name)
    xs, M = exact_solution(g)
    keys = [k[:-2] for k in g if k.endswith("_K")]
    tol = max(float(g["precision"]) * np.linalg.norm(g["b"]), 2.0 ** -26)
    for key in keys:
        K, x, res, info = _run_dropin(g, key)
        K_ref = int(g[key + "_K"])
        n = len(g["A"]) - 1
        # the reference stops at K = N without converging on the smallest Laplacians (Chebyshev);
        # conjugate residuals test "energy negative" before "energy small" (:1804-1812), so a
        # round-off negative energy at convergence ends the solve through the breakdown branch
        if key in ("cr", "crt") and info["status"] == 1:
            assert info["final_norm"] < tol, (key, info)
        else:
            assert info["status"] == (3 if K_ref == n else 0), (key, info)
        assert abs(K - K_ref) <= max(1, int(np.ceil(0.02 * K_ref))), (key, K, K_ref)
        x_ref = g[key + "_x"]
        own_err = np.linalg.norm(x_ref - xs) / np.linalg.norm(xs)
        diff = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
        assert diff <= max(1e-9, 2.0 * own_err), (key, diff, own_err)
        if key.startswith("eis"):
            # the Eisenstat drivers return the residual of the L-solved system; it satisfies
            # the reference's stopping rule |z.r| < tol^2 with z = r D (2 - omega) / omega
            om = float(g[key + "_omega"])
            zr = float(np.sum(res * res * g["diag"] * (2.0 - om) / om))
            assert abs(zr) < tol * tol * 1.0001, (key, zr, tol)
        elif key == "cheb":
            # as in the reference, x is the iterate before the one the residual belongs to
            assert np.linalg.norm(res - g[key + "_res"]) <= 1e-6 * np.linalg.norm(g["b"]) + 1e-12, key
        else:
            # the residual array is the recursive residual; it must describe x
            true_r = g["b"] - M @ x
            assert np.linalg.norm(res - true_r) <= 1e-6 * np.linalg.norm(g["b"]) + 1e-12


def test_dropin_nonzero_initial_guess_and_omega(cuda):
    import simplefem_gb300 as S
    from oracle import oracle
    g = load_golden("fem3d_p1_l3")
    n = len(g["A"]) - 1
    x0 = np.linspace(-1, 1, n)
    rb = (int(g["rb_nc"]), g["rb_F"], g["rb_B"], g["rb_R"])
    for om in (0.7, 1.5):
        K_o, x_o, _ = oracle.cg_rainbow(g["A"], g["C"], g["V"], g["b"], g["diag"], rb, om, x0=x0, precision=1e-10)
        x = x0.copy(); res = np.zeros(n)
        K = S.ConjugateGradientSolverCSR_Rainbow(n, x, g["b"], g["A"], g["C"], g["V"], res, 1e-10, -3, g["diag"], om,
                                                 *rb)
        assert abs(K - K_o) <= max(1, int(np.ceil(0.02 * K_o)))
        assert np.linalg.norm(x - x_o) / np.linalg.norm(x_o) < 1e-8


def test_zero_rhs_returns_immediately(cuda):
    """b = 0 and x0 = 0: the reference stops before the first iteration (K = 0)."""
    import simplefem_gb300 as S
    g = load_golden("lap5_n8")
    n = len(g["A"]) - 1
    x = np.zeros(n); res = np.zeros(n)
    K = S.ConjugateGradientSolverCSR(n, x, np.zeros(n), g["A"], g["C"], g["V"], res, 1e-10, -3)
    assert K == 0 and not np.any(x)


def test_nan_rhs_reports_breakdown(cuda):
    """Non-finite r.r takes the reference's breakdown branch (sparsesolver.cpp:148-151)."""
    import simplefem_gb300 as S
    g = load_golden("lap5_n8")
    n = len(g["A"]) - 1
    b = np.array(g["b"]); b[3] = np.nan
    x = np.zeros(n); res = np.zeros(n)
    K = S.ConjugateGradientSolverCSR(n, x, b, g["A"], g["C"], g["V"], res, 1e-10, -3)
    assert S.last_info()["status"] in (1, 2) and K == 0


def test_one_by_one_system(cuda):
    import simplefem_gb300 as S
    x = np.zeros(1); res = np.zeros(1)
    K = S.ConjugateGradientSolverCSR(1, x, np.array([3.0]), [0, 1], [0], [2.0], res, 1e-10, -3)
    assert K == 1 and abs(x[0] - 1.5) < 1e-15


def test_zero_diagonal_rows_are_skipped_like_reference(cuda):
    """Rows with diagonal 0 are skipped by the SSOR sweeps (sparsesolver.cpp:1094, 1106 ...)."""
    import simplefem_gb300 as S
    from oracle import oracle
    g = load_golden("lap5_n8")
    n = len(g["A"]) - 1
    diag = np.array(g["diag"]); diag[[5, 17]] = 0.0
    x = np.zeros(n); res = np.array(g["b"])
    K = S.ConjugateGradientSolverCSR_SSOR(n, x, g["b"], g["A"], g["C"], g["V"], res, 1e-10, -3, diag, 1.0)
    K_o, x_o, r_o = oracle.cg_ssor(g["A"], g["C"], g["V"], g["b"], diag, 1.0, precision=1e-10)
    assert abs(K - K_o) <= 1
    assert np.linalg.norm(x - x_o) <= 1e-8 * np.linalg.norm(x_o)


@pytest.mark.parametrize("dim,r,L", [(3, 2, 3), (2, 1, 7), (3, 1, 4)])
def test_rainbow_and_ssor_match_oracle_on_lattice(cuda, dim, r, L):
    import simplefem_gb300 as S
    from oracle import oracle
    from simplefem_gb300 import workloads
    A, C, V = workloads.lattice_matrix(dim, r, L)
    n = len(A) - 1
    b = workloads.uniform_vector(1234, n)
    diag = oracle.csr_diagonal(A, C, V)
    rb = oracle.rainbow(A, C)
    K_o, x_o, _ = oracle.cg_rainbow(A, C, V, b, diag, rb, 1.0, precision=1e-10)
    x = np.zeros(n); res = np.zeros(n)
    K = S.ConjugateGradientSolverCSR_Rainbow(n, x, b, A, C, V, res, 1e-10, -3, diag, 1.0, *rb)
    assert abs(K - K_o) <= max(1, int(np.ceil(0.02 * K_o)))
    assert np.linalg.norm(x - x_o) / np.linalg.norm(x_o) < 1e-9
    K_o, x_o, _ = oracle.cg_ssor(A, C, V, b, diag, 1.0, precision=1e-10)
    x = np.zeros(n); res = np.zeros(n)
    K = S.ConjugateGradientSolverCSR_SSOR(n, x, b, A, C, V, res, 1e-10, -3, diag, 1.0)
    assert abs(K - K_o) <= max(1, int(np.ceil(0.02 * K_o)))
    assert np.linalg.norm(x - x_o) / np.linalg.norm(x_o) < 1e-9


def _system(dim, r, L, method):
    from oracle import oracle
    from simplefem_gb300 import workloads
    from simplefem_gb300.system import System
    A, C, V = workloads.lattice_matrix(dim, r, L)
    sysm = System(A, C, V)
    diag = oracle.csr_diagonal(A, C, V)
    if method == "rainbow":
        nc, F, B, R = oracle.rainbow(A, C)
        sysm.set_rainbow(diag, 1.0, nc, F, B, R)
    elif method == "ssor":
        sysm.set_ssor(diag, 1.0)
    return sysm, (A, C, V)


@pytest.mark.parametrize("method", ["cg", "rainbow", "ssor"])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_product_modes_reach_true_residual(cuda, method, mode):
    torch = cuda
    from simplefem_gb300 import workloads
    sysm, (A, C, V) = _system(3, 2, 3, method)
    n = sysm.n
    b = workloads.uniform_vector(99, n)
    bt = torch.from_numpy(b).cuda()
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    info = sysm.solve(bt, x, method=method, mode=mode, precision=1e-10)
    assert info["status"] == 0, info
    xs = sla.spsolve(sp.csr_matrix((V, C, A), shape=(n, n)).tocsc(), b)
    xh = x.cpu().numpy()
    relres = np.linalg.norm(b - sp.csr_matrix((V, C, A), shape=(n, n)) @ xh) / np.linalg.norm(b)
    assert relres <= 1e-10 and info["true_relres"] <= 1e-10
    assert np.linalg.norm(xh - xs) / np.linalg.norm(xs) < 1e-9
    sysm.close()


def test_full_size_rainbow_cfg2_matches_oracle(cuda):
    """3D P2 refined 5 times (N = 274,625): iteration count within 2% of the oracle's
    and the same solution to 1e-9."""
    import simplefem_gb300 as S
    from oracle import oracle
    from simplefem_gb300 import workloads
    A, C, V = workloads.lattice_matrix(3, 2, 5)
    n = len(A) - 1
    b = workloads.uniform_vector(2025, n)
    diag = oracle.csr_diagonal(A, C, V)
    rb = oracle.rainbow(A, C)
    oracle.set_threads(oracle.max_threads())
    K_o, x_o, _ = oracle.cg_rainbow(A, C, V, b, diag, rb, 1.0, precision=1e-10)
    x = np.zeros(n); res = np.zeros(n)
    K = S.ConjugateGradientSolverCSR_Rainbow(n, x, b, A, C, V, res, 1e-10, -3, diag, 1.0, *rb)
    assert abs(K - K_o) <= max(1, int(np.ceil(0.02 * K_o)))
    assert np.linalg.norm(x - x_o) / np.linalg.norm(x_o) < 1e-9


def test_launch_counter_counts_kernels(cuda):
    from simplefem_gb300 import _native
    import simplefem_gb300 as S
    g = load_golden("lap5_n4")
    before = _native.gpu().feec_kernel_launches()
    n = len(g["A"]) - 1
    S.ConjugateGradientSolverCSR(n, np.zeros(n), g["b"], g["A"], g["C"], g["V"], np.zeros(n), 1e-10, -3)
    assert _native.gpu().feec_kernel_launches() > before


@pytest.mark.parametrize("name", ["fem3d_p2_l3", "fem2d_p1_l6", "fem2d_p3_l2_coef", "lap5_n32"])
def test_system_apply_sell_matches_reference(cuda, name):
    """Resident SpMV (SELL-32, FP64 and FP32 values) against MatrixCSR::apply's output."""
    torch = cuda
    from simplefem_gb300.system import System
    g = load_golden(name)
    n = len(g["A"]) - 1
    sysm = System(g["A"], g["C"], g["V"])
    x = torch.from_numpy(g["b"]).cuda()
    y = torch.empty(n, dtype=torch.float64, device="cuda")
    sysm.apply(x, y, 0.7)
    ref = g["apply_out"]
    assert np.max(np.abs(y.cpu().numpy() - ref)) <= 1e-13 * np.max(np.abs(ref))
    y32 = torch.empty(n, dtype=torch.float32, device="cuda")
    sysm.apply(x.float(), y32, 0.7)
    assert np.max(np.abs(y32.double().cpu().numpy() - ref)) <= 2e-6 * np.max(np.abs(ref))
    for lanes in (1, 4, 8):                      # CSR kernel through the launch-shape override
        sysm.set_launch(0, lanes)
        sysm.apply(x, y, 0.7)
        assert np.max(np.abs(y.cpu().numpy() - ref)) <= 1e-13 * np.max(np.abs(ref))
    sysm.close()


@pytest.mark.parametrize("method", ["ssor", "rainbow"])
def test_one_block_shared_memory_solver_matches_grid_solver(cuda, method):
    """Small systems run the reference-rule SSOR / Rainbow PCG in one block with the
    gathered vectors in shared memory; a launch-shape override sends the same solve to
    the grid-wide persistent kernel. Both follow the reference: same K (+-1), same x."""
    torch = cuda
    from simplefem_gb300 import workloads
    sysm, (A, C, V) = _system(2, 1, 6, method)
    n = sysm.n
    b = torch.from_numpy(workloads.uniform_vector(31, n)).cuda()
    xs = []
    infos = []
    for override in (False, True):
        if override:
            sysm.set_launch(16, 4)
        x = torch.zeros(n, dtype=torch.float64, device="cuda")
        infos.append(sysm.solve(b, x, method=method, mode="reference", precision=1e-10))
        xs.append(x.cpu().numpy())
    assert infos[0]["grid_blocks"] == 1 and infos[1]["grid_blocks"] == 16, infos
    assert infos[0]["status"] == 0 and infos[1]["status"] == 0
    assert abs(infos[0]["iterations"] - infos[1]["iterations"]) <= 1, infos
    assert np.linalg.norm(xs[0] - xs[1]) / np.linalg.norm(xs[1]) < 1e-11
    sysm.close()
