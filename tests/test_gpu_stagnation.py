"""Mixed precision on an operator too ill-conditioned for FP32 arithmetic (the 1D
Dirichlet Laplacian tridiag(-1, 2, -1) with N = 3000, condition number about 3.6e6,
so condition number times FP32 roundoff is about 0.2): the FP64 defect correction sees
that an FP32 inner solve gained less than half the digits it was asked for and
finishes the solve in FP64. Every entry point still reaches the requested true FP64
relative residual (1e-8, checked on the host) and reports fp64_fallback = 1; a well
conditioned operator (3D P2, 3 refinements) never falls back."""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

N = 3000
TOL = 1e-8
MAX_IT = 20 * N


def _laplace_1d(n):
    M = sp.diags([-np.ones(n - 1), 2.0 * np.ones(n), -np.ones(n - 1)], [-1, 0, 1]).tocsr()
    M.sort_indices()
    return M.indptr.astype(np.int32), M.indices.astype(np.int32), M.data.astype(np.float64), M


def _system(A, C, V, method):
    import simplefem_gb300 as S
    from simplefem_gb300.system import System
    n = len(A) - 1
    sysm = System(A, C, V)
    if method == "rainbow":
        mat = S.MatrixCSR(n, n, A, C, V)
        rb = S.Rainbow(mat)
        sysm.set_rainbow(mat.getDiagonal().raw(), 1.0, rb.num_colors, rb.F, rb.B, rb.R)
    return sysm


def _relres(M, b, x):
    return np.linalg.norm(b - M @ x) / np.linalg.norm(b)


@pytest.mark.parametrize("method", ["cg", "rainbow"])
def test_single_solve_falls_back_to_fp64(cuda, method):
    torch = cuda
    from simplefem_gb300 import workloads
    A, C, V, M = _laplace_1d(N)
    sysm = _system(A, C, V, method)
    b = workloads.uniform_vector(7, N)
    x = torch.zeros(N, dtype=torch.float64, device="cuda")
    info = sysm.solve(torch.from_numpy(b).cuda(), x, method=method, mode="mixed", precision=TOL, max_iter=MAX_IT)
    assert info["status"] == 0, info
    assert info["fp64_fallback"] == 1, info
    assert _relres(M, b, x.cpu().numpy()) <= TOL
    sysm.close()


def test_well_conditioned_stays_in_fp32(cuda):
    torch = cuda
    from simplefem_gb300 import workloads
    A, C, V = workloads.lattice_matrix(3, 2, 3, 0)
    n = len(A) - 1
    sysm = _system(A, C, V, "rainbow")
    b = workloads.uniform_vector(8, n)
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    info = sysm.solve(torch.from_numpy(b).cuda(), x, method="rainbow", mode="mixed", precision=1e-10)
    assert info["status"] == 0 and info["fp64_fallback"] == 0, info
    X = torch.zeros((2, n), dtype=torch.float64, device="cuda")
    B = torch.from_numpy(np.stack([b, -b])).cuda()
    infos = sysm.solve_batch(B, X, method="rainbow", mode="mixed", precision=1e-10)
    assert all(i["status"] == 0 and i["fp64_fallback"] == 0 for i in infos), infos
    sysm.close()


@pytest.mark.parametrize("method", ["cg", "rainbow"])
def test_batched_columns_fall_back_to_fp64(cuda, method):
    torch = cuda
    from simplefem_gb300 import workloads
    A, C, V, M = _laplace_1d(N)
    sysm = _system(A, C, V, method)
    Bh = np.stack([workloads.uniform_vector(20 + j, N) for j in range(3)])
    X = torch.zeros((3, N), dtype=torch.float64, device="cuda")
    infos = sysm.solve_batch(torch.from_numpy(Bh).cuda(), X, method=method, mode="mixed", precision=TOL,
                             max_iter=MAX_IT, rhs_per_team=2)
    Xh = X.cpu().numpy()
    for j in range(3):
        assert infos[j]["status"] == 0, infos[j]
        assert infos[j]["fp64_fallback"] == 1, infos[j]
        assert _relres(M, Bh[j], Xh[j]) <= TOL
    sysm.close()


def test_many_systems_and_graph_batch_fall_back_only_where_needed(cuda):
    torch = cuda
    from simplefem_gb300 import workloads
    from simplefem_gb300.system import Batch, solve_many
    A1, C1, V1, M1 = _laplace_1d(N)
    A2, C2, V2 = workloads.lattice_matrix(3, 2, 3, 0)
    n2 = len(A2) - 1
    M2 = sp.csr_matrix((V2, C2, A2), shape=(n2, n2))
    systems = [_system(A1, C1, V1, "rainbow"), _system(A2, C2, V2, "rainbow")]
    bh = [workloads.uniform_vector(31, N), workloads.uniform_vector(32, n2)]
    for use_graph in (False, True):
        bs = [torch.from_numpy(v).cuda() for v in bh]
        xs = [torch.zeros_like(v) for v in bs]
        if use_graph:
            bt = Batch(systems, bs, xs, method="rainbow", mode="mixed", precision=TOL, max_iter=MAX_IT)
            infos, _ = bt.run()
            bt.close()
        else:
            infos = solve_many(systems, bs, xs, method="rainbow", mode="mixed", precision=TOL, max_iter=MAX_IT)
        assert [i["status"] for i in infos] == [0, 0], infos
        if use_graph and infos[0]["inner_fp64"]:
            # the reusable batch measured FP64 inner iterations faster at creation
            assert [i["inner_fp64"] for i in infos] == [1, 1], infos
        else:
            assert [i["fp64_fallback"] for i in infos] == [1, 0], infos
        assert _relres(M1, bh[0], xs[0].cpu().numpy()) <= TOL
        assert _relres(M2, bh[1], xs[1].cpu().numpy()) <= TOL
    for s in systems:
        s.close()


def test_server_request_falls_back_to_fp64(cuda):
    from simplefem_gb300 import workloads
    from simplefem_gb300.serving import Server
    A, C, V, M = _laplace_1d(N)
    b = workloads.uniform_vector(41, N)
    A2, C2, V2 = workloads.lattice_matrix(3, 2, 3, 0)
    b2 = workloads.uniform_vector(42, len(A2) - 1)
    srv = Server(hbm_budget_bytes=10**9, slots=2, method="rainbow", mode="mixed")
    rid = srv.submit(A, C, V, b, TOL)
    rid2 = srv.submit(A2, C2, V2, b2, TOL)
    assert srv.wait(300)
    res = {r["id"]: r for r in srv.poll()}
    srv.close()
    assert res[rid]["status"] == 0, res[rid]
    assert res[rid]["fp64_fallback"] == 1, res[rid]
    assert _relres(M, b, res[rid]["x"]) <= TOL
    assert res[rid2]["status"] == 0 and res[rid2]["fp64_fallback"] == 0, res[rid2]
