"""Batched engine (one thread block per work item, K right-hand sides in lockstep):
every column reaches the requested true FP64 relative residual 1e-10 and agrees
with an exact solve to 1e-9; the multicolor preconditioner is the reference's
(iteration counts of the FP64 batched Rainbow solve match the single-system
solver's within 2%); mixed systems of different sizes in one launch."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

pytestmark = pytest.mark.gpu


def _prepared(dim, r, L, seed=0, method="rainbow"):
    import simplefem_gb300 as S
    from simplefem_gb300 import workloads
    from simplefem_gb300.system import System
    A, C, V = workloads.lattice_matrix(dim, r, L, seed)
    n = len(A) - 1
    mat = S.MatrixCSR(n, n, A, C, V)
    sysm = System(A, C, V)
    if method == "rainbow":
        rb = S.Rainbow(mat)
        sysm.set_rainbow(mat.getDiagonal().raw(), 1.0, rb.num_colors, rb.F, rb.B, rb.R)
    return sysm, sp.csr_matrix((V, C, A), shape=(n, n))


@pytest.mark.parametrize("method,mode,k", [("rainbow", "mixed", 4), ("rainbow", "mixed", 1), ("rainbow", "fp64", 2),
                                           ("cg", "mixed", 4), ("cg", "fp64", 1), ("rainbow", "mixed", 2),
                                           ("rainbow", "mixed", 8), ("cg", "mixed", 8)])
def test_batch_of_rhs_reaches_tolerance(cuda, method, mode, k):
    torch = cuda
    from simplefem_gb300 import workloads
    sysm, M = _prepared(3, 2, 3, method=method)
    n = sysm.n
    nrhs = 7
    Bh = np.stack([workloads.uniform_vector(100 + j, n) for j in range(nrhs)])
    B = torch.from_numpy(Bh).cuda()
    X = torch.zeros_like(B)
    infos = sysm.solve_batch(B, X, method=method, mode=mode, precision=1e-10, rhs_per_team=k)
    Xh = X.cpu().numpy()
    lu = sla.splu(M.tocsc())
    for j in range(nrhs):
        assert infos[j]["status"] == 0, (j, infos[j])
        relres = np.linalg.norm(Bh[j] - M @ Xh[j]) / np.linalg.norm(Bh[j])
        assert relres <= 1e-10, (j, relres)
        xs = lu.solve(Bh[j])
        assert np.linalg.norm(Xh[j] - xs) / np.linalg.norm(xs) < 1e-9
    sysm.close()


def test_batched_fp64_rainbow_iterations_match_single_solver(cuda):
    """Same preconditioner as the single-system Rainbow solver: FP64 iteration counts agree within 2%."""
    torch = cuda
    from simplefem_gb300 import workloads
    sysm, M = _prepared(3, 2, 3)
    n = sysm.n
    b = workloads.uniform_vector(5, n)
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    single = sysm.solve(torch.from_numpy(b).cuda(), x, method="rainbow", mode="fp64", precision=1e-10)
    X = torch.zeros((1, n), dtype=torch.float64, device="cuda")
    batched = sysm.solve_batch(torch.from_numpy(b[None, :]).cuda(), X, method="rainbow", mode="fp64",
                               precision=1e-10, rhs_per_team=1)[0]
    assert abs(batched["iterations"] - single["iterations"]) <= max(1, int(np.ceil(0.02 * single["iterations"])))
    assert torch.allclose(X[0], x, rtol=0, atol=1e-9 * float(x.abs().max()))
    sysm.close()


def test_nonzero_initial_guess_batch(cuda):
    torch = cuda
    from simplefem_gb300 import workloads
    sysm, M = _prepared(2, 2, 5, seed=3)
    n = sysm.n
    Bh = np.stack([workloads.uniform_vector(7 + j, n) for j in range(3)])
    X0 = np.stack([workloads.uniform_vector(70 + j, n) for j in range(3)])
    X = torch.from_numpy(X0.copy()).cuda()
    infos = sysm.solve_batch(torch.from_numpy(Bh).cuda(), X, method="rainbow", mode="mixed", precision=1e-10)
    Xh = X.cpu().numpy()
    for j in range(3):
        assert infos[j]["status"] == 0
        assert np.linalg.norm(Bh[j] - M @ Xh[j]) / np.linalg.norm(Bh[j]) <= 1e-10
    sysm.close()


def test_solve_many_uneven_systems(cuda):
    """Uneven systems (2D P1/P2, coefficient mass, refinements 2-6) in one launch."""
    torch = cuda
    from simplefem_gb300 import workloads
    from simplefem_gb300.system import solve_many
    specs = [(2, 1, 2, 11), (2, 2, 5, 12), (2, 1, 6, 13), (2, 2, 3, 14), (2, 1, 4, 15), (3, 1, 3, 16)]
    systems, mats, bs, xs = [], [], [], []
    for (d, r, L, seed) in specs:
        s, M = _prepared(d, r, L, seed)
        systems.append(s); mats.append(M)
        b = workloads.uniform_vector(seed, s.n)
        bs.append(torch.from_numpy(b).cuda())
        xs.append(torch.zeros(s.n, dtype=torch.float64, device="cuda"))
    infos = solve_many(systems, bs, xs, method="rainbow", mode="mixed", precision=1e-10)
    for i, M in enumerate(mats):
        b = bs[i].cpu().numpy(); x = xs[i].cpu().numpy()
        assert infos[i]["status"] == 0, (i, infos[i])
        assert np.linalg.norm(b - M @ x) / np.linalg.norm(b) <= 1e-10
    for s in systems:
        s.close()


def test_batch_column_equals_alone(cuda):
    """A column's result does not depend on the other columns it shares a team with
    (same solution within the 1e-9 solution tolerance; in practice bit-identical)."""
    torch = cuda
    from simplefem_gb300 import workloads
    sysm, M = _prepared(3, 1, 4)
    n = sysm.n
    Bh = np.stack([workloads.uniform_vector(300 + j, n) for j in range(4)])
    X4 = torch.zeros((4, n), dtype=torch.float64, device="cuda")
    sysm.solve_batch(torch.from_numpy(Bh).cuda(), X4, method="rainbow", mode="mixed", rhs_per_team=4)
    X1 = torch.zeros((1, n), dtype=torch.float64, device="cuda")
    sysm.solve_batch(torch.from_numpy(Bh[2:3].copy()).cuda(), X1, method="rainbow", mode="mixed", rhs_per_team=1)
    diff = float((X4[2] - X1[0]).norm() / X1[0].norm())
    assert diff <= 1e-9, diff
    sysm.close()


def test_graph_captured_batch_replays(cuda):
    """The reusable batch (CUDA-graph replay) solves uneven coefficient systems, and a
    second replay with new right-hand sides is as correct as the first."""
    torch = cuda
    from simplefem_gb300 import workloads
    from simplefem_gb300.system import Batch
    specs = [(2, 1, 3, 21), (2, 2, 4, 22), (2, 1, 5, 23), (2, 2, 3, 24), (2, 1, 6, 25), (2, 2, 5, 26)]
    systems, mats = [], []
    for (d, r, L, seed) in specs:
        s, M = _prepared(d, r, L, seed)
        systems.append(s); mats.append(M)
    bs = [torch.zeros(s.n, dtype=torch.float64, device="cuda") for s in systems]
    xs = [torch.zeros(s.n, dtype=torch.float64, device="cuda") for s in systems]
    batch = Batch(systems, bs, xs, method="rainbow", mode="mixed", precision=1e-10)
    for rep in range(2):
        for i, s in enumerate(systems):
            bs[i].copy_(torch.from_numpy(workloads.uniform_vector(500 * rep + i, s.n)))
            xs[i].zero_()
        infos, ms = batch.run()
        assert ms > 0
        for i, M in enumerate(mats):
            b = bs[i].cpu().numpy(); x = xs[i].cpu().numpy()
            assert infos[i]["status"] == 0
            assert np.linalg.norm(b - M @ x) / np.linalg.norm(b) <= 1e-10
    batch.close()
    for s in systems:
        s.close()


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_graph_batch_launch_finish_double_buffered(cuda, mode):
    """The two halves of a replay (feec_batch_launch / feec_batch_finish): two batches over
    separate right-hand sides of the same systems are in flight at once from one host
    thread, each reaches 1e-10 with the solution and iteration count of a synchronous
    replay of the same inputs, and a second launch before the finish or a finish without
    a launch is refused."""
    torch = cuda
    from simplefem_gb300 import _native, workloads
    from simplefem_gb300.system import Batch
    specs = [(2, 1, 4, 31), (2, 2, 3, 32), (2, 1, 5, 33), (2, 2, 4, 34)]
    systems, mats = [], []
    for (d, r, L, seed) in specs:
        s, M = _prepared(d, r, L, seed)
        systems.append(s); mats.append(M)

    def buffers(seed):
        bs = [torch.from_numpy(workloads.uniform_vector(seed + i, s.n)).cuda() for i, s in enumerate(systems)]
        return bs, [torch.zeros(s.n, dtype=torch.float64, device="cuda") for s in systems]

    (bs0, xs0), (bs1, xs1) = buffers(700), buffers(800)
    b0 = Batch(systems, bs0, xs0, method="rainbow", mode=mode, precision=1e-10)
    b1 = Batch(systems, bs1, xs1, method="rainbow", mode=mode, precision=1e-10)
    with pytest.raises(_native.FeecError):
        b0.finish()                                   # nothing launched yet
    b0.launch()
    with pytest.raises(_native.FeecError):
        b0.launch()                                   # the first replay is still pending
    b1.launch()
    infos0, ms0 = b0.finish()
    infos1, ms1 = b1.finish()
    assert ms0 > 0 and ms1 > 0
    got = [[x.cpu().numpy() for x in xs0], [x.cpu().numpy() for x in xs1]]
    # the same inputs through synchronous replays, one batch at a time
    for (bt, bs, xs, infos, x_async) in ((b0, bs0, xs0, infos0, got[0]), (b1, bs1, xs1, infos1, got[1])):
        for x in xs:
            x.zero_()
        infos_sync, _ = bt.run()
        for i, M in enumerate(mats):
            b = bs[i].cpu().numpy(); x_sync = xs[i].cpu().numpy()
            assert infos[i]["status"] == 0
            assert np.linalg.norm(b - M @ x_async[i]) / np.linalg.norm(b) <= 1e-10
            assert abs(infos[i]["iterations"] - infos_sync[i]["iterations"]) <= max(1, 0.02 * infos_sync[i]["iterations"])
            assert np.linalg.norm(x_async[i] - x_sync) <= 1e-9 * np.linalg.norm(x_sync)
    b0.close(); b1.close()
    for s in systems:
        s.close()


@pytest.mark.parametrize("mode,k,blocks", [("mixed", 4, 4), ("mixed", 2, 8), ("mixed", 1, 2), ("fp64", 2, 4),
                                           ("fp64", 1, 16), ("mixed", 8, 4)])
def test_cluster_teams_reach_tolerance(cuda, mode, k, blocks):
    """Cluster teams (2-16 blocks per work item, sums over distributed shared memory):
    every column reaches 1e-10 and agrees with an exact solve to 1e-9; FP64 iteration
    counts equal those of one-block teams within 2% (only the summation order differs)."""
    torch = cuda
    from simplefem_gb300 import workloads
    sysm, M = _prepared(2, 2, 5, seed=4)
    n = sysm.n
    nrhs = 6
    Bh = np.stack([workloads.uniform_vector(900 + j, n) for j in range(nrhs)])
    X = torch.zeros((nrhs, n), dtype=torch.float64, device="cuda")
    sysm.set_batch_config("rainbow", mode, rhs_per_team=k, team_blocks=blocks)
    infos = sysm.solve_batch(torch.from_numpy(Bh).cuda(), X, method="rainbow", mode=mode, precision=1e-10)
    assert all(i["grid_blocks"] % blocks == 0 for i in infos)
    sysm.set_batch_config("rainbow", mode, rhs_per_team=0)
    X1 = torch.zeros((nrhs, n), dtype=torch.float64, device="cuda")
    ref = sysm.solve_batch(torch.from_numpy(Bh).cuda(), X1, method="rainbow", mode=mode, precision=1e-10,
                           rhs_per_team=k)
    Xh = X.cpu().numpy()
    lu = sla.splu(M.tocsc())
    for j in range(nrhs):
        assert infos[j]["status"] == 0, (j, infos[j])
        assert np.linalg.norm(Bh[j] - M @ Xh[j]) / np.linalg.norm(Bh[j]) <= 1e-10
        xs = lu.solve(Bh[j])
        assert np.linalg.norm(Xh[j] - xs) / np.linalg.norm(xs) < 1e-9
        if mode == "fp64":
            a, b = infos[j]["iterations"], ref[j]["iterations"]
            assert abs(a - b) <= max(1, int(np.ceil(0.02 * b))), (a, b)
    sysm.close()


def test_autotuner_choice_is_used_and_correct(cuda):
    """The autotuner returns a valid configuration (cluster teams allowed when the batch
    has few work items), and solve_batch with rhs_per_team=0 runs it to 1e-10."""
    torch = cuda
    from simplefem_gb300 import workloads
    sysm, M = _prepared(2, 2, 6, seed=5)
    n = sysm.n
    for hint in (8, 0):
        cfg = sysm.tune_batch("rainbow", "mixed", nrhs_hint=hint)
        assert cfg["rhs_per_team"] in (1, 2, 4) and cfg["team_blocks"] in (1, 2, 4, 8, 16), cfg
        assert cfg["rhs_iters_per_s"] > 0
        if cfg["team_blocks"] == 1:
            assert cfg["team_threads"] in (128, 256, 512, 1024)
        nrhs = 8
        Bh = np.stack([workloads.uniform_vector(950 + j, n) for j in range(nrhs)])
        X = torch.zeros((nrhs, n), dtype=torch.float64, device="cuda")
        infos = sysm.solve_batch(torch.from_numpy(Bh).cuda(), X, method="rainbow", mode="mixed", precision=1e-10)
        Xh = X.cpu().numpy()
        for j in range(nrhs):
            assert infos[j]["status"] == 0
            assert np.linalg.norm(Bh[j] - M @ Xh[j]) / np.linalg.norm(Bh[j]) <= 1e-10
    sysm.close()


def test_batch_config_rejects_invalid(cuda):
    from simplefem_gb300 import FeecError
    sysm, _ = _prepared(2, 1, 3)
    for kw in (dict(rhs_per_team=3), dict(rhs_per_team=4, team_blocks=3), dict(rhs_per_team=4, team_blocks=32),
               dict(rhs_per_team=4, team_threads=100), dict(rhs_per_team=8, team_threads=1024),
               dict(rhs_per_team=16)):
        with pytest.raises(FeecError):
            sysm.set_batch_config("rainbow", "mixed", **kw)
    with pytest.raises(FeecError):
        sysm.set_batch_config("rainbow", "fp64", rhs_per_team=4)
    sysm.close()
