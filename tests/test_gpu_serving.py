"""Serving loop (continuous batching): mixed-size requests overlap on the device, each
reaches its requested true FP64 relative residual, the device memory budget is
respected, and a request's result is the same alone and in a mix (tolerance: 1e-9
relative in the solution, the solution tolerance of the other GPU tests)."""
import time

import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

SPECS = [(2, 1, 4, 1), (3, 2, 3, 2), (2, 3, 3, 3), (3, 1, 4, 4), (2, 2, 6, 5), (3, 2, 4, 6), (2, 1, 7, 7),
         (3, 3, 2, 8), (2, 2, 4, 9), (3, 1, 5, 10)]


def _problem(dim, r, L, seed):
    from simplefem_gb300 import workloads
    A, C, V = workloads.lattice_matrix(dim, r, L, seed)
    b = workloads.uniform_vector(1000 + seed, len(A) - 1)
    return A, C, V, b


def _relres(A, C, V, b, x):
    n = len(A) - 1
    M = sp.csr_matrix((V, C, A), shape=(n, n))
    return np.linalg.norm(b - M @ x) / np.linalg.norm(b)


@pytest.mark.parametrize("method,mode", [("rainbow", "mixed"), ("cg", "fp64")])
def test_mixed_sizes_all_reach_tolerance(cuda, method, mode):
    from simplefem_gb300.serving import Server
    srv = Server(hbm_budget_bytes=40 * 10**9, slots=6, method=method, mode=mode)
    probs = {}
    tols = [1e-8, 1e-10, 1e-12]
    for i, spec in enumerate(SPECS):
        A, C, V, b = _problem(*spec)
        tol = tols[i % 3]
        rid = srv.submit(A, C, V, b, tol)
        probs[rid] = (A, C, V, b, tol)
    assert srv.wait(600)
    res = srv.poll()
    assert len(res) == len(SPECS)
    for r in res:
        A, C, V, b, tol = probs[r["id"]]
        assert r["status"] == 0, r
        assert _relres(A, C, V, b, r["x"]) <= tol, r
        assert r["true_relres"] <= tol
    srv.close()


def test_result_same_alone_and_in_mix(cuda):
    from simplefem_gb300.serving import Server
    A, C, V, b = _problem(3, 2, 4, 42)
    alone = Server(hbm_budget_bytes=10 * 10**9, slots=1)
    alone.submit(A, C, V, b, 1e-10)
    assert alone.wait(300)
    x_alone = alone.poll()[0]["x"]
    alone.close()
    mix = Server(hbm_budget_bytes=40 * 10**9, slots=8)
    ids = []
    for spec in SPECS[:5]:
        mix.submit(*_problem(*spec), 1e-10)
    target = mix.submit(A, C, V, b, 1e-10)
    for spec in SPECS[5:]:
        mix.submit(*_problem(*spec), 1e-10)
    assert mix.wait(600)
    res = {r["id"]: r for r in mix.poll()}
    x_mix = res[target]["x"]
    diff = np.linalg.norm(x_mix - x_alone) / np.linalg.norm(x_alone)
    assert diff <= 1e-9, diff
    assert _relres(A, C, V, b, x_mix) <= 1e-10
    mix.close()


def test_budget_limits_admission(cuda):
    """With a budget that holds about two of these requests, the bytes in use never
    exceed it, and every request still completes."""
    from simplefem_gb300.serving import Server
    probs = [_problem(3, 2, 4, s) for s in range(6)]
    srv = Server(hbm_budget_bytes=400 * 10**6, slots=6)
    for A, C, V, b in probs:
        srv.submit(A, C, V, b, 1e-10)
    seen = 0
    t_end = time.time() + 300
    while time.time() < t_end:
        st = srv.stats()
        assert st["bytes_in_use"] <= 400 * 10**6
        seen = max(seen, st["inflight"])
        if srv.wait(0.01):
            break
    assert srv.stats()["peak_bytes"] <= 400 * 10**6
    res = srv.poll()
    assert len(res) == 6 and all(r["status"] == 0 for r in res)
    srv.close()


def test_oversized_request_is_rejected(cuda):
    from simplefem_gb300 import FeecError
    from simplefem_gb300.serving import Server
    A, C, V, b = _problem(3, 2, 4, 1)
    srv = Server(hbm_budget_bytes=10**6, slots=1)
    with pytest.raises(FeecError):
        srv.submit(A, C, V, b, 1e-10)
    srv.close()


def _laplace_1d(n):
    """tridiag(-1, 2, -1): condition number about 3.6e6 at n = 3000, too ill-conditioned
    for FP32 arithmetic, so a mixed-precision request finishes in FP64."""
    M = sp.diags([-np.ones(n - 1), 2.0 * np.ones(n), -np.ones(n - 1)], [-1, 0, 1]).tocsr()
    M.sort_indices()
    return M.indptr.astype(np.int32), M.indices.astype(np.int32), M.data.astype(np.float64)


def test_whole_gpu_and_fp64_fallback_requests_same_alone_and_in_mix(cuda):
    """A request above the whole-GPU threshold (3D P1 refined 6 times, 4.0 M stored
    entries: the persistent solver on every SM) and one whose FP32 iterations stagnate
    (finished in FP64) give the same solution alone and in a mix of cluster requests,
    and each reaches its tolerance."""
    from simplefem_gb300 import workloads
    from simplefem_gb300.serving import Server
    big = _problem(3, 1, 6, 11)
    A1, C1, V1 = _laplace_1d(3000)
    b1 = workloads.uniform_vector(7, 3000)
    cases = [(big, 1e-10), ((A1, C1, V1, b1), 1e-8)]
    alone = []
    for prob, tol in cases:
        srv = Server(hbm_budget_bytes=20 * 10**9, slots=1)
        srv.submit(*prob, tol)
        assert srv.wait(600)
        alone.append(srv.poll()[0])
        srv.close()
    assert alone[0]["cluster_blocks"] < 0, alone[0]          # whole-GPU persistent grid
    assert alone[1]["fp64_fallback"] == 1, alone[1]
    mix = Server(hbm_budget_bytes=60 * 10**9, slots=8)
    for spec in SPECS[:4]:
        mix.submit(*_problem(*spec), 1e-10)
    ids = [mix.submit(*prob, tol) for prob, tol in cases]
    for spec in SPECS[4:8]:
        mix.submit(*_problem(*spec), 1e-10)
    assert mix.wait(900)
    res = {r["id"]: r for r in mix.poll()}
    assert len(res) == 10 and all(r["status"] == 0 for r in res.values())
    for (prob, tol), rid, a in zip(cases, ids, alone):
        r = res[rid]
        assert r["cluster_blocks"] == a["cluster_blocks"] and r["fp64_fallback"] == a["fp64_fallback"], (r, a)
        diff = np.linalg.norm(r["x"] - a["x"]) / np.linalg.norm(a["x"])
        assert diff <= 1e-9, diff
        assert _relres(*prob, r["x"]) <= tol
    mix.close()


def test_repeated_pattern_reuses_its_coloring(cuda):
    """The same operator submitted twice (a coloring cached by pattern the second time)
    gives the same solution both times."""
    from simplefem_gb300.serving import Server
    A, C, V, b = _problem(3, 2, 3, 5)
    srv = Server(hbm_budget_bytes=10 * 10**9, slots=1)
    srv.submit(A, C, V, b, 1e-10)
    srv.submit(A, C, V, b, 1e-10)
    assert srv.wait(300)
    res = srv.poll()
    assert len(res) == 2 and all(r["status"] == 0 for r in res)
    assert np.array_equal(res[0]["x"], res[1]["x"])
    srv.close()


def test_resident_operators_serve_right_hand_sides(cuda):
    """Resident operators: a matrix added once serves many right-hand sides, several of them
    in flight at the same time on the cluster path, and a large one (above the whole-GPU
    threshold) on the whole-GPU solver; every result reaches its tolerance and equals the
    one-request-one-matrix path's (1e-9). The operator's bytes are held while it is
    registered; removing it with requests outstanding is refused, afterwards it works and
    the bytes come back."""
    from simplefem_gb300 import _native, workloads
    from simplefem_gb300.serving import Server
    A, C, V, _ = _problem(3, 2, 4, 51)
    Ab, Cb, Vb = workloads.lattice_matrix(2, 1, 10, 1)      # 7.3 M entries: whole-GPU solver
    srv = Server(hbm_budget_bytes=60 * 10**9, slots=6)
    before = srv.stats()["bytes_in_use"]
    op = srv.add_operator(A, C, V)
    opb = srv.add_operator(Ab, Cb, Vb)
    assert srv.stats()["bytes_in_use"] > before
    rhs = {}
    for k in range(8):
        b = workloads.uniform_vector(600 + k, len(A) - 1)
        rhs[srv.submit_rhs(op, b, 1e-10)] = (A, C, V, b, 1e-10)
    for k in range(2):
        b = workloads.uniform_vector(700 + k, len(Ab) - 1)
        rhs[srv.submit_rhs(opb, b, 1e-10)] = (Ab, Cb, Vb, b, 1e-10)
    with pytest.raises(_native.FeecError):
        srv.remove_operator(op)                              # requests outstanding
    assert srv.wait(600)
    res = {r["id"]: r for r in srv.poll()}
    assert len(res) == len(rhs)
    for rid, (A_, C_, V_, b, tol) in rhs.items():
        r = res[rid]
        assert r["status"] == 0, r
        assert _relres(A_, C_, V_, b, r["x"]) <= tol, r
    big = [res[rid] for rid, v in rhs.items() if v[0] is Ab]
    assert all(r["cluster_blocks"] < 0 for r in big), big       # negative: the whole-GPU grid
    # the same right-hand side through the one-request-one-matrix path
    rid0 = next(iter(rhs))
    A_, C_, V_, b, tol = rhs[rid0]
    ref = Server(hbm_budget_bytes=10 * 10**9, slots=1)
    ref.submit(A_, C_, V_, b, tol)
    assert ref.wait(300)
    x_ref = ref.poll()[0]["x"]
    ref.close()
    x = res[rid0]["x"]
    assert np.linalg.norm(x - x_ref) <= 1e-9 * np.linalg.norm(x_ref)
    srv.remove_operator(op)
    srv.remove_operator(opb)
    assert srv.stats()["bytes_in_use"] == before
    with pytest.raises(ValueError):
        srv.submit_rhs(op, np.ones(len(A) - 1), 1e-10)        # removed
    srv.close()
