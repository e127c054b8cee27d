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
