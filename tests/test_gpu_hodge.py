"""Hodge conjugate residual solvers on the GPU (solver/systemsparsesolver.cpp:18-1120)
through the C ABI: against the fixture the reference's own drivers wrote and against the
oracle (pinned bit-exact to that fixture). Bar: solution within max(1e-9, 2 x the reference's
own error against a dense solve); outer iteration count within the band that rounding-level
changes alone produce in the reference's algorithm, plus one: the oracle's K under
perturbations of b by one unit in the last place (scaled by 1 +- 1e-15, or with random
one-ulp noise). On the fixture system that band is up to 6 of 58 (57 -> 53 for the diagonal
variant, 58 -> 52 for the textbook one): outer conjugate residuals over inexact inner solves
amplify rounding."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

VARIANTS = (("diagonal", "HodgeConjugateResidualSolverCSR_diagonal", 0),
            ("ssor", "HodgeConjugateResidualSolverCSR_SSOR", 1),
            ("textbook", "HodgeConjugateResidualSolverCSR_textbook", 2),
            ("plain", "HodgeConjugateResidualSolverCSR", 1))


def _dense(M, rows, cols):
    D = np.zeros((rows, cols))
    np.add.at(D, (np.repeat(np.arange(rows), np.diff(M[0])), M[1]), M[2])
    return D


def _schur_solution(A, B, Bt, C, b):
    L = len(A[0]) - 1
    N = len(C[0]) - 1
    Ad, Bd, Btd, Cd = _dense(A, L, L), _dense(B, N, L), _dense(Bt, L, N), _dense(C, N, N)
    return np.linalg.solve(Bd @ np.linalg.solve(Ad, Btd) + Cd, b)


def _close_K(K, K_o):
    return abs(K - K_o) <= max(1, int(np.ceil(0.02 * K_o)))


def _order_band(variant, A, B, Bt, C, b, K_ref, prec, inner):
    """Spread of the oracle's K under one-ulp perturbations of b."""
    from oracle import oracle
    oracle.set_threads(1)
    rng = np.random.default_rng(0)
    perturbed = [b * (1 + 1e-15), b * (1 - 1e-15)]
    perturbed += [b + np.spacing(b) * rng.integers(-1, 2, len(b)) for _ in range(2)]
    band = 0
    for bp in perturbed:
        K_p, _, _ = oracle.hodge_cr(variant, A, B, Bt, C, bp, precision=prec, inner_precision=inner)
        band = max(band, abs(K_p - K_ref))
    return band


def test_hodge_matches_reference_fixture(cuda):
    import simplefem_gb300 as S
    g = load_golden("hodge")
    M = lambda k: (g[k + "_A"], g[k + "_C"], g[k + "_V"])  # noqa: E731
    N, L = len(g["C_A"]) - 1, len(g["A_A"]) - 1
    xs = _schur_solution(M("A"), M("B"), M("Bt"), M("C"), g["b"])
    prec, inner = float(g["precision"]), float(g["inner_precision"])
    for key, fn, variant in VARIANTS:
        x = np.zeros(N); res = np.zeros(N)
        K = getattr(S, fn)(N, L, x, g["b"], M("A"), M("B"), M("Bt"), M("C"), res, prec, -3, inner, -3)
        info = S.last_info()
        assert info["status"] == 0, (key, info)
        K_ref = int(g[key + "_K"])
        band = _order_band(variant, M("A"), M("B"), M("Bt"), M("C"), g["b"], K_ref, prec, inner)
        assert _close_K(K, K_ref) or abs(K - K_ref) <= band + 1, (key, K, K_ref, band)
        own = np.linalg.norm(g[key + "_x"] - xs) / np.linalg.norm(xs)
        diff = np.linalg.norm(x - g[key + "_x"]) / np.linalg.norm(g[key + "_x"])
        assert diff <= max(1e-9, 2.0 * own), (key, diff, own)
        assert info["outer_iterations"] > K          # the inner iterations, summed


def test_hodge_matches_oracle_on_larger_system(cuda):
    import simplefem_gb300 as S
    from oracle import oracle
    from simplefem_gb300 import workloads
    rng = np.random.default_rng(8)
    A = workloads.lattice_matrix(3, 1, 3, 2)                 # L = 729
    C = workloads.lattice_matrix(2, 1, 4, 6)                 # N = 289
    L, N = len(A[0]) - 1, len(C[0]) - 1
    cols = np.concatenate([np.sort(rng.choice(L, 5, replace=False)) for _ in range(N)]).astype(np.int32)
    B = (np.arange(0, 5 * N + 1, 5, dtype=np.int32), cols, rng.uniform(-1, 1, 5 * N))
    Bt = oracle.csr_transpose(*B, L)
    b = rng.uniform(-1, 1, N)
    xs = _schur_solution(A, B, Bt, C, b)
    for key, fn, variant in VARIANTS[:3]:
        x = np.zeros(N); res = np.zeros(N)
        K = getattr(S, fn)(N, L, x, b, A, B, Bt, C, res, 1e-10, -3, 1e-12, -3)
        assert S.last_info()["status"] == 0, key
        oracle.set_threads(1)
        K_o, x_o, _ = oracle.hodge_cr(variant, A, B, Bt, C, b, precision=1e-10, inner_precision=1e-12)
        band = _order_band(variant, A, B, Bt, C, b, K_o, 1e-10, 1e-12)
        assert _close_K(K, K_o) or abs(K - K_o) <= band + 1, (key, K, K_o, band)
        own = np.linalg.norm(x_o - xs) / np.linalg.norm(xs)
        assert np.linalg.norm(x - x_o) / np.linalg.norm(x_o) <= max(1e-9, 2.0 * own), key
        # the residual array is the recursive residual of the Schur system
        assert np.linalg.norm(res) < 1e-6 * np.linalg.norm(b)


def test_hodge_rejects_out_of_range_columns(cuda):
    from simplefem_gb300 import _native
    g = load_golden("hodge")
    N, L = len(g["C_A"]) - 1, len(g["A_A"]) - 1
    Bc = g["B_C"].copy(); Bc[3] = L + 4                       # a column beyond A's size
    info = _native.FeecSolveInfo()
    st = _native.gpu().feec_hodge_cr_csr_textbook(N, L, np.zeros(N), g["b"], g["A_A"], g["A_C"], g["A_V"],
                                                  g["B_A"], Bc, g["B_V"], g["Bt_A"], g["Bt_C"], g["Bt_V"],
                                                  g["C_A"], g["C_C"], g["C_V"], np.zeros(N), 1e-10, -3, 1e-12, -3,
                                                  ctypes.byref(info))
    assert st == _native.FEEC_BADARG


def test_herzog_soodhalter_matches_reference_fixture(cuda):
    """HodgeHerzogSoodhalterMethod with both, one and no block preconditioners: solution
    within max(1e-9, 2 x the reference's own error against a dense solve of the saddle-point
    system); iteration count within the oracle's one-ulp band plus one."""
    import simplefem_gb300 as S
    from oracle import oracle
    g = load_golden("hodge")
    M = lambda k: (g[k + "_A"], g[k + "_C"], g[k + "_V"])  # noqa: E731
    dC, dA = len(g["C_A"]) - 1, len(g["A_A"]) - 1
    K_full = np.block([[-_dense(M("A"), dA, dA), _dense(M("Bt"), dA, dC)],
                       [_dense(M("B"), dC, dA), _dense(M("C"), dC, dC)]])
    xs = np.linalg.solve(K_full, np.concatenate([g["hhs_bA"], g["hhs_bC"]]))
    prec, inner = float(g["precision"]), float(g["inner_precision"])
    oracle.set_threads(1)
    for case, PA, PC in (("hhs_pp", M("A"), M("C")), ("hhs_pn", M("A"), None), ("hhs_nn", None, None)):
        xA = np.zeros(dA); xC = np.zeros(dC)
        K = S.HodgeHerzogSoodhalterMethod(dA, dC, xA, xC, g["hhs_bA"], g["hhs_bC"], M("A"), M("B"), M("Bt"), M("C"),
                                          prec, -3, PA, PC, inner, -3)
        info = S.last_info()
        K_ref = int(g[case + "_K"])
        assert info["status"] == (0 if K_ref < dA + dC else 3), (case, info)
        band = 0
        for sc in (1 + 1e-15, 1 - 1e-15):
            K_p, _, _ = oracle.hodge_hs(M("A"), M("B"), M("Bt"), M("C"), g["hhs_bA"] * sc, g["hhs_bC"] * sc, PA, PC,
                                        prec, inner)
            band = max(band, abs(K_p - K_ref))
        assert _close_K(K, K_ref) or abs(K - K_ref) <= band + 1, (case, K, K_ref, band)
        x_ref = np.concatenate([g[case + "_xA"], g[case + "_xC"]])
        own = np.linalg.norm(x_ref - xs) / np.linalg.norm(xs)
        diff = np.linalg.norm(np.concatenate([xA, xC]) - x_ref) / np.linalg.norm(x_ref)
        assert diff <= max(1e-9, 2.0 * own), (case, diff, own)
