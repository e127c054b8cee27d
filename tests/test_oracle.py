"""Pins the oracle (the C restatement in oracle/feec_oracle.c) to the reference's own
outputs stored in tests/golden (written by tests/golden/make_golden.py from the
compiled reference). At one OpenMP thread the restatement must reproduce the
reference bit for bit: iteration counts, solutions, residual arrays, SpMV,
diagonal and the Rainbow ordering, for all six CG drivers (plain, diagonal
preconditioner, SSOR, Rainbow, SSOR-Eisenstat, Eisenstat-Rainbow)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden

NAMES = golden_names()


@pytest.fixture(scope="module")
def O(built):
    from oracle import oracle
    oracle.set_threads(1)
    return oracle


@pytest.mark.parametrize("name", NAMES)
def test_oracle_spmv_diagonal_rainbow_bitexact(O, name):
    g = load_golden(name)
    A, C, V, b = g["A"], g["C"], g["V"], g["b"]
    assert np.array_equal(O.csr_apply(A, C, V, b, 0.7), g["apply_out"])
    assert np.array_equal(O.csr_diagonal(A, C, V), g["diag"])
    nc, F, B, R = O.rainbow(A, C)
    assert nc == int(g["rb_nc"])
    assert np.array_equal(F, g["rb_F"]) and np.array_equal(B, g["rb_B"]) and np.array_equal(R, g["rb_R"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_solvers_bitexact(O, name):
    g = load_golden(name)
    A, C, V, b = g["A"], g["C"], g["V"], g["b"]
    prec = float(g["precision"])
    diag = g["diag"]
    rb = (int(g["rb_nc"]), g["rb_F"], g["rb_B"], g["rb_R"])
    for key in [k[:-2] for k in g if k.endswith("_K")]:
        om = float(g[key + "_omega"])
        if key == "cg":
            K, x, r = O.cg(A, C, V, b, precision=prec)
        elif key == "jac":
            K, x, r = O.cg_diag(A, C, V, b, np.where(diag != 0, 1.0 / np.where(diag != 0, diag, 1.0), 0.0),
                                precision=prec)
        elif key in ("cr", "crt"):
            K, x, r = O.cr(A, C, V, b, precision=prec)
        elif key == "minres":
            K, x, r = O.minres(A, C, V, b, precision=prec)
        elif key == "cheb":
            K, x, r = O.chebyshev(A, C, V, b, np.where(diag != 0, 1.0 / np.where(diag != 0, diag, 1.0), 0.0),
                                  float(g["cheb_lower"]), float(g["cheb_upper"]), precision=prec)
        elif key.startswith("ssor"):
            K, x, r = O.cg_ssor(A, C, V, b, diag, om, precision=prec)
        elif key.startswith("eisrb"):
            K, x, r = O.cg_eisenstat_rainbow(A, C, V, b, diag, rb, om, precision=prec)
        elif key.startswith("eis"):
            K, x, r = O.cg_ssor_eisenstat(A, C, V, b, diag, om, precision=prec)
        else:
            K, x, r = O.cg_rainbow(A, C, V, b, diag, rb, om, precision=prec)
        assert K == int(g[key + "_K"]), key
        assert np.array_equal(x, g[key + "_x"]), key
        assert np.array_equal(r, g[key + "_res"]), key


def test_oracle_planted_mistake_is_caught(O):
    """A wrong matrix entry planted in the oracle's input must change its answer."""
    g = load_golden("fem2d_p1_l6")
    V = g["V"].copy()
    V[100] *= 1.0 + 1e-6
    K, x, _ = O.cg(g["A"], g["C"], V, g["b"], precision=float(g["precision"]))
    assert not np.array_equal(x, g["cg_x"])


def test_oracle_csr_algebra_bitexact(O):
    """MatrixCSRAddition, MatrixCSRMultiplication (square and rectangular),
    MatrixCSR::getTranspose and MatrixCSR(SparseMatrix) exactly as the reference wrote them."""
    g = load_golden("csr_algebra")
    X = (g["X_A"], g["X_C"], g["X_V"]); Y = (g["Y_A"], g["Y_C"], g["Y_V"]); Xr = (g["Xr_A"], g["Xr_C"], g["Xr_V"])
    cases = {
        "add": O.csr_add(*X, *Y, 0.7, -1.3),
        "mul": O.csr_multiply(*X, *Y),
        "mulr": O.csr_multiply(*Xr, *Y),
        "tr": O.csr_transpose(*Xr, int(g["Xr_ncols"])),
        "coo": O.coo_to_csr(len(g["X_A"]) - 1, g["coo_in_r"], g["coo_in_c"], g["coo_in_v"]),
    }
    for case, (A, C, V) in cases.items():
        assert np.array_equal(A, g[case + "_A"]), case
        assert np.array_equal(C, g[case + "_C"]), case
        assert np.array_equal(V, g[case + "_V"]), case


def test_oracle_coo_multiply_against_reference(O):
    """SparseMatrixMultiplication (sparse/sparsematrix.cpp:609-722) against the reference's
    own output: the structure bit for bit, entries with one product bit for bit, and sums
    of several products within 16 eps of the sum of their magnitudes (the reference's
    std::sort leaves the order of equal positions, hence the summation order, unspecified;
    the oracle sums in emission order)."""
    g = load_golden("csr_algebra")
    inner = int(len(g["Y_A"]) - 1)
    L = (g["coomul_l_r"], g["coomul_l_c"], g["coomul_l_v"])
    R = (g["coomul_r_r"], g["coomul_r_c"], g["coomul_r_v"])
    r, c, v = O.coo_multiply(inner, L, R)
    assert np.array_equal(r, g["coomul_out_r"]) and np.array_equal(c, g["coomul_out_c"])
    _, _, mag = O.coo_multiply(inner, (L[0], L[1], np.abs(L[2])), (R[0], R[1], np.abs(R[2])))
    ref = g["coomul_out_v"]
    assert np.all(np.abs(v - ref) <= 16 * np.finfo(float).eps * mag)
    # products per entry: the product of the compressed operands' patterns
    rows = int(g["coomul_shape"][0])
    Al, Cl, _ = O.coo_to_csr(rows, *L)
    Ar, Cr, _ = O.coo_to_csr(inner, *R)
    Ap, Cp, count = O.csr_multiply(Al, Cl, np.ones(len(Cl)), Ar, Cr, np.ones(len(Cr)))
    assert np.array_equal(Cp, c) and np.array_equal(np.repeat(np.arange(rows), np.diff(Ap)), r)
    single = count == 1.0
    assert 0 < single.sum() < len(v)
    assert np.array_equal(v[single], ref[single])


def test_oracle_hodge_cr_bitexact(O):
    """The Hodge conjugate residual solvers (solver/systemsparsesolver.cpp:18-1120) exactly
    as the reference's own code computed them: K, x and the residual."""
    g = load_golden("hodge")
    M = lambda k: (g[k + "_A"], g[k + "_C"], g[k + "_V"])  # noqa: E731
    for key, variant in (("diagonal", 0), ("ssor", 1), ("textbook", 2), ("plain", 1)):
        K, x, r = O.hodge_cr(variant, M("A"), M("B"), M("Bt"), M("C"), g["b"], precision=float(g["precision"]),
                             inner_precision=float(g["inner_precision"]))
        assert K == int(g[key + "_K"]), key
        assert np.array_equal(x, g[key + "_x"]), key
        assert np.array_equal(r, g[key + "_res"]), key


def test_oracle_hodge_herzog_soodhalter_bitexact(O):
    """HodgeHerzogSoodhalterMethod (solver/systemsparsesolver.cpp:1122-1575) exactly as the
    reference computed it, with both block preconditioners, with PA only and with none."""
    g = load_golden("hodge")
    M = lambda k: (g[k + "_A"], g[k + "_C"], g[k + "_V"])  # noqa: E731
    for case, PA, PC in (("hhs_pp", M("A"), M("C")), ("hhs_pn", M("A"), None), ("hhs_nn", None, None)):
        K, xA, xC = O.hodge_hs(M("A"), M("B"), M("Bt"), M("C"), g["hhs_bA"], g["hhs_bC"], PA, PC,
                               float(g["precision"]), float(g["inner_precision"]))
        assert K == int(g[case + "_K"]), case
        assert np.array_equal(xA, g[case + "_xA"]) and np.array_equal(xC, g[case + "_xC"]), case


def test_oracle_algebra_and_solvers_agree_with_independent_references(O):
    """Beyond the pins: the oracle's CSR algebra against scipy.sparse, and its further
    drivers and block solvers against dense solves (independent arithmetic)."""
    sp = pytest.importorskip("scipy.sparse")
    g = load_golden("fem2d_p2_l4_coef")
    A, C, V = g["A"], g["C"], g["V"]
    n = len(A) - 1
    M = sp.csr_matrix((V, C, A), shape=(n, n))
    rng = np.random.default_rng(7)
    V2 = V * rng.uniform(0.5, 1.5, len(V))
    M2 = sp.csr_matrix((V2, C, A), shape=(n, n))
    for (Ao, Co, Vo), ref in ((O.csr_add(A, C, V, A, C, V2, 0.3, -1.7), 0.3 * M - 1.7 * M2),
                              (O.csr_multiply(A, C, V, A, C, V2), M @ M2),
                              (O.csr_transpose(A, C, V2, n), M2.T.tocsr())):
        got = sp.csr_matrix((Vo, Co, Ao), shape=ref.shape)
        assert abs(got - ref).max() <= 1e-12 * abs(ref).max()
    r, c, v = sp.find(M)
    rr, cc, vv = O.coo_multiply(n, (r.astype(np.int32), c.astype(np.int32), v),
                                (r.astype(np.int32), c.astype(np.int32), v))
    P = sp.csr_matrix((vv, (rr, cc)), shape=(n, n))
    assert abs(P - M @ M).max() <= 1e-12 * abs(M @ M).max()
    # further drivers against a dense solve (the operator is SPD)
    b = g["b"]
    xs = np.linalg.solve(M.toarray(), b)
    d = M.diagonal()
    ev = np.linalg.eigvalsh((M.multiply(1.0 / np.sqrt(np.outer(d, d)))).toarray())
    for K, x, _ in (O.cr(A, C, V, b, precision=1e-12), O.minres(A, C, V, b, precision=1e-12),
                    O.chebyshev(A, C, V, b, 1.0 / d, 0.99 * ev[0], 1.01 * ev[-1], precision=1e-12)):
        assert 0 < K < n and np.linalg.norm(x - xs) <= 1e-6 * np.linalg.norm(xs)
    # Hodge: conjugate residuals on B A^-1 Bt + C, and the block MINRES on [[-A, Bt], [B, C]]
    h = load_golden("hodge")
    Mh = lambda k: (h[k + "_A"], h[k + "_C"], h[k + "_V"])  # noqa: E731
    L, N = len(h["A_A"]) - 1, len(h["C_A"]) - 1
    Ad = sp.csr_matrix((h["A_V"], h["A_C"], h["A_A"]), shape=(L, L)).toarray()
    Bd = sp.csr_matrix((h["B_V"], h["B_C"], h["B_A"]), shape=(N, L)).toarray()
    Cd = sp.csr_matrix((h["C_V"], h["C_C"], h["C_A"]), shape=(N, N)).toarray()
    xs = np.linalg.solve(Bd @ np.linalg.solve(Ad, Bd.T) + Cd, h["b"])
    K, x, _ = O.hodge_cr(2, Mh("A"), Mh("B"), Mh("Bt"), Mh("C"), h["b"], precision=1e-12, inner_precision=1e-14)
    assert np.linalg.norm(x - xs) <= 1e-6 * np.linalg.norm(xs)
    Kb = np.block([[-Ad, Bd.T], [Bd, Cd]])
    zs = np.linalg.solve(Kb, np.concatenate([h["hhs_bA"], h["hhs_bC"]]))
    K, xA, xC = O.hodge_hs(Mh("A"), Mh("B"), Mh("Bt"), Mh("C"), h["hhs_bA"], h["hhs_bC"], Mh("A"), Mh("C"),
                           1e-12, 1e-14)
    assert np.linalg.norm(np.concatenate([xA, xC]) - zs) <= 1e-6 * np.linalg.norm(zs)


@pytest.mark.parametrize("shape", [(7, 5, 9), (1, 1, 1), (6, 0, 4), (0, 3, 2), (40, 33, 17)])
def test_oracle_rectangular_and_empty_algebra_against_scipy(O, shape):
    """Rectangular, empty-inner and zero-row shapes, random sparse operands with duplicated
    columns inside rows, exact cancellations and explicit zeros: the oracle's sum, product,
    transpose and COO -> CSR agree with scipy.sparse (structure free of zeros, as the
    reference compresses them away)."""
    sp = pytest.importorskip("scipy.sparse")
    m, k, n = shape
    rng = np.random.default_rng(m * 1000 + k * 10 + n)

    def rand_csr(r, c, dens):
        if r == 0 or c == 0:
            return np.zeros(r + 1, np.int32), np.zeros(0, np.int32), np.zeros(0)
        lens = rng.binomial(max(1, int(c * dens * 2)), 0.5, r)
        A = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
        C = rng.integers(0, c, A[-1]).astype(np.int32)
        V = rng.integers(-3, 4, A[-1]).astype(np.float64)      # integers: exact cancellations, zeros
        return A, C, V

    def dense(A, C, V, r, c):
        D = np.zeros((r, c))
        for i in range(r):
            for j in range(A[i], A[i + 1]):
                D[i, C[j]] += V[j]
        return D

    def check(got, D):
        A, C, V = got
        assert A[0] == 0 and np.all(np.diff(A) >= 0) and A[-1] == len(C) == len(V)
        assert np.all(V != 0)
        for i in range(len(A) - 1):
            assert np.all(np.diff(C[A[i]:A[i + 1]]) > 0)     # sorted, merged rows
        np.testing.assert_array_equal(dense(A, C, V, len(A) - 1, D.shape[1]), D)

    X1, X2, Y = rand_csr(m, k, 0.4), rand_csr(m, k, 0.3), rand_csr(k, n, 0.4)
    D1, D2, DY = dense(*X1, m, k), dense(*X2, m, k), dense(*Y, k, n)
    check(O.csr_add(*X1, *X2, 2.0, -1.0), 2.0 * D1 - D2)
    check(O.csr_multiply(*X1, *Y), D1 @ DY)
    check(O.csr_transpose(*X1, k), D1.T)
    r = rng.integers(0, max(m, 1), 3 * m).astype(np.int32) if m else np.zeros(0, np.int32)
    c = rng.integers(0, max(k, 1), 3 * m).astype(np.int32) if m else np.zeros(0, np.int32)
    v = rng.integers(-2, 3, 3 * m).astype(np.float64) if m else np.zeros(0)
    if k:
        ref = sp.coo_matrix((v, (r, c)), shape=(m, k)).toarray()
        check(O.coo_to_csr(m, r, c, v), ref)
