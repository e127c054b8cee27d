"""CSR algebra on the GPU through the C ABI: MatrixCSRAddition, MatrixCSRMultiplication,
MatrixCSR::getTranspose (sparse/matcsr.cpp:291-350, 707-849) and MatrixCSR(SparseMatrix)
(sparse/matcsr.cpp:43-89). Bar: bit-identical row pointers, columns and values against the
fixture the reference's own code wrote and against the oracle on lattice operators."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _mat(S, g, key):
    return S.MatrixCSR(len(g[key + "_A"]) - 1, int(g[key + "_ncols"]), g[key + "_A"], g[key + "_C"], g[key + "_V"])


def _same(M, A, C, V, what):
    assert np.array_equal(M.A, A), what
    assert np.array_equal(M.C, C), what
    assert np.array_equal(M.V, V), what   # bit-exact (array_equal on float64 compares values)
    assert np.array_equal(M.V.view(np.int64), np.asarray(V, np.float64).view(np.int64)), what


def test_csr_algebra_matches_reference_fixture(cuda):
    import simplefem_gb300 as S
    g = load_golden("csr_algebra")
    X, Y, Xr = _mat(S, g, "X"), _mat(S, g, "Y"), _mat(S, g, "Xr")
    _same(S.MatrixCSRAddition(X, Y, 0.7, -1.3), g["add_A"], g["add_C"], g["add_V"], "add")
    _same(S.MatrixCSRMultiplication(X, Y), g["mul_A"], g["mul_C"], g["mul_V"], "mul")
    _same(S.MatrixCSRMultiplication(Xr, Y), g["mulr_A"], g["mulr_C"], g["mulr_V"], "mulr")
    _same(Xr.getTranspose(), g["tr_A"], g["tr_C"], g["tr_V"], "tr")
    T = S.MatrixCSR.from_coo(len(g["X_A"]) - 1, int(g["X_ncols"]), g["coo_in_r"], g["coo_in_c"], g["coo_in_v"])
    _same(T, g["coo_A"], g["coo_C"], g["coo_V"], "coo")


def _lattice(dim, r, L, seed):
    from simplefem_gb300 import workloads
    return workloads.lattice_matrix(dim, r, L, seed)


def _rows(A, C, V, m):
    """The first m rows of a CSR (a rectangular operator m x n)."""
    e = int(A[m])
    return A[: m + 1].copy(), C[:e].copy(), V[:e].copy()


@pytest.mark.parametrize("dim,r,L", [(2, 1, 6), (3, 1, 3), (2, 2, 4), (2, 3, 2)])
def test_csr_algebra_matches_oracle_on_lattice(cuda, dim, r, L):
    import simplefem_gb300 as S
    from oracle import oracle
    A1, C1, V1 = _lattice(dim, r, L, 3)
    A2, C2, V2 = _lattice(dim, r, L, 4)
    n = len(A1) - 1
    m = (2 * n) // 3
    X, Y = S.MatrixCSR(n, n, A1, C1, V1), S.MatrixCSR(n, n, A2, C2, V2)
    Ar, Cr, Vr = _rows(A1, C1, V1, m)
    Xr = S.MatrixCSR(m, n, Ar, Cr, Vr)
    _same(S.MatrixCSRAddition(X, Y, 0.3, -2.1), *oracle.csr_add(A1, C1, V1, A2, C2, V2, 0.3, -2.1), "add")
    _same(S.MatrixCSRMultiplication(X, Y), *oracle.csr_multiply(A1, C1, V1, A2, C2, V2), "mul")
    _same(S.MatrixCSRMultiplication(Xr, Y), *oracle.csr_multiply(Ar, Cr, Vr, A2, C2, V2), "mulr")
    _same(Xr.getTranspose(), *oracle.csr_transpose(Ar, Cr, Vr, n), "tr")
    # Xr^T * Xr: the product of a transpose, as in B^T M B assemblies
    T = Xr.getTranspose()
    _same(S.MatrixCSRMultiplication(T, Xr), *oracle.csr_multiply(T.A, T.C, T.V, Ar, Cr, Vr), "trmul")


def test_coo_to_csr_matches_oracle_with_duplicates_and_zeros(cuda):
    import simplefem_gb300 as S
    from oracle import oracle
    rng = np.random.default_rng(11)
    rows, cols, count = 700, 500, 40_000
    r = rng.integers(0, rows, count).astype(np.int32)
    c = rng.integers(0, cols, count).astype(np.int32)
    v = rng.standard_normal(count)
    v[rng.random(count) < 0.05] = 0.0                      # dropped before sorting
    r[:50] = 3; c[:50] = 7                                  # one position hit 50 times
    M = S.MatrixCSR.from_coo(rows, cols, r, c, v)
    _same(M, *oracle.coo_to_csr(rows, r, c, v), "coo")
    # positions are unique and sorted within each row
    assert np.all(np.diff(M.A) >= 0)
    for i in range(0, rows, 97):
        assert np.all(np.diff(M.C[M.A[i]:M.A[i + 1]]) > 0)


def test_csr_algebra_edge_cases(cuda):
    import simplefem_gb300 as S
    from oracle import oracle
    A, C, V = _lattice(2, 1, 4, 1)
    n = len(A) - 1
    X = S.MatrixCSR(n, n, A, C, V)
    # X - X: every entry cancels, the result has no entries at all
    Z = S.MatrixCSRAddition(X, X, 1.0, -1.0)
    assert Z.getnumberofentries() == 0 and np.all(Z.A == 0)
    # X + 0 * X: the zero products are dropped, X comes back bit for bit
    _same(S.MatrixCSRAddition(X, X, 1.0, 0.0), A, C, V, "x+0")
    # double transpose of a compressed CSR is the identity
    _same(X.getTranspose().getTranspose(), A, C, V, "tt")
    # rows without entries, in the middle and at the end
    Ae = A.copy()
    keep = np.ones(len(C), bool)
    for row in (0, 5, n - 1):
        keep[A[row]:A[row + 1]] = False
    lens = np.diff(A) * np.array([0 if row in (0, 5, n - 1) else 1 for row in range(n)])
    Ae = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    Ce, Ve = C[keep], V[keep]
    E = S.MatrixCSR(n, n, Ae, Ce, Ve)
    _same(S.MatrixCSRMultiplication(E, X), *oracle.csr_multiply(Ae, Ce, Ve, A, C, V), "empty rows mul")
    _same(E.getTranspose(), *oracle.csr_transpose(Ae, Ce, Ve, n), "empty rows tr")
    # no rows / no entries
    N0 = S.MatrixCSR(0, 4, np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0))
    assert S.MatrixCSRAddition(N0, N0).getnumberofentries() == 0
    T0 = N0.getTranspose()
    assert T0.rows == 4 and T0.getnumberofentries() == 0 and np.all(T0.A == 0)
    assert S.MatrixCSR.from_coo(3, 3, [], [], []).getnumberofentries() == 0
    assert S.MatrixCSR.from_coo(3, 3, [1, 2], [0, 2], [0.0, 0.0]).getnumberofentries() == 0


def test_csr_algebra_rejects_bad_input(cuda):
    """Indices out of range and broken row pointers are refused on the host, before
    any kernel indexes through them."""
    from simplefem_gb300 import _native
    L = _native.gpu()
    A = np.array([0, 2, 3], np.int32); C = np.array([0, 5, 1], np.int32); V = np.ones(3)
    B = np.empty(8, np.int32); D = np.empty(3, np.int32); W = np.empty(3)
    nnz = ctypes.c_int(0)
    assert L.feec_csr_transpose(2, 3, A, C, V, B, D, W, ctypes.byref(nnz)) == _native.FEEC_BADARG
    Ab = np.array([0, 3, 2], np.int32); Cb = np.array([0, 1, 1], np.int32)
    assert L.feec_csr_transpose(2, 3, Ab, Cb, V, B, D, W, ctypes.byref(nnz)) == _native.FEEC_BADARG
    r = np.array([0, 2], np.int32); c = np.array([0, 0], np.int32); v = np.ones(2)
    assert L.feec_coo_to_csr(2, 2, 2, r, c, v, B, D, W, ctypes.byref(nnz)) == _native.FEEC_BADARG
    Ca = np.array([0, 1, 1], np.int32)
    out_C = np.empty(6, np.int32); out_V = np.empty(6)
    assert L.feec_csr_add(2, 2, A, Ca, V, A, C, V, 1.0, 1.0, B, out_C, out_V, ctypes.byref(nnz)) == _native.FEEC_BADARG
    assert L.feec_csr_add(2, 2, A, Ca, V, A, Ca, V, 1.0, 1.0, B, out_C, out_V, ctypes.byref(nnz)) == _native.FEEC_OK
    assert nnz.value == 3


def test_transpose_full_size_symmetric_operator(cuda):
    """At solver size (3D P2 lattice operator, 274,625 rows, 7.7M entries) the transpose
    of the symmetric operator is the operator itself, bit for bit."""
    import simplefem_gb300 as S
    A, C, V = _lattice(3, 2, 5, 0)
    n = len(A) - 1
    X = S.MatrixCSR(n, n, A, C, V)
    _same(X.getTranspose(), A, C, V, "symmetric transpose")


def test_multiply_long_rows_match_oracle(cuda):
    """Product rows longer than one warp's shared-memory stage (1600 entries before
    compression, many equal columns) take the in-place path; still bit-identical."""
    import simplefem_gb300 as S
    from oracle import oracle
    rng = np.random.default_rng(5)
    n, per_row = 200, 40
    C = np.concatenate([np.sort(rng.choice(n, per_row, replace=False)) for _ in range(n)]).astype(np.int32)
    A = np.arange(0, n * per_row + 1, per_row, dtype=np.int32)
    V = rng.standard_normal(n * per_row)
    X = S.MatrixCSR(n, n, A, C, V)
    _same(S.MatrixCSRMultiplication(X, X), *oracle.csr_multiply(A, C, V, A, C, V), "long rows")


def _coo_of(A, C, V, rng, split=0.25, zeros=0, cols=None):
    """COO entries of a CSR, shuffled, some split into two exact halves, explicit zeros."""
    n = len(A) - 1
    r = np.repeat(np.arange(n, dtype=np.int32), np.diff(A)); c = C.copy(); v = V.copy()
    s = rng.random(len(v)) < split
    v[s] *= 0.5
    r = np.concatenate([r, r[s], rng.integers(0, n, zeros).astype(np.int32)])
    c = np.concatenate([c, c[s], rng.integers(0, cols or n, zeros).astype(np.int32)])
    v = np.concatenate([v, v[s], np.zeros(zeros)])
    p = rng.permutation(len(r))
    return r[p], c[p], v[p]


def test_coo_multiply_matches_reference_fixture_and_oracle(cuda):
    """SparseMatrixMultiplication: bit-identical to the oracle; against the reference's
    own output the structure and single-product entries bit for bit, sums of several
    products within 16 eps of the sum of magnitudes (unspecified std::sort order)."""
    import simplefem_gb300 as S
    from oracle import oracle
    g = load_golden("csr_algebra")
    rows, cols = (int(x) for x in g["coomul_shape"])
    inner = len(g["Y_A"]) - 1
    L = S.SparseMatrix(rows, inner, g["coomul_l_r"], g["coomul_l_c"], g["coomul_l_v"])
    R = S.SparseMatrix(inner, cols, g["coomul_r_r"], g["coomul_r_c"], g["coomul_r_v"])
    P = S.SparseMatrixMultiplication(L, R)
    r_o, c_o, v_o = oracle.coo_multiply(inner, (L.r, L.c, L.v), (R.r, R.c, R.v))
    assert np.array_equal(P.r, r_o) and np.array_equal(P.c, c_o)
    assert np.array_equal(P.v.view(np.int64), v_o.view(np.int64))
    assert np.array_equal(P.r, g["coomul_out_r"]) and np.array_equal(P.c, g["coomul_out_c"])
    _, _, mag = oracle.coo_multiply(inner, (L.r, L.c, np.abs(L.v)), (R.r, R.c, np.abs(R.v)))
    assert np.all(np.abs(P.v - g["coomul_out_v"]) <= 16 * np.finfo(float).eps * mag)


@pytest.mark.parametrize("dim,r,L", [(2, 2, 5), (3, 1, 4), (2, 3, 3)])
def test_coo_multiply_matches_oracle_on_lattice(cuda, dim, r, L):
    import simplefem_gb300 as S
    from oracle import oracle
    rng = np.random.default_rng(100 + dim * 10 + r)
    A1, C1, V1 = _lattice(dim, r, L, 1)
    A2, C2, V2 = _lattice(dim, r, L, 2)
    n = len(A1) - 1
    l = _coo_of(A1, C1, V1, rng, zeros=50)
    rr = _coo_of(A2, C2, V2, rng, zeros=50)
    P = S.SparseMatrixMultiplication(S.SparseMatrix(n, n, *l), S.SparseMatrix(n, n, *rr))
    r_o, c_o, v_o = oracle.coo_multiply(n, l, rr)
    assert np.array_equal(P.r, r_o) and np.array_equal(P.c, c_o)
    assert np.array_equal(P.v.view(np.int64), v_o.view(np.int64))


def test_coo_multiply_wide_rows_and_edge_cases(cuda):
    """Product rows with more distinct columns than the shared-memory table holds take
    the global-table pass; zero products are dropped before merging; empty operands."""
    import simplefem_gb300 as S
    from oracle import oracle
    rng = np.random.default_rng(9)
    inner, cols = 2000, 3000
    # left: row 0 touches 300 columns k, rows 1..9 a few; right: 20 random columns per row
    lr = np.concatenate([np.zeros(300, np.int32), rng.integers(1, 10, 60).astype(np.int32)])
    lc = np.concatenate([rng.choice(inner, 300, replace=False), rng.integers(0, inner, 60)]).astype(np.int32)
    lv = rng.standard_normal(len(lr))
    rr = np.repeat(np.arange(inner, dtype=np.int32), 20)
    rc = np.concatenate([rng.choice(cols, 20, replace=False) for _ in range(inner)]).astype(np.int32)
    rv = rng.standard_normal(len(rr))
    # two products that underflow to zero: entry (9, rc[0..]) gets only those
    lr = np.concatenate([lr, [9]]).astype(np.int32); lc = np.concatenate([lc, [0]]).astype(np.int32)
    lv = np.concatenate([lv, [1e-200]]); rv[:20] = np.where(np.arange(20) < 2, 1e-200, rv[:20])
    left, right = S.SparseMatrix(10, inner, lr, lc, lv), S.SparseMatrix(inner, cols, rr, rc, rv)
    P = S.SparseMatrixMultiplication(left, right)
    assert np.sum(P.r == 0) > 1536            # row 0 overflowed the shared table
    r_o, c_o, v_o = oracle.coo_multiply(inner, (lr, lc, lv), (rr, rc, rv))
    assert np.array_equal(P.r, r_o) and np.array_equal(P.c, c_o)
    assert np.array_equal(P.v.view(np.int64), v_o.view(np.int64))
    E = S.SparseMatrixMultiplication(S.SparseMatrix(4, 5, [], [], []), S.SparseMatrix(5, 6, [1], [2], [3.0]))
    assert E.getnumberofentries() == 0
    from simplefem_gb300 import _native
    cnt = ctypes.c_longlong(0)
    bad = np.array([7], np.int32)
    out_i = np.empty(4, np.int32); out_v = np.empty(4)
    st = _native.gpu().feec_coo_multiply(4, 5, 6, 1, np.array([0], np.int32), bad, np.ones(1), 1,
                                         np.array([1], np.int32), np.array([2], np.int32), np.ones(1),
                                         out_i, out_i.copy(), out_v, ctypes.byref(cnt))
    assert st == _native.FEEC_BADARG
