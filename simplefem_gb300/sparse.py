"""MatrixCSR / Rainbow / FloatVector surface of the reference, over the GPU library.

Mirrors the parts of sparse/matcsr.hpp:25-121, sparse/rainbow.hpp:13-31 and
operators/floatvector.hpp:21-338 that the CSR Krylov path touches: the CSR arrays
(``getA``/``getC``/``getV``), ``apply`` (SpMV on the GPU), ``getDiagonal``,
``check``, and the Rainbow coloring with its ``F``/``B``/``R`` members.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native


class FloatVector:
    """Owned float64 buffer with ``raw()`` access (operators/floatvector.hpp:21-338)."""

    def __init__(self, dim_or_data, initialvalue=float("nan")):
        if np.isscalar(dim_or_data):
            self._d = np.full(int(dim_or_data), initialvalue, np.float64)
        else:
            self._d = np.array(dim_or_data, np.float64)

    def raw(self) -> np.ndarray:
        return self._d

    def getdimension(self) -> int:
        return int(self._d.shape[0])

    def zero(self):
        self._d[:] = 0.0

    def norm_sq(self) -> float:
        # the reference accumulates in long double (floatvector.cpp:619-626)
        return float(np.sum(self._d.astype(np.longdouble) ** 2))

    def norm(self) -> float:
        return float(np.sqrt(np.longdouble(self.norm_sq())))

    def scalarproductwith(self, other: "FloatVector") -> float:
        return float(np.sum(self._d.astype(np.longdouble) * other._d.astype(np.longdouble)))

    def __len__(self):
        return self.getdimension()


class MatrixCSR:
    """CSR matrix with int32 row pointers ``A``, column indices ``C`` and float64 values ``V``."""

    def __init__(self, rows, columns, A, C, V):
        self.rows = int(rows)
        self.columns = int(columns)
        self.A = np.ascontiguousarray(A, np.int32)
        self.C = np.ascontiguousarray(C, np.int32)
        self.V = np.ascontiguousarray(V, np.float64)
        self.check()

    # access (sparse/matcsr.hpp:89-93)
    def getA(self): return self.A
    def getC(self): return self.C
    def getV(self): return self.V
    def getdimout(self): return self.rows
    def getdimin(self): return self.columns
    def getnumberofentries(self): return int(self.C.shape[0])
    def is_square(self): return self.rows == self.columns

    def check(self):
        """Structural invariants of MatrixCSR::check (sparse/matcsr.cpp:178-194)."""
        if (self.A.ndim != 1 or self.A.shape[0] != self.rows + 1 or self.C.shape[0] != self.V.shape[0]
                or int(self.A[self.rows]) != self.C.shape[0]):
            raise ValueError("MatrixCSR: array sizes do not match the dimensions")
        st = _native.gpu().feec_csr_check(self.rows, self.columns, self.A, self.C, self.V)
        if st != _native.FEEC_OK:
            raise ValueError("MatrixCSR: invalid CSR arrays (row pointers, column range or non-finite values)")

    def apply(self, dest, src, scaling=1.0):
        """dest = scaling * A * src on the GPU (MatrixCSR::apply, sparse/matcsr.cpp:216-244)."""
        d = dest.raw() if isinstance(dest, FloatVector) else dest
        s = src.raw() if isinstance(src, FloatVector) else src
        if d is s:
            raise ValueError("MatrixCSR::apply: dest and src must differ")
        if not (isinstance(d, np.ndarray) and d.dtype == np.float64 and d.flags.c_contiguous):
            raise TypeError("dest must be a C-contiguous float64 array")
        if d.shape[0] != self.rows or len(s) != self.columns:
            raise ValueError("MatrixCSR::apply: dimension mismatch")
        st = _native.gpu().feec_csr_apply(self.rows, self.columns, self.A, self.C, self.V,
                                          np.ascontiguousarray(s, np.float64), d, float(scaling))
        _native.check(st, "MatrixCSR::apply")
        return dest

    def __matmul__(self, vec):
        out = np.empty(self.rows)
        self.apply(out, np.ascontiguousarray(vec, np.float64))
        return out

    def getDiagonal(self) -> FloatVector:
        """Sum of the stored diagonal entries per row (sparse/matcsr.cpp:266-286), on the GPU."""
        if not self.is_square():
            raise ValueError("getDiagonal needs a square matrix")
        d = np.empty(self.rows)
        _native.check(_native.gpu().feec_csr_diagonal(self.rows, self.A, self.C, self.V, d), "getDiagonal")
        return FloatVector(d)

    def getTranspose(self) -> "MatrixCSR":
        """Transpose on the GPU (MatrixCSR::getTranspose, sparse/matcsr.cpp:291-350), bit-identical."""
        B = np.empty(self.columns + 1, np.int32)
        D = np.empty(max(self.getnumberofentries(), 1), np.int32)
        W = np.empty(max(self.getnumberofentries(), 1), np.float64)
        nnz = ctypes.c_int(0)
        st = _native.gpu().feec_csr_transpose(self.rows, self.columns, self.A, self.C, self.V, B, D, W,
                                              ctypes.byref(nnz))
        _native.check(st, "MatrixCSR::getTranspose")
        return MatrixCSR(self.columns, self.rows, B, D[:nnz.value], W[:nnz.value])

    @classmethod
    def from_coo(cls, rows, columns, r, c, v) -> "MatrixCSR":
        """CSR from coordinate entries (MatrixCSR(const SparseMatrix&), sparse/matcsr.cpp:43-89 with
        SparseMatrix::sortandcompressentries, sparse/sparsematrix.cpp:405-458) on the GPU: zero
        values dropped, entries at one position summed in input order."""
        r = np.ascontiguousarray(r, np.int32)
        c = np.ascontiguousarray(c, np.int32)
        v = np.ascontiguousarray(v, np.float64)
        if not (r.shape == c.shape == v.shape) or r.ndim != 1:
            raise ValueError("from_coo: r, c and v must be 1-D arrays of one length")
        A = np.empty(int(rows) + 1, np.int32)
        C = np.empty(max(r.shape[0], 1), np.int32)
        V = np.empty(max(r.shape[0], 1), np.float64)
        nnz = ctypes.c_int(0)
        st = _native.gpu().feec_coo_to_csr(int(rows), int(columns), r.shape[0], r, c, v, A, C, V, ctypes.byref(nnz))
        _native.check(st, "MatrixCSR(SparseMatrix)")
        return cls(rows, columns, A, C[:nnz.value], V[:nnz.value])


def MatrixCSRAddition(mat1: MatrixCSR, mat2: MatrixCSR, s1: float = 1.0, s2: float = 1.0) -> MatrixCSR:
    """s1 * mat1 + s2 * mat2 on the GPU (sparse/matcsr.cpp:707-765), bit-identical to the reference."""
    if mat1.rows != mat2.rows or mat1.columns != mat2.columns:
        raise ValueError("MatrixCSRAddition: dimension mismatch")
    cap = max(mat1.getnumberofentries() + mat2.getnumberofentries(), 1)
    A = np.empty(mat1.rows + 1, np.int32)
    C = np.empty(cap, np.int32)
    V = np.empty(cap, np.float64)
    nnz = ctypes.c_int(0)
    st = _native.gpu().feec_csr_add(mat1.rows, mat1.columns, mat1.A, mat1.C, mat1.V, mat2.A, mat2.C, mat2.V,
                                    float(s1), float(s2), A, C, V, ctypes.byref(nnz))
    _native.check(st, "MatrixCSRAddition")
    return MatrixCSR(mat1.rows, mat1.columns, A, C[:nnz.value], V[:nnz.value])


def MatrixCSRMultiplication(mat1: MatrixCSR, mat2: MatrixCSR) -> MatrixCSR:
    """mat1 * mat2 on the GPU (sparse/matcsr.cpp:767-849), bit-identical to the reference."""
    if mat1.columns != mat2.rows:
        raise ValueError("MatrixCSRMultiplication: dimension mismatch")
    L = _native.gpu()
    size = ctypes.c_longlong(0)
    _native.check(L.feec_csr_multiply_size(mat1.rows, mat1.columns, mat1.A, mat1.C, mat2.A, ctypes.byref(size)),
                  "MatrixCSRMultiplication")
    cap = max(int(size.value), 1)
    A = np.empty(mat1.rows + 1, np.int32)
    C = np.empty(cap, np.int32)
    V = np.empty(cap, np.float64)
    nnz = ctypes.c_int(0)
    st = L.feec_csr_multiply(mat1.rows, mat1.columns, mat2.columns, mat1.A, mat1.C, mat1.V, mat2.A, mat2.C, mat2.V,
                             A, C, V, ctypes.byref(nnz))
    _native.check(st, "MatrixCSRMultiplication")
    return MatrixCSR(mat1.rows, mat2.columns, A, C[:nnz.value], V[:nnz.value])


class Rainbow:
    """Greedy multicolor ordering of a CSR graph (sparse/rainbow.hpp:13-31, rainbow.cpp:14-130).

    ``F[r]`` is the color of row r, ``B`` the color pointers and ``R`` the rows listed
    color by color (descending within a color), bit-identical to the reference with
    ``do_shuffle = False``.
    """

    def __init__(self, mat: MatrixCSR, do_shuffle: bool = False):
        if do_shuffle:
            raise NotImplementedError("do_shuffle=True draws from std::random_device in the reference and is not "
                                      "reproducible; only the deterministic ordering is provided")
        if not mat.is_square():
            raise ValueError("Rainbow needs a square matrix")
        n = mat.getdimout()
        self.num_rows = n
        self.F = np.empty(n, np.int32)
        B = np.empty(n + 1, np.int32)
        self.R = np.empty(n, np.int32)
        nc = ctypes.c_int(0)
        _native.check(_native.gpu().feec_rainbow(n, mat.A, mat.C, ctypes.byref(nc), self.F, B, self.R), "Rainbow")
        self.num_colors = int(nc.value)
        self.B = B[: self.num_colors + 1].copy()
        self.check()

    def check(self):
        """Rainbow::check (sparse/rainbow.cpp:133-152): R lists every row once under its color."""
        for c in range(self.num_colors):
            if not np.all(self.F[self.R[self.B[c]:self.B[c + 1]]] == c):
                raise AssertionError(f"Rainbow: row listed under the wrong color {c}")
        if not np.array_equal(np.sort(self.R), np.arange(self.num_rows)):
            raise AssertionError("Rainbow: R is not a permutation")

    def text(self) -> str:
        return f"num_colors: {self.num_colors}"


class SparseMatrix:
    """Coordinate-format matrix (sparse/sparsematrix.hpp): ``rows x columns`` with entries
    ``(r[i], c[i], v[i])`` in any order, duplicates allowed."""

    def __init__(self, rows, columns, r, c, v):
        self.rows = int(rows)
        self.columns = int(columns)
        self.r = np.ascontiguousarray(r, np.int32)
        self.c = np.ascontiguousarray(c, np.int32)
        self.v = np.ascontiguousarray(v, np.float64)
        if not (self.r.shape == self.c.shape == self.v.shape) or self.r.ndim != 1:
            raise ValueError("SparseMatrix: r, c and v must be 1-D arrays of one length")

    def getdimout(self): return self.rows
    def getdimin(self): return self.columns
    def getnumberofentries(self): return int(self.r.shape[0])

    def to_csr(self) -> MatrixCSR:
        """MatrixCSR(const SparseMatrix&) (sparse/matcsr.cpp:43-89) on the GPU."""
        return MatrixCSR.from_coo(self.rows, self.columns, self.r, self.c, self.v)


def SparseMatrixMultiplication(left: SparseMatrix, right: SparseMatrix) -> SparseMatrix:
    """left * right on the GPU (sparse/sparsematrix.cpp:609-722); entries row-wise sorted."""
    if left.columns != right.rows:
        raise ValueError("SparseMatrixMultiplication: dimension mismatch")
    L = _native.gpu()
    size = ctypes.c_longlong(0)
    _native.check(L.feec_coo_multiply_size(left.columns, left.getnumberofentries(), left.c,
                                           right.getnumberofentries(), right.r, ctypes.byref(size)),
                  "SparseMatrixMultiplication")
    cap = max(int(size.value), 1)
    r = np.empty(cap, np.int32); c = np.empty(cap, np.int32); v = np.empty(cap, np.float64)
    count = ctypes.c_longlong(0)
    st = L.feec_coo_multiply(left.rows, left.columns, right.columns, left.getnumberofentries(), left.r, left.c, left.v,
                             right.getnumberofentries(), right.r, right.c, right.v, r, c, v, ctypes.byref(count))
    _native.check(st, "SparseMatrixMultiplication")
    n = int(count.value)
    return SparseMatrix(left.rows, right.columns, r[:n].copy(), c[:n].copy(), v[:n].copy())
