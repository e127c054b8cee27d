"""ORACLE — test infrastructure, not product code.

ctypes binding of ``oracle/_build/libfeec_oracle.so`` (the plain-C restatement of the
reference's CSR Krylov path, ``oracle/feec_oracle.c``). Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (CPU-baseline and reference legs) import
this module, and only to compare results against or as the timed CPU baseline.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libfeec_oracle.so")
_lib = None

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def build(verbose: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP, no FMA contraction)."""
    out = subprocess.run(["make", "-C", _HERE, "-s"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if verbose and out.stdout:
        print(out.stdout)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.oracle_csr_apply.argtypes = [ctypes.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, ctypes.c_double]
        L.oracle_csr_diagonal.argtypes = [ctypes.c_int, _i32p, _i32p, _f64p, _f64p]
        L.oracle_rainbow.argtypes = [ctypes.c_int, _i32p, _i32p, _i32p, _i32p, _i32p]
        L.oracle_rainbow.restype = ctypes.c_int
        L.oracle_cg.argtypes = [ctypes.c_int, _f64p, _f64p, _i32p, _i32p, _f64p, _f64p, ctypes.c_double, ctypes.c_int]
        L.oracle_cg_ssor.argtypes = L.oracle_cg.argtypes + [_f64p, ctypes.c_double]
        L.oracle_cg_rainbow.argtypes = L.oracle_cg_ssor.argtypes + [ctypes.c_int, _i32p, _i32p, _i32p]
        L.oracle_cg_ssor_eisenstat.argtypes = L.oracle_cg_ssor.argtypes
        L.oracle_cg_diag.argtypes = L.oracle_cg.argtypes + [_f64p]
        L.oracle_cg_eisenstat_rainbow.argtypes = L.oracle_cg_rainbow.argtypes
        L.oracle_csr_compress.argtypes = [ctypes.c_int, _i32p, _i32p, _f64p]
        L.oracle_csr_add.argtypes = [ctypes.c_int, _i32p, _i32p, _f64p, _i32p, _i32p, _f64p, ctypes.c_double,
                                     ctypes.c_double, _i32p, _i32p, _f64p]
        L.oracle_csr_multiply_size.argtypes = [ctypes.c_int, _i32p, _i32p, _i32p]
        L.oracle_csr_multiply_size.restype = ctypes.c_longlong
        L.oracle_csr_multiply.argtypes = [ctypes.c_int, _i32p, _i32p, _f64p, _i32p, _i32p, _f64p, _i32p, _i32p, _f64p]
        L.oracle_csr_transpose.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f64p, _i32p, _i32p, _f64p]
        L.oracle_coo_to_csr.argtypes = [ctypes.c_int, ctypes.c_longlong, _i32p, _i32p, _f64p, _i32p, _i32p, _f64p]
        L.oracle_coo_multiply_size.argtypes = [ctypes.c_int, ctypes.c_longlong, _i32p, ctypes.c_longlong, _i32p]
        L.oracle_coo_multiply_size.restype = ctypes.c_longlong
        L.oracle_coo_multiply.argtypes = [ctypes.c_longlong, _i32p, _i32p, _f64p, ctypes.c_longlong, _i32p, _i32p,
                                          _f64p, _i32p, _i32p, _f64p]
        L.oracle_coo_multiply.restype = ctypes.c_longlong
        L.oracle_cr.argtypes = L.oracle_cg.argtypes
        L.oracle_minres.argtypes = L.oracle_cg.argtypes
        L.oracle_chebyshev.argtypes = L.oracle_cg.argtypes + [_f64p, ctypes.c_double, ctypes.c_double]
        L.oracle_hodge_cr.argtypes = ([ctypes.c_int, ctypes.c_int, ctypes.c_int, _f64p, _f64p] + [_i32p, _i32p, _f64p] * 4
                                      + [_f64p, ctypes.c_double, ctypes.c_double])
        _ip32 = ctypes.POINTER(ctypes.c_int); _dp64 = ctypes.POINTER(ctypes.c_double)
        L.oracle_hodge_hs.argtypes = ([ctypes.c_int, ctypes.c_int, _f64p, _f64p, _f64p, _f64p]
                                      + [_i32p, _i32p, _f64p] * 4 + [ctypes.c_double]
                                      + [_ip32, _ip32, _dp64] * 2 + [ctypes.c_double])
        L.oracle_max_threads.restype = ctypes.c_int
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def csr_apply(A, C, V, src, scaling=1.0):
    dest = np.empty(len(A) - 1)
    lib().oracle_csr_apply(len(A) - 1, A, C, V, np.ascontiguousarray(src, np.float64), dest, float(scaling))
    return dest


def csr_diagonal(A, C, V):
    d = np.empty(len(A) - 1)
    lib().oracle_csr_diagonal(len(A) - 1, A, C, V, d)
    return d


def rainbow(A, C):
    n = len(A) - 1
    F = np.empty(n, np.int32); B = np.empty(n + 1, np.int32); R = np.empty(n, np.int32)
    nc = lib().oracle_rainbow(n, A, C, F, B, R)
    if nc < 0:
        raise RuntimeError("oracle rainbow failed")
    return nc, F, B[: nc + 1].copy(), R


def cg(A, C, V, b, x0=None, precision=1e-10):
    n = len(A) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    res = np.array(b, np.float64)
    K = lib().oracle_cg(n, x, np.ascontiguousarray(b, np.float64), A, C, V, res, float(precision), -3)
    return K, x, res


def cr(A, C, V, b, x0=None, precision=1e-10):
    """ConjugateResidualSolverCSR (and _textbook, the same arithmetic): (K, x, residual)."""
    n = len(A) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    res = np.array(b, np.float64)
    K = lib().oracle_cr(n, x, np.ascontiguousarray(b, np.float64), A, C, V, res, float(precision), -3)
    return K, x, res


def minres(A, C, V, b, x0=None, precision=1e-10):
    """MINRESCSR: (K, x, b - A x)."""
    n = len(A) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    res = np.array(b, np.float64)
    K = lib().oracle_minres(n, x, np.ascontiguousarray(b, np.float64), A, C, V, res, float(precision), -3)
    return K, x, res


def chebyshev(A, C, V, b, precon, lower, upper, x0=None, precision=1e-10):
    """ChebyshevIteration_DiagonalPreconditioner: (K, x, residual)."""
    n = len(A) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    res = np.array(b, np.float64)
    K = lib().oracle_chebyshev(n, x, np.ascontiguousarray(b, np.float64), A, C, V, res, float(precision), -3,
                               np.ascontiguousarray(precon, np.float64), float(lower), float(upper))
    return K, x, res


def cg_ssor(A, C, V, b, diag, omega=1.0, x0=None, precision=1e-10):
    n = len(A) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    res = np.array(b, np.float64)
    K = lib().oracle_cg_ssor(n, x, np.ascontiguousarray(b, np.float64), A, C, V, res, float(precision), -3,
                             np.ascontiguousarray(diag, np.float64), float(omega))
    return K, x, res


def cg_rainbow(A, C, V, b, diag, rb, omega=1.0, x0=None, precision=1e-10):
    n = len(A) - 1
    nc, F, B, R = rb
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    res = np.array(b, np.float64)
    K = lib().oracle_cg_rainbow(n, x, np.ascontiguousarray(b, np.float64), A, C, V, res, float(precision), -3,
                                np.ascontiguousarray(diag, np.float64), float(omega), int(nc),
                                np.ascontiguousarray(F, np.int32), np.ascontiguousarray(B, np.int32),
                                np.ascontiguousarray(R, np.int32))
    return K, x, res


def cg_ssor_eisenstat(A, C, V, b, diag, omega=1.0, x0=None, precision=1e-10):
    n = len(A) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    res = np.array(b, np.float64)
    K = lib().oracle_cg_ssor_eisenstat(n, x, np.ascontiguousarray(b, np.float64), A, C, V, res, float(precision),
                                       -3, np.ascontiguousarray(diag, np.float64), float(omega))
    return K, x, res


def cg_eisenstat_rainbow(A, C, V, b, diag, rb, omega=1.0, x0=None, precision=1e-10):
    n = len(A) - 1
    nc, F, B, R = rb
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    res = np.array(b, np.float64)
    K = lib().oracle_cg_eisenstat_rainbow(n, x, np.ascontiguousarray(b, np.float64), A, C, V, res, float(precision),
                                          -3, np.ascontiguousarray(diag, np.float64), float(omega), int(nc),
                                          np.ascontiguousarray(F, np.int32), np.ascontiguousarray(B, np.int32),
                                          np.ascontiguousarray(R, np.int32))
    return K, x, res


def cg_diag(A, C, V, b, precon, x0=None, precision=1e-10):
    n = len(A) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    res = np.array(b, np.float64)
    K = lib().oracle_cg_diag(n, x, np.ascontiguousarray(b, np.float64), A, C, V, res, float(precision), -3,
                             np.ascontiguousarray(precon, np.float64))
    return K, x, res


def _i32(a):
    return np.ascontiguousarray(a, np.int32)


def _f64(a):
    return np.ascontiguousarray(a, np.float64)


def csr_add(A1, C1, V1, A2, C2, V2, s1, s2):
    rows = len(A1) - 1
    cap = int(A1[-1]) + int(A2[-1])
    A = np.empty(rows + 1, np.int32); C = np.empty(max(cap, 1), np.int32); V = np.empty(max(cap, 1))
    n = lib().oracle_csr_add(rows, _i32(A1), _i32(C1), _f64(V1), _i32(A2), _i32(C2), _f64(V2), float(s1), float(s2),
                             A, C, V)
    return A, C[:n].copy(), V[:n].copy()


def csr_multiply(A1, C1, V1, A2, C2, V2):
    rows = len(A1) - 1
    cap = int(lib().oracle_csr_multiply_size(rows, _i32(A1), _i32(C1), _i32(A2)))
    A = np.empty(rows + 1, np.int32); C = np.empty(max(cap, 1), np.int32); V = np.empty(max(cap, 1))
    n = lib().oracle_csr_multiply(rows, _i32(A1), _i32(C1), _f64(V1), _i32(A2), _i32(C2), _f64(V2), A, C, V)
    return A, C[:n].copy(), V[:n].copy()


def csr_transpose(A, C, V, cols):
    rows = len(A) - 1
    nnz = int(A[-1])
    B = np.empty(cols + 1, np.int32); D = np.empty(max(nnz, 1), np.int32); W = np.empty(max(nnz, 1))
    n = lib().oracle_csr_transpose(rows, int(cols), _i32(A), _i32(C), _f64(V), B, D, W)
    return B, D[:n].copy(), W[:n].copy()


def coo_to_csr(rows, r, c, v):
    count = len(r)
    A = np.empty(rows + 1, np.int32); C = np.empty(max(count, 1), np.int32); V = np.empty(max(count, 1))
    n = lib().oracle_coo_to_csr(int(rows), count, _i32(r), _i32(c), _f64(v), A, C, V)
    return A, C[:n].copy(), V[:n].copy()


def coo_multiply(inner, left, right):
    """SparseMatrixMultiplication of two COO operands given as (r, c, v): the product's
    entries (r, c, v), sorted by row then column."""
    lr, lc, lv = (_i32(left[0]), _i32(left[1]), _f64(left[2]))
    rr, rc, rv = (_i32(right[0]), _i32(right[1]), _f64(right[2]))
    cap = int(lib().oracle_coo_multiply_size(int(inner), len(lr), lc, len(rr), rr))
    r = np.empty(max(cap, 1), np.int32); c = np.empty(max(cap, 1), np.int32); v = np.empty(max(cap, 1))
    n = int(lib().oracle_coo_multiply(len(lr), lr, lc, lv, len(rr), rr, rc, rv, r, c, v))
    return r[:n].copy(), c[:n].copy(), v[:n].copy()


def hodge_cr(variant, Amat, Bmat, Btmat, Cmat, b, x0=None, precision=1e-10, inner_precision=1e-12):
    """Hodge conjugate residuals (variant 0 diagonal, 1 SSOR, 2 plain inner CG); matrices
    are (A, C, V) triples: A L x L, B N x L, Bt L x N, C N x N. Returns (K, x, residual)."""
    N = len(Cmat[0]) - 1
    L = len(Amat[0]) - 1
    x = np.zeros(N) if x0 is None else np.array(x0, np.float64)
    res = np.zeros(N)
    mats = []
    for M in (Amat, Bmat, Btmat, Cmat):
        mats += [_i32(M[0]), _i32(M[1]), _f64(M[2])]
    K = lib().oracle_hodge_cr(int(variant), N, L, x, _f64(b), *mats, res, float(precision), float(inner_precision))
    return K, x, res


def hodge_hs(Amat, Bmat, Btmat, Cmat, b_A, b_C, PA=None, PC=None, precision=1e-10, inner_precision=1e-12):
    """HodgeHerzogSoodhalterMethod from x = 0: (K, x_A, x_C). PA / PC are (rows, columns,
    values) triples or None."""
    dA, dC = len(Amat[0]) - 1, len(Cmat[0]) - 1
    xA, xC = np.zeros(dA), np.zeros(dC)
    mats = []
    for M in (Amat, Bmat, Btmat, Cmat):
        mats += [_i32(M[0]), _i32(M[1]), _f64(M[2])]
    keep = []

    def opt(P):
        if P is None:
            return [None, None, None]
        a, c, v = _i32(P[0]), _i32(P[1]), _f64(P[2])
        keep.extend([a, c, v])
        return [a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), c.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                v.ctypes.data_as(ctypes.POINTER(ctypes.c_double))]
    K = lib().oracle_hodge_hs(dA, dC, xA, xC, _f64(b_A), _f64(b_C), *mats, float(precision), *opt(PA), *opt(PC),
                              float(inner_precision))
    return K, xA, xC
