"""The reference's raw-pointer CSR Krylov drivers, running on the GPU.

Same names, argument order and meaning as solver/sparsesolver.hpp:11-70: ``x`` is the
initial guess and receives the solution, ``residual`` receives the final recursive
residual, and the return value is the iteration count K. Arrays are NumPy arrays
(float64 vectors, int32 CSR arrays) standing in for the raw pointers; ``x`` and
``residual`` are written in place. Where the reference asserts on an argument
(sparsesolver.cpp:32-43) these functions raise ``FeecError``; numerical breakdowns
return the current K as the reference does, and the last call's details
(status, timing, tolerance) are kept in ``last_info()``.
"""
from __future__ import annotations

import numpy as np

from . import _native

_last_info = None


def last_info() -> dict | None:
    """Details of the most recent solve: status, iterations, tolerance, device time."""
    return None if _last_info is None else _last_info.as_dict()


def _vec(a, name, n=None, writable=False):
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
        if writable:
            raise TypeError(f"{name} must be a C-contiguous float64 numpy array (it is written in place)")
        a = np.ascontiguousarray(a, np.float64)
    if a.ndim != 1:
        raise ValueError(f"{name} must be one-dimensional, not of shape {a.shape}")
    if n is not None and a.shape[0] < n:
        raise ValueError(f"{name} has {a.shape[0]} entries, expected {n}")
    return a


def _ints(a, name, n=None):
    a = np.ascontiguousarray(a, np.int32)
    if n is not None and (a.ndim != 1 or a.shape[0] < n):
        raise ValueError(f"{name} has {a.shape[0] if a.ndim == 1 else a.shape} entries, expected {n}")
    return a


def _coloring(N, num_colors, F, B, R):
    """Rainbow's F (color of each row), B (color offsets) and R (rows by color) arrays."""
    return _ints(F, "F", N), _ints(B, "B", int(num_colors) + 1), _ints(R, "R", N)


def _csr(rows, csrrows, csrcolumns, csrvalues, name=""):
    """The CSR arrays of a matrix with `rows` rows, checked to be as long as the row
    pointers say (the library reads rows + 1 pointers and A[rows] columns and values
    through the raw pointers); the pointers' contents are validated by the library."""
    A = _ints(csrrows, name + "rows", int(rows) + 1)
    nnz = int(A[int(rows)]) if int(rows) >= 0 else 0
    if nnz < 0:
        raise ValueError(f"{name}rows[{int(rows)}] = {nnz} is negative")
    return A, _ints(csrcolumns, name + "columns", nnz), _vec(csrvalues, name + "values", nnz)


_DONE = (_native.FEEC_OK, _native.FEEC_BREAKDOWN, _native.FEEC_SMALL_ENERGY, _native.FEEC_MAXITER)


def _finish(status, info, where):
    global _last_info
    _last_info = info
    if status not in _DONE:
        raise _native.FeecError(status, where)
    return int(info.iterations)


def ConjugateGradientSolverCSR(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision, print_modulo=-3):
    """GPU replacement of ConjugateGradientSolverCSR (solver/sparsesolver.cpp:26-201)."""
    x = _vec(x, "x", N, True); residual = _vec(residual, "residual", N, True)
    csr = _csr(N, csrrows, csrcolumns, csrvalues)
    info = _native.FeecSolveInfo()
    st = _native.gpu().feec_cg_csr(int(N), x, _vec(b, "b", N), *csr, residual, float(precision), int(print_modulo),
                                   info)
    return _finish(st, info, "ConjugateGradientSolverCSR")


def ConjugateGradientSolverCSR_SSOR(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision, print_modulo,
                                    diagonal, omega):
    """GPU replacement of ConjugateGradientSolverCSR_SSOR (solver/sparsesolver.cpp:446-724)."""
    x = _vec(x, "x", N, True); residual = _vec(residual, "residual", N, True)
    csr = _csr(N, csrrows, csrcolumns, csrvalues)
    info = _native.FeecSolveInfo()
    st = _native.gpu().feec_cg_csr_ssor(int(N), x, _vec(b, "b", N), *csr, residual, float(precision), int(print_modulo),
                                        _vec(diagonal, "diagonal", N), float(omega), info)
    return _finish(st, info, "ConjugateGradientSolverCSR_SSOR")


def ConjugateGradientSolverCSR_Rainbow(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision, print_modulo,
                                       diagonal, omega, num_colors, F, B, R):
    """GPU replacement of ConjugateGradientSolverCSR_Rainbow (solver/sparsesolver.cpp:1002-1335)."""
    x = _vec(x, "x", N, True); residual = _vec(residual, "residual", N, True)
    csr = _csr(N, csrrows, csrcolumns, csrvalues)
    info = _native.FeecSolveInfo()
    st = _native.gpu().feec_cg_csr_rainbow(int(N), x, _vec(b, "b", N), *csr, residual, float(precision),
                                           int(print_modulo), _vec(diagonal, "diagonal", N), float(omega),
                                           int(num_colors), *_coloring(N, num_colors, F, B, R), info)
    return _finish(st, info, "ConjugateGradientSolverCSR_Rainbow")


def ConjugateGradientSolverCSR_SSOR_Eisenstat(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision,
                                              print_modulo, diagonal, omega):
    """GPU replacement of ConjugateGradientSolverCSR_SSOR_Eisenstat (solver/sparsesolver.cpp:726-995);
    `residual` receives the residual of the L-solved system, as in the reference."""
    x = _vec(x, "x", N, True); residual = _vec(residual, "residual", N, True)
    csr = _csr(N, csrrows, csrcolumns, csrvalues)
    info = _native.FeecSolveInfo()
    st = _native.gpu().feec_cg_csr_ssor_eisenstat(int(N), x, _vec(b, "b", N), *csr, residual,
                                                  float(precision), int(print_modulo), _vec(diagonal, "diagonal", N),
                                                  float(omega), info)
    return _finish(st, info, "ConjugateGradientSolverCSR_SSOR_Eisenstat")


def ConjugateGradientSolverCSR_Eisenstat_Rainbow(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision,
                                                 print_modulo, diagonal, omega, num_colors, F, B, R):
    """GPU replacement of ConjugateGradientSolverCSR_Eisenstat_Rainbow (solver/sparsesolver.cpp:1338-1645)."""
    x = _vec(x, "x", N, True); residual = _vec(residual, "residual", N, True)
    csr = _csr(N, csrrows, csrcolumns, csrvalues)
    info = _native.FeecSolveInfo()
    st = _native.gpu().feec_cg_csr_eisenstat_rainbow(int(N), x, _vec(b, "b", N), *csr, residual,
                                                     float(precision), int(print_modulo),
                                                     _vec(diagonal, "diagonal", N), float(omega), int(num_colors),
                                                     *_coloring(N, num_colors, F, B, R), info)
    return _finish(st, info, "ConjugateGradientSolverCSR_Eisenstat_Rainbow")


def ConjugateGradientSolverCSR_DiagonalPreconditioner(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision,
                                                      print_modulo, precon):
    """GPU replacement of ConjugateGradientSolverCSR_DiagonalPreconditioner (solver/sparsesolver.cpp:221-416)."""
    x = _vec(x, "x", N, True); residual = _vec(residual, "residual", N, True)
    csr = _csr(N, csrrows, csrcolumns, csrvalues)
    info = _native.FeecSolveInfo()
    st = _native.gpu().feec_cg_csr_diagonal_precon(int(N), x, _vec(b, "b", N), *csr, residual,
                                                   float(precision), int(print_modulo), _vec(precon, "precon", N),
                                                   info)
    return _finish(st, info, "ConjugateGradientSolverCSR_DiagonalPreconditioner")


def _plain(fn, where, N, x, b, csrrows, csrcolumns, csrvalues, residual, precision, print_modulo):
    x = _vec(x, "x", N, True); residual = _vec(residual, "residual", N, True)
    csr = _csr(N, csrrows, csrcolumns, csrvalues)
    info = _native.FeecSolveInfo()
    st = fn(int(N), x, _vec(b, "b", N), *csr, residual,
            float(precision), int(print_modulo), info)
    return _finish(st, info, where)


def ConjugateResidualSolverCSR(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision, print_modulo=-3):
    """GPU replacement of ConjugateResidualSolverCSR (solver/sparsesolver.cpp:1687-1915)."""
    return _plain(_native.gpu().feec_cr_csr, "ConjugateResidualSolverCSR", N, x, b, csrrows, csrcolumns, csrvalues,
                  residual, precision, print_modulo)


def ConjugateResidualSolverCSR_textbook(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision,
                                        print_modulo=-3):
    """GPU replacement of ConjugateResidualSolverCSR_textbook (solver/sparsesolver.cpp:1918-2156)."""
    return _plain(_native.gpu().feec_cr_csr_textbook, "ConjugateResidualSolverCSR_textbook", N, x, b, csrrows,
                  csrcolumns, csrvalues, residual, precision, print_modulo)


def MINRESCSR(N, x, b, csrrows, csrcolumns, csrvalues, res, precision, print_modulo=-3):
    """GPU replacement of MINRESCSR (solver/sparsesolver.cpp:2159-2425)."""
    return _plain(_native.gpu().feec_minres_csr, "MINRESCSR", N, x, b, csrrows, csrcolumns, csrvalues, res,
                  precision, print_modulo)


def ChebyshevIteration_DiagonalPreconditioner(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision,
                                              print_modulo, precon, lower, upper):
    """GPU replacement of ChebyshevIteration_DiagonalPreconditioner (solver/sparsesolver.cpp:2428-2590)."""
    x = _vec(x, "x", N, True); residual = _vec(residual, "residual", N, True)
    csr = _csr(N, csrrows, csrcolumns, csrvalues)
    info = _native.FeecSolveInfo()
    st = _native.gpu().feec_chebyshev_diag(int(N), x, _vec(b, "b", N), *csr, residual, float(precision),
                                           int(print_modulo), _vec(precon, "precon", N), float(lower), float(upper),
                                           info)
    return _finish(st, info, "ChebyshevIteration_DiagonalPreconditioner")


def _hodge(entry, where, N, L, x, b, A, B, Bt, C, residual, precision, print_modulo, inner_precision,
           inner_print_modulo):
    x = _vec(x, "x", N, True); residual = _vec(residual, "residual", N, True)
    mats = []
    for name, rows, M in (("A", L, A), ("B", N, B), ("Bt", L, Bt), ("C", N, C)):
        mats += [*_csr(rows, *M, name=name)]
    info = _native.FeecSolveInfo()
    st = getattr(_native.gpu(), entry)(int(N), int(L), x, _vec(b, "b", N), *mats, residual, float(precision),
                                       int(print_modulo), float(inner_precision), int(inner_print_modulo), info)
    return _finish(st, info, where)


def HodgeConjugateResidualSolverCSR(N, L, x, b, A, B, Bt, C, residual, precision, print_modulo,
                                    inneriteration_precision, inneriteration_print_modulo=-3):
    """GPU replacement of HodgeConjugateResidualSolverCSR (solver/systemsparsesolver.cpp:18-50):
    conjugate residuals on B A^-1 Bt + C, inner SSOR-PCG. A, B, Bt, C are (rows, columns, values)."""
    return _hodge("feec_hodge_cr_csr", "HodgeConjugateResidualSolverCSR", N, L, x, b, A, B, Bt, C, residual,
                  precision, print_modulo, inneriteration_precision, inneriteration_print_modulo)


def HodgeConjugateResidualSolverCSR_diagonal(N, L, x, b, A, B, Bt, C, residual, precision, print_modulo,
                                             inneriteration_precision, inneriteration_print_modulo=-3):
    """GPU replacement of HodgeConjugateResidualSolverCSR_diagonal (systemsparsesolver.cpp:52-424)."""
    return _hodge("feec_hodge_cr_csr_diagonal", "HodgeConjugateResidualSolverCSR_diagonal", N, L, x, b, A, B, Bt, C,
                  residual, precision, print_modulo, inneriteration_precision, inneriteration_print_modulo)


def HodgeConjugateResidualSolverCSR_SSOR(N, L, x, b, A, B, Bt, C, residual, precision, print_modulo,
                                         inneriteration_precision, inneriteration_print_modulo=-3):
    """GPU replacement of HodgeConjugateResidualSolverCSR_SSOR (systemsparsesolver.cpp:426-796)."""
    return _hodge("feec_hodge_cr_csr_ssor", "HodgeConjugateResidualSolverCSR_SSOR", N, L, x, b, A, B, Bt, C,
                  residual, precision, print_modulo, inneriteration_precision, inneriteration_print_modulo)


def HodgeConjugateResidualSolverCSR_textbook(N, L, x, b, A, B, Bt, C, residual, precision, print_modulo,
                                             inneriteration_precision, inneriteration_print_modulo=-3):
    """GPU replacement of HodgeConjugateResidualSolverCSR_textbook (systemsparsesolver.cpp:798-1120)."""
    return _hodge("feec_hodge_cr_csr_textbook", "HodgeConjugateResidualSolverCSR_textbook", N, L, x, b, A, B, Bt, C,
                  residual, precision, print_modulo, inneriteration_precision, inneriteration_print_modulo)


def HodgeHerzogSoodhalterMethod(dimension_A, dimension_C, x_A, x_C, b_A, b_C, A, B, Bt, C, precision, print_modulo,
                                PA, PC, inneriteration_precision, inneriteration_print_modulo=-3):
    """GPU replacement of HodgeHerzogSoodhalterMethod (solver/systemsparsesolver.cpp:1122-1575):
    block-preconditioned MINRES on [[-A, Bt], [B, C]]. A, B, Bt, C (and PA, PC, or None) are
    (rows, columns, values) triples."""
    import ctypes
    dA, dC = int(dimension_A), int(dimension_C)
    x_A = _vec(x_A, "x_A", dA, True); x_C = _vec(x_C, "x_C", dC, True)
    mats = []
    for name, rows, M in (("A", dA, A), ("B", dC, B), ("Bt", dA, Bt), ("C", dC, C)):
        mats += [*_csr(rows, *M, name=name)]
    keep = []

    def opt(P, name, rows):
        if P is None:
            return [None, None, None]
        r, c, v = _csr(rows, *P, name=name)
        keep.extend([r, c, v])
        return [r.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), c.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                v.ctypes.data_as(ctypes.POINTER(ctypes.c_double))]
    info = _native.FeecSolveInfo()
    st = _native.gpu().feec_hodge_herzog_soodhalter(dA, dC, x_A, x_C, _vec(b_A, "b_A", dA), _vec(b_C, "b_C", dC),
                                                    *mats, float(precision), int(print_modulo), *opt(PA, "PA", dA),
                                                    *opt(PC, "PC", dC), float(inneriteration_precision),
                                                    int(inneriteration_print_modulo), info)
    return _finish(st, info, "HodgeHerzogSoodhalterMethod")
