"""GB300-native sparse-CSR Krylov path of FEEC++ (martinlicht/simplefem).

CSR SpMV, the ConjugateGradientSolverCSR drivers (plain, diagonal, SSOR, multicolor
"Rainbow" SSOR, and both with Eisenstat's trick), conjugate residuals, MINRES, the
diagonally preconditioned Chebyshev iteration, the CSR/COO algebra (sums, products,
transposes, COO -> CSR) and the Rainbow coloring, as hand-written sm_103a kernels behind
the C ABI of ``include/feec_gpu.h``. This package is the Python host side of that
ABI; it mirrors the reference's MatrixCSR / Rainbow / raw-pointer solver surface.
"""
from ._native import FeecError, FeecSolveInfo  # noqa: F401
from .solver import (ConjugateGradientSolverCSR, ConjugateGradientSolverCSR_DiagonalPreconditioner,  # noqa: F401
                     ConjugateGradientSolverCSR_Eisenstat_Rainbow, ConjugateGradientSolverCSR_Rainbow, ConjugateGradientSolverCSR_SSOR,
                     ConjugateGradientSolverCSR_SSOR_Eisenstat, ConjugateResidualSolverCSR,
                     ConjugateResidualSolverCSR_textbook, MINRESCSR, ChebyshevIteration_DiagonalPreconditioner,
                     HodgeConjugateResidualSolverCSR, HodgeConjugateResidualSolverCSR_diagonal,
                     HodgeConjugateResidualSolverCSR_SSOR, HodgeConjugateResidualSolverCSR_textbook,
                     HodgeHerzogSoodhalterMethod, last_info)
from .sparse import (FloatVector, MatrixCSR, MatrixCSRAddition, MatrixCSRMultiplication, Rainbow,  # noqa: F401
                     SparseMatrix, SparseMatrixMultiplication)

# Constants of base/base.hpp:121-131 (Float = double)
machine_epsilon = 2.220446049250313080847263336181640625e-16
desired_precision = 1.490116119384765625e-08

__all__ = ["MatrixCSR", "MatrixCSRAddition", "MatrixCSRMultiplication", "SparseMatrix", "SparseMatrixMultiplication", "Rainbow", "FloatVector", "ConjugateGradientSolverCSR",
           "ConjugateGradientSolverCSR_DiagonalPreconditioner", "ConjugateGradientSolverCSR_SSOR",
           "ConjugateGradientSolverCSR_Rainbow", "ConjugateGradientSolverCSR_SSOR_Eisenstat",
           "ConjugateGradientSolverCSR_Eisenstat_Rainbow", "ConjugateResidualSolverCSR",
           "ConjugateResidualSolverCSR_textbook", "MINRESCSR", "ChebyshevIteration_DiagonalPreconditioner",
           "HodgeConjugateResidualSolverCSR", "HodgeConjugateResidualSolverCSR_diagonal",
           "HodgeConjugateResidualSolverCSR_SSOR", "HodgeConjugateResidualSolverCSR_textbook",
           "HodgeHerzogSoodhalterMethod", "last_info", "FeecError", "machine_epsilon", "desired_precision"]
