"""CPU-only checks of the library boundary and the host-side parts of the path:
the C ABI loads and exports every symbol include/feec_gpu.h declares, the
drop-in shim exports the reference's mangled C++ names, the Rainbow coloring is
bit-identical to the reference's, CSR checks and argument validation behave like
the reference's asserts, and the lattice workload assembler reproduces the
reference's FEM matrices up to the numbering of unknowns."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_names, load_golden

HEADER = os.path.join(ROOT, "include", "feec_gpu.h")


def declared_symbols():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_ ]+\*?\s*\**\s*(feec_[a-z0-9_]+)\s*\(", src, re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ["feec_cg_csr", "feec_cg_csr_ssor", "feec_cg_csr_rainbow", "feec_csr_apply", "feec_rainbow",
              "feec_system_solve"]:
        assert s in syms


def test_library_exports_every_declared_symbol(built):
    from simplefem_gb300 import _native
    lib = _native.gpu()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_dropin_exports_reference_mangled_names(built):
    from simplefem_gb300 import build
    out = subprocess.run(["nm", "-D", "--defined-only", build.lib_path("libfeec_dropin.so")], capture_output=True,
                         text=True, check=True).stdout
    # C++ names of solver/sparsesolver.hpp:11-19, 33-43, 59-70 with Float = double
    for mangled in ["_Z26ConjugateGradientSolverCSRiPdPKdPKiS3_S1_S_di",
                    "_Z31ConjugateGradientSolverCSR_SSORiPdPKdPKiS3_S1_S_diS1_d",
                    "_Z34ConjugateGradientSolverCSR_RainbowiPdPKdPKiS3_S1_S_diS1_diS3_S3_S3_",
                    "_Z41ConjugateGradientSolverCSR_SSOR_EisenstatiPdPKdPKiS3_S1_S_diS1_d",
                    "_Z49ConjugateGradientSolverCSR_DiagonalPreconditioneriPdPKdPKiS3_S1_S_diS1_",
                    "_Z44ConjugateGradientSolverCSR_Eisenstat_RainbowiPdPKdPKiS3_S1_S_diS1_diS3_S3_S3_",
                    "_Z26ConjugateResidualSolverCSRiPdPKdPKiS3_S1_S_di",
                    "_Z35ConjugateResidualSolverCSR_textbookiPdPKdPKiS3_S1_S_di",
                    "_Z9MINRESCSRiPdPKdPKiS3_S1_S_di",
                    "_Z41ChebyshevIteration_DiagonalPreconditioneriPdPKdPKiS3_S1_S_diS1_dd",
                    "_Z31HodgeConjugateResidualSolverCSRiiPdPKdPKiS3_S1_S3_S3_S1_S3_S3_S1_S3_S3_S1_S_didi",
                    "_Z40HodgeConjugateResidualSolverCSR_diagonaliiPdPKdPKiS3_S1_S3_S3_S1_S3_S3_S1_S3_S3_S1_S_didi",
                    "_Z36HodgeConjugateResidualSolverCSR_SSORiiPdPKdPKiS3_S1_S3_S3_S1_S3_S3_S1_S3_S3_S1_S_didi",
                    "_Z40HodgeConjugateResidualSolverCSR_textbookiiPdPKdPKiS3_S1_S3_S3_S1_S3_S3_S1_S3_S3_S1_S_didi",
                    "_Z27HodgeHerzogSoodhalterMethodiiPdS_PKdS1_PKiS3_S1_S3_S3_S1_S3_S3_S1_S3_S3_S1_diS3_S3_S1_S3_S3_S1_di"]:
        assert mangled in out, mangled


REF_SOLVER_OBJECT = os.path.join(ROOT, "oracle", "_ref", "solver.o")


@pytest.mark.skipif(not os.path.exists(REF_SOLVER_OBJECT),
                    reason="the reference's own solver object is built only where its sources are mounted")
def test_dropin_exports_the_reference_objects_csr_solver_names(built):
    """Every CSR Krylov driver the reference's compiled solver module defines (its own
    object file, oracle/_ref/solver.o) is exported by the shim under the same symbol,
    and the shim exports nothing else of that family."""
    from simplefem_gb300 import build
    family = re.compile(r"(CSR|MINRES|Chebyshev|Hodge)")

    def defined(cmd):
        out = subprocess.run(cmd, capture_output=True, text=True, check=True).stdout
        return {ln.split()[-1] for ln in out.splitlines()
                if len(ln.split()) == 3 and ln.split()[1] == "T" and family.search(ln.split()[-1])}

    ref = defined(["nm", "--defined-only", REF_SOLVER_OBJECT])
    shim = defined(["nm", "-D", "--defined-only", build.lib_path("libfeec_dropin.so")])
    assert ref, "no CSR drivers found in the reference object"
    assert shim == ref, (sorted(ref - shim), sorted(shim - ref))


def test_shim_aborts_like_a_checked_build_when_no_gpu_is_usable(built, tmp_path):
    """A C++ caller linked against the shim alone: where no GPU is usable the C ABI
    returns FEEC_NO_DEVICE and the shim prints it and aborts (it never falls back to
    the CPU). On a GPU machine this runs the same driver's argument-check abort."""
    import torch
    from test_gpu_dropin_shim import build_driver, write_input
    g = load_golden("lap5_n8")
    exe = build_driver(tmp_path)
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    has_gpu = torch.cuda.is_available()
    write_input(inp, g, precision=-1.0 if has_gpu else None)
    res = subprocess.run([exe, inp, outp], capture_output=True, text=True, timeout=120)
    assert res.returncode == -6, (res.returncode, res.stderr)
    assert "ConjugateGradientSolverCSR:" in res.stderr


@pytest.mark.parametrize("name", golden_names())
def test_rainbow_bitexact_against_reference(built, name):
    from simplefem_gb300 import MatrixCSR, Rainbow
    g = load_golden(name)
    n = len(g["A"]) - 1
    rb = Rainbow(MatrixCSR(n, n, g["A"], g["C"], g["V"]))
    assert rb.num_colors == int(g["rb_nc"])
    assert np.array_equal(rb.F, g["rb_F"])
    assert np.array_equal(rb.B, g["rb_B"])
    assert np.array_equal(rb.R, g["rb_R"])


def test_rainbow_matches_oracle_on_large_lattice(built):
    from oracle import oracle
    from simplefem_gb300 import MatrixCSR, Rainbow, workloads
    A, C, V = workloads.lattice_matrix(3, 2, 4)
    n = len(A) - 1
    rb = Rainbow(MatrixCSR(n, n, A, C, V))
    nc, F, B, R = oracle.rainbow(A, C)
    assert rb.num_colors == nc and np.array_equal(rb.F, F) and np.array_equal(rb.B, B) and np.array_equal(rb.R, R)


def test_rainbow_edge_cases(built):
    from simplefem_gb300 import MatrixCSR, Rainbow
    # single row, diagonal only: one color
    rb = Rainbow(MatrixCSR(1, 1, [0, 1], [0], [2.0]))
    assert rb.num_colors == 1 and list(rb.R) == [0]
    # empty rows: every row gets color 0
    rb = Rainbow(MatrixCSR(3, 3, [0, 0, 0, 0], [], []))
    assert rb.num_colors == 1 and list(rb.R) == [2, 1, 0]
    # a path 0-1-2: unvisited neighbours block color 0
    A = [0, 2, 5, 7]; C = [0, 1, 0, 1, 2, 1, 2]; V = [2.0, -1, -1, 2, -1, -1, 2]
    rb = Rainbow(MatrixCSR(3, 3, A, C, V))
    assert list(rb.F) == [1, 2, 0] and rb.num_colors == 3


def test_csr_check_rejects_bad_arrays(built):
    from simplefem_gb300 import MatrixCSR
    with pytest.raises(ValueError):
        MatrixCSR(2, 2, [0, 2, 1], [0, 1], [1.0, 1.0])          # decreasing row pointer
    with pytest.raises(ValueError):
        MatrixCSR(2, 2, [0, 1, 2], [0, 2], [1.0, 1.0])          # column out of range
    with pytest.raises(ValueError):
        MatrixCSR(2, 2, [0, 1, 2], [0, 1], [1.0, np.nan])       # non-finite value
    with pytest.raises(ValueError):
        MatrixCSR(2, 2, [0, 1, 3], [0, 1], [1.0, 1.0])          # A[rows] beyond the stored entries


def test_solver_argument_checks_fail_like_asserts(built):
    """The reference asserts N > 0 and precision > 0 (sparsesolver.cpp:32-43)."""
    from simplefem_gb300 import ConjugateGradientSolverCSR, FeecError
    x = np.zeros(1); r = np.zeros(1)
    with pytest.raises(FeecError):
        ConjugateGradientSolverCSR(0, x, np.zeros(1), [0, 1], [0], [1.0], r, 1e-10, -3)
    with pytest.raises(FeecError):
        ConjugateGradientSolverCSR(1, x, np.zeros(1), [0, 1], [0], [1.0], r, 0.0, -3)


@pytest.mark.parametrize("name", [n for n in golden_names() if not n.startswith("lap5")])
def test_lattice_assembler_reproduces_reference_matrix(built, name):
    """Same operator as the reference's FEEC assembly, up to the numbering of unknowns:
    every entry (mapped through the degree-of-freedom positions) agrees to 1e-12 of its
    row's largest entry, and the sparsity patterns are identical."""
    from simplefem_gb300 import workloads
    g = load_golden(name)
    dim, r, L, seed = (int(v) for v in g["lattice"])
    A, C, V = workloads.lattice_matrix(dim, r, L, seed)
    assert len(A) == len(g["A"]) and len(C) == len(g["C"])
    m = r * 2 ** L + 1
    ip = np.rint(g["pos"] * (m - 1)).astype(np.int64)
    assert np.abs(g["pos"] * (m - 1) - ip).max() < 1e-9
    lidx = ip[:, 0] + m * ip[:, 1] + (m * m * ip[:, 2] if dim == 3 else 0)
    n = len(A) - 1
    assert np.array_equal(np.sort(lidx), np.arange(n))
    # reference entries mapped into lattice numbering, then compared row by row
    rrow = np.repeat(lidx, np.diff(g["A"]))
    rcol = lidx[g["C"]]
    order = np.lexsort((rcol, rrow))
    mrow = np.repeat(np.arange(n), np.diff(A))
    assert np.array_equal(rrow[order], mrow) and np.array_equal(rcol[order], C)
    rv = g["V"][order]
    rowmax = np.maximum.reduceat(np.abs(V), A[:-1])
    assert np.all(np.abs(rv - V) <= 1e-12 * rowmax[mrow])


def test_uniform_vector_reproducible(built):
    from simplefem_gb300 import workloads
    a = workloads.uniform_vector(7, 1000)
    b = workloads.uniform_vector(7, 1000)
    assert np.array_equal(a, b) and a.min() >= -1.0 and a.max() < 1.0 and abs(a.mean()) < 0.1


def test_algebra_and_solver_entry_points_check_arguments_on_the_host(built):
    """The CSR algebra, the COO product, CR/MINRES/Chebyshev and the Hodge solvers refuse
    invalid arguments on the host, before any device work (FEEC_BADARG without a GPU)."""
    from simplefem_gb300 import _native
    L = _native.gpu()
    BAD = _native.FEEC_BADARG
    A = np.array([0, 2, 3], np.int32); C = np.array([0, 1, 1], np.int32); V = np.ones(3)
    Cbad = np.array([0, 5, 1], np.int32); Abad = np.array([0, 3, 2], np.int32)
    oA = np.empty(8, np.int32); oC = np.empty(16, np.int32); oV = np.empty(16)
    nnz = ctypes.c_int(0); cnt = ctypes.c_longlong(0)
    assert L.feec_csr_add(2, 2, A, Cbad, V, A, C, V, 1.0, 1.0, oA, oC, oV, ctypes.byref(nnz)) == BAD
    assert L.feec_csr_add(2, 2, Abad, C, V, A, C, V, 1.0, 1.0, oA, oC, oV, ctypes.byref(nnz)) == BAD
    assert L.feec_csr_multiply(2, 2, 2, A, Cbad, V, A, C, V, oA, oC, oV, ctypes.byref(nnz)) == BAD
    assert L.feec_csr_transpose(2, 2, A, Cbad, V, oA, oC, oV, ctypes.byref(nnz)) == BAD
    r = np.array([0, 3], np.int32); c = np.array([0, 1], np.int32)
    assert L.feec_coo_to_csr(2, 2, 2, r, c, np.ones(2), oA, oC, oV, ctypes.byref(nnz)) == BAD
    assert L.feec_coo_multiply(2, 2, 2, 2, r, c, np.ones(2), 2, c, c, np.ones(2), oC, oC.copy(), oV,
                               ctypes.byref(cnt)) == BAD
    size = ctypes.c_longlong(0)
    assert L.feec_coo_multiply_size(2, 2, np.array([0, 1], np.int32), 2, np.array([0, 1], np.int32),
                                    ctypes.byref(size)) == _native.FEEC_OK and size.value == 2
    info = _native.FeecSolveInfo()
    x = np.zeros(2); res = np.zeros(2); b = np.ones(2)
    for fn in (L.feec_cr_csr, L.feec_cr_csr_textbook, L.feec_minres_csr):
        assert fn(0, x, b, A, C, V, res, 1e-10, -3, ctypes.byref(info)) == BAD          # N > 0 (:1699)
        assert fn(2, x, b, A, C, V, res, 0.0, -3, ctypes.byref(info)) == BAD            # precision > 0
    assert L.feec_chebyshev_diag(2, x, b, A, C, V, res, 0.0, -3, np.ones(2), 0.5, 2.0, ctypes.byref(info)) == BAD
    args = [2, 0, x, b] + [A, C, V] * 4 + [res, 1e-10, -3, 1e-12, -3, ctypes.byref(info)]
    for name in ("feec_hodge_cr_csr", "feec_hodge_cr_csr_diagonal", "feec_hodge_cr_csr_ssor",
                 "feec_hodge_cr_csr_textbook"):
        assert getattr(L, name)(*args) == BAD                                          # L > 0 (:76-77)
    assert L.feec_hodge_herzog_soodhalter(0, 2, x, x.copy(), b, b, *([A, C, V] * 4), 1e-10, -3,
                                          None, None, None, None, None, None, 1e-12, -3, ctypes.byref(info)) == BAD
    # the batch replay halves refuse a missing batch before touching the device
    ms = ctypes.c_double(0.0)
    assert L.feec_batch_launch(None) == BAD
    assert L.feec_batch_finish(None, ctypes.byref(info), ctypes.byref(ms)) == BAD
    assert L.feec_batch_run(None, ctypes.byref(info), ctypes.byref(ms)) == BAD


def test_python_surface_checks_shapes(built):
    from simplefem_gb300 import MatrixCSR, MatrixCSRAddition, MatrixCSRMultiplication, SparseMatrix
    with pytest.raises(ValueError):
        SparseMatrix(2, 2, [0, 1], [0], [1.0])
    X = MatrixCSR(2, 3, [0, 1, 2], [0, 2], [1.0, 2.0])
    Y = MatrixCSR(2, 2, [0, 1, 2], [0, 1], [1.0, 2.0])
    with pytest.raises(ValueError):
        MatrixCSRAddition(X, Y)
    with pytest.raises(ValueError):
        MatrixCSRMultiplication(X, Y)


def test_public_header_compiles_as_c_and_cpp():
    """include/feec_gpu.h is plain C (the boundary a cgo / FFI / C caller includes)."""
    import shutil
    header = os.path.join(ROOT, "include", "feec_gpu.h")
    if shutil.which("gcc"):
        subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only", "-x", "c",
                        header], check=True)
    if shutil.which("g++"):
        subprocess.run(["g++", "-std=c++14", "-Wall", "-Werror", "-fsyntax-only", "-x", "c++", header], check=True)


def test_device_arrays_are_checked_before_the_library():
    """The System / Batch / solve_many mirror refuses host tensors, wrong dtypes, wrong
    shapes and non-contiguous views with a ValueError before any pointer reaches a kernel."""
    torch = pytest.importorskip("torch")
    from simplefem_gb300.system import _device_array, _system_vectors
    with pytest.raises(ValueError, match="dtype"):
        _device_array(torch.zeros(4, dtype=torch.float32), "x", (4,))
    with pytest.raises(ValueError, match="ndarray, expected a CUDA tensor"):
        _device_array(np.zeros(4), "x", (4,))
    with pytest.raises(ValueError, match="shape"):
        _device_array(torch.zeros(5, dtype=torch.float64), "x", (4,))
    with pytest.raises(ValueError, match="shape"):
        _device_array(torch.zeros((4, 3), dtype=torch.float64), "B", (3, 4))
    with pytest.raises(ValueError, match="contiguous"):
        _device_array(torch.zeros((4, 3), dtype=torch.float64).t(), "B", (3, 4))
    with pytest.raises(ValueError, match="CUDA"):
        _device_array(torch.zeros(4, dtype=torch.float64), "x", (4,))

    class _Sys:
        n, _h = 4, None
    with pytest.raises(ValueError, match="one each"):
        _system_vectors([_Sys(), _Sys()], [torch.zeros(4, dtype=torch.float64)] * 2, [])
    with pytest.raises(ValueError, match=r"xs\[0\]: shape"):
        _system_vectors([_Sys(), _Sys()], [torch.zeros(4, dtype=torch.float64)] * 2,
                        [torch.zeros(3, dtype=torch.float64), torch.zeros(4, dtype=torch.float64)])


def test_raw_pointer_mirror_checks_array_lengths(built):
    """The raw-pointer drivers read N + 1 row pointers, A[N] columns and values, and the
    Rainbow arrays through their pointers: NumPy arrays shorter than that are a ValueError
    in the Python mirror (the library would read past them on the host)."""
    import simplefem_gb300 as S
    n = 3
    A = np.array([0, 1, 2, 3], np.int32); C = np.array([0, 1, 2], np.int32); V = np.ones(3)
    x, r, b = np.zeros(n), np.zeros(n), np.ones(n)
    with pytest.raises(ValueError, match="columns has 2 entries, expected 3"):
        S.ConjugateGradientSolverCSR(n, x, b, A, C[:2], V, r, 1e-10, -3)
    with pytest.raises(ValueError, match="values has 2 entries, expected 3"):
        S.MINRESCSR(n, x, b, A, C, V[:2], r, 1e-10, -3)
    with pytest.raises(ValueError, match="x must be one-dimensional"):
        S.ConjugateGradientSolverCSR(n, np.zeros((n, 1)), b, A, C, V, r, 1e-10, -3)
    with pytest.raises(ValueError, match="rows has 3 entries, expected 4"):
        S.ConjugateResidualSolverCSR(n, x, b, A[:3], C, V, r, 1e-10, -3)
    with pytest.raises(ValueError, match="R has 2 entries, expected 3"):
        S.ConjugateGradientSolverCSR_Rainbow(n, x, b, A, C, V, r, 1e-10, -3, np.ones(n), 1.0, 1,
                                             np.zeros(n, np.int32), np.array([0, 3], np.int32),
                                             np.array([2, 1], np.int32))
    with pytest.raises(ValueError, match="B has 1 entries, expected 2"):
        S.ConjugateGradientSolverCSR_Eisenstat_Rainbow(n, x, b, A, C, V, r, 1e-10, -3, np.ones(n), 1.0, 1,
                                                       np.zeros(n, np.int32), np.array([0], np.int32),
                                                       np.array([2, 1, 0], np.int32))
    # Hodge: B has N rows, Bt has L rows
    L = 2
    Ah = (np.array([0, 1, 2], np.int32), np.array([0, 1], np.int32), np.ones(2))
    Bh = (np.array([0, 1, 2, 3], np.int32), np.array([0, 1, 0], np.int32), np.ones(3))
    Bth = (np.array([0, 2, 3], np.int32), np.array([0, 2, 1], np.int32), np.ones(3))
    with pytest.raises(ValueError, match="Btrows has 2 entries, expected 3"):
        S.HodgeConjugateResidualSolverCSR_diagonal(n, L, x, b, Ah, Bh, (Bth[0][:2], Bth[1], Bth[2]), (A, C, V), r,
                                                   1e-10, -3, 1e-12)
    with pytest.raises(ValueError, match="Bcolumns has 2 entries, expected 3"):
        S.HodgeConjugateResidualSolverCSR_textbook(n, L, x, b, Ah, (Bh[0], Bh[1][:2], Bh[2]), Bth, (A, C, V), r,
                                                   1e-10, -3, 1e-12)
    with pytest.raises(ValueError, match="PArows has 2 entries, expected 3"):
        S.HodgeHerzogSoodhalterMethod(L, n, np.zeros(L), np.zeros(n), np.ones(L), b, Ah, Bh, Bth, (A, C, V),
                                      1e-10, -3, (Ah[0][:2], Ah[1], Ah[2]), None, 1e-12)


def test_server_submit_checks_arrays_before_queueing(built):
    """A request's CSR arrays and right-hand side are read later by a worker thread: arrays
    shorter than the row pointers say are refused at submit with a ValueError."""
    from simplefem_gb300.serving import Server
    srv = object.__new__(Server)                       # no device here: only the host checks run
    A = np.array([0, 1, 2], np.int32); C = np.array([0, 1], np.int32); V = np.ones(2)
    with pytest.raises(ValueError, match="at least one row"):
        srv.submit(np.array([0], np.int32), C[:0], V[:0], np.ones(0))
    with pytest.raises(ValueError, match="columns has 1 entries, expected 2"):
        srv.submit(A, C[:1], V, np.ones(2))
    with pytest.raises(ValueError, match="b has 1 entries, expected 2"):
        srv.submit(A, C, V, np.ones(1))
