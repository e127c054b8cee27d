"""The drop-in shim (libfeec_dropin.so) driven the way a FEEC++ program drives the
reference: tests/dropin_driver.cpp declares ConjugateGradientSolverCSR, _SSOR and
_Rainbow exactly as solver/sparsesolver.hpp:11-70 does, links against the shim alone,
and calls them on the golden fixtures. K and x must match the reference's own outputs
(cg_K/cg_x, ssor_K/ssor_x, rainbow_K/rainbow_x) at the drop-in parity bar: K within 2%
(at least +-1) and the solution as close to the reference's as the reference's own
solution is to the exact one (never looser than 1e-9 relative).
"""
import os
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

from conftest import ROOT, load_golden

DRIVER_SRC = os.path.join(ROOT, "tests", "dropin_driver.cpp")


def build_driver(tmpdir):
    from simplefem_gb300 import build
    exe = os.path.join(str(tmpdir), "dropin_driver")
    libdir = os.path.dirname(build.lib_path("libfeec_dropin.so"))
    subprocess.run(["g++", "-O2", "-std=c++14", DRIVER_SRC, "-o", exe, "-L" + libdir, "-lfeec_dropin",
                    "-Wl,-rpath," + libdir], check=True, capture_output=True, text=True)
    return exe


def write_input(path, g, precision=None, print_modulo=-3):
    n = len(g["A"]) - 1
    nnz = len(g["C"])
    nc = int(g["rb_nc"])
    prec = float(g["precision"]) if precision is None else precision
    with open(path, "wb") as f:
        np.array([n, nnz, nc, print_modulo], np.int32).tofile(f)
        np.array([prec, float(g["rainbow_omega"])], np.float64).tofile(f)
        for arr, dt in ((g["A"], np.int32), (g["C"], np.int32), (g["V"], np.float64), (g["b"], np.float64),
                        (g["diag"], np.float64), (g["rb_F"], np.int32), (g["rb_B"], np.int32), (g["rb_R"], np.int32)):
            np.ascontiguousarray(arr, dt).tofile(f)


def read_output(path, n):
    raw = open(path, "rb").read()
    out, off = [], 0
    for _ in range(3):
        K = int(np.frombuffer(raw, np.int32, 1, off)[0]); off += 4
        x = np.frombuffer(raw, np.float64, n, off).copy(); off += 8 * n
        r = np.frombuffer(raw, np.float64, n, off).copy(); off += 8 * n
        out.append((K, x, r))
    assert off == len(raw)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["fem2d_p1_l6", "fem3d_p2_l3", "lap5_n32", "fem2d_p2_l4_coef"])
def test_reference_caller_through_shim_matches_reference(cuda, tmp_path, name):
    g = load_golden(name)
    n = len(g["A"]) - 1
    assert float(g["ssor_omega"]) == float(g["rainbow_omega"])
    exe = build_driver(tmp_path)
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_input(inp, g)
    res = subprocess.run([exe, inp, outp], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    M = sp.csr_matrix((g["V"], g["C"], g["A"]), shape=(n, n))
    xs = sla.spsolve(M.tocsc(), g["b"])
    for key, (K, x, r) in zip(("cg", "ssor", "rainbow"), read_output(outp, n)):
        K_ref = int(g[key + "_K"])
        assert abs(K - K_ref) <= max(1, int(np.ceil(0.02 * K_ref))), (key, K, K_ref)
        x_ref = g[key + "_x"]
        own_err = np.linalg.norm(x_ref - xs) / np.linalg.norm(xs)
        diff = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
        assert diff <= max(1e-9, 2.0 * own_err), (key, diff, own_err)
        # the residual array is the recursive residual of x
        assert np.linalg.norm(r - (g["b"] - M @ x)) <= 1e-6 * np.linalg.norm(g["b"]) + 1e-12, key


@pytest.mark.gpu
def test_shim_aborts_on_rejected_argument_like_a_checked_build(cuda, tmp_path):
    """precision <= 0 is an assert in the reference (sparsesolver.cpp:43): the shim prints
    the status and aborts, as a checked reference build does. Host-side check only."""
    g = load_golden("lap5_n8")
    exe = build_driver(tmp_path)
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_input(inp, g, precision=-1.0)
    res = subprocess.run([exe, inp, outp], capture_output=True, text=True, timeout=120)
    assert res.returncode < 0 and res.returncode == -6, (res.returncode, res.stderr)
    assert "ConjugateGradientSolverCSR:" in res.stderr
