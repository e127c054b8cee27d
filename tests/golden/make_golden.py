"""Writes the golden fixtures in this directory from the FEEC++ reference itself.

Runs ``oracle/_ref/ref_harness`` (the unmodified reference modules linked with a small
driver, built by ``make -C oracle -f Makefile.ref`` with FEEC_REFERENCE_DIR naming the
reference sources) and stores, per case, one
compressed ``.npz`` holding:

* the matrix exactly as the reference assembles it (``A``, ``C``, ``V``; plus ``pos``,
  the position of every unknown, for the numbering-independent check of the package's
  lattice assembler), or the 5-point Laplacian of tests/solver/solvespd_csr.cpp:155-177;
* the right-hand side ``b`` (seeded U[-1,1], or ``A @ sol`` for the Laplacians);
* ``MatrixCSR::getDiagonal`` (``diag``) and ``MatrixCSR::apply`` of ``b`` with scaling
  0.7 (``apply_out``);
* ``Rainbow(A)``: ``rb_nc``, ``rb_F``, ``rb_B``, ``rb_R``;
* for each solver ``cg``, ``jac`` (diagonal preconditioner 1/diagonal), ``ssor``, ``rainbow``,
  ``eis`` (SSOR-Eisenstat), ``eisrb`` (Eisenstat-Rainbow), ``cr`` / ``crt``
  (ConjugateResidualSolverCSR and its _textbook twin), ``minres`` (MINRESCSR) and
  ``cheb`` (ChebyshevIteration_DiagonalPreconditioner with precon = 1/diagonal and the
  spectral bounds ``cheb_lower`` / ``cheb_upper`` of D^-1 A widened by 1 %, from a dense
  eigensolve) (and ``ssor13``/``rainbow13``/``eis13``/``eisrb13`` at
  omega = 1.3 where listed): the returned iteration count ``<s>_K``, the solution
  ``<s>_x`` and the residual array ``<s>_res`` written by the reference, at one
  OpenMP thread (the plain CG is only correct there).

Usage: python tests/golden/make_golden.py   (needs the reference sources; run once).
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from simplefem_gb300 import csrio  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
PRECISION = 1e-10

# name, (dim, r, L, coef_seed) or ("lap5", n), rhs seed, extra omegas
CASES = [
    ("lap5_n4", ("lap5", 4), 11, []),
    ("lap5_n8", ("lap5", 8), 12, []),
    ("lap5_n16", ("lap5", 16), 13, []),
    ("lap5_n32", ("lap5", 32), 14, []),
    ("fem2d_p1_l6", (2, 1, 6, 0), 2024, [1.3]),
    ("fem2d_p2_l4_coef", (2, 2, 4, 3), 77, []),
    ("fem2d_p3_l2_coef", (2, 3, 2, 7), 5, []),
    ("fem3d_p1_l3", (3, 1, 3, 0), 31, [1.3]),
    ("fem3d_p2_l2", (3, 2, 2, 0), 32, []),
    ("fem3d_p2_l3", (3, 2, 3, 0), 33, []),
    ("fem3d_p3_l1_coef", (3, 3, 1, 9), 34, []),
]


def run(*args):
    subprocess.run([HARNESS, *map(str, args)], check=True, capture_output=True,
                   env=dict(os.environ, OMP_NUM_THREADS="1"))


def lap5(n):
    """5-point Laplacian of tests/solver/solvespd_csr.cpp:155-177 (row e = x*n + y)."""
    h = 1.0 / (n + 1)
    h2 = h * h
    A = [0]; C = []; V = []
    for e in range(n * n):
        x, y = divmod(e, n)
        ent = [(e, 4.0 / h2)]
        if x != 0: ent.append(((x - 1) * n + y, -1.0 / h2))
        if x != n - 1: ent.append(((x + 1) * n + y, -1.0 / h2))
        if y != 0: ent.append((x * n + y - 1, -1.0 / h2))
        if y != n - 1: ent.append((x * n + y + 1, -1.0 / h2))
        ent.sort()
        C += [c for c, _ in ent]; V += [v for _, v in ent]
        A.append(len(C))
    return csrio.CsrData(np.array(A, np.int32), np.array(C, np.int32), np.array(V), n * n)


def spectral_bounds(m):
    """[0.99 lambda_min, 1.01 lambda_max] of D^-1 A (dense symmetric eigensolve of
    D^-1/2 A D^-1/2; every fixture has positive diagonal)."""
    M = np.zeros((m.n, m.n))
    rows = np.repeat(np.arange(m.n), np.diff(m.A))
    np.add.at(M, (rows, m.C), m.V)
    d = 1.0 / np.sqrt(np.diag(M))
    ev = np.linalg.eigvalsh(d[:, None] * M * d[None, :])
    return 0.99 * float(ev[0]), 1.01 * float(ev[-1])


def main():
    if not os.path.exists(HARNESS):
        sys.exit("build the reference harness first: FEEC_REFERENCE_DIR=<reference sources> make -C oracle -f Makefile.ref")
    with tempfile.TemporaryDirectory() as tmp:
        t = lambda name: os.path.join(tmp, name)  # noqa: E731
        for name, spec, seed, omegas in CASES:
            out = {}
            if spec[0] == "lap5":
                m = lap5(spec[1])
                csrio.write_csr(t("m.csr"), m)
                sol = np.random.default_rng(seed).uniform(-1.0, 1.0, m.n)
                sol /= np.linalg.norm(sol)
                csrio.write_vec(t("sol.vec"), sol)
                run("apply", t("m.csr"), t("sol.vec"), "1.0", t("b.vec"))
                b = csrio.read_vec(t("b.vec"), m.n)
                out["sol"] = sol
            else:
                run("assemble", *spec, t("m.csr"))
                m = csrio.read_csr(t("m.csr"))
                out["pos"] = m.pos
                out["lattice"] = np.array(spec, np.int64)
                b = np.random.default_rng(seed).uniform(-1.0, 1.0, m.n)
            out.update(A=m.A, C=m.C, V=m.V, b=b)
            csrio.write_vec(t("b.vec"), b)
            csrio.write_vec(t("x0.vec"), np.zeros(m.n))
            run("diag", t("m.csr"), t("d.vec"))
            out["diag"] = csrio.read_vec(t("d.vec"), m.n)
            run("apply", t("m.csr"), t("b.vec"), "0.7", t("y.vec"))
            out["apply_out"] = csrio.read_vec(t("y.vec"), m.n)
            run("rainbow", t("m.csr"), t("rb.rb"))
            nc, F, B, R = csrio.read_rainbow(t("rb.rb"))
            out.update(rb_nc=np.int64(nc), rb_F=F, rb_B=B, rb_R=R)
            solves = [("cg", "cg", 1.0), ("jac", "diag", 1.0), ("ssor", "ssor", 1.0), ("rainbow", "rainbow", 1.0),
                      ("eis", "eisenstat", 1.0), ("eisrb", "eisenstat_rainbow", 1.0)]
            for om in omegas:
                tag = str(om).replace(".", "")
                solves += [(f"ssor{tag}", "ssor", om), (f"rainbow{tag}", "rainbow", om),
                           (f"eis{tag}", "eisenstat", om), (f"eisrb{tag}", "eisenstat_rainbow", om)]
            solves += [("cr", "cr", 1.0), ("crt", "cr_textbook", 1.0), ("minres", "minres", 1.0)]
            lo, hi = spectral_bounds(m)
            out["cheb_lower"] = np.float64(lo); out["cheb_upper"] = np.float64(hi)
            solves += [("cheb", "chebyshev", f"{lo!r}:{hi!r}")]
            for key, kind, om in solves:
                run("solve", kind, t("m.csr"), t("b.vec"), t("x0.vec"), repr(PRECISION),
                    om if isinstance(om, str) else repr(om), t("s.sol"))
                K, x, res, _ = csrio.read_sol(t("s.sol"))
                out[f"{key}_K"] = np.int64(K); out[f"{key}_x"] = x; out[f"{key}_res"] = res
                out[f"{key}_omega"] = np.float64(1.0 if isinstance(om, str) else om)
            out["precision"] = np.float64(PRECISION)
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
            print(f"{name}: N={m.n} nnz={m.nnz} colors={nc} K(cg/ssor/rainbow/eis/eisrb)="
                  f"{out['cg_K']}/{out['ssor_K']}/{out['rainbow_K']}/{out['eis_K']}/{out['eisrb_K']}")


if __name__ == "__main__":
    main()
