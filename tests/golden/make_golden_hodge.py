"""Writes ``hodge.npz`` in this directory from the FEEC++ reference itself: the Hodge
conjugate residual solvers (solver/systemsparsesolver.cpp:18-1120), run by
``oracle/_ref/ref_harness`` on a system of the block structure they solve, conjugate
residuals on M = B A^-1 Bt + C:

* ``A``  (L x L): the reference's 2D P1 Lagrange stiffness + mass, refined 4 times (L = 289);
* ``C``  (N x N): the same refined 3 times, cell coefficients from seed 5 (N = 81);
* ``B``  (N x L): 6 entries per row, seeded columns and U[-1, 1] values;
* ``Bt`` (L x N): the reference's transpose of B (MatrixCSR::getTranspose);
* ``b``: seeded U[-1, 1].

Stored per variant ``diagonal``, ``ssor``, ``textbook`` and ``plain``
(HodgeConjugateResidualSolverCSR): ``<v>_K``, ``<v>_x``, ``<v>_res``, at precision 1e-10
with inner precision 1e-12, from x0 = 0, one OpenMP thread.

HodgeHerzogSoodhalterMethod (systemsparsesolver.cpp:1122-1575) on [[-A, Bt], [B, C]] with
right-hand sides ``hhs_bA`` (L), ``hhs_bC`` (N) (seeded U[-1, 1]), for the preconditioner
cases ``hhs_pp`` (PA = A, PC = C), ``hhs_pn`` (PA = A only) and ``hhs_nn`` (none):
``<case>_K``, ``<case>_xA``, ``<case>_xC`` (precision 1e-10, inner precision 1e-12).

Usage: python tests/golden/make_golden_hodge.py   (needs the reference sources; run once).
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
PRECISION, INNER = 1e-10, 1e-12


def run(*args):
    subprocess.run([HARNESS, *map(str, args)], check=True, capture_output=True,
                   env=dict(os.environ, OMP_NUM_THREADS="1"))


def main():
    if not os.path.exists(HARNESS):
        sys.exit("build the reference harness first: FEEC_REFERENCE_DIR=<reference sources> make -C oracle -f Makefile.ref")
    out = {}
    rng = np.random.default_rng(4242)
    with tempfile.TemporaryDirectory() as tmp:
        t = lambda name: os.path.join(tmp, name)  # noqa: E731
        run("assemble", 2, 1, 4, 0, t("a.csr"))
        run("assemble", 2, 1, 3, 5, t("c.csr"))
        A = csrio.read_csr(t("a.csr")); C = csrio.read_csr(t("c.csr"))
        A.pos = None; C.pos = None
        csrio.write_csr(t("a.csr"), A); csrio.write_csr(t("c.csr"), C)
        N, L = C.n, A.n
        cols = np.concatenate([np.sort(rng.choice(L, 6, replace=False)) for _ in range(N)]).astype(np.int32)
        B = csrio.CsrData(np.arange(0, 6 * N + 1, 6, dtype=np.int32), cols, rng.uniform(-1.0, 1.0, 6 * N), L)
        csrio.write_csr(t("b.csr"), B)
        run("csrtrans", t("b.csr"), t("bt.csr"))
        Bt = csrio.read_csr(t("bt.csr"))
        b = rng.uniform(-1.0, 1.0, N)
        csrio.write_vec(t("b.vec"), b)
        for key, m in (("A", A), ("B", B), ("Bt", Bt), ("C", C)):
            out[key + "_A"] = m.A; out[key + "_C"] = m.C; out[key + "_V"] = m.V
        out["b"] = b
        out["precision"] = np.float64(PRECISION); out["inner_precision"] = np.float64(INNER)
        for variant in ("diagonal", "ssor", "textbook", "plain"):
            run("hodge", variant, t("a.csr"), t("b.csr"), t("bt.csr"), t("c.csr"), t("b.vec"), repr(PRECISION),
                repr(INNER), t("s.sol"))
            K, x, res, _ = csrio.read_sol(t("s.sol"))
            out[f"{variant}_K"] = np.int64(K); out[f"{variant}_x"] = x; out[f"{variant}_res"] = res
            print(f"{variant}: N={N} L={L} K={K}")
        rng2 = np.random.default_rng(4343)
        bA = rng2.uniform(-1.0, 1.0, L); bC = rng2.uniform(-1.0, 1.0, N)
        csrio.write_vec(t("ba.vec"), bA); csrio.write_vec(t("bc.vec"), bC)
        out["hhs_bA"] = bA; out["hhs_bC"] = bC
        for case, pa, pc in (("hhs_pp", t("a.csr"), t("c.csr")), ("hhs_pn", t("a.csr"), "-"), ("hhs_nn", "-", "-")):
            run("hhs", t("a.csr"), t("b.csr"), t("bt.csr"), t("c.csr"), pa, pc, t("ba.vec"), t("bc.vec"),
                repr(PRECISION), repr(INNER), t("h.out"))
            with open(t("h.out"), "rb") as f:
                buf = f.read()
            dA, dC, K = (int(v) for v in np.frombuffer(buf, np.int64, 3, 0))
            out[case + "_K"] = np.int64(K)
            out[case + "_xA"] = np.frombuffer(buf, np.float64, dA, 24).copy()
            out[case + "_xC"] = np.frombuffer(buf, np.float64, dC, 24 + 8 * dA).copy()
            print(f"{case}: K={K}")
    np.savez_compressed(os.path.join(HERE, "hodge.npz"), **out)


if __name__ == "__main__":
    main()
