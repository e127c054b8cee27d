"""Writes ``csr_algebra.npz`` in this directory from the FEEC++ reference itself: the CSR
algebra one step before the solver path (MatrixCSRAddition, MatrixCSRMultiplication,
MatrixCSR::getTranspose, and MatrixCSR(SparseMatrix), i.e. COO -> CSR), run by
``oracle/_ref/ref_harness`` on operators the reference assembles (2D P2 refined 4 times,
two cell coefficients).

Stored (prefix per case): inputs ``<case>_in*`` and the reference's output CSR
``<case>_A``, ``<case>_C``, ``<case>_V``.
* ``add``  : X + Y with s1 = 0.7, s2 = -1.3 (both 1089 x 1089);
* ``mul``  : X Y (1089 x 1089);
* ``mulr`` : X[:700] Y (rectangular, 700 x 1089);
* ``tr``   : transpose of X[:700] (1089 x 700);
* ``coo``  : COO -> CSR of X's entries, shuffled, a third of them split into two equal
  halves (the two halves sum to the entry exactly in either order) and 500 explicit
  zeros (the reference drops them).
* ``coomul``: SparseMatrixMultiplication (sparse/sparsematrix.cpp:609-722) of X[:700] and
  Y, both given as shuffled COO with split halves and explicit zeros; inputs
  ``coomul_l_{r,c,v}``, ``coomul_r_{r,c,v}``, output ``coomul_out_{r,c,v}`` (row-wise).

Usage: python tests/golden/make_golden_csr.py   (needs the reference sources; run once).
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


def run(*args):
    subprocess.run([HARNESS, *map(str, args)], check=True, capture_output=True,
                   env=dict(os.environ, OMP_NUM_THREADS="1"))


def first_rows(m, k):
    A = m.A[: k + 1].copy()
    return csrio.CsrData(A, m.C[: A[-1]].copy(), m.V[: A[-1]].copy(), m.ncols)


def main():
    if not os.path.exists(HARNESS):
        sys.exit("build the reference harness first: FEEC_REFERENCE_DIR=<reference sources> make -C oracle -f Makefile.ref")
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        t = lambda name: os.path.join(tmp, name)  # noqa: E731
        run("assemble", 2, 2, 4, 3, t("x.csr"))
        run("assemble", 2, 2, 4, 8, t("y.csr"))
        X = csrio.read_csr(t("x.csr")); Y = csrio.read_csr(t("y.csr"))
        X.pos = None; Y.pos = None
        csrio.write_csr(t("x.csr"), X); csrio.write_csr(t("y.csr"), Y)
        Xr = first_rows(X, 700)
        csrio.write_csr(t("xr.csr"), Xr)
        for key, m in (("X", X), ("Y", Y), ("Xr", Xr)):
            out[f"{key}_A"] = m.A; out[f"{key}_C"] = m.C; out[f"{key}_V"] = m.V; out[f"{key}_ncols"] = np.int64(m.ncols)

        def store(case, path):
            m = csrio.read_csr(path)
            out[f"{case}_A"] = m.A; out[f"{case}_C"] = m.C; out[f"{case}_V"] = m.V
            out[f"{case}_ncols"] = np.int64(m.ncols)
            print(f"{case}: {m.n} x {m.ncols}, nnz {m.nnz}")

        run("csradd", t("x.csr"), t("y.csr"), "0.7", "-1.3", t("o.csr")); store("add", t("o.csr"))
        run("csrmul", t("x.csr"), t("y.csr"), t("o.csr")); store("mul", t("o.csr"))
        run("csrmul", t("xr.csr"), t("y.csr"), t("o.csr")); store("mulr", t("o.csr"))
        run("csrtrans", t("xr.csr"), t("o.csr")); store("tr", t("o.csr"))

        rng = np.random.default_rng(2026)
        rows = np.repeat(np.arange(X.n, dtype=np.int32), np.diff(X.A))
        r, c, v = list(rows), list(X.C), list(X.V)
        split = rng.random(len(v)) < 1.0 / 3.0
        for i in np.nonzero(split)[0]:
            h = v[i] * 0.5
            v[i] = h
            r.append(rows[i]); c.append(X.C[i]); v.append(h)
        zr = rng.integers(0, X.n, 500); zc = rng.integers(0, X.n, 500)
        r += list(zr); c += list(zc); v += [0.0] * 500
        order = rng.permutation(len(r))
        r = np.array(r, np.int32)[order]; c = np.array(c, np.int32)[order]; v = np.array(v)[order]
        out["coo_in_r"] = r; out["coo_in_c"] = c; out["coo_in_v"] = v
        csrio.write_coo(t("m.coo"), X.n, X.n, r, c, v)
        run("coo2csr", t("m.coo"), t("o.csr")); store("coo", t("o.csr"))

        rng2 = np.random.default_rng(2027)

        def scrambled(m, zeros):
            rows_m = np.repeat(np.arange(m.n, dtype=np.int32), np.diff(m.A))
            rr, cc, vv = list(rows_m), list(m.C), list(m.V)
            for i in np.nonzero(rng2.random(len(vv)) < 0.25)[0]:
                h = vv[i] * 0.5
                vv[i] = h
                rr.append(rows_m[i]); cc.append(m.C[i]); vv.append(h)
            rr += list(rng2.integers(0, m.n, zeros)); cc += list(rng2.integers(0, m.ncols, zeros)); vv += [0.0] * zeros
            perm = rng2.permutation(len(rr))
            return np.array(rr, np.int32)[perm], np.array(cc, np.int32)[perm], np.array(vv)[perm]

        L_ = scrambled(Xr, 200)
        R_ = scrambled(Y, 300)
        csrio.write_coo(t("l.coo"), Xr.n, Xr.ncols, *L_)
        csrio.write_coo(t("r.coo"), Y.n, Y.ncols, *R_)
        for key, arrs in (("coomul_l", L_), ("coomul_r", R_)):
            out[key + "_r"], out[key + "_c"], out[key + "_v"] = arrs
        run("coomul", t("l.coo"), t("r.coo"), t("p.coo"))
        pr, pc, pv, prow, pcol = csrio.read_coo(t("p.coo"))
        out["coomul_out_r"] = pr; out["coomul_out_c"] = pc; out["coomul_out_v"] = pv
        out["coomul_shape"] = np.array([prow, pcol], np.int64)
        print(f"coomul: {prow} x {pcol}, {len(pr)} entries")
    np.savez_compressed(os.path.join(HERE, "csr_algebra.npz"), **out)


if __name__ == "__main__":
    main()
